// prop_rows_fwd.cu -- dispatch of pass 1 (forward row FFTs) of the fused
// propagation over the power-of-two lengths and launch variants; the
// instantiations live here so that they compile in parallel with the others.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "propk.cuh"

namespace olg {

int rows_fwd_pass_pow2(const PropParams &P, cudaStream_t st) { OLG_SIZE_SWITCH(P.NX, launch_rows_fwd, P, st) }

} // namespace olg
