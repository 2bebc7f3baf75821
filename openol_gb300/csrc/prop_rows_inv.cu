// prop_rows_inv.cu -- dispatch of pass 3 (inverse row FFTs) of the fused
// propagation over the power-of-two lengths and launch variants.
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

int rows_inv_pass_pow2(const PropParams &P, cudaStream_t st) { OLG_SIZE_SWITCH(P.NX, launch_rows_inv, P, st) }

} // namespace olg
