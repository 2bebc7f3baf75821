// prop_cols.cu -- dispatch of pass 2 (column FFT, transfer function,
// inverse column FFT) of the fused propagation over the power-of-two lengths
// and launch variants.
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

int cols_pass_pow2(const PropParams &P, cudaStream_t st) { OLG_SIZE_SWITCH(P.NY, launch_cols, P, st) }

} // namespace olg
