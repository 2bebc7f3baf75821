// prop_aux.cu -- the per-axis chirp-spectrum kernels (Fresnel / ARSS set-up)
// and the fused seed row pass of the phase optimiser, dispatched over the
// power-of-two lengths.
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

int chirp_axis_pow2(const ChirpAxis &A, cudaStream_t st) { OLG_SIZE_SWITCH(A.L, launch_chirp, A, st) }

// forward pass 3 (OP_SEED) and adjoint pass 1 of one plane, fused; padded
// widths 256..8192 (the first and last radix-16 stages need N >= 256)
int rows_seed_pass(const PropParams &P, cudaStream_t st)
{
    switch (P.NX) {
    case 256: return launch_rows_seed<256>(P, st);
    case 512: return launch_rows_seed<512>(P, st);
    case 1024: return launch_rows_seed<1024>(P, st);
    case 2048: return launch_rows_seed<2048>(P, st);
    case 4096: return launch_rows_seed<4096>(P, st);
    case 8192: return launch_rows_seed<8192>(P, st);
    default: return fail(OLG_ERR_UNSUPPORTED_SIZE, "fused seed pass: padded width 256..8192");
    }
}

} // namespace olg
