// fft2.cuh -- register-resident end stages for the propagation passes.
//
// For N = 16 * M * 16 (M in {1, 2, 4, 8, 16, 32}: N = 256 .. 8192) the
// Stockham FFT is split as
//   first stage : radix 16, Ns = 1     -- inputs j + r N/16 read straight from
//                 global memory (or registers); half of them are the zero
//                 padding and are skipped (dft16_in_mid)
//   middle      : radix-M stage(s) in shared memory (fft.cuh fft_stage)
//   last stage  : radix 16, Ns = N/16  -- outputs j + k N/16 written straight
//                 to global memory; for a crop only k in [4, 12) is formed
//                 (dft16_out_mid)
// The first stage's inputs and the last stage's outputs of butterfly j are
// the same index set {j + r N/16}, so a forward last stage can feed an
// inverse first stage in registers (the column pass multiplies by the
// transfer function in between and never touches shared memory there).
#pragma once
#include "fft.cuh"

namespace olg {

// radix-16 DFT with inputs only at r in [4, 12) (the rest zero)
template <int DIR>
__device__ __forceinline__ void dft16_in_mid(float2 (&v)[16])
{
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
        const float2 a = v[n2 + 4], b = v[n2 + 8];
        const float2 ia = mul_di<DIR>(a);
        v[n2] = cadd(a, b);
        v[n2 + 4] = csub(ia, b);
        v[n2 + 8] = csub(b, a);
        v[n2 + 12] = make_float2(-b.x - ia.x, -b.y - ia.y);
    }
    v[5] = w16<DIR, 1>(v[5]);
    v[9] = w16<DIR, 2>(v[9]);
    v[13] = w16<DIR, 3>(v[13]);
    v[6] = w16<DIR, 2>(v[6]);
    v[10] = w16<DIR, 4>(v[10]);
    v[14] = w16<DIR, 6>(v[14]);
    v[7] = w16<DIR, 3>(v[7]);
    v[11] = w16<DIR, 6>(v[11]);
    v[15] = w16<DIR, 9>(v[15]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4<DIR>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
}

// radix-16 DFT forming only the outputs k in [4, 12): X[k] left at v[outpos<16>(k)]
// (outputs k = k1 + 4 k2 with k2 in {1, 2}); the other entries are garbage.
template <int DIR>
__device__ __forceinline__ void dft16_out_mid(float2 (&v)[16])
{
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4<DIR>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
    v[5] = w16<DIR, 1>(v[5]);
    v[9] = w16<DIR, 2>(v[9]);
    v[13] = w16<DIR, 3>(v[13]);
    v[6] = w16<DIR, 2>(v[6]);
    v[10] = w16<DIR, 4>(v[10]);
    v[14] = w16<DIR, 6>(v[14]);
    v[7] = w16<DIR, 3>(v[7]);
    v[11] = w16<DIR, 6>(v[11]);
    v[15] = w16<DIR, 9>(v[15]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        // DFT4 over n2 of (v[4k1], ..., v[4k1+3]) evaluated at k2 = 1 and 2 only
        const float2 a = v[4 * k1], b = v[4 * k1 + 1], c = v[4 * k1 + 2], d = v[4 * k1 + 3];
        const float2 s02 = cadd(a, c), d02 = csub(a, c), s13 = cadd(b, d), d13 = mul_di<DIR>(csub(b, d));
        v[4 * k1 + 1] = cadd(d02, d13);
        v[4 * k1 + 2] = csub(s02, s13);
    }
}

// Twiddle for the last stage (Ns = N/16): exp(DIR 2 pi i r j / N)
template <int N, int DIR>
__device__ __forceinline__ void last_twiddle(float2 (&v)[16], int j, const float2 *__restrict__ tw)
{
    constexpr int STEP = FFT_MAX / N;
    twiddle_powers<16, DIR>(v, tw, j * STEP);
}

// Middle stages: Stockham from Ns = 16 up to Ns = N/16 (none when N == 256).
template <int N, int NS, int DIR, int NT, bool COLS, int NSEQ>
struct MidRun {
    static __device__ __forceinline__ void run(float2 *s, int ss, const float2 *__restrict__ tw, int tid)
    {
        constexpr int REM = N / 16 / NS; // radix product still to apply before the last stage
        constexpr int R = REM >= 16 ? 16 : REM;
        fft_stage<N, R, NS, DIR, NT, COLS, NSEQ>(s, ss, tw, tid);
        MidRun<N, NS * R, DIR, NT, COLS, NSEQ>::run(s, ss, tw, tid);
    }
};
template <int N, int DIR, int NT, bool COLS, int NSEQ>
struct MidRun<N, N / 16, DIR, NT, COLS, NSEQ> {
    static __device__ __forceinline__ void run(float2 *, int, const float2 *__restrict__, int) {}
};

template <int N, int DIR, int NT, bool COLS, int NSEQ>
__device__ __forceinline__ void mid_stages(float2 *s, int ss, const float2 *__restrict__ tw, int tid)
{
    if constexpr (N > 256) MidRun<N, 16, DIR, NT, COLS, NSEQ>::run(s, ss, tw, tid);
}

} // namespace olg
