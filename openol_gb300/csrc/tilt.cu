// tilt.cu -- the column FFTs of tilted-plane propagation for power-of-two
// padded heights, on the tuned column-tile FFT (fft.cuh / fft2.cuh): a
// zero-pruned first radix-16 stage straight from global memory, the
// shared-memory middle stages, and a register-resident last stage.
//   k_tilt_cols_fwd2  ny stored row spectra (D rows 0..ny-1) -> centred full
//                     spectrum C, x 1/N (x the unrotated transfer function,
//                     reference form)
//   k_tilt_cols_inv2  resampled spectrum D (natural order) -> inverse column
//                     FFTs, central ny rows x 1/N back into D's first rows
// Heights 256..8192 (the first and last radix-16 stages need N >= 256);
// other heights take the mixed-radix kernels in propmr.cu.
#include "common.cuh"
#include "fft.cuh"
#include "fft2.cuh"
#include "propmr.cuh"

namespace olg {

// from N = 2048: 1024 threads over C = 16384 / N columns per CTA (one
// butterfly per thread; one CTA per SM); below: 512 threads, C = 8192 / N
template <int N>
struct TiltCol {
    static constexpr bool BIG = N >= 2048;
    static constexpr int NT = BIG ? 1024 : 512, C = (BIG ? 16384 : 8192) / N, B = N / 16, BPT = C * B / NT;
    static constexpr int SMEM = padded_len(N) * C * (int)sizeof(float2);
    static_assert((C * B) % NT == 0, "threads must divide the butterflies");
};

template <int N>
__global__ void __launch_bounds__(TiltCol<N>::NT) k_tilt_cols_fwd2(TiltArgs T, const float2 *__restrict__ tw)
{
    using S = TiltCol<N>;
    constexpr int B = S::B, C = S::C, NT = S::NT;
    extern __shared__ float2 sm[];
    const int NX = T.NX, c0 = blockIdx.x * C, tid = threadIdx.x;
#pragma unroll
    for (int t = 0; t < S::BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 4; r < 12; ++r)
            v[r] = kx < NX ? T.D[(size_t)(j + (r - 4) * B) * NX + kx] : make_float2(0.f, 0.f);
        dft16_in_mid<-1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[17 * C * j + c + k * C] = v[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, -1, NT, true, C>(sm, 0, tw, tid);
#pragma unroll
    for (int t = 0; t < S::BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[pidx(j) * C + c + r * (pstride<B>() * C)];
        last_twiddle<N, -1>(v, j, tw);
        dft<16, -1>(v);
        if (kx >= NX) continue;
        const int m = kx < NX / 2 ? kx + NX / 2 : kx - NX / 2;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int ky = j + k * B;
            float2 x = cscale(v[outpos<16>(k)], T.invN);
            if (T.reference) x = cmul(x, tf_at(T.tf, ky, kx, N));
            const int n = ky < N / 2 ? ky + N / 2 : ky - N / 2;
            T.C[(size_t)n * NX + m] = x;
        }
    }
}

template <int N>
__global__ void __launch_bounds__(TiltCol<N>::NT) k_tilt_cols_inv2(TiltArgs T, const float2 *__restrict__ tw)
{
    using S = TiltCol<N>;
    constexpr int B = S::B, C = S::C, NT = S::NT;
    extern __shared__ float2 sm[];
    const int NX = T.NX, c0 = blockIdx.x * C, tid = threadIdx.x;
#pragma unroll
    for (int t = 0; t < S::BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r)
            v[r] = kx < NX ? T.D[(size_t)(j + r * B) * NX + kx] : make_float2(0.f, 0.f);
        dft<16, +1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[17 * C * j + c + k * C] = v[outpos<16>(k)];
    }
    // every column of this tile is now in shared memory: the writes below go
    // back into the same columns of D
    __syncthreads();
    mid_stages<N, +1, NT, true, C>(sm, 0, tw, tid);
#pragma unroll
    for (int t = 0; t < S::BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[pidx(j) * C + c + r * (pstride<B>() * C)];
        last_twiddle<N, +1>(v, j, tw);
        dft16_out_mid<+1>(v);
        if (kx >= NX) continue;
#pragma unroll
        for (int k = 4; k < 12; ++k) T.D[(size_t)(j + (k - 4) * B) * NX + kx] = cscale(v[outpos<16>(k)], T.invN);
    }
}

namespace {

template <int N>
int launch_tilt_cols(const TiltArgs &T, bool inverse, const float2 *tw, cudaStream_t st)
{
    using S = TiltCol<N>;
    auto kern = inverse ? k_tilt_cols_inv2<N> : k_tilt_cols_fwd2<N>;
    if (S::SMEM > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    }
    kern<<<(T.NX + S::C - 1) / S::C, S::NT, S::SMEM, st>>>(T, tw);
    count_launch();
    return check_launch(inverse ? "k_tilt_cols_inv2" : "k_tilt_cols_fwd2");
}

} // namespace

int tilt_cols_pow2(const TiltArgs &T, bool inverse, cudaStream_t st)
{
    const float2 *tw = twiddle_table();
    if (!tw) return fail(OLG_ERR_CUDA, "twiddle table unavailable");
    switch (T.NY) {
    case 256: return launch_tilt_cols<256>(T, inverse, tw, st);
    case 512: return launch_tilt_cols<512>(T, inverse, tw, st);
    case 1024: return launch_tilt_cols<1024>(T, inverse, tw, st);
    case 2048: return launch_tilt_cols<2048>(T, inverse, tw, st);
    case 4096: return launch_tilt_cols<4096>(T, inverse, tw, st);
    case 8192: return launch_tilt_cols<8192>(T, inverse, tw, st);
    default: return fail(OLG_ERR_UNSUPPORTED_SIZE, "power-of-two column length out of range");
    }
}

} // namespace olg
