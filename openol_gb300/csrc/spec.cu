// spec.cu -- column FFTs between a half-padded row spectrum S (the ny stored
// rows x NX, as pass 1 leaves it) and a full padded spectrum F (NY x NX),
// for power-of-two heights 256..8192, on the tuned column-tile
// FFT (zero-pruned first stage from global memory, shared-memory middle
// stages, register-resident last stage):
//   spec_cols forward  F  = FFT_col(S)  [x T(ky, kx)]  [+ F]
//   spec_cols inverse  S' = central ny rows of IFFT_col(F [x T(ky, kx)])
// with T the propagation's transfer function (tf_at: ASM phase in registers,
// its 1/Np and, for the adjoint, its conjugate).  The multi-plane phase
// gradient uses them to share one forward spectrum across the planes and to
// sum the planes' adjoints in the spectral domain.
//
// F is private to these kernels and is stored by column tiles: tile
// t = kx / C holds rows ky = 0..NY-1 of its C columns contiguously
// (F[t NY C + ky C + kx % C]), so that every CTA reads and writes one
// contiguous block.
#include "common.cuh"
#include "fft.cuh"
#include "fft2.cuh"
#include "propmr.cuh"

namespace olg {

// Launch shape: from N = 2048, one 1024-thread CTA per SM over 16384
// elements (one butterfly per thread; 139 KB of shared memory), which took
// the 2048^2 phase-gradient step from 2.48 to 2.38 ms against two 512-thread
// CTAs of 8192 elements; below, the latter.
template <int N>
struct SpecCol {
    static constexpr bool BIG = N >= 2048;
    static constexpr int NT = BIG ? 1024 : 512, MINB = BIG ? 1 : 2;
    static constexpr int C = (BIG ? 16384 : 8192) / N, B = N / 16, BPT = C * B / NT;
    static constexpr int SMEM = padded_len(N) * C * (int)sizeof(float2);
    static_assert((C * B) % NT == 0, "threads must divide the butterflies");
};

template <int N>
__global__ void __launch_bounds__(SpecCol<N>::NT, SpecCol<N>::MINB) k_spec_cols_fwd(SpecArgs A, const float2 *__restrict__ tw)
{
    using S = SpecCol<N>;
    constexpr int B = S::B, C = S::C, NT = S::NT;
    extern __shared__ float2 sm[];
    const int NX = A.NX, c0 = blockIdx.x * C, tid = threadIdx.x;
#pragma unroll
    for (int t = 0; t < S::BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 4; r < 12; ++r)
            v[r] = kx < NX ? __ldcg(A.in + (size_t)(j + (r - 4) * B) * NX + kx) : make_float2(0.f, 0.f);
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
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const int ky = j + k * B;
            float2 x = v[outpos<16>(k)];
            if (A.tf) x = cmul(x, tf_at(A.P, ky, kx, N));
            float2 *o = A.out + (size_t)blockIdx.x * N * C + (size_t)ky * C + c;
            if (A.accumulate) {
                const float2 y = __ldcg(o);
                x.x += y.x;
                x.y += y.y;
            }
            __stcg(o, x);
        }
    }
}

template <int N>
__global__ void __launch_bounds__(SpecCol<N>::NT, SpecCol<N>::MINB) k_spec_cols_inv(SpecArgs A, const float2 *__restrict__ tw)
{
    using S = SpecCol<N>;
    constexpr int B = S::B, C = S::C, NT = S::NT;
    extern __shared__ float2 sm[];
    const int NX = A.NX, c0 = blockIdx.x * C, tid = threadIdx.x;
#pragma unroll
    for (int t = 0; t < S::BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            float2 x = make_float2(0.f, 0.f);
            if (kx < NX) {
                x = __ldcg(A.in + (size_t)blockIdx.x * N * C + (size_t)(j + r * B) * C + c);
                if (A.tf) x = cmul(x, tf_at(A.P, j + r * B, kx, N));
            }
            v[r] = x;
        }
        dft<16, +1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[17 * C * j + c + k * C] = v[outpos<16>(k)];
    }
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
        for (int k = 4; k < 12; ++k) __stcg(A.out + (size_t)(j + (k - 4) * B) * NX + kx, v[outpos<16>(k)]);
    }
}

namespace {

template <int N>
int launch_spec_cols(const SpecArgs &A, bool inverse, const float2 *tw, cudaStream_t st)
{
    using S = SpecCol<N>;
    auto kern = inverse ? k_spec_cols_inv<N> : k_spec_cols_fwd<N>;
    if (S::SMEM > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    }
    kern<<<(A.NX + S::C - 1) / S::C, S::NT, S::SMEM, st>>>(A, tw);
    count_launch();
    return check_launch(inverse ? "k_spec_cols_inv" : "k_spec_cols_fwd");
}

} // namespace

bool spec_cols_ok(int NY) { return is_pow2(NY) && NY >= 256 && NY <= FFT_MAX; }

int spec_cols(const SpecArgs &A, bool inverse, cudaStream_t st)
{
    const float2 *tw = twiddle_table();
    if (!tw) return fail(OLG_ERR_CUDA, "twiddle table unavailable");
    switch (A.NY) {
    case 256: return launch_spec_cols<256>(A, inverse, tw, st);
    case 512: return launch_spec_cols<512>(A, inverse, tw, st);
    case 1024: return launch_spec_cols<1024>(A, inverse, tw, st);
    case 2048: return launch_spec_cols<2048>(A, inverse, tw, st);
    case 4096: return launch_spec_cols<4096>(A, inverse, tw, st);
    case 8192: return launch_spec_cols<8192>(A, inverse, tw, st);
    default: return fail(OLG_ERR_UNSUPPORTED_SIZE, "spectral column pass: power-of-two height 256..8192");
    }
}

} // namespace olg
