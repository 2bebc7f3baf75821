// prop.cu -- fused ASM / Fresnel / ARSS propagation on GB300 (sm_103a).
//
// The reference runs each propagation as ~8 full-size elementwise kernels
// plus 2-3 cuFFT calls over a 2x zero-padded grid (golprop.h:507-534 for ASM,
// 167-198 Fresnel, 941-995 ARSS), synchronising after every step.  Here one
// propagation of an ny x nx field (padded NY = 2ny, NX = 2nx) is three passes
// over HBM, with the padding, transfer function / chirp products and the
// crop folded into the FFT passes:
//
//   pass 1 (k_rows_fwd): the ny non-zero rows: load (x pre-chirp), zero-pad to
//          NX in shared memory, row FFT, store to scratch S (ny x NX).
//   pass 2 (k_cols):     tiles of C adjacent columns of S: load the ny rows
//          into the centre of an NY-long column (zeros around), column FFT,
//          x T(ky, kx), inverse column FFT, keep the central ny rows, store
//          back in place.
//   pass 3 (k_rows_inv): rows of S: inverse row FFT, keep the central nx
//          columns (x post-chirp), store the ny x nx result.
//
// Algorithmic HBM traffic per propagation: 8n + 16n + 16n + 16n + 16n + 8n =
// 80 n bytes (n = ny * nx), against ~71 n complex64 reads/writes in the
// reference's chain.  Transfer functions are evaluated in registers (ASM) or
// from two 1-D spectra of the separable chirp (Fresnel, ARSS): the 2-D FFT of
// the sampled chirp exp(i pi (x^2 + y^2) / (lambda z)) is the outer product of
// two 1-D FFTs, which k_chirp computes per call (exactly the DFT of the sampled
// response the reference builds, golprop.h:184-187, olprop.h:133-137).
#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>
#include <cmath>
#include <cstdio>

#include "common.cuh"
#include "fft.cuh"
#include "fft2.cuh"
#include "fftp.cuh"
#include "propdev.cuh"
#include "propmr.cuh"

namespace olg {

static __device__ float2 g_tw[FFT_MAX];
// the same table as (c, c, s, s) for the paired-sequence passes
static __device__ float4 g_tw4[FFT_MAX];

// ---------------------------------------------------------------- launch shapes
template <int N>
struct RowCfg {
    static constexpr int NT = N >= 2048 ? N / 16 : 128;
    static constexpr int NSEQ = N >= 2048 ? 1 : 2048 / N;
    static constexpr int SMEM = NSEQ * padded_len(N) * 8;
};
template <int N>
struct ColCfg {
    static constexpr int E = N >= 4096 ? 2 * N : 8192; // elements per CTA
    static constexpr int C = E / N;                    // columns per CTA
    static constexpr int NT = E / 16;                  // 1 radix-16 butterfly per thread per stage
    static constexpr int SMEM = padded_len(N) * C * 8;
};

// ------------------------------------------------------------------- pass 1
template <int N>
__global__ void __launch_bounds__(RowCfg<N>::NT) k_rows_fwd(PropParams P)
{
    pdl_enter();
    using Cfg = RowCfg<N>;
    extern __shared__ float2 sm[];
    constexpr int SS = padded_len(N);
    const int tid = threadIdx.x;
    const int r0 = blockIdx.x * Cfg::NSEQ;
    const int nx = P.nx, off = N / 4;
    // zero the pad regions [0, N/4) and [3N/4, N) of every row
    for (int e = tid; e < Cfg::NSEQ * (N / 2); e += Cfg::NT) {
        const int q = e / (N / 2), i = e % (N / 2);
        const int idx = i < N / 4 ? i : i + N / 2;
        sm[q * SS + pidx(idx)] = make_float2(0.f, 0.f);
    }
    // load the nx input samples of each row (two complex per float4)
    const int hx = nx / 2;
    for (int e = tid; e < Cfg::NSEQ * hx; e += Cfg::NT) {
        const int q = e / hx, w2 = (e % hx) * 2;
        const int h = r0 + q;
        float2 a = make_float2(0.f, 0.f), b = a;
        if (h < P.ny) {
            if (P.in_phase) {
                const float2 ph = __ldg(reinterpret_cast<const float2 *>(P.in_phase + (size_t)h * P.in_ld + w2));
                sincosf(ph.x, &a.y, &a.x);
                sincosf(ph.y, &b.y, &b.x);
            } else {
                const float4 v = __ldg(reinterpret_cast<const float4 *>(P.in + (size_t)h * P.in_ld + w2));
                a = make_float2(v.x, v.y);
                b = make_float2(v.z, v.w);
            }
            a = apply_op(a, P.pre_mode, P.prex, P.prey, h, w2, P.ny, nx, P.pre_hlim, P.pre_wlim);
            b = apply_op(b, P.pre_mode, P.prex, P.prey, h, w2 + 1, P.ny, nx, P.pre_hlim, P.pre_wlim);
        }
        sm[q * SS + pidx(off + w2)] = a;
        sm[q * SS + pidx(off + w2 + 1)] = b;
    }
    __syncthreads();
    smem_fft<N, -1, Cfg::NT, false, Cfg::NSEQ>(sm, SS, g_tw, tid);
    // store full rows to S
    for (int e = tid; e < Cfg::NSEQ * (N / 2); e += Cfg::NT) {
        const int q = e / (N / 2), i2 = (e % (N / 2)) * 2;
        const int h = r0 + q;
        if (h >= P.ny) continue;
        const float2 a = sm[q * SS + pidx(i2)], b = sm[q * SS + pidx(i2 + 1)];
        *reinterpret_cast<float4 *>(P.S + (size_t)h * N + i2) = make_float4(a.x, a.y, b.x, b.y);
    }
}

// ------------------------------------------------------------------- pass 3
template <int N>
__global__ void __launch_bounds__(RowCfg<N>::NT) k_rows_inv(PropParams P)
{
    pdl_enter();
    using Cfg = RowCfg<N>;
    extern __shared__ float2 sm[];
    constexpr int SS = padded_len(N);
    const int tid = threadIdx.x;
    const int r0 = blockIdx.x * Cfg::NSEQ;
    for (int e = tid; e < Cfg::NSEQ * (N / 2); e += Cfg::NT) {
        const int q = e / (N / 2), i2 = (e % (N / 2)) * 2;
        const int h = r0 + q;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (h < P.ny) v = *reinterpret_cast<const float4 *>(P.S + (size_t)h * N + i2);
        sm[q * SS + pidx(i2)] = make_float2(v.x, v.y);
        sm[q * SS + pidx(i2 + 1)] = make_float2(v.z, v.w);
    }
    __syncthreads();
    smem_fft<N, +1, Cfg::NT, false, Cfg::NSEQ>(sm, SS, g_tw, tid);
    const int nx = P.nx, off = N / 4, hx = nx / 2;
    float lsum = 0.f;
    for (int e = tid; e < Cfg::NSEQ * hx; e += Cfg::NT) {
        const int q = e / hx, w2 = (e % hx) * 2;
        const int h = r0 + q;
        if (h >= P.ny) continue;
        float2 a = sm[q * SS + pidx(off + w2)], b = sm[q * SS + pidx(off + w2 + 1)];
        if (P.post_mode == OP_SEED) {
            const float2 t = __ldg(reinterpret_cast<const float2 *>(P.target + (size_t)h * nx + w2));
            const float ra = a.x * a.x + a.y * a.y - t.x, rb = b.x * b.x + b.y * b.y - t.y;
            lsum = fmaf(ra, ra, fmaf(rb, rb, lsum));
            a = cscale(a, P.seed_scale * ra);
            b = cscale(b, P.seed_scale * rb);
        } else {
            a = apply_op(a, P.post_mode, P.postx, P.posty, h, w2, P.ny, nx, P.post_hlim, P.post_wlim);
            b = apply_op(b, P.post_mode, P.postx, P.posty, h, w2 + 1, P.ny, nx, P.post_hlim, P.post_wlim);
        }
        float4 *dst = reinterpret_cast<float4 *>(P.out + (size_t)h * P.out_ld + w2);
        if (P.accumulate) {
            const float4 o = *dst;
            a.x += o.x; a.y += o.y; b.x += o.z; b.y += o.w;
        }
        *dst = make_float4(a.x, a.y, b.x, b.y);
    }
    if (P.post_mode == OP_SEED) {
        __shared__ float red[32];
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        if ((tid & 31) == 0) red[tid >> 5] = lsum;
        __syncthreads();
        if (tid < 32) {
            float v = tid < Cfg::NT / 32 ? red[tid] : 0.f;
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (tid == 0) atomicAdd(P.loss, (double)v);
        }
    }
}

// ------------------------------------------------------------------- pass 2
template <int N>
__global__ void __launch_bounds__(ColCfg<N>::NT) k_cols(PropParams P)
{
    pdl_enter();
    using Cfg = ColCfg<N>;
    constexpr int C = Cfg::C, NT = Cfg::NT;
    extern __shared__ float2 sm[];
    const int tid = threadIdx.x;
    const int c0 = blockIdx.x * C;
    const int NX = P.NX, ny = P.ny, off = N / 4;
    // zero rows [0, N/4) and [3N/4, N)
    for (int e = tid; e < (N / 2) * C; e += NT) {
        const int i = e / C, c = e % C;
        const int idx = i < N / 4 ? i : i + N / 2;
        sm[pidx(idx) * C + c] = make_float2(0.f, 0.f);
    }
    // load the ny stored rows into the centre
    constexpr int C2 = C / 2;
    for (int e = tid; e < ny * C2; e += NT) {
        const int h = e / C2, c = (e % C2) * 2;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c0 + c < NX) v = *reinterpret_cast<const float4 *>(P.S + (size_t)h * NX + c0 + c);
        sm[pidx(off + h) * C + c] = make_float2(v.x, v.y);
        sm[pidx(off + h) * C + c + 1] = make_float2(v.z, v.w);
    }
    __syncthreads();
    smem_fft<N, -1, NT, true, C>(sm, 0, g_tw, tid);
    // multiply by the transfer function
    for (int e = tid; e < N * C; e += NT) {
        const int ky = e / C, c = e % C;
        const int kx = c0 + c;
        float2 T;
        if (P.method == M_ASM) {
            const int fx = kx < NX / 2 ? kx : kx - NX;
            const int fy = ky < N / 2 ? ky : ky - N;
            T = asm_tf(P, fx, fy);
        } else {
            T = cmul(__ldg(P.Hx + (kx < NX ? kx : 0)), __ldg(P.Hy + ky));
            if (P.conj) T = cconj(T);
        }
        float2 &x = sm[pidx(ky) * C + c];
        x = cmul(x, T);
    }
    __syncthreads();
    smem_fft<N, +1, NT, true, C>(sm, 0, g_tw, tid);
    for (int e = tid; e < ny * C2; e += NT) {
        const int h = e / C2, c = (e % C2) * 2;
        if (c0 + c >= NX) continue;
        const float2 a = sm[pidx(off + h) * C + c], b = sm[pidx(off + h) * C + c + 1];
        *reinterpret_cast<float4 *>(P.S + (size_t)h * NX + c0 + c) = make_float4(a.x, a.y, b.x, b.y);
    }
}

// =========================================================== v2 passes
// N >= 256: register-resident first / last radix-16 stages (fft2.cuh).
template <int N, int NT, int NSEQ>
__device__ __forceinline__ void rows_fwd_body(const PropParams &P, int r0, float2 *sm, int tid)
{
    constexpr int SS = padded_len(N), B = N / 16;
    static_assert((NSEQ * B) % NT == 0, "threads must divide the butterflies");
    constexpr int BPT = NSEQ * B / NT;
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 4; r < 12; ++r) v[r] = h < P.ny ? load_in(P, h, j + (r - 4) * B) : make_float2(0.f, 0.f);
        dft16_in_mid<-1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[q * SS + pidx(j * 16 + k)] = v[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, -1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j + r * B)];
        last_twiddle<N, -1>(v, j, g_tw);
        dft<16, -1>(v);
        if (h < P.ny) {
#pragma unroll
            for (int k = 0; k < 16; ++k) __stcg(P.S + (size_t)h * N + j + k * B, v[outpos<16>(k)]);
        }
    }
}

template <int N, int NT, int NSEQ>
__device__ __forceinline__ void rows_inv_body(const PropParams &P, int r0, float2 *sm, int tid, float &lsum)
{
    constexpr int SS = padded_len(N), B = N / 16;
    constexpr int BPT = NSEQ * B / NT;
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r)
            v[r] = h < P.ny ? __ldcg(P.S + (size_t)h * N + j + r * B) : make_float2(0.f, 0.f);
        dft<16, +1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[q * SS + pidx(j * 16 + k)] = v[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, +1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j + r * B)];
        last_twiddle<N, +1>(v, j, g_tw);
        dft16_out_mid<+1>(v);
        if (h >= P.ny) continue;
#pragma unroll
        for (int k = 4; k < 12; ++k) {
            const int w = j + (k - 4) * B;
            float2 a = v[outpos<16>(k)];
            store_out(P, h, w, a, lsum);
        }
    }
}

template <int N, int NT, int C>
__device__ __forceinline__ void cols_body(const PropParams &P, int c0, float2 *sm, int tid)
{
    constexpr int B = N / 16;
    static_assert((C * B) % NT == 0, "threads must divide the butterflies");
    constexpr int BPT = C * B / NT;
    const int NX = P.NX;
    // forward first stage, straight from the ny stored rows (the rest is zero padding)
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 4; r < 12; ++r)
            v[r] = kx < NX ? __ldcg(P.S + (size_t)(j + (r - 4) * B) * NX + kx) : make_float2(0.f, 0.f);
        dft16_in_mid<-1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[pidx(j * 16 + k) * C + c] = v[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, -1, NT, true, C>(sm, 0, g_tw, tid);
    // forward last stage -> x T(ky, kx) -> inverse first stage, in registers
    float2 vv[BPT][16];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C;
#pragma unroll
        for (int r = 0; r < 16; ++r) vv[t][r] = sm[pidx(j + r * B) * C + c];
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        last_twiddle<N, -1>(vv[t], j, g_tw);
        dft<16, -1>(vv[t]);
        float2 w[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) w[k] = kx < NX ? cmul(vv[t][outpos<16>(k)], tf_at(P, j + k * B, kx, N)) : vv[t][outpos<16>(k)];
        dft<16, +1>(w);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[pidx(j * 16 + k) * C + c] = w[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, +1, NT, true, C>(sm, 0, g_tw, tid);
    // inverse last stage: only the central ny rows, back in place
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[pidx(j + r * B) * C + c];
        last_twiddle<N, +1>(v, j, g_tw);
        dft16_out_mid<+1>(v);
        if (kx < NX) {
#pragma unroll
            for (int k = 4; k < 12; ++k) __stcg(P.S + (size_t)(j + (k - 4) * B) * NX + kx, v[outpos<16>(k)]);
        }
    }
}

// ======================================================= persistent row passes
// The same row transforms as rows_fwd_body / rows_inv_body, but each CTA loops
// over row groups g = blockIdx.x, + gridDim.x, ... and issues the global loads
// of its next group into registers before it runs the current group through
// shared memory, so that the loads' latency overlaps the butterflies.
template <int N, int NT, int NSEQ>
__device__ __forceinline__ void rows_fwd_body_persist(const PropParams &P, float2 *sm, int tid)
{
    constexpr int SS = padded_len(N), B = N / 16;
    constexpr int BPT = NSEQ * B / NT;
    const int groups = (P.ny + NSEQ - 1) / NSEQ;
    float2 nv[BPT][8];
    auto fetch = [&](int g) {
#pragma unroll
        for (int t = 0; t < BPT; ++t) {
            const int b = tid + t * NT, q = b / B, j = b % B, h = g * NSEQ + q;
            const bool live = g < groups && h < P.ny;
#pragma unroll
            for (int r = 0; r < 8; ++r) nv[t][r] = live ? load_in(P, h, j + r * B) : make_float2(0.f, 0.f);
        }
    };
    fetch(blockIdx.x);
    for (int g = blockIdx.x; g < groups; g += gridDim.x) {
#pragma unroll
        for (int t = 0; t < BPT; ++t) {
            const int b = tid + t * NT, q = b / B, j = b % B;
            float2 v[16];
#pragma unroll
            for (int r = 4; r < 12; ++r) v[r] = nv[t][r - 4];
            dft16_in_mid<-1>(v);
#pragma unroll
            for (int k = 0; k < 16; ++k) sm[q * SS + pidx(j * 16 + k)] = v[outpos<16>(k)];
        }
        fetch(g + gridDim.x);
        __syncthreads();
        mid_stages<N, -1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
        for (int t = 0; t < BPT; ++t) {
            const int b = tid + t * NT, q = b / B, j = b % B, h = g * NSEQ + q;
            float2 v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j + r * B)];
            last_twiddle<N, -1>(v, j, g_tw);
            dft<16, -1>(v);
            if (h < P.ny) {
#pragma unroll
                for (int k = 0; k < 16; ++k) __stcg(P.S + (size_t)h * N + j + k * B, v[outpos<16>(k)]);
            }
        }
        __syncthreads();
    }
}

template <int N, int NT, int NSEQ>
__device__ __forceinline__ void rows_inv_body_persist(const PropParams &P, float2 *sm, int tid, float &lsum)
{
    constexpr int SS = padded_len(N), B = N / 16;
    constexpr int BPT = NSEQ * B / NT;
    const int groups = (P.ny + NSEQ - 1) / NSEQ;
    float2 nv[BPT][16];
    auto fetch = [&](int g) {
#pragma unroll
        for (int t = 0; t < BPT; ++t) {
            const int b = tid + t * NT, q = b / B, j = b % B, h = g * NSEQ + q;
            const bool live = g < groups && h < P.ny;
#pragma unroll
            for (int r = 0; r < 16; ++r)
                nv[t][r] = live ? __ldcg(P.S + (size_t)h * N + j + r * B) : make_float2(0.f, 0.f);
        }
    };
    fetch(blockIdx.x);
    for (int g = blockIdx.x; g < groups; g += gridDim.x) {
#pragma unroll
        for (int t = 0; t < BPT; ++t) {
            const int b = tid + t * NT, q = b / B, j = b % B;
            float2 v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = nv[t][r];
            dft<16, +1>(v);
#pragma unroll
            for (int k = 0; k < 16; ++k) sm[q * SS + pidx(j * 16 + k)] = v[outpos<16>(k)];
        }
        fetch(g + gridDim.x);
        __syncthreads();
        mid_stages<N, +1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
        for (int t = 0; t < BPT; ++t) {
            const int b = tid + t * NT, q = b / B, j = b % B, h = g * NSEQ + q;
            float2 v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j + r * B)];
            last_twiddle<N, +1>(v, j, g_tw);
            dft16_out_mid<+1>(v);
            if (h < P.ny) {
#pragma unroll
                for (int k = 4; k < 12; ++k) store_out(P, h, j + (k - 4) * B, v[outpos<16>(k)], lsum);
            }
        }
        __syncthreads();
    }
}

// ======================================================= seed round trip
// The multi-plane gradient's forward pass 3 and adjoint pass 1 in one pass:
// per row, the inverse row FFT of S, the crop, the seed (2/n)(|v|^2 - t) v
// and the loss (OP_SEED), then the zero-padded forward row FFT of the seed
// back into the same row of S.  The thread that ends the inverse transform
// with the central outputs w = j + (k - 4) B (k = 4..11) is the one that
// starts the forward transform from inputs j + r B (r = 4..11): the seed
// stays in its registers.
template <int N, int NT, int NSEQ>
__device__ __forceinline__ void rows_seed_body(const PropParams &P, int r0, float2 *sm, int tid, float &lsum)
{
    constexpr int SS = padded_len(N), B = N / 16;
    constexpr int BPT = NSEQ * B / NT;
    float2 u[BPT][16];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r)
            v[r] = h < P.ny ? __ldcg(P.S + (size_t)h * N + j + r * B) : make_float2(0.f, 0.f);
        dft<16, +1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[q * SS + pidx(j * 16 + k)] = v[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, +1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j + r * B)];
        last_twiddle<N, +1>(v, j, g_tw);
        dft16_out_mid<+1>(v);
#pragma unroll
        for (int k = 4; k < 12; ++k) {
            float2 a = v[outpos<16>(k)];
            if (h < P.ny) {
                const float r2 = a.x * a.x + a.y * a.y - __ldg(P.target + (size_t)h * P.nx + j + (k - 4) * B);
                lsum = fmaf(r2, r2, lsum);
                a = cscale(a, P.seed_scale * r2);
            } else {
                a = make_float2(0.f, 0.f);
            }
            u[t][k] = a;
        }
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B;
        dft16_in_mid<-1>(u[t]);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[q * SS + pidx(j * 16 + k)] = u[t][outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, -1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j + r * B)];
        last_twiddle<N, -1>(v, j, g_tw);
        dft<16, -1>(v);
        if (h < P.ny) {
#pragma unroll
            for (int k = 0; k < 16; ++k) __stcg(P.S + (size_t)h * N + j + k * B, v[outpos<16>(k)]);
        }
    }
}

// one shape for every length: 256 threads, 4096 elements (NSEQ rows) per CTA
template <int N>
struct SeedCfg {
    static constexpr int NT = 256, NSEQ = N >= 4096 ? 1 : 4096 / N;
    static constexpr int SMEM = NSEQ * padded_len(N) * 8;
};

template <int N>
__global__ void __launch_bounds__(256) k_rows_seed(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    using C = SeedCfg<N>;
    float lsum = 0.f;
    rows_seed_body<N, C::NT, C::NSEQ>(P, blockIdx.x * C::NSEQ, sm, threadIdx.x, lsum);
    loss_reduce(lsum, P.loss, threadIdx.x, C::NT);
}

// ======================================================= paired passes
// Two rows (passes 1 and 3) or two adjacent columns (pass 2) per butterfly,
// in planar pairs on the paired FP32 pipe (fftp.cuh).  Same stages, pruning
// and fusion as the v2 passes.
template <int N, int NT, int NSP>
__device__ __forceinline__ void rows_fwd_body_p(const PropParams &P, int r0, float4 *sm, int tid)
{
    constexpr int SS = padded_len(N), B = N / 16;
    static_assert((NSP * B) % NT == 0, "threads must divide the butterflies");
    constexpr int BPT = NSP * B / NT;
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + 2 * q;
        cpair v[16];
#pragma unroll
        for (int r = 4; r < 12; ++r) {
            const int w = j + (r - 4) * B;
            const float2 x0 = h < P.ny ? load_in(P, h, w) : make_float2(0.f, 0.f);
            const float2 x1 = h + 1 < P.ny ? load_in(P, h + 1, w) : make_float2(0.f, 0.f);
            v[r] = cp_pack(x0, x1);
        }
        cp_dft16_in_mid<-1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) cp_st(sm + q * SS + pidx(j * 16 + k), v[outpos<16>(k)]);
    }
    __syncthreads();
    cp_mid_stages<N, -1, NT, false, NSP>(sm, SS, g_tw4, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + 2 * q;
        cpair v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = cp_ld(sm + q * SS + pidx(j + r * B));
        cp_last_twiddle<N, -1>(v, j, g_tw4);
        cp_dft<16, -1>(v);
        if (h < P.ny) {
#pragma unroll
            for (int k = 0; k < 16; ++k) __stcg(P.S + (size_t)h * N + j + k * B, cp_lane0(v[outpos<16>(k)]));
        }
        if (h + 1 < P.ny) {
#pragma unroll
            for (int k = 0; k < 16; ++k) __stcg(P.S + (size_t)(h + 1) * N + j + k * B, cp_lane1(v[outpos<16>(k)]));
        }
    }
}


template <int N, int NT, int NSP>
__device__ __forceinline__ void rows_inv_body_p(const PropParams &P, int r0, float4 *sm, int tid, float &lsum)
{
    constexpr int SS = padded_len(N), B = N / 16;
    constexpr int BPT = NSP * B / NT;
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + 2 * q;
        cpair v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            const float2 x0 = h < P.ny ? __ldcg(P.S + (size_t)h * N + j + r * B) : make_float2(0.f, 0.f);
            const float2 x1 = h + 1 < P.ny ? __ldcg(P.S + (size_t)(h + 1) * N + j + r * B) : make_float2(0.f, 0.f);
            v[r] = cp_pack(x0, x1);
        }
        cp_dft<16, +1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) cp_st(sm + q * SS + pidx(j * 16 + k), v[outpos<16>(k)]);
    }
    __syncthreads();
    cp_mid_stages<N, +1, NT, false, NSP>(sm, SS, g_tw4, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + 2 * q;
        cpair v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = cp_ld(sm + q * SS + pidx(j + r * B));
        cp_last_twiddle<N, +1>(v, j, g_tw4);
        cp_dft16_out_mid<+1>(v);
        if (h < P.ny) {
#pragma unroll
            for (int k = 4; k < 12; ++k) store_out(P, h, j + (k - 4) * B, cp_lane0(v[outpos<16>(k)]), lsum);
        }
        if (h + 1 < P.ny) {
#pragma unroll
            for (int k = 4; k < 12; ++k) store_out(P, h + 1, j + (k - 4) * B, cp_lane1(v[outpos<16>(k)]), lsum);
        }
    }
}

template <int N, int NT, int CP>
__device__ __forceinline__ void cols_body_p(const PropParams &P, int c0, float4 *sm, int tid)
{
    constexpr int B = N / 16;
    static_assert((CP * B) % NT == 0, "threads must divide the butterflies");
    constexpr int BPT = CP * B / NT;
    const int NX = P.NX;
    // forward first stage, straight from the ny stored rows (the rest is zero padding)
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % CP, j = b / CP, kx = c0 + 2 * c;
        cpair v[16];
#pragma unroll
        for (int r = 4; r < 12; ++r) {
            const float4 f = kx < NX ? __ldcg(reinterpret_cast<const float4 *>(P.S + (size_t)(j + (r - 4) * B) * NX + kx))
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
            v[r] = {make_float2(f.x, f.z), make_float2(f.y, f.w)};
        }
        cp_dft16_in_mid<-1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) cp_st(sm + pidx(j * 16 + k) * CP + c, v[outpos<16>(k)]);
    }
    __syncthreads();
    cp_mid_stages<N, -1, NT, true, CP>(sm, 0, g_tw4, tid);
    // forward last stage -> x T(ky, kx) -> inverse first stage, in registers
    cpair vv[BPT][16];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % CP, j = b / CP;
#pragma unroll
        for (int r = 0; r < 16; ++r) vv[t][r] = cp_ld(sm + pidx(j + r * B) * CP + c);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % CP, j = b / CP, kx = c0 + 2 * c;
        cp_last_twiddle<N, -1>(vv[t], j, g_tw4);
        cp_dft<16, -1>(vv[t]);
        cpair w[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            const cpair x = vv[t][outpos<16>(k)];
            if (kx < NX) {
                const int ky = j + k * B;
                const cpair T = cp_pack(tf_at(P, ky, kx, N), tf_at(P, ky, kx + 1, N));
                w[k] = {__ffma2_rn(x.im, pneg(T.im), __fmul2_rn(x.re, T.re)),
                        __ffma2_rn(x.re, T.im, __fmul2_rn(x.im, T.re))};
            } else {
                w[k] = x;
            }
        }
        cp_dft<16, +1>(w);
#pragma unroll
        for (int k = 0; k < 16; ++k) cp_st(sm + pidx(j * 16 + k) * CP + c, w[outpos<16>(k)]);
    }
    __syncthreads();
    cp_mid_stages<N, +1, NT, true, CP>(sm, 0, g_tw4, tid);
    // inverse last stage: only the central ny rows, back in place
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % CP, j = b / CP, kx = c0 + 2 * c;
        cpair v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = cp_ld(sm + pidx(j + r * B) * CP + c);
        cp_last_twiddle<N, +1>(v, j, g_tw4);
        cp_dft16_out_mid<+1>(v);
        if (kx < NX) {
#pragma unroll
            for (int k = 4; k < 12; ++k) {
                const cpair x = v[outpos<16>(k)];
                __stcg(reinterpret_cast<float4 *>(P.S + (size_t)(j + (k - 4) * B) * NX + kx),
                       make_float4(x.re.x, x.im.x, x.re.y, x.im.y));
            }
        }
    }
}


// Launch-shape variants of the v2 passes (threads, elements per CTA, minimum
// resident CTAs); olg_autotune_prop times them on the device and keeps the
// fastest per FFT length.
template <int NT_, int E_, int MINB_, bool PAIRED_ = false, bool PERSIST_ = false>
struct Shape {
    static constexpr int NT = NT_, E = E_, MINB = MINB_;
    static constexpr bool PAIRED = PAIRED_, PERSIST = PERSIST_;
};
// rows: E = row elements per CTA (NSEQ = E / N rows, at least one; paired
// variants: NSEQ = E / 2N row pairs, at least one)
template <int I> struct RowVar;
template <> struct RowVar<0> : Shape<256, 4096, 2> {};
template <> struct RowVar<1> : Shape<256, 4096, 4> {};
template <> struct RowVar<2> : Shape<512, 8192, 2> {};
template <> struct RowVar<3> : Shape<128, 2048, 4> {};
template <> struct RowVar<4> : Shape<128, 4096, 4, true> {};
template <> struct RowVar<5> : Shape<256, 8192, 2, true> {};
template <> struct RowVar<6> : Shape<512, 16384, 1, true> {};
template <> struct RowVar<7> : Shape<64, 2048, 8, true> {};
// persistent: one grid of SMs x MINB CTAs looping over row groups
template <> struct RowVar<8> : Shape<128, 2048, 4, false, true> {};
template <> struct RowVar<9> : Shape<256, 4096, 2, false, true> {};
constexpr int N_ROW_VARIANTS = 10;
// columns: E = elements per CTA (C = E / N adjacent columns; paired variants:
// C = E / 2N adjacent column pairs)
template <int I> struct ColVar;
template <> struct ColVar<0> : Shape<512, 8192, 1> {};
template <> struct ColVar<1> : Shape<512, 16384, 1> {};
template <> struct ColVar<2> : Shape<256, 4096, 2> {};
template <> struct ColVar<3> : Shape<256, 8192, 2> {};
template <> struct ColVar<4> : Shape<256, 8192, 2, true> {};
template <> struct ColVar<5> : Shape<512, 16384, 1, true> {};
template <> struct ColVar<6> : Shape<128, 4096, 4, true> {};
template <> struct ColVar<7> : Shape<64, 2048, 8, true> {};
// register-capped shapes: two / four CTAs per SM for more resident warps
template <> struct ColVar<8> : Shape<512, 8192, 2> {};
template <> struct ColVar<9> : Shape<256, 4096, 4> {};
constexpr int N_COL_VARIANTS = 10;

template <int N, class V>
struct RowShape {
    static constexpr int NT = V::NT;
    static constexpr bool PAIRED = V::PAIRED, PERSIST = V::PERSIST;
    static constexpr int MINB = V::MINB;
    static constexpr int NSEQ = PAIRED ? (V::E >= 2 * N ? V::E / (2 * N) : 1) : (V::E >= N ? V::E / N : 1);
    static constexpr int ROWS = PAIRED ? 2 * NSEQ : NSEQ; // field rows per CTA
    static constexpr int SMEM = NSEQ * padded_len(N) * (PAIRED ? 16 : 8);
    // paired variants: exactly one butterfly pair per thread in the end stages
    static constexpr bool valid = (NSEQ * (N / 16)) % NT == 0 && SMEM <= 200 * 1024 &&
                                  (!PAIRED || (NSEQ * (N / 16) == NT && cp_mid_bpt<N, NT, NSEQ>() <= 32));
};
template <int N, class V>
struct ColShape {
    static constexpr int NT = V::NT;
    static constexpr bool PAIRED = V::PAIRED;
    static constexpr int C = PAIRED ? V::E / (2 * N) : V::E / N;
    static constexpr int COLS = PAIRED ? 2 * C : C; // field columns per CTA
    static constexpr int SMEM = padded_len(N) * (C > 0 ? C : 1) * (PAIRED ? 16 : 8);
    static constexpr bool valid = C >= 1 && (C * (N / 16)) % NT == 0 && SMEM <= 200 * 1024 &&
                                  (!PAIRED || (C * (N / 16) == NT && cp_mid_bpt<N, NT, (C > 0 ? C : 1)>() <= 32));
};

template <int N, class V>
__global__ void __launch_bounds__(V::NT, V::MINB) k_rows_fwd2(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    using S = RowShape<N, V>;
    if constexpr (S::valid && S::PERSIST) rows_fwd_body_persist<N, S::NT, S::NSEQ>(P, sm, threadIdx.x);
    else if constexpr (S::valid) rows_fwd_body<N, S::NT, S::NSEQ>(P, blockIdx.x * S::NSEQ, sm, threadIdx.x);
}

template <int N, class V>
__global__ void __launch_bounds__(V::NT, V::MINB) k_rows_inv2(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    using S = RowShape<N, V>;
    if constexpr (S::valid) {
        float lsum = 0.f;
        if constexpr (S::PERSIST) rows_inv_body_persist<N, S::NT, S::NSEQ>(P, sm, threadIdx.x, lsum);
        else rows_inv_body<N, S::NT, S::NSEQ>(P, blockIdx.x * S::NSEQ, sm, threadIdx.x, lsum);
        if (P.post_mode == OP_SEED) loss_reduce(lsum, P.loss, threadIdx.x, S::NT);
    }
}

template <int N, class V>
__global__ void __launch_bounds__(V::NT, V::MINB) k_cols2(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    using S = ColShape<N, V>;
    if constexpr (S::valid) cols_body<N, S::NT, S::C>(P, blockIdx.x * S::C, sm, threadIdx.x);
}

template <int N, class V>
__global__ void __launch_bounds__(V::NT, V::MINB) k_rows_fwd3(PropParams P)
{
    pdl_enter();
    extern __shared__ float4 sm4[];
    using S = RowShape<N, V>;
    if constexpr (S::valid && S::PAIRED) rows_fwd_body_p<N, S::NT, S::NSEQ>(P, blockIdx.x * S::ROWS, sm4, threadIdx.x);
}

template <int N, class V>
__global__ void __launch_bounds__(V::NT, V::MINB) k_rows_inv3(PropParams P)
{
    pdl_enter();
    extern __shared__ float4 sm4[];
    using S = RowShape<N, V>;
    if constexpr (S::valid && S::PAIRED) {
        float lsum = 0.f;
        rows_inv_body_p<N, S::NT, S::NSEQ>(P, blockIdx.x * S::ROWS, sm4, threadIdx.x, lsum);
        if (P.post_mode == OP_SEED) loss_reduce(lsum, P.loss, threadIdx.x, S::NT);
    }
}

template <int N, class V>
__global__ void __launch_bounds__(V::NT, V::MINB) k_cols3(PropParams P)
{
    pdl_enter();
    extern __shared__ float4 sm4[];
    using S = ColShape<N, V>;
    if constexpr (S::valid && S::PAIRED) cols_body_p<N, S::NT, S::C>(P, blockIdx.x * S::COLS, sm4, threadIdx.x);
}

// ------------------------------------------------------------- chirp tables
// Per axis (blockIdx.x == 0): the 1-D spectrum H[k] = sum_j c(j') e^{-2 pi i j k / L},
// j' = j for j < L/2 else j - L (the fftshift'ed centred response), with
// c(m) = exp(2 pi i (kap m^2 + lin m)) and c = 0 for |m| >= lim (lim < 0: no window).
// blockIdx.x == 1: the pass-1 / pass-3 tables along this axis:
//   a[m] = [|m'| < alim] exp(2 pi i (a2 m'^2 + a1 m' + a0))  (m' = m - n/2), and b[] likewise.
template <int N>
struct ChirpCfg {
    static constexpr int NT = N / 16 < 256 ? N / 16 : 256;
    static constexpr int SMEM = padded_len(N) * 8;
};

template <int N, int NT>
__device__ __forceinline__ void chirp_body(const ChirpAxis &A, int part, float2 *sm, int tid)
{
    if (part == 0) {
        for (int j = tid; j < N; j += NT) {
            const int m = j < N / 2 ? j : j - N;
            sm[pidx(j)] = chirp_sample(A, m);
        }
        __syncthreads();
        smem_fft<N, -1, NT, false, 1>(sm, padded_len(N), g_tw, tid);
        for (int j = tid; j < N; j += NT) {
            const float2 v = cscale(sm[pidx(j)], A.scale);
            A.H[j] = A.conj_spec ? cconj(v) : v;
        }
    } else {
        chirp_tables(A, tid, NT);
    }
}

template <int N>
__global__ void __launch_bounds__(ChirpCfg<N>::NT) k_chirp(ChirpAxis A)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    chirp_body<N, ChirpCfg<N>::NT>(A, blockIdx.x, sm, threadIdx.x);
}

// ===================================================================== host
namespace {

std::mutex g_tw_mu;
bool g_tw_ready[64] = {};

int ensure_twiddles()
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return fail(OLG_ERR_INVALID_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_tw_mu);
    if (g_tw_ready[dev]) return OLG_OK;
    std::vector<float2> t(FFT_MAX);
    for (int m = 0; m < FFT_MAX; ++m) {
        const double a = -2.0 * M_PI * (double)m / (double)FFT_MAX;
        t[m] = make_float2((float)cos(a), (float)sin(a));
    }
    e = cudaMemcpyToSymbol(g_tw, t.data(), sizeof(float2) * FFT_MAX);
    if (e != cudaSuccess) return cuda_fail(e, "twiddle table upload");
    std::vector<float4> t4(FFT_MAX);
    for (int m = 0; m < FFT_MAX; ++m) t4[m] = make_float4(t[m].x, t[m].x, t[m].y, t[m].y);
    e = cudaMemcpyToSymbol(g_tw4, t4.data(), sizeof(float4) * FFT_MAX);
    if (e != cudaSuccess) return cuda_fail(e, "paired twiddle table upload");
    g_tw_ready[dev] = true;
    return OLG_OK;
}

template <typename K>
int prep_smem(K kern, int bytes)
{
    if (bytes <= 48 * 1024) return OLG_OK;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, "cudaFuncSetAttribute");
}

// Launch with programmatic stream serialisation (see pdl_enter).
template <typename Arg>
int launch_pdl(void (*kern)(Arg), int grid, int block, int smem, cudaStream_t st, const Arg &a, const char *what)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, a);
    if (e != cudaSuccess) return cuda_fail(e, what);
    count_launch();
    return check_launch(what);
}

// selected variant per FFT length (index log2 N) and pass kind (0 rows fwd, 1 cols, 2 rows inv);
// atomic so that a set or an autotune on one host thread races no launch on another
std::atomic<int> g_variant[3][14];

// SMs of the current device (cached per device; 152 on GB300)
int sm_count()
{
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        cache[dev] = n;
    }
    return cache[dev];
}

template <int N, int I>
int launch_rows_v(const PropParams &P, bool inverse, cudaStream_t st)
{
    using S = RowShape<N, RowVar<I>>;
    if constexpr (!S::valid) {
        return fail(OLG_ERR_INVALID_ARG, "row variant not valid for this length");
    } else if constexpr (S::PAIRED) {
        const int grid = (P.ny + S::ROWS - 1) / S::ROWS;
        if (!inverse) {
            if (int rc = prep_smem(k_rows_fwd3<N, RowVar<I>>, S::SMEM)) return rc;
            return launch_pdl(k_rows_fwd3<N, RowVar<I>>, grid, S::NT, S::SMEM, st, P, "k_rows_fwd3");
        }
        if (int rc = prep_smem(k_rows_inv3<N, RowVar<I>>, S::SMEM)) return rc;
        return launch_pdl(k_rows_inv3<N, RowVar<I>>, grid, S::NT, S::SMEM, st, P, "k_rows_inv3");
    } else {
        int grid = (P.ny + S::ROWS - 1) / S::ROWS;
        if constexpr (S::PERSIST) grid = std::min(grid, sm_count() * S::MINB);
        if (!inverse) {
            if (int rc = prep_smem(k_rows_fwd2<N, RowVar<I>>, S::SMEM)) return rc;
            return launch_pdl(k_rows_fwd2<N, RowVar<I>>, grid, S::NT, S::SMEM, st, P, "k_rows_fwd2");
        }
        if (int rc = prep_smem(k_rows_inv2<N, RowVar<I>>, S::SMEM)) return rc;
        return launch_pdl(k_rows_inv2<N, RowVar<I>>, grid, S::NT, S::SMEM, st, P, "k_rows_inv2");
    }
}

template <int N, int I>
int launch_cols_v(const PropParams &P, cudaStream_t st)
{
    using S = ColShape<N, ColVar<I>>;
    if constexpr (!S::valid) {
        return fail(OLG_ERR_INVALID_ARG, "column variant not valid for this length");
    } else if constexpr (S::PAIRED) {
        const int grid = (P.NX + S::COLS - 1) / S::COLS;
        if (int rc = prep_smem(k_cols3<N, ColVar<I>>, S::SMEM)) return rc;
        return launch_pdl(k_cols3<N, ColVar<I>>, grid, S::NT, S::SMEM, st, P, "k_cols3");
    } else {
        const int grid = (P.NX + S::COLS - 1) / S::COLS;
        if (int rc = prep_smem(k_cols2<N, ColVar<I>>, S::SMEM)) return rc;
        return launch_pdl(k_cols2<N, ColVar<I>>, grid, S::NT, S::SMEM, st, P, "k_cols2");
    }
}

template <int N>
bool row_variant_valid(int i)
{
    switch (i) {
    case 0: return RowShape<N, RowVar<0>>::valid;
    case 1: return RowShape<N, RowVar<1>>::valid;
    case 2: return RowShape<N, RowVar<2>>::valid;
    case 3: return RowShape<N, RowVar<3>>::valid;
    case 4: return RowShape<N, RowVar<4>>::valid;
    case 5: return RowShape<N, RowVar<5>>::valid;
    case 6: return RowShape<N, RowVar<6>>::valid;
    case 7: return RowShape<N, RowVar<7>>::valid;
    case 8: return RowShape<N, RowVar<8>>::valid;
    case 9: return RowShape<N, RowVar<9>>::valid;
    default: return false;
    }
}
template <int N>
bool col_variant_valid(int i)
{
    switch (i) {
    case 0: return ColShape<N, ColVar<0>>::valid;
    case 1: return ColShape<N, ColVar<1>>::valid;
    case 2: return ColShape<N, ColVar<2>>::valid;
    case 3: return ColShape<N, ColVar<3>>::valid;
    case 4: return ColShape<N, ColVar<4>>::valid;
    case 5: return ColShape<N, ColVar<5>>::valid;
    case 6: return ColShape<N, ColVar<6>>::valid;
    case 7: return ColShape<N, ColVar<7>>::valid;
    case 8: return ColShape<N, ColVar<8>>::valid;
    case 9: return ColShape<N, ColVar<9>>::valid;
    default: return false;
    }
}

constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

template <int N>
int launch_rows(const PropParams &P, bool inverse, cudaStream_t st)
{
    if constexpr (N >= 256) {
        switch (g_variant[inverse ? 2 : 0][ilog2(N)]) {
        case 1: return launch_rows_v<N, 1>(P, inverse, st);
        case 2: return launch_rows_v<N, 2>(P, inverse, st);
        case 3: return launch_rows_v<N, 3>(P, inverse, st);
        case 4: return launch_rows_v<N, 4>(P, inverse, st);
        case 5: return launch_rows_v<N, 5>(P, inverse, st);
        case 6: return launch_rows_v<N, 6>(P, inverse, st);
        case 7: return launch_rows_v<N, 7>(P, inverse, st);
        case 8: return launch_rows_v<N, 8>(P, inverse, st);
        case 9: return launch_rows_v<N, 9>(P, inverse, st);
        default: return launch_rows_v<N, 0>(P, inverse, st);
        }
    } else {
        using C = RowCfg<N>;
        const int grid = (P.ny + C::NSEQ - 1) / C::NSEQ;
        if (!inverse) {
            if (int rc = prep_smem(k_rows_fwd<N>, C::SMEM)) return rc;
            return launch_pdl(k_rows_fwd<N>, grid, C::NT, C::SMEM, st, P, "k_rows_fwd");
        }
        if (int rc = prep_smem(k_rows_inv<N>, C::SMEM)) return rc;
        return launch_pdl(k_rows_inv<N>, grid, C::NT, C::SMEM, st, P, "k_rows_inv");
    }
}

template <int N>
int launch_cols(const PropParams &P, cudaStream_t st)
{
    if constexpr (N >= 256) {
        switch (g_variant[1][ilog2(N)]) {
        case 1: return launch_cols_v<N, 1>(P, st);
        case 2: return launch_cols_v<N, 2>(P, st);
        case 3: return launch_cols_v<N, 3>(P, st);
        case 4: return launch_cols_v<N, 4>(P, st);
        case 5: return launch_cols_v<N, 5>(P, st);
        case 6: return launch_cols_v<N, 6>(P, st);
        case 7: return launch_cols_v<N, 7>(P, st);
        case 8: return launch_cols_v<N, 8>(P, st);
        case 9: return launch_cols_v<N, 9>(P, st);
        default: return launch_cols_v<N, 0>(P, st);
        }
    } else {
        using C = ColCfg<N>;
        const int grid = (P.NX + C::C - 1) / C::C;
        if (int rc = prep_smem(k_cols<N>, C::SMEM)) return rc;
        return launch_pdl(k_cols<N>, grid, C::NT, C::SMEM, st, P, "k_cols");
    }
}

template <int N>
int launch_rows_seed(const PropParams &P, cudaStream_t st)
{
    using C = SeedCfg<N>;
    if (int rc = prep_smem(k_rows_seed<N>, C::SMEM)) return rc;
    return launch_pdl(k_rows_seed<N>, (P.ny + C::NSEQ - 1) / C::NSEQ, C::NT, C::SMEM, st, P, "k_rows_seed");
}

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

template <int N>
int launch_chirp(const ChirpAxis &A, cudaStream_t st)
{
    using C = ChirpCfg<N>;
    if (int rc = prep_smem(k_chirp<N>, C::SMEM)) return rc;
    const int grid = (A.ta || A.tb) ? 2 : 1;
    k_chirp<N><<<grid, C::NT, C::SMEM, st>>>(A);
    count_launch();
    return check_launch("k_chirp");
}

#define OLG_SIZE_SWITCH(n, FN, ...)                                                                              \
    switch (n) {                                                                                                 \
    case 32: return FN<32>(__VA_ARGS__);                                                                         \
    case 64: return FN<64>(__VA_ARGS__);                                                                         \
    case 128: return FN<128>(__VA_ARGS__);                                                                       \
    case 256: return FN<256>(__VA_ARGS__);                                                                       \
    case 512: return FN<512>(__VA_ARGS__);                                                                       \
    case 1024: return FN<1024>(__VA_ARGS__);                                                                     \
    case 2048: return FN<2048>(__VA_ARGS__);                                                                     \
    case 4096: return FN<4096>(__VA_ARGS__);                                                                     \
    case 8192: return FN<8192>(__VA_ARGS__);                                                                     \
    default: return fail(OLG_ERR_UNSUPPORTED_SIZE, "FFT length not supported");                                \
    }

// lengths that are not powers of two take the mixed-radix passes (propmr.cu)
int rows_pass(const PropParams &P, bool inverse, cudaStream_t st)
{
    if (!is_pow2(P.NX)) return mr_rows_pass(P, inverse, st);
    OLG_SIZE_SWITCH(P.NX, launch_rows, P, inverse, st)
}
int cols_pass(const PropParams &P, cudaStream_t st)
{
    if (!is_pow2(P.NY)) return mr_cols_pass(P, st);
    OLG_SIZE_SWITCH(P.NY, launch_cols, P, st)
}
int chirp_axis(const ChirpAxis &A, cudaStream_t st)
{
    if (!is_pow2(A.L)) return mr_chirp_axis(A, st);
    OLG_SIZE_SWITCH(A.L, launch_chirp, A, st)
}

struct Layout {
    float2 *S, *Hx, *Hy, *tax, *tay, *tbx, *tby;
};

size_t layout_bytes(int ny, int nx, Layout *L, char *base)
{
    size_t off = 0;
    auto take = [&](size_t elems) {
        char *p = base ? base + off : nullptr;
        off += align_up(elems * sizeof(float2), 256);
        return (float2 *)p;
    };
    Layout l;
    l.S = take((size_t)ny * 2 * nx);
    l.Hx = take(2 * (size_t)nx);
    l.Hy = take(2 * (size_t)ny);
    l.tax = take(nx);
    l.tay = take(ny);
    l.tbx = take(nx);
    l.tby = take(ny);
    if (L) *L = l;
    return off;
}

// A field axis n is supported when the padded length 2n is a power of two in
// [32, 8192] (the tuned passes) or 2^a 3^b 5^c with n >= 8 that one CTA holds
// (mixed radix, up to 7680).
bool axis_ok(int n) { return is_pow2(n) ? (n >= 16 && 2 * n <= FFT_MAX) : (n >= 8 && mr_length_ok(2 * n)); }

int validate(const void *a, const void *b, int ny, int nx)
{
    if (!a || !b) return fail(OLG_ERR_INVALID_ARG, "null field pointer");
    if (((uintptr_t)a & 15) || ((uintptr_t)b & 15)) return fail(OLG_ERR_INVALID_ARG, "field pointers must be 16-byte aligned");
    if (!axis_ok(ny) || !axis_ok(nx))
        return fail(OLG_ERR_UNSUPPORTED_SIZE,
                    "ny, nx must be powers of two in [16, 4096] or have 2n = 2^a 3^b 5^c <= 7680 (n >= 8)");
    return OLG_OK;
}

PropParams base_params(const void *in, void *out, int ny, int nx, const Layout &L)
{
    PropParams P{};
    P.ny = ny; P.nx = nx; P.NY = 2 * ny; P.NX = 2 * nx;
    P.in = (const float2 *)in;
    P.out = (float2 *)out;
    P.S = L.S;
    P.Hx = L.Hx; P.Hy = L.Hy;
    P.pre_mode = OP_NONE; P.post_mode = OP_NONE;
    P.in_ld = nx;
    P.out_ld = nx;
    return P;
}

int run_passes(const PropParams &P, cudaStream_t st)
{
    if (int rc = rows_pass(P, false, st)) return rc;
    if (int rc = cols_pass(P, st)) return rc;
    return rows_pass(P, true, st);
}

long floor_lim(double v)
{
    double f = std::floor(v);
    if (!(f < 1073741824.0)) f = 1073741824.0;
    if (f < -1073741824.0) f = -1073741824.0;
    return (long)f;
}

void set_quad(float &hi, float &lo, double v)
{
    DF d = split_df(v);
    hi = d.hi;
    lo = d.lo;
}

// frac(v) in [-0.5, 0.5]
float frac_host(double v) { return (float)(v - std::nearbyint(v)); }

ChirpAxis chirp_axis_params(int L, int n, double d, double lambda, double z, double s_factor, int lim, double scale,
                            float2 *H)
{
    ChirpAxis A{};
    A.L = L;
    A.n = n;
    set_quad(A.kap_hi, A.kap_lo, s_factor * d * d / (2.0 * lambda * z));
    A.lim = lim;
    A.scale = (float)scale;
    A.conj_spec = 0;
    A.H = H;
    A.alim = A.blim = -1;
    return A;
}

} // namespace
} // namespace olg

using namespace olg;

extern "C" size_t olg_prop_workspace_bytes(int ny, int nx)
{
    if (ny <= 0 || nx <= 0) return 0;
    return layout_bytes(ny, nx, nullptr, nullptr);
}

namespace olg {
namespace {

// Parameters of one propagation: the three passes plus the per-axis chirp
// jobs (none for ASM; spectra for Fresnel; spectra and pre/post tables for ARSS).
struct PropSetup {
    PropParams P;
    ChirpAxis ax, ay;
    bool chirps = false;
};

int check_phys(double dy, double dx, double lambda, double z, bool nonzero_z)
{
    if (!(dy > 0) || !(dx > 0) || !(lambda > 0) || !std::isfinite(z) || (nonzero_z && z == 0.0))
        return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    return OLG_OK;
}

int setup_asm(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z, int flags,
              const Layout &L, PropSetup *S)
{
    if (int rc = check_phys(dy, dx, lambda, z, false)) return rc;
    PropParams P = base_params(in, out, ny, nx, L);
    if (int rc = mr_prepare(P)) return rc;
    const double NX = 2.0 * nx, NY = 2.0 * ny;
    const double du = 1.0 / (dx * NX), dv = 1.0 / (dy * NY);
    const double zl = z / lambda;
    P.method = M_ASM;
    P.conj = (flags & OLG_CONJ) ? 1 : 0;
    P.scale = (flags & OLG_NO_NORMALIZE) ? 1.0f : (float)(1.0 / (NX * NY));
    P.c0 = frac_host(zl);
    set_quad(P.ax_hi, P.ax_lo, z * lambda * du * du / 2.0);
    set_quad(P.ay_hi, P.ay_lo, z * lambda * dv * dv / 2.0);
    P.tx = (float)(lambda * lambda * du * du);
    P.ty = (float)(lambda * lambda * dv * dv);
    P.zl = (float)zl;
    S->P = P;
    S->chirps = false;
    return OLG_OK;
}

// Shifted ASM (golprop.h:335-420, 536-576): T gains the phase ox u + oy v,
// an integer multiple of (lx, ly) = (ox du, oy dv) cycles per frequency index.
// OLG_BANDLIMIT adds the band window of the host overload (olprop.h:251-300):
// T = 0 unless |u - u0| 2 < uw and |v - v0| 2 < vw, decided here in double
// for every frequency index exactly as that code decides it.
// T = double decides in double; T = float mirrors the PREC_T = float
// instantiation operation by operation (float operands, std::pow(float, int)
// and the sqrt in double, results stored to float; this file is compiled with
// -ffp-contract=off).  Adjacent split blocks sit exactly on a branch boundary
// (offset == 0.5 / du), so the precision decides which branch is taken.
template <typename T>
void shifted_window(double pitch, int L, double o_, double z_, double lambda_, int *lo, int *hi)
{
    const T d = (T)1 / ((T)pitch * (T)L);
    const T o = (T)o_, z = (T)z_, lambda = (T)lambda_;
    const T s0 = (T)0.5 / d;
    const T tm = o - (T)0.5 / d, tp = o + (T)0.5 / d;
    const T lm = (T)(1 / std::sqrt(std::pow((double)tm, -2.0) * z * z + 1.0) / lambda);
    const T lp = (T)(1 / std::sqrt(std::pow((double)tp, -2.0) * z * z + 1.0) / lambda);
    T c, w;
    if (s0 < o) {
        c = (T)0.5 * (lp + lm);
        w = lp - lm;
    } else if (-s0 <= o && o < s0) {
        c = (T)0.5 * (lp - lm);
        w = lp + lm;
    } else {
        c = (T)-0.5 * (lp + lm);
        w = lm - lp;
    }
    *lo = 1;
    *hi = 0;
    bool any = false;
    for (int m = 0; m < L; ++m) {
        const int f = m - L / 2;
        const T u = (T)f * d;
        if (std::fabs(u - c) * 2 < w) {
            if (!any) *lo = f;
            *hi = f;
            any = true;
        }
    }
}

int setup_shifted_asm(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z,
                      double oy, double ox, int flags, const Layout &L, PropSetup *S)
{
    if (!std::isfinite(oy) || !std::isfinite(ox)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if (int rc = setup_asm(in, out, ny, nx, dy, dx, lambda, z, flags, L, S)) return rc;
    PropParams &P = S->P;
    const double du = 1.0 / (dx * 2.0 * nx), dv = 1.0 / (dy * 2.0 * ny);
    P.shift = 1;
    set_quad(P.lx_hi, P.lx_lo, ox * du);
    set_quad(P.ly_hi, P.ly_lo, oy * dv);
    if (flags & OLG_BANDLIMIT) {
        P.band = 1;
        if (flags & OLG_CHECK_F32) {
            shifted_window<float>(dx, 2 * nx, ox, z, lambda, &P.fx_lo, &P.fx_hi);
            shifted_window<float>(dy, 2 * ny, oy, z, lambda, &P.fy_lo, &P.fy_hi);
        } else {
            shifted_window<double>(dx, 2 * nx, ox, z, lambda, &P.fx_lo, &P.fx_hi);
            shifted_window<double>(dy, 2 * ny, oy, z, lambda, &P.fy_lo, &P.fy_hi);
        }
    }
    return OLG_OK;
}

int setup_fresnel(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z,
                  int bandlimit, int flags, const Layout &L, PropSetup *S)
{
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (bandlimit < 0 || bandlimit > 2) return fail(OLG_ERR_INVALID_ARG, "bandlimit must be 0, 1 or 2");
    PropParams P = base_params(in, out, ny, nx, L);
    if (int rc = mr_prepare(P)) return rc;
    const int NX = 2 * nx, NY = 2 * ny;
    const double np = (double)NX * (double)NY;
    const double sc1 = (flags & OLG_NO_NORMALIZE) ? 1.0 : 1.0 / np;
    int limx = -1, limy = -1;
    if (bandlimit == 1) { // golprop.h:227-233: one limit, from x, on both axes
        limx = limy = (int)floor_lim(std::fabs(lambda * z * 0.5 / dx) / dx);
    } else if (bandlimit == 2) { // olprop.h:34-39
        limx = (int)floor_lim(std::fabs(lambda * z * 0.5 / dx) / dx);
        limy = (int)floor_lim(std::fabs(lambda * z * 0.5 / dy) / dy);
    }
    S->ax = chirp_axis_params(NX, nx, dx, lambda, z, 1.0, limx, sc1, L.Hx);
    S->ay = chirp_axis_params(NY, ny, dy, lambda, z, 1.0, limy, sc1, L.Hy);
    S->chirps = true;
    P.method = M_CHIRP;
    P.conj = (flags & OLG_CONJ) ? 1 : 0;
    P.scale = 1.0f;
    S->P = P;
    return OLG_OK;
}

// windows == false: the shifted Fresnel propagation (golprop.h:606-752), the
// same three chirps without any window.
int setup_arss(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx, double lambda, double z,
               double s, double oy, double ox, int flags, const Layout &L, PropSetup *S, bool windows = true)
{
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (!std::isfinite(s) || !std::isfinite(oy) || !std::isfinite(ox))
        return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if (windows && (s == 0.0 || s == 1.0))
        return fail(OLG_ERR_INVALID_ARG, "ARSS is undefined for s = 0 or s = 1 (window limits divide by s|s-1|)");
    PropParams P = base_params(u_src, u_dst, ny, nx, L);
    if (int rc = mr_prepare(P)) return rc;
    const int NX = 2 * nx, NY = 2 * ny;
    const double np = (double)NX * (double)NY;
    // windows, golprop.h:849-852, 891-892, 928-931 (-1: none)
    int hlim_u = -1, wlim_u = -1, lim_h = -1, hlim_c = -1, wlim_c = -1;
    if (windows) {
        hlim_u = (int)floor_lim((lambda * std::fabs(z) * 0.5 / (s * std::fabs(s - 1) * dy)) / dy);
        wlim_u = (int)floor_lim((lambda * std::fabs(z) * 0.5 / (s * std::fabs(s - 1) * dx)) / dx);
        lim_h = (int)floor_lim(std::fabs(lambda * z * 0.5 / (dx * s)) / dx);
        hlim_c = (int)floor_lim((lambda * std::fabs(z) * 0.5 / (std::fabs(1 - s) * dy)) / dy);
        wlim_c = (int)floor_lim((lambda * std::fabs(z) * 0.5 / (std::fabs(1 - s) * dx)) / dx);
    }
    const bool adj = (flags & OLG_CONJ) != 0;
    const double lz2 = 2.0 * lambda * z;
    ChirpAxis ax = chirp_axis_params(NX, nx, dx, lambda, z, s, lim_h, 1.0 / np, L.Hx);
    ChirpAxis ay = chirp_axis_params(NY, ny, dy, lambda, z, s, lim_h, 1.0 / np, L.Hy);
    // pre-chirp (golprop.h:830-841) and post-chirp (golprop.h:910-920) coefficients, cycles
    struct Q {
        double a2, a1, a0;
    };
    const Q prex{(s * s - s) * dx * dx / lz2, -2.0 * s * ox * dx / lz2, 0.0};
    const Q prey{(s * s - s) * dy * dy / lz2, -2.0 * s * oy * dy / lz2, 0.0};
    const Q postx{(1 - s) * dx * dx / lz2, 2.0 * ox * dx / lz2, (ox * ox + oy * oy) / lz2};
    const Q posty{(1 - s) * dy * dy / lz2, 2.0 * oy * dy / lz2, 0.0};
    auto fill = [&](ChirpAxis &A, float2 *ta, float2 *tb, const Q &qa, int alim, int aconj, const Q &qb, int blim,
                    int bconj) {
        A.ta = ta;
        A.tb = tb;
        set_quad(A.a2_hi, A.a2_lo, qa.a2);
        set_quad(A.a1_hi, A.a1_lo, qa.a1);
        A.a0 = frac_host(qa.a0);
        A.alim = alim;
        A.aconj = aconj;
        set_quad(A.b2_hi, A.b2_lo, qb.a2);
        set_quad(A.b1_hi, A.b1_lo, qb.a1);
        A.b0 = frac_host(qb.a0);
        A.blim = blim;
        A.bconj = bconj;
    };
    if (!adj) {
        // pass 1: pre-chirp, zero outside its window; pass 3: post-chirp inside its window
        fill(ax, L.tax, L.tbx, prex, wlim_u, 0, postx, -1, 0);
        fill(ay, L.tay, L.tby, prey, hlim_u, 0, posty, -1, 0);
        P.pre_mode = OP_TABLE;
        P.post_mode = windows ? OP_TABLE_IN_WINDOW : OP_TABLE;
        P.post_hlim = hlim_c;
        P.post_wlim = wlim_c;
    } else {
        // adjoint: conj(post-chirp) inside the Cz window first, conj(pre-chirp) with its window last
        fill(ax, L.tax, L.tbx, postx, -1, 1, prex, wlim_u, 1);
        fill(ay, L.tay, L.tby, posty, -1, 1, prey, hlim_u, 1);
        P.pre_mode = windows ? OP_TABLE_IN_WINDOW : OP_TABLE;
        P.pre_hlim = hlim_c;
        P.pre_wlim = wlim_c;
        P.post_mode = OP_TABLE;
    }
    P.prex = L.tax;
    P.prey = L.tay;
    P.postx = L.tbx;
    P.posty = L.tby;
    P.method = M_CHIRP;
    P.conj = adj ? 1 : 0;
    P.scale = 1.0f;
    S->P = P;
    S->ax = ax;
    S->ay = ay;
    S->chirps = true;
    return OLG_OK;
}

int run_setup(const PropSetup &S, cudaStream_t st)
{
    if (S.chirps) {
        if (int rc = chirp_axis(S.ax, st)) return rc;
        if (int rc = chirp_axis(S.ay, st)) return rc;
    }
    return run_passes(S.P, st);
}

} // namespace
} // namespace olg

extern "C" int olg_asm_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                                double z, int flags, void *work, size_t work_bytes, olg_stream_t stream)
{
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, false)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_asm(u_in, u_out, ny, nx, dy, dx, lambda, z, flags, L, &S)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_fresnel_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                                    double z, int bandlimit, int flags, void *work, size_t work_bytes,
                                    olg_stream_t stream)
{
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (bandlimit < 0 || bandlimit > 2) return fail(OLG_ERR_INVALID_ARG, "bandlimit must be 0, 1 or 2");
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_fresnel(u_in, u_out, ny, nx, dy, dx, lambda, z, bandlimit, flags, L, &S)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_arss_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx, double lambda,
                                 double z, double s, double oy, double ox, int flags, void *work, size_t work_bytes,
                                 olg_stream_t stream)
{
    if (int rc = validate(u_src, u_dst, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (!std::isfinite(s)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if (s == 0.0 || s == 1.0)
        return fail(OLG_ERR_INVALID_ARG, "ARSS is undefined for s = 0 or s = 1 (window limits divide by s|s-1|)");
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_arss(u_src, u_dst, ny, nx, dy, dx, lambda, z, s, oy, ox, flags, L, &S)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_shifted_asm_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx,
                                        double lambda, double z, double oy, double ox, int flags, void *work,
                                        size_t work_bytes, olg_stream_t stream)
{
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, false)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_shifted_asm(u_in, u_out, ny, nx, dy, dx, lambda, z, oy, ox, flags, L, &S)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_shifted_fresnel_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx,
                                            double lambda, double z, double s, double oy, double ox, int flags,
                                            void *work, size_t work_bytes, olg_stream_t stream)
{
    if (int rc = validate(u_src, u_dst, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_arss(u_src, u_dst, ny, nx, dy, dx, lambda, z, s, oy, ox, flags, L, &S, false)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_shifted_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx,
                                    double lambda, double z, double oy, double ox, int propmode, int flags, void *work,
                                    size_t work_bytes, olg_stream_t stream)
{
    if (propmode == OLG_ASM)
        return olg_shifted_asm_prop_c64(u_src, u_dst, ny, nx, dy, dx, lambda, z, oy, ox, flags, work, work_bytes,
                                        stream);
    if (propmode == OLG_FRESNEL)
        return olg_shifted_fresnel_prop_c64(u_src, u_dst, ny, nx, dy, dx, lambda, z, 1.0, oy, ox, flags, work,
                                            work_bytes, stream);
    return fail(OLG_ERR_INVALID_ARG, "shifted propagation takes OLG_ASM or OLG_FRESNEL");
}

extern "C" size_t olg_split_prop_workspace_bytes(int ny, int nx, int blocks_y, int blocks_x)
{
    if (ny <= 0 || nx <= 0 || blocks_y <= 0 || blocks_x <= 0) return 0;
    return layout_bytes(ny / blocks_y, nx / blocks_x, nullptr, nullptr);
}

// Split propagation (golprop.h:772-813, olprop.h:618-654): the field is cut
// into blocks_y x blocks_x blocks; every (source block, destination block)
// pair adds a shifted propagation of the source block, offset by the blocks'
// distance, into the destination block.  Blocks are read and written in place
// through row strides; u_out must not overlap u_in.
extern "C" int olg_split_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                                  double z, int propmode, int blocks_y, int blocks_x, int flags, void *work,
                                  size_t work_bytes, olg_stream_t stream)
{
    if (!u_in || !u_out || blocks_y <= 0 || blocks_x <= 0 || ny % blocks_y || nx % blocks_x)
        return fail(OLG_ERR_INVALID_ARG, "blocks must divide the field");
    const int bh = ny / blocks_y, bw = nx / blocks_x;
    if (int rc = validate(u_in, u_out, bh, bw)) return rc;
    if (propmode != OLG_ASM && propmode != OLG_FRESNEL)
        return fail(OLG_ERR_INVALID_ARG, "split propagation takes OLG_ASM or OLG_FRESNEL");
    const size_t bytes = (size_t)ny * nx * sizeof(float2);
    const char *a = (const char *)u_in, *b = (const char *)u_out;
    if (a < b + bytes && b < a + bytes) return fail(OLG_ERR_INVALID_ARG, "u_out must not overlap u_in");
    if (int rc = check_phys(dy, dx, lambda, z, propmode == OLG_FRESNEL)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(bh, bw, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(bh, bw, &L, (char *)sc.ptr);
    if (!(flags & OLG_ACCUMULATE)) {
        const cudaError_t e = cudaMemsetAsync(u_out, 0, bytes, st);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    }
    const int pflags = flags & (OLG_CONJ | OLG_NO_NORMALIZE | OLG_BANDLIMIT | OLG_CHECK_F32);
    for (int gn = 0; gn < blocks_y; ++gn)
        for (int gm = 0; gm < blocks_x; ++gm) {
            const float2 *src = (const float2 *)u_in + (size_t)gn * bh * nx + (size_t)gm * bw;
            for (int dn = 0; dn < blocks_y; ++dn)
                for (int dm = 0; dm < blocks_x; ++dm) {
                    float2 *dst = (float2 *)u_out + (size_t)dn * bh * nx + (size_t)dm * bw;
                    // offsets as the reference forms them: an int times a float pitch, in float
                    const double oy = (double)((float)((gn - dn) * bh) * (float)dy);
                    const double ox = (double)((float)((gm - dm) * bw) * (float)dx);
                    PropSetup S;
                    int rc = propmode == OLG_ASM
                                 ? setup_shifted_asm(src, dst, bh, bw, dy, dx, lambda, z, oy, ox, pflags, L, &S)
                                 : setup_arss(src, dst, bh, bw, dy, dx, lambda, z, 1.0, oy, ox, pflags, L, &S, false);
                    if (rc) return rc;
                    S.P.in_ld = nx;
                    S.P.out_ld = nx;
                    S.P.accumulate = 1;
                    if ((rc = run_setup(S, st))) return rc;
                }
        }
    return OLG_OK;
}

// ------------------------------------------------------------- tilted
namespace olg {

const float2 *twiddle_table()
{
    static std::atomic<const float2 *> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    if (!cache[dev]) {
        if (ensure_twiddles() != OLG_OK) return nullptr;
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_tw) != cudaSuccess) return nullptr;
        cache[dev] = (const float2 *)p;
    }
    return cache[dev];
}

namespace {

struct TiltLayout {
    float2 *C, *D, *Hx, *Hy;
};

size_t tilt_layout(int ny, int nx, TiltLayout *L, char *base)
{
    size_t off = 0;
    auto take = [&](size_t elems) {
        char *p = base ? base + off : nullptr;
        off += align_up(elems * sizeof(float2), 256);
        return (float2 *)p;
    };
    const size_t full = (size_t)4 * ny * nx;
    TiltLayout l;
    l.C = take(full);
    l.D = take(full);
    l.Hx = take(2 * (size_t)nx);
    l.Hy = take(2 * (size_t)ny);
    if (L) *L = l;
    return off;
}

} // namespace
} // namespace olg

extern "C" size_t olg_tilted_workspace_bytes(int ny, int nx)
{
    if (ny <= 0 || nx <= 0) return 0;
    return tilt_layout(ny, nx, nullptr, nullptr);
}

// Tilted-plane propagation (olprop.h:414-600).  reference == 0:
// TiltedSourceProp, the destination plane rotated by `angle` about the y axis
// as seen from the source; the spectrum is resampled on the rotated grid and
// then propagated.  reference != 0: TiltedReferenceProp, propagated first and
// then resampled for a plane rotated by `angle`.  Every frequency of the 2x
// padded grid must propagate (no evanescent sample), as the reference's
// square roots require.  u_out may equal u_in.
extern "C" int olg_tilted_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                                   double z, double angle, int interp, int propmode, int reference, void *work,
                                   size_t work_bytes, olg_stream_t stream)
{
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    if (propmode != OLG_ASM && propmode != OLG_FRESNEL)
        return fail(OLG_ERR_INVALID_ARG, "tilted propagation takes OLG_ASM or OLG_FRESNEL");
    if (interp != OLG_BILINEAR && interp != OLG_BICUBIC)
        return fail(OLG_ERR_INVALID_ARG, "interp must be OLG_BILINEAR or OLG_BICUBIC");
    if (int rc = check_phys(dy, dx, lambda, z, propmode == OLG_FRESNEL)) return rc;
    if (!std::isfinite(angle)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    const int NY = 2 * ny, NX = 2 * nx;
    const double N = (double)NY * (double)NX;
    const double du = 1 / (dx * NX), dv = 1 / (dy * NY);
    const double fsqr = 1 / (lambda * lambda), f0 = 1 / lambda;
    const double ang = reference ? angle : -angle;
    const double a11 = std::cos(ang), a13 = -std::sin(ang);
    const double a13f0 = reference ? 0.0 : a13 * f0;
    // the largest |fpx|, |fpy| (and |fpx + a13 f0| for the shifted ASM) sit on the grid's corners
    for (int cm = 0; cm < 2; ++cm)
        for (int cn = 0; cn < 2; ++cn) {
            const double fpx = (double)((cm ? NX - 1 : 0) - NX / 2) * du, fpy = (double)((cn ? NY - 1 : 0) - NY / 2) * dv;
            const double uu = fpx + a13f0;
            if (!(fsqr - fpx * fpx - fpy * fpy > 0) ||
                (!reference && propmode == OLG_ASM && !(fsqr - uu * uu - fpy * fpy >= 0)))
                return fail(OLG_ERR_INVALID_ARG, "tilted propagation: the padded grid reaches evanescent frequencies");
        }
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, tilt_layout(ny, nx, nullptr, nullptr), st)) return rc;
    TiltLayout TL;
    tilt_layout(ny, nx, &TL, (char *)sc.ptr);
    Layout L{};
    L.S = TL.D;
    PropParams P = base_params(u_in, u_out, ny, nx, L);
    if (int rc = mr_prepare(P)) return rc;

    TiltArgs T{};
    T.ny = ny; T.nx = nx; T.NY = NY; T.NX = NX;
    T.reference = reference ? 1 : 0;
    T.interp = interp;
    T.fresnel = propmode == OLG_FRESNEL ? 1 : 0;
    T.du = du; T.dv = dv; T.fsqr = fsqr; T.a11 = a11; T.a13 = a13; T.a13f0 = a13f0; T.z = z;
    T.J0 = (float)a11;
    T.Jb = (float)(-a13);
    T.invN = (float)(1.0 / N);
    {
        // a11 - 1 = -2 sin^2(ang / 2), without cancellation
        const double sh = std::sin(ang / 2);
        set_quad(T.c1_hi, T.c1_lo, -2.0 * sh * sh);
        const double K = reference ? a13 * f0 / du : 0.0;
        const double Ki = std::nearbyint(K);
        T.Ki = (int)Ki;
        T.Kf = (float)(K - Ki);
        T.a13f = (float)a13;
        T.duf = (float)du;
        T.dvf = (float)dv;
        T.dv2du = (float)(dv * dv / du);
        T.f0f = (float)f0;
        T.f0sq = (float)(f0 * f0);
        set_quad(T.du_hi, T.du_lo, du);
        set_quad(T.dv_hi, T.dv_lo, dv);
        set_quad(T.c_hi, T.c_lo, a13 * f0);
        set_quad(T.f0sq_hi, T.f0sq_lo, fsqr);
        set_quad(T.z_hi, T.z_lo, z);
    }
    T.Hx = TL.Hx; T.Hy = TL.Hy;
    T.C = TL.C; T.D = TL.D;
    PropParams &tf = T.tf;
    tf.ny = ny; tf.nx = nx; tf.NY = NY; tf.NX = NX;
    tf.scale = 1.0f;
    if (propmode == OLG_FRESNEL) {
        tf.method = M_CHIRP;
        tf.Hx = TL.Hx;
        tf.Hy = TL.Hy;
    } else {
        const double zl = z / lambda;
        tf.method = M_ASM;
        tf.c0 = frac_host(zl);
        set_quad(tf.ax_hi, tf.ax_lo, z * lambda * du * du / 2.0);
        set_quad(tf.ay_hi, tf.ay_lo, z * lambda * dv * dv / 2.0);
        tf.tx = (float)(lambda * lambda * du * du);
        tf.ty = (float)(lambda * lambda * dv * dv);
        tf.zl = (float)zl;
    }

    if (int rc = rows_pass(P, false, st)) return rc;
    if (propmode == OLG_FRESNEL) {
        // the Fresnel response's spectrum, fftshift'ed, 1/N (on x), with the
        // source form's linear phase exp(-2 pi i x a13 f0) along x
        ChirpAxis ax = chirp_axis_params(NX, nx, dx, lambda, z, 1.0, -1, 1.0 / N, TL.Hx);
        if (!reference) set_quad(ax.lin_hi, ax.lin_lo, -a13 * f0 * dx);
        ChirpAxis ay = chirp_axis_params(NY, ny, dy, lambda, z, 1.0, -1, 1.0, TL.Hy);
        if (int rc = chirp_axis(ax, st)) return rc;
        if (int rc = chirp_axis(ay, st)) return rc;
    }
    if (int rc = tilt_middle(T, st)) return rc;
    return rows_pass(P, true, st);
}

// ------------------------------------------------------------- autotuner
namespace olg {
namespace {

#define OLG_N_SWITCH(n, EXPR)                                                                                           \
    switch (n) {                                                                                                       \
    case 256: { constexpr int NN = 256; EXPR; }                                                                        \
    case 512: { constexpr int NN = 512; EXPR; }                                                                        \
    case 1024: { constexpr int NN = 1024; EXPR; }                                                                      \
    case 2048: { constexpr int NN = 2048; EXPR; }                                                                      \
    case 4096: { constexpr int NN = 4096; EXPR; }                                                                      \
    case 8192: { constexpr int NN = 8192; EXPR; }                                                                      \
    default: return false;                                                                                             \
    }

bool variant_valid(int kind, int n, int i)
{
    if (kind == 1) { OLG_N_SWITCH(n, return col_variant_valid<NN>(i)) }
    OLG_N_SWITCH(n, return row_variant_valid<NN>(i))
}

int log2i(int n)
{
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

} // namespace
} // namespace olg

extern "C" int olg_prop_variant_count(void) { return N_ROW_VARIANTS > N_COL_VARIANTS ? N_ROW_VARIANTS : N_COL_VARIANTS; }

extern "C" int olg_prop_get_variant(int kind, int n)
{
    if (kind < 0 || kind > 2 || !is_pow2(n) || n < 256 || n > FFT_MAX) return -1;
    return g_variant[kind][log2i(n)];
}

extern "C" int olg_prop_set_variant(int kind, int n, int idx)
{
    if (kind < 0 || kind > 2 || !is_pow2(n) || n < 256 || n > FFT_MAX) return fail(OLG_ERR_INVALID_ARG, "bad pass kind or length");
    if (!variant_valid(kind, n, idx)) return fail(OLG_ERR_INVALID_ARG, "launch variant not valid for this length");
    g_variant[kind][log2i(n)] = idx;
    return OLG_OK;
}

// Times every valid launch variant of the three passes on an ny x nx ASM
// propagation (the real kernels on the real shapes) and keeps the fastest.
extern "C" int olg_autotune_prop(int ny, int nx, int reps, olg_stream_t stream)
{
    if (!is_pow2(nx) || !is_pow2(ny) || nx < 128 || ny < 128 || 2 * nx > FFT_MAX || 2 * ny > FFT_MAX)
        return fail(OLG_ERR_UNSUPPORTED_SIZE, "autotuning covers fields with ny, nx powers of two in [128, 4096]");
    if (reps < 1) reps = 5;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch buf, sc;
    if (int rc = buf.acquire(nullptr, 0, (size_t)ny * nx * sizeof(float2), st)) return rc;
    if (int rc = sc.acquire(nullptr, 0, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    cudaError_t e = cudaMemsetAsync(buf.ptr, 0, (size_t)ny * nx * sizeof(float2), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_asm(buf.ptr, buf.ptr, ny, nx, 8e-6, 8e-6, 532e-9, 0.05, 0, L, &S)) return rc;
    // events released on every return path
    struct Events {
        cudaEvent_t a = nullptr, b = nullptr;
        ~Events()
        {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev;
    if ((e = cudaEventCreate(&ev.a)) != cudaSuccess || (e = cudaEventCreate(&ev.b)) != cudaSuccess)
        return cuda_fail(e, "cudaEventCreate");
    // Coordinate descent over the three passes, timing whole propagations:
    // a pass's speed depends on its neighbours (L2 contents, dependent-launch
    // overlap), so passes are not timed alone.
    const int lens[3] = {2 * nx, 2 * ny, 2 * nx};
    int lns[3];
    for (int k = 0; k < 3; ++k) lns[k] = log2i(lens[k]);
    // Each timed propagation starts from a cold L2 (a 256 MiB write first),
    // like a propagation of a field that was not just touched.
    const size_t flush_bytes = (size_t)256 << 20;
    Scratch flush;
    if (int rc = flush.acquire(nullptr, 0, flush_bytes, st)) return rc;
    auto time_prop = [&](float *ms) -> int {
        int rc = run_passes(S.P, st);
        *ms = 0.f;
        for (int r = 0; r < reps && !rc; ++r) {
            cudaError_t te = cudaMemsetAsync(flush.ptr, r & 0xff, flush_bytes, st);
            if (te != cudaSuccess) return cuda_fail(te, "cudaMemsetAsync (L2 flush)");
            if ((te = cudaEventRecord(ev.a, st)) != cudaSuccess) return cuda_fail(te, "cudaEventRecord");
            rc = run_passes(S.P, st);
            if (rc) break;
            if ((te = cudaEventRecord(ev.b, st)) != cudaSuccess) return cuda_fail(te, "cudaEventRecord");
            if ((te = cudaEventSynchronize(ev.b)) != cudaSuccess) return cuda_fail(te, "cudaEventSynchronize");
            float t = 0.f;
            if ((te = cudaEventElapsedTime(&t, ev.a, ev.b)) != cudaSuccess) return cuda_fail(te, "cudaEventElapsedTime");
            *ms += t;
        }
        return rc;
    };
    for (int round = 0; round < 2; ++round) {
        for (int kind = 0; kind < 3; ++kind) {
            const int n = lens[kind], ln = lns[kind];
            float best = 1e30f;
            int best_i = g_variant[kind][ln];
            for (int i = 0; i < olg_prop_variant_count(); ++i) {
                if (!variant_valid(kind, n, i)) continue;
                g_variant[kind][ln] = i;
                float ms = 0.f;
                if (int rc = time_prop(&ms)) {
                    g_variant[kind][ln] = best_i; // keep the last good choice
                    return rc;
                }
                if (ms < best) {
                    best = ms;
                    best_i = i;
                }
            }
            g_variant[kind][ln] = best_i;
        }
    }
    return OLG_OK;
}

// ---------------------------------------------------------------- AUTO checks
// AsmPropCheck olprop.h:209-225 and FresnelPropCheck olprop.h:109-123 in the
// caller's precision.  This file is compiled with -ffp-contract=off so the
// float versions round each operation like the reference's float build.
template <typename T>
static int asm_check_t(int ny, int nx, T dy, T dx, T lambda, T z)
{
    const int64_t nx2 = 2 * (int64_t)nx, ny2 = 2 * (int64_t)ny;
    const T du = 1 / (dx * nx2);
    const T dv = 1 / (dy * ny2);
    const T umax = du * nx2 / 2;
    const T vmax = dv * ny2 / 2;
    const T tmpsqrt = std::sqrt(1 / (lambda * lambda) - umax * umax - vmax * vmax);
    const T zmax_u = tmpsqrt / (2 * umax * du);
    const T zmax_v = tmpsqrt / (2 * vmax * dv);
    return (zmax_u < std::abs(z) || zmax_v < std::abs(z)) ? 0 : 1;
}
template <typename T>
static int fresnel_check_t(int ny, int nx, T dy, T dx, T lambda, T z)
{
    const size_t nx2 = 2 * (size_t)nx, ny2 = 2 * (size_t)ny;
    const T xmax = dx * nx2 / 2;
    const T ymax = dy * ny2 / 2;
    const T zmin_x = 2 * xmax * dx / lambda;
    const T zmin_y = 2 * ymax * dy / lambda;
    return (zmin_x > std::abs(z) || zmin_y > std::abs(z)) ? 0 : 1;
}

extern "C" int olg_asm_prop_check(int ny, int nx, double dy, double dx, double lambda, double z, int single_precision)
{
    if (single_precision) return asm_check_t<float>(ny, nx, (float)dy, (float)dx, (float)lambda, (float)z);
    return asm_check_t<double>(ny, nx, dy, dx, lambda, z);
}

extern "C" int olg_fresnel_prop_check(int ny, int nx, double dy, double dx, double lambda, double z, int single_precision)
{
    if (single_precision) return fresnel_check_t<float>(ny, nx, (float)dy, (float)dx, (float)lambda, (float)z);
    return fresnel_check_t<double>(ny, nx, dy, dx, lambda, z);
}

extern "C" int olg_prop_c64(void *u, int ny, int nx, double dy, double dx, double lambda, double z, int mode, int flags,
                            int *chosen, void *work, size_t work_bytes, olg_stream_t stream)
{
    const bool verbose = (flags & OLG_VERBOSE) != 0;
    const int f = flags & (OLG_CONJ | OLG_NO_NORMALIZE);
    const int sp = (flags & OLG_CHECK_F32) ? 1 : 0;
    int pick;
    if (mode == OLG_FRESNEL) pick = 1;
    else if (mode == OLG_ASM) pick = 0;
    else if (mode == OLG_AUTO) {
        if (olg_asm_prop_check(ny, nx, dy, dx, lambda, z, sp)) pick = 0;
        else if (!olg_fresnel_prop_check(ny, nx, dy, dx, lambda, z, sp)) pick = 2;
        else pick = 1;
    } else {
        return fail(OLG_ERR_INVALID_ARG, "invalid PROPMODE");
    }
    if (chosen) *chosen = pick;
    if (verbose) {
        if (pick == 0) printf("AsmProp\n");
        else if (pick == 1) printf("FresnelProp\n");
        else printf("warning!!\neither AsmProp or FresnelProp does not meet the condition.\n");
    }
    if (pick == 0) return olg_asm_prop_c64(u, u, ny, nx, dy, dx, lambda, z, f, work, work_bytes, stream);
    return olg_fresnel_prop_c64(u, u, ny, nx, dy, dx, lambda, z, pick == 2 ? 1 : 0, f, work, work_bytes, stream);
}

// ======================================================= batched persistent
// Many propagations of uneven sizes, methods and wavelengths in one launch.
// Work items, in queue order: every chirp job, then every pass-1 row group,
// every pass-2 column tile, every pass-3 row group (large fields first within
// each pass).  A CTA (one per SM, 512 threads) takes the next item with an
// atomic ticket, waits until the item's field has finished the pass it depends
// on (per-field counters; the wait is bounded and only ever on items taken
// earlier by running CTAs, so it cannot deadlock), runs it with the same pass
// bodies as the single-call kernels, then publishes its completion.
namespace olg {

constexpr int BATCH_NT = 512;
constexpr int BATCH_CTAS_PER_SM = 1;
// rows per row unit and columns per column tile: 16384 elements per unit
// (two 8192-point columns, as the fastest single-call column shape)
constexpr int BATCH_TILE = 2 * FFT_MAX;
__host__ __device__ constexpr int brow_nseq(int N) { return BATCH_TILE / N; }
__host__ __device__ constexpr int bcol_c(int N) { return BATCH_TILE / N; }
constexpr int BATCH_SMEM = padded_len(FFT_MAX) * 2 * 8; // the largest pass tile
constexpr long long BATCH_WAIT = 4000000000LL;           // ~2 s of SM clock

enum : int { BK_CHIRP = 0, BK_FWD = 1, BK_COLS = 2, BK_INV = 3 };

struct BatchItem {
    int field, kind, unit, n; // n: FFT length that selects the instantiation
    int count;                // consecutive units processed by this item
};
constexpr int BATCH_UNITS_PER_ITEM = 8; // 8 x 16384 elements per item

struct BatchDev {
    const PropParams *P;
    const ChirpAxis *jobs;
    const BatchItem *items;
    int n_items;
    int *head;
    int *done;         // per field: chirp jobs, pass-1 units, pass-2 units finished
    const int *target; // per field: how many of each there are
    int *err;
};

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ bool wait_at_least(const int *p, int target, long long budget)
{
    const long long t0 = clock64();
    while (ld_acquire(p) < target) {
        __nanosleep(100);
        if (clock64() - t0 > budget) return false;
    }
    return true;
}

template <int N>
__device__ __forceinline__ void batch_run(const PropParams &P, const ChirpAxis *jobs, const BatchItem &I, float2 *sm,
                                          int tid)
{
    if (I.kind == BK_CHIRP) {
        chirp_body<N, BATCH_NT>(jobs[I.unit >> 1], I.unit & 1, sm, tid);
    } else if (I.kind == BK_FWD) {
        rows_fwd_body<N, BATCH_NT, brow_nseq(N)>(P, I.unit * brow_nseq(N), sm, tid);
    } else if (I.kind == BK_COLS) {
        cols_body<N, BATCH_NT, bcol_c(N)>(P, I.unit * bcol_c(N), sm, tid);
    } else {
        float lsum = 0.f;
        rows_inv_body<N, BATCH_NT, brow_nseq(N)>(P, I.unit * brow_nseq(N), sm, tid, lsum);
    }
}

__global__ void __launch_bounds__(BATCH_NT, BATCH_CTAS_PER_SM) k_batch(BatchDev D)
{
    extern __shared__ float2 sm[];
    __shared__ int s_item, s_ok;
    __shared__ PropParams sP;
    const int tid = threadIdx.x;
    int loaded_field = -1;
    for (;;) {
        if (tid == 0) s_item = atomicAdd(D.head, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= D.n_items) break;
        const BatchItem I = D.items[it];
        const int f = I.field;
        if (tid == 0) {
            bool ok = true;
            if (I.kind == BK_FWD) ok = wait_at_least(D.done + 3 * f, D.target[3 * f], BATCH_WAIT);
            else if (I.kind == BK_COLS)
                ok = wait_at_least(D.done + 3 * f + 1, D.target[3 * f + 1], BATCH_WAIT) &&
                     wait_at_least(D.done + 3 * f, D.target[3 * f], BATCH_WAIT);
            else if (I.kind == BK_INV) ok = wait_at_least(D.done + 3 * f + 2, D.target[3 * f + 2], BATCH_WAIT);
            if (!ok) atomicExch(D.err, 1);
            __threadfence();
            s_ok = ok;
        }
        if (f != loaded_field) {
            const int *src = reinterpret_cast<const int *>(D.P + f);
            int *dst = reinterpret_cast<int *>(&sP);
            for (int w = tid; w < (int)(sizeof(PropParams) / 4); w += BATCH_NT) dst[w] = src[w];
            loaded_field = f;
        }
        __syncthreads();
        if (s_ok) {
            for (int u = 0; u < I.count; ++u) {
                BatchItem J = I;
                J.unit = I.unit + u;
                switch (I.n) {
                case 512: batch_run<512>(sP, D.jobs, J, sm, tid); break;
                case 1024: batch_run<1024>(sP, D.jobs, J, sm, tid); break;
                case 2048: batch_run<2048>(sP, D.jobs, J, sm, tid); break;
                case 4096: batch_run<4096>(sP, D.jobs, J, sm, tid); break;
                case 8192: batch_run<8192>(sP, D.jobs, J, sm, tid); break;
                default: break;
                }
                __syncthreads();
            }
        }
        __syncthreads();
        if (tid == 0 && I.kind != BK_INV) {
            __threadfence();
            atomicAdd(D.done + 3 * f + (I.kind == BK_CHIRP ? 0 : I.kind == BK_FWD ? 1 : 2), I.count);
        }
    }
}

} // namespace olg

struct olg_batch_plan_s {
    int dev = 0, n = 0, n_items = 0, grid = 0;
    std::vector<olg_field> fields;
    std::vector<char> direct; // per field: run through the tuned per-field passes, not k_batch
    std::vector<size_t> ws_off;
    char *mem = nullptr;
    size_t bytes = 0;
    BatchDev D{};
    size_t counters_off = 0, counters_bytes = 0;
};

namespace olg {
namespace {

bool batch_size_ok(int n) { return n >= 256 && n <= FFT_MAX / 2 && is_pow2(n); }

// Fields of at least this many pixels leave the persistent kernel: each fills
// the GPU on its own, and the per-field passes (autotuned launch shapes, no
// register cap shared with the largest length) run them faster; the
// persistent launch keeps the many small fields, where launches would cost
// more than the work.
std::atomic<long long> g_batch_direct_pixels{2048LL * 2048LL};

int field_setup(const olg_field &F, const Layout &L, PropSetup *S)
{
    switch (F.method) {
    case OLG_BATCH_ASM: return setup_asm(F.in, F.out, F.ny, F.nx, F.dy, F.dx, F.lambda, F.z, F.flags, L, S);
    case OLG_BATCH_FRESNEL: return setup_fresnel(F.in, F.out, F.ny, F.nx, F.dy, F.dx, F.lambda, F.z, 0, F.flags, L, S);
    case OLG_BATCH_FRESNEL_BANDLIMIT:
        return setup_fresnel(F.in, F.out, F.ny, F.nx, F.dy, F.dx, F.lambda, F.z, 1, F.flags, L, S);
    case OLG_BATCH_ARSS:
        return setup_arss(F.in, F.out, F.ny, F.nx, F.dy, F.dx, F.lambda, F.z, F.s, F.oy, F.ox, F.flags, L, S);
    default: return fail(OLG_ERR_INVALID_ARG, "unknown batch method");
    }
}

} // namespace
} // namespace olg

extern "C" int olg_batch_plan_create(const olg_field *fields, int n_fields, olg_batch_plan *out)
{
    if (!out || !fields || n_fields <= 0) return fail(OLG_ERR_INVALID_ARG, "no fields");
    *out = nullptr;
    for (int i = 0; i < n_fields; ++i) {
        const olg_field &F = fields[i];
        if (int rc = validate(F.in, F.out, F.ny, F.nx)) return rc;
        if (!batch_size_ok(F.ny) || !batch_size_ok(F.nx))
            return fail(OLG_ERR_UNSUPPORTED_SIZE, "batched fields must be powers of two in [256, 4096]");
    }
    if (int rc = ensure_twiddles()) return rc;
    int dev = 0;
    if (cudaError_t e = cudaGetDevice(&dev); e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    auto *plan = new olg_batch_plan_s();
    plan->n = n_fields;
    plan->fields.assign(fields, fields + n_fields);
    plan->dev = dev;
    const long long direct_px = g_batch_direct_pixels.load();
    plan->direct.resize(n_fields);
    for (int i = 0; i < n_fields; ++i) plan->direct[i] = (long long)fields[i].ny * fields[i].nx >= direct_px;
    // device memory: [PropParams x n][ChirpAxis jobs][items][done 3n][target 3n][head, err][per-field scratch]
    std::vector<PropSetup> setups(n_fields);
    std::vector<ChirpAxis> jobs;
    std::vector<BatchItem> items;
    std::vector<int> target(3 * n_fields, 0);
    size_t o = 0;
    const size_t offP = o; o += align_up(sizeof(PropParams) * n_fields, 256);
    // at most two axes per field
    const size_t offJ = o; o += align_up(sizeof(ChirpAxis) * 2 * n_fields, 256);
    // item count: chirp <= 4 per field, rows and column tiles per field
    size_t n_items_max = 0;
    for (auto &F : plan->fields) {
        const int NX = 2 * F.nx, NY = 2 * F.ny;
        const int rows = (F.ny + brow_nseq(NX) - 1) / brow_nseq(NX);
        const int cols = (NX + bcol_c(NY) - 1) / bcol_c(NY);
        n_items_max += 4 + 2 * rows + cols;
    }
    const size_t offI = o; o += align_up(sizeof(BatchItem) * n_items_max, 256);
    const size_t offC = o; o += align_up(sizeof(int) * (6 * n_fields + 2), 256);
    plan->ws_off.resize(n_fields);
    for (int i = 0; i < n_fields; ++i) {
        plan->ws_off[i] = o;
        o += align_up(layout_bytes(plan->fields[i].ny, plan->fields[i].nx, nullptr, nullptr), 256);
    }
    plan->bytes = o;
    cudaError_t e = cudaMalloc(&plan->mem, plan->bytes);
    if (e != cudaSuccess) {
        delete plan;
        return cuda_fail(e, "cudaMalloc (batch plan)");
    }
    // per-field setup, chirp jobs and the item queue
    std::vector<int> order(n_fields);
    for (int i = 0; i < n_fields; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (long)plan->fields[a].ny * plan->fields[a].nx > (long)plan->fields[b].ny * plan->fields[b].nx;
    });
    for (int i = 0; i < n_fields; ++i) {
        const olg_field &F = plan->fields[i];
        Layout L;
        layout_bytes(F.ny, F.nx, &L, plan->mem + plan->ws_off[i]);
        if (int rc = field_setup(F, L, &setups[i])) {
            cudaFree(plan->mem);
            delete plan;
            return rc;
        }
        setups[i].P.coherent = 1;
        if (setups[i].chirps && !plan->direct[i]) {
            for (int a = 0; a < 2; ++a) {
                const ChirpAxis &A = a ? setups[i].ay : setups[i].ax;
                const int jidx = (int)jobs.size();
                jobs.push_back(A);
                items.push_back({i, BK_CHIRP, 2 * jidx + 0, A.L, 1});
                target[3 * i] += 1;
                if (A.ta || A.tb) {
                    items.push_back({i, BK_CHIRP, 2 * jidx + 1, A.L, 1});
                    target[3 * i] += 1;
                }
            }
        }
    }
    for (int kind = BK_FWD; kind <= BK_INV; ++kind)
        for (int i : order) {
            if (plan->direct[i]) continue;
            const olg_field &F = plan->fields[i];
            const int NX = 2 * F.nx, NY = 2 * F.ny;
            if (kind == BK_COLS) {
                const int C = bcol_c(NY), units = (NX + C - 1) / C;
                for (int u = 0; u < units; u += BATCH_UNITS_PER_ITEM)
                    items.push_back({i, kind, u, NY, std::min(BATCH_UNITS_PER_ITEM, units - u)});
                target[3 * i + 2] = units;
            } else {
                const int R = brow_nseq(NX), units = (F.ny + R - 1) / R;
                for (int u = 0; u < units; u += BATCH_UNITS_PER_ITEM)
                    items.push_back({i, kind, u, NX, std::min(BATCH_UNITS_PER_ITEM, units - u)});
                if (kind == BK_FWD) target[3 * i + 1] = units;
            }
        }
    plan->n_items = (int)items.size();
    std::vector<PropParams> Ps(n_fields);
    for (int i = 0; i < n_fields; ++i) Ps[i] = setups[i].P;
    e = cudaMemcpy(plan->mem + offP, Ps.data(), sizeof(PropParams) * n_fields, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !jobs.empty())
        e = cudaMemcpy(plan->mem + offJ, jobs.data(), sizeof(ChirpAxis) * jobs.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(plan->mem + offI, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(plan->mem + offC + sizeof(int) * 3 * n_fields, target.data(), sizeof(int) * 3 * n_fields,
                       cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(plan->mem);
        delete plan;
        return cuda_fail(e, "uploading the batch plan");
    }
    int* C = (int *)(plan->mem + offC);
    plan->D.P = (const PropParams *)(plan->mem + offP);
    plan->D.jobs = (const ChirpAxis *)(plan->mem + offJ);
    plan->D.items = (const BatchItem *)(plan->mem + offI);
    plan->D.n_items = plan->n_items;
    plan->D.done = C;
    plan->D.target = C + 3 * n_fields;
    plan->D.head = C + 6 * n_fields;
    plan->D.err = C + 6 * n_fields + 1;
    plan->counters_off = offC;
    plan->counters_bytes = sizeof(int) * 3 * n_fields;
    plan->grid = sm_count() * BATCH_CTAS_PER_SM;
    e = cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, BATCH_SMEM);
    if (e != cudaSuccess) {
        cudaFree(plan->mem);
        delete plan;
        return cuda_fail(e, "cudaFuncSetAttribute(k_batch)");
    }
    *out = plan;
    return OLG_OK;
}

namespace olg {
namespace {

// one field through the single-field passes, in the plan's workspace
int batch_field_direct(olg_batch_plan plan, int i, cudaStream_t st)
{
    const olg_field &F = plan->fields[i];
    Layout L;
    layout_bytes(F.ny, F.nx, &L, plan->mem + plan->ws_off[i]);
    PropSetup S;
    if (int rc = field_setup(F, L, &S)) return rc;
    return run_setup(S, st);
}

} // namespace
} // namespace olg

extern "C" int olg_batch_execute(olg_batch_plan plan, olg_stream_t stream)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    cudaStream_t st = (cudaStream_t)stream;
    // reset the done counters, the ticket and the error word (target stays)
    cudaError_t e = cudaMemsetAsync(plan->D.done, 0, plan->counters_bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(plan->D.head, 0, 2 * sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync (batch counters)");
    if (plan->n_items > 0) {
        k_batch<<<plan->grid, BATCH_NT, BATCH_SMEM, st>>>(plan->D);
        count_launch();
        if (int rc = check_launch("k_batch")) return rc;
    }
    for (int i = 0; i < plan->n; ++i)
        if (plan->direct[i])
            if (int rc = batch_field_direct(plan, i, st)) return rc;
    return OLG_OK;
}

extern "C" int olg_batch_execute_serial(olg_batch_plan plan, olg_stream_t stream)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    cudaStream_t st = (cudaStream_t)stream;
    for (int i = 0; i < plan->n; ++i)
        if (int rc = batch_field_direct(plan, i, st)) return rc;
    return OLG_OK;
}

extern "C" long long olg_batch_direct_pixels(long long pixels)
{
    if (pixels > 0) return g_batch_direct_pixels.exchange(pixels);
    return g_batch_direct_pixels.load();
}

extern "C" int olg_batch_plan_direct_fields(olg_batch_plan plan)
{
    if (!plan) return 0;
    int n = 0;
    for (char d : plan->direct) n += d ? 1 : 0;
    return n;
}

extern "C" int olg_batch_check(olg_batch_plan plan)
{
    if (!plan) return fail(OLG_ERR_INVALID_ARG, "null plan");
    int err = 0;
    cudaError_t e = cudaMemcpy(&err, plan->D.err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "reading the batch error word");
    return err ? fail(OLG_ERR_CUDA, "a batched item gave up on a bounded wait") : OLG_OK;
}

extern "C" int olg_batch_plan_items(olg_batch_plan plan) { return plan ? plan->n_items : 0; }

extern "C" int olg_batch_plan_destroy(olg_batch_plan plan)
{
    if (!plan) return OLG_OK;
    cudaError_t e = cudaFree(plan->mem);
    delete plan;
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, "cudaFree (batch plan)");
}

// ------------------------------------------- multi-plane phase optimisation
// Phase-only hologram phi (ny x nx) propagated by ASM to P depth planes;
// loss L = sum_p mean((|A_p e^{i phi}|^2 - t_p)^2).  Per plane: the forward
// propagation, whose pass 3 writes the seed dL/dv* = (2/n)(|v|^2 - t) v (and
// sums the loss), then the adjoint propagation (conjugate transfer function)
// of the seed, accumulated into g = dL/du*.  No plane's field is stored.
// dL/dphi = -2 Im(u conj(g)).  For padded heights 256..8192 the planes share
// the forward spectrum of e^{i phi} and sum their adjoint spectra (spec.cu);
// otherwise each plane runs two full three-pass propagations.
namespace olg {

__global__ void k_phase_grad(const float *phi, const float2 *g, float *grad, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float s, c;
        sincosf(phi[i], &s, &c);
        const float2 G = g[i];
        grad[i] = 2.0f * (c * G.y - s * G.x);
    }
}

__global__ void k_adam(float *phi, float *m, float *v, const float2 *g, long n, float lr, float b1, float b2, float eps,
                       float bc1, float bc2)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float ph = phi[i];
        float s, c;
        sincosf(ph, &s, &c);
        const float2 G = g[i];
        const float gr = 2.0f * (c * G.y - s * G.x);
        const float mm = b1 * m[i] + (1.0f - b1) * gr;
        const float vv = b2 * v[i] + (1.0f - b2) * gr * gr;
        m[i] = mm;
        v[i] = vv;
        phi[i] = ph - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
    }
}

__global__ void k_loss_scale(double *loss, double s) { *loss *= s; }

int elem_grid(long n)
{
    long g = (n + 255) / 256;
    return (int)(g > 152 * 8 ? 152 * 8 : (g < 1 ? 1 : g));
}

PropParams asm_params(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z, bool conj,
                      const Layout &L)
{
    PropParams P = base_params(in, out, ny, nx, L);
    const double NX = 2.0 * nx, NY = 2.0 * ny;
    const double du = 1.0 / (dx * NX), dv = 1.0 / (dy * NY);
    const double zl = z / lambda;
    P.method = M_ASM;
    P.conj = conj ? 1 : 0;
    P.scale = (float)(1.0 / (NX * NY));
    P.c0 = frac_host(zl);
    set_quad(P.ax_hi, P.ax_lo, z * lambda * du * du / 2.0);
    set_quad(P.ay_hi, P.ay_lo, z * lambda * dv * dv / 2.0);
    P.tx = (float)(lambda * lambda * du * du);
    P.ty = (float)(lambda * lambda * dv * dv);
    P.zl = (float)zl;
    return P;
}

// [propagation layout][seed][g][loss][F0: NY x NX][G: NY x NX]
size_t phase_ws(int ny, int nx, size_t *off_seed, size_t *off_g, size_t *off_loss, size_t *off_spec = nullptr)
{
    const size_t lb = layout_bytes(ny, nx, nullptr, nullptr);
    const size_t f = align_up((size_t)ny * nx * sizeof(float2), 256);
    if (off_seed) *off_seed = lb;
    if (off_g) *off_g = lb + f;
    if (off_loss) *off_loss = lb + 2 * f;
    if (off_spec) *off_spec = lb + 2 * f + 256;
    return lb + 2 * f + 256 + 2 * 4 * f;
}

int phase_loss_grad(const float *phi, const float *targets, const double *z, int np, int ny, int nx, double dy,
                    double dx, double lambda, char *ws, float2 *g, double *loss, cudaStream_t st)
{
    size_t os, og, ol;
    phase_ws(ny, nx, &os, &og, &ol);
    Layout L;
    layout_bytes(ny, nx, &L, ws);
    float2 *seed = (float2 *)(ws + os);
    const long n = (long)ny * nx;
    cudaError_t e = cudaMemsetAsync(loss, 0, sizeof(double), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(loss)");
    if (spec_cols_ok(2 * ny)) {
        // Every plane's forward propagation starts from the same e^{i phi}: its
        // padded spectrum F0 is formed once.  The adjoints are linear in their
        // seeds, so their conjugate-transfer-function spectra add into G and
        // one inverse transform gives g.  Per plane this leaves one inverse
        // and one forward column transform and two row passes.
        size_t ospec;
        phase_ws(ny, nx, nullptr, nullptr, nullptr, &ospec);
        float2 *F0 = (float2 *)(ws + ospec);
        float2 *G = F0 + (size_t)4 * n;
        SpecArgs A{};
        A.ny = ny; A.NY = 2 * ny; A.NX = 2 * nx;
        PropParams R = asm_params(nullptr, nullptr, ny, nx, dy, dx, lambda, z[0], false, L);
        R.in_phase = phi;
        if (int rc = rows_pass(R, false, st)) return rc;
        A.in = L.S; A.out = F0; A.tf = 0; A.accumulate = 0;
        if (int rc = spec_cols(A, false, st)) return rc;
        for (int p = 0; p < np; ++p) {
            PropParams F = asm_params(nullptr, seed, ny, nx, dy, dx, lambda, z[p], false, L);
            F.post_mode = OP_SEED;
            F.target = targets + (size_t)p * n;
            F.seed_scale = (float)(2.0 / (double)n);
            F.loss = loss;
            A.in = F0; A.out = L.S; A.tf = 1; A.accumulate = 0; A.P = F;
            if (int rc = spec_cols(A, true, st)) return rc;
            PropParams B = asm_params(seed, nullptr, ny, nx, dy, dx, lambda, z[p], true, L);
            if (2 * nx >= 256) {
                // the seed goes from the forward's inverse row FFT to the
                // adjoint's forward row FFT in registers
                if (int rc = rows_seed_pass(F, st)) return rc;
            } else {
                if (int rc = rows_pass(F, true, st)) return rc;
                if (int rc = rows_pass(B, false, st)) return rc;
            }
            A.in = L.S; A.out = G; A.tf = 1; A.accumulate = p > 0 ? 1 : 0; A.P = B;
            if (int rc = spec_cols(A, false, st)) return rc;
        }
        A.in = G; A.out = L.S; A.tf = 0; A.accumulate = 0;
        if (int rc = spec_cols(A, true, st)) return rc;
        PropParams Gp = asm_params(nullptr, g, ny, nx, dy, dx, lambda, z[0], false, L);
        if (int rc = rows_pass(Gp, true, st)) return rc;
        k_loss_scale<<<1, 1, 0, st>>>(loss, 1.0 / (double)n);
        count_launch();
        return check_launch("k_loss_scale");
    }
    for (int p = 0; p < np; ++p) {
        PropParams F = asm_params(nullptr, seed, ny, nx, dy, dx, lambda, z[p], false, L);
        F.in_phase = phi;
        F.post_mode = OP_SEED;
        F.target = targets + (size_t)p * n;
        F.seed_scale = (float)(2.0 / (double)n);
        F.loss = loss;
        if (int rc = run_passes(F, st)) return rc;
        PropParams B = asm_params(seed, g, ny, nx, dy, dx, lambda, z[p], true, L);
        B.accumulate = p > 0 ? 1 : 0;
        if (int rc = run_passes(B, st)) return rc;
    }
    k_loss_scale<<<1, 1, 0, st>>>(loss, 1.0 / (double)n);
    count_launch();
    return check_launch("k_loss_scale");
}

int phase_checks(const void *phi, const void *targets, const double *z, int np, int ny, int nx)
{
    if (!phi || !targets || !z || np <= 0) return fail(OLG_ERR_INVALID_ARG, "null pointer or no planes");
    if (((uintptr_t)phi & 7) || ((uintptr_t)targets & 7)) return fail(OLG_ERR_INVALID_ARG, "phi / targets must be 8-byte aligned");
    if (!is_pow2(nx) || !is_pow2(ny) || nx < 16 || ny < 16 || 2 * nx > FFT_MAX || 2 * ny > FFT_MAX)
        return fail(OLG_ERR_UNSUPPORTED_SIZE, "ny, nx must be powers of two in [16, 4096]");
    return OLG_OK;
}

} // namespace olg

extern "C" size_t olg_phase_opt_workspace_bytes(int ny, int nx)
{
    if (ny <= 0 || nx <= 0) return 0;
    return phase_ws(ny, nx, nullptr, nullptr, nullptr);
}

extern "C" int olg_phase_loss_grad(const float *phi, const float *targets, const double *z, int n_planes, int ny,
                                   int nx, double dy, double dx, double lambda, float *grad, double *loss,
                                   void *work, size_t work_bytes, olg_stream_t stream)
{
    if (int rc = phase_checks(phi, targets, z, n_planes, ny, nx)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, phase_ws(ny, nx, nullptr, nullptr, nullptr), st)) return rc;
    size_t os, og, ol;
    phase_ws(ny, nx, &os, &og, &ol);
    char *ws = (char *)sc.ptr;
    float2 *g = (float2 *)(ws + og);
    double *dl = loss ? loss : (double *)(ws + ol);
    if (int rc = phase_loss_grad(phi, targets, z, n_planes, ny, nx, dy, dx, lambda, ws, g, dl, st)) return rc;
    if (grad) {
        const long n = (long)ny * nx;
        k_phase_grad<<<elem_grid(n), 256, 0, st>>>(phi, g, grad, n);
        count_launch();
        return check_launch("k_phase_grad");
    }
    return OLG_OK;
}

extern "C" int olg_phase_adam_step(float *phi, float *m, float *v, const float *targets, const double *z, int n_planes,
                                   int ny, int nx, double dy, double dx, double lambda, double lr, double beta1,
                                   double beta2, double eps, int step, double *loss, void *work, size_t work_bytes,
                                   olg_stream_t stream)
{
    if (int rc = phase_checks(phi, targets, z, n_planes, ny, nx)) return rc;
    if (!m || !v || step < 1) return fail(OLG_ERR_INVALID_ARG, "Adam state missing or step < 1");
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, phase_ws(ny, nx, nullptr, nullptr, nullptr), st)) return rc;
    size_t os, og, ol;
    phase_ws(ny, nx, &os, &og, &ol);
    char *ws = (char *)sc.ptr;
    float2 *g = (float2 *)(ws + og);
    double *dl = loss ? loss : (double *)(ws + ol);
    if (int rc = phase_loss_grad(phi, targets, z, n_planes, ny, nx, dy, dx, lambda, ws, g, dl, st)) return rc;
    const long n = (long)ny * nx;
    const float bc1 = (float)(1.0 - std::pow(beta1, step)), bc2 = (float)(1.0 - std::pow(beta2, step));
    k_adam<<<elem_grid(n), 256, 0, st>>>(phi, m, v, g, n, (float)lr, (float)beta1, (float)beta2, (float)eps, bc1, bc2);
    count_launch();
    return check_launch("k_adam");
}

// ------------------------------------------------------- no-allocation entry
// Scratch for olg_asm_prop_noalloc_c64, owned by the library module itself:
// 17 MiB per device, enough for any field with ny * nx <= 1,048,576
// (1024 x 1024, 512 x 2048, ...).  Every device that loads the library keeps
// this array until the process exits.
namespace {
constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)17 << 20;
constexpr long NOALLOC_MAX_PIXELS = 1L << 20;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {};
} // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch on the current device.  The name
// g_noalloc_scratch in host code is only a host-side handle for the symbol,
// so the address is looked up once per device (with that device current) and
// cached; kernels receive this pointer like any caller-provided workspace.
static int noalloc_scratch(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return fail(OLG_ERR_INVALID_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return OLG_OK;
}

extern "C" int olg_asm_prop_noalloc_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx,
                                        double lambda, double z, int flags, olg_stream_t stream)
{
    if ((long)ny * (long)nx > NOALLOC_MAX_PIXELS || layout_bytes(ny, nx, nullptr, nullptr) > NOALLOC_SCRATCH_BYTES)
        return fail(OLG_ERR_WORKSPACE, "olg_asm_prop_noalloc_c64: ny * nx must be <= 1048576 (its static scratch is "
                                       "17 MiB); use olg_asm_prop_c64 with a workspace for larger fields");
    // mixed-radix lengths allocate their twiddle table on first use
    if (!is_pow2(ny) || !is_pow2(nx))
        return fail(OLG_ERR_UNSUPPORTED_SIZE, "olg_asm_prop_noalloc_c64 takes power-of-two ny, nx");
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    void *scratch = nullptr;
    if (int rc = noalloc_scratch(&scratch)) return rc;
    // Pass 1 writes every element of the scratch spectrum before passes 2 and 3
    // read it, so the previous call's contents never leak into this one and
    // nothing needs clearing.
    return olg_asm_prop_c64(u_in, u_out, ny, nx, dy, dx, lambda, z, flags, scratch, NOALLOC_SCRATCH_BYTES, stream);
}
