// propk.cuh -- device side of the fused propagation passes: launch shapes,
// the pass kernels, the chirp kernels, and the host templates that launch
// them.  Each translation unit that includes it holds its own copy of the
// twiddle tables (the library is built without relocatable device code) and
// registers it with ensure_twiddles(), which uploads every copy once per
// CUDA context.
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>

#include "common.cuh"
#include "fft.cuh"
#include "fft2.cuh"
#include "fftp.cuh"
#include "propdev.cuh"
#include "prophost.cuh"
#include "propmr.cuh"

namespace olg {

static __device__ float2 g_tw[FFT_MAX];
// the same table as (c, c, s, s) for the paired-sequence passes
static __device__ float4 g_tw4[FFT_MAX];

static int upload_twiddles_here(const float2 *t, const float4 *t4)
{
    cudaError_t e = cudaMemcpyToSymbol(g_tw, t, sizeof(float2) * FFT_MAX);
    if (e != cudaSuccess) return cuda_fail(e, "twiddle table upload");
    e = cudaMemcpyToSymbol(g_tw4, t4, sizeof(float4) * FFT_MAX);
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, "paired twiddle table upload");
}
[[maybe_unused]] static const int g_tw_registered = register_twiddle_uploader(&upload_twiddles_here);

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
        for (int k = 0; k < 16; ++k) sm[q * SS + 17 * j + k] = v[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, -1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j) + r * pstride<B>()];
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
        for (int k = 0; k < 16; ++k) sm[q * SS + 17 * j + k] = v[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, +1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j) + r * pstride<B>()];
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
        for (int k = 0; k < 16; ++k) sm[17 * C * j + c + k * C] = v[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, -1, NT, true, C>(sm, 0, g_tw, tid);
    // forward last stage -> x T(ky, kx) -> inverse first stage, in registers
    float2 vv[BPT][16];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C;
#pragma unroll
        for (int r = 0; r < 16; ++r) vv[t][r] = sm[pidx(j) * C + c + r * (pstride<B>() * C)];
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
        for (int k = 0; k < 16; ++k) sm[17 * C * j + c + k * C] = w[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, +1, NT, true, C>(sm, 0, g_tw, tid);
    // inverse last stage: only the central ny rows, back in place
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[pidx(j) * C + c + r * (pstride<B>() * C)];
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
            for (int k = 0; k < 16; ++k) sm[q * SS + 17 * j + k] = v[outpos<16>(k)];
        }
        fetch(g + gridDim.x);
        __syncthreads();
        mid_stages<N, -1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
        for (int t = 0; t < BPT; ++t) {
            const int b = tid + t * NT, q = b / B, j = b % B, h = g * NSEQ + q;
            float2 v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j) + r * pstride<B>()];
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
            for (int k = 0; k < 16; ++k) sm[q * SS + 17 * j + k] = v[outpos<16>(k)];
        }
        fetch(g + gridDim.x);
        __syncthreads();
        mid_stages<N, +1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
        for (int t = 0; t < BPT; ++t) {
            const int b = tid + t * NT, q = b / B, j = b % B, h = g * NSEQ + q;
            float2 v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j) + r * pstride<B>()];
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
        for (int k = 0; k < 16; ++k) sm[q * SS + 17 * j + k] = v[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, +1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j) + r * pstride<B>()];
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
        for (int k = 0; k < 16; ++k) sm[q * SS + 17 * j + k] = u[t][outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, -1, NT, false, NSEQ>(sm, SS, g_tw, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[q * SS + pidx(j) + r * pstride<B>()];
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
        for (int k = 0; k < 16; ++k) cp_st(sm + q * SS + 17 * j + k, v[outpos<16>(k)]);
    }
    __syncthreads();
    cp_mid_stages<N, -1, NT, false, NSP>(sm, SS, g_tw4, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + 2 * q;
        cpair v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = cp_ld(sm + q * SS + pidx(j) + r * pstride<B>());
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
        for (int k = 0; k < 16; ++k) cp_st(sm + q * SS + 17 * j + k, v[outpos<16>(k)]);
    }
    __syncthreads();
    cp_mid_stages<N, +1, NT, false, NSP>(sm, SS, g_tw4, tid);
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, q = b / B, j = b % B, h = r0 + 2 * q;
        cpair v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = cp_ld(sm + q * SS + pidx(j) + r * pstride<B>());
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
        for (int k = 0; k < 16; ++k) cp_st(sm + 17 * CP * j + c + k * CP, v[outpos<16>(k)]);
    }
    __syncthreads();
    cp_mid_stages<N, -1, NT, true, CP>(sm, 0, g_tw4, tid);
    // forward last stage -> x T(ky, kx) -> inverse first stage, in registers
    cpair vv[BPT][16];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % CP, j = b / CP;
#pragma unroll
        for (int r = 0; r < 16; ++r) vv[t][r] = cp_ld(sm + pidx(j) * CP + c + r * (pstride<B>() * CP));
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
        for (int k = 0; k < 16; ++k) cp_st(sm + 17 * CP * j + c + k * CP, w[outpos<16>(k)]);
    }
    __syncthreads();
    cp_mid_stages<N, +1, NT, true, CP>(sm, 0, g_tw4, tid);
    // inverse last stage: only the central ny rows, back in place
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % CP, j = b / CP, kx = c0 + 2 * c;
        cpair v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = cp_ld(sm + pidx(j) * CP + c + r * (pstride<B>() * CP));
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
// 1024 threads, one butterfly each: twice the resident warps of ColVar<1> at
// the same 64 KB-per-column tile (64 registers, no spills up to 8192)
template <> struct ColVar<11> : Shape<1024, 16384, 1> {};
// variant 10: the persistent TMA-staged column pass (prop_cols_tma.cu),
// padded heights 2048..8192
constexpr int COL_VARIANT_TMA = 10;
constexpr int N_COL_VARIANTS = 12;

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

// ----------------------------------------------------------- launch helpers
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

template <int N, int I, bool INV>
int launch_rows_v(const PropParams &P, cudaStream_t st)
{
    using S = RowShape<N, RowVar<I>>;
    if constexpr (!S::valid) {
        return fail(OLG_ERR_INVALID_ARG, "row variant not valid for this length");
    } else if constexpr (S::PAIRED) {
        const int grid = (P.ny + S::ROWS - 1) / S::ROWS;
        if constexpr (!INV) {
            if (int rc = prep_smem(k_rows_fwd3<N, RowVar<I>>, S::SMEM)) return rc;
            return launch_pdl(k_rows_fwd3<N, RowVar<I>>, grid, S::NT, S::SMEM, st, P, "k_rows_fwd3");
        }
        if (int rc = prep_smem(k_rows_inv3<N, RowVar<I>>, S::SMEM)) return rc;
        return launch_pdl(k_rows_inv3<N, RowVar<I>>, grid, S::NT, S::SMEM, st, P, "k_rows_inv3");
    } else {
        int grid = (P.ny + S::ROWS - 1) / S::ROWS;
        if constexpr (S::PERSIST) grid = std::min(grid, sm_count() * S::MINB);
        if constexpr (!INV) {
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
    case COL_VARIANT_TMA: return N >= 2048 && N <= 8192;
    case 11: return ColShape<N, ColVar<11>>::valid;
    default: return false;
    }
}

constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

template <int N, bool INV>
int launch_rows(const PropParams &P, cudaStream_t st)
{
    if constexpr (N >= 256) {
        switch (g_variant[INV ? 2 : 0][ilog2(N)]) {
        case 1: return launch_rows_v<N, 1, INV>(P, st);
        case 2: return launch_rows_v<N, 2, INV>(P, st);
        case 3: return launch_rows_v<N, 3, INV>(P, st);
        case 4: return launch_rows_v<N, 4, INV>(P, st);
        case 5: return launch_rows_v<N, 5, INV>(P, st);
        case 6: return launch_rows_v<N, 6, INV>(P, st);
        case 7: return launch_rows_v<N, 7, INV>(P, st);
        case 8: return launch_rows_v<N, 8, INV>(P, st);
        case 9: return launch_rows_v<N, 9, INV>(P, st);
        default: return launch_rows_v<N, 0, INV>(P, st);
        }
    } else {
        using C = RowCfg<N>;
        const int grid = (P.ny + C::NSEQ - 1) / C::NSEQ;
        if constexpr (!INV) {
            if (int rc = prep_smem(k_rows_fwd<N>, C::SMEM)) return rc;
            return launch_pdl(k_rows_fwd<N>, grid, C::NT, C::SMEM, st, P, "k_rows_fwd");
        }
        if (int rc = prep_smem(k_rows_inv<N>, C::SMEM)) return rc;
        return launch_pdl(k_rows_inv<N>, grid, C::NT, C::SMEM, st, P, "k_rows_inv");
    }
}

template <int N>
int launch_rows_fwd(const PropParams &P, cudaStream_t st) { return launch_rows<N, false>(P, st); }
template <int N>
int launch_rows_inv(const PropParams &P, cudaStream_t st) { return launch_rows<N, true>(P, st); }

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
        case COL_VARIANT_TMA:
            if constexpr (N >= 2048) return cols_pass_tma(P, st);
            else return fail(OLG_ERR_INVALID_ARG, "TMA column pass: padded heights 2048..8192");
        case 11: return launch_cols_v<N, 11>(P, st);
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


} // namespace olg
