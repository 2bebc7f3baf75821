// cgh_gemm.cu -- Fresnel-form point-cloud CGH as a split-FP16 complex GEMM on
// the 5th-generation tensor cores (tcgen05 + TMA + TMEM, sm_103a).
//
// The Fresnel kernel of the reference (golcgh.h:47-145) is separable per
// point:  exp(i pi ((px w - x_j)^2 + (py h - y_j)^2) / (lambda z_j))
//       = X[w, j] * Y[h, j],   so   U = Y' X^T  with Y'[h, j] = a_j e^{i phi_j} Y[h, j],
// a complex GEMM with M = ny, N = nx, K = n points.  As one real GEMM with the
// real / imaginary parts interleaved on the M side:
//   A (2M x 2K): row 2h = [Re Y', -Im Y'] per point, row 2h+1 = [Im Y', Re Y']
//   B (N  x 2K): row w  = [Re X,  Im X ]
//   D = A B^T (2M x N): D[2h, w] = Re U[h, w], D[2h+1, w] = Im U[h, w].
// Precision: each operand is split into f16 hi + lo (22 significant bits);
// D = A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T accumulated in f32 in TMEM
// (three K segments of one accumulation).  Issued tensor work 3 x 2 x 2M N 2K
// = 24 M N K flop for 8 M N K useful.
//
// k_cgh_gemm_prep  per point, FP64: the x / y phase polynomials as 64-bit
//                  fixed-point fractions of a cycle
// k_cgh_gemm_ops   builds A_hi/A_lo/B_hi/B_lo (f16, K-contiguous, zero padded):
//                  phases stepped row to row exactly in 64-bit integers,
//                  MUFU sin/cos
// k_cgh_gemm<BN>   warp-specialised tcgen05 GEMM, one CTA per tile plus CTAs on
//                  the spare SMs that take the tiles' K tails: warp 0 issues TMA loads into a
//                  2-stage ring, each stage the four f16 tiles of one 64-wide K
//                  range (A hi, A lo: 128 x 64; B hi, B lo: BN x 64; 128-byte
//                  swizzle); warp 1 owns TMEM (two f32 accumulators of BN
//                  columns) and issues the three split products' 128 x BN x 16
//                  MMAs from each stage, chunk by chunk; warps 2-9 add each
//                  finished chunk into f32 registers and add every finished
//                  piece of a tile into the complex64 output.  BN in
//                  {128, ..., 256} is the N tile that pads nx least
//                  (1920 = 8 x 240).
#include <cuda.h>
#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "tc.cuh"

namespace olg {

constexpr int GB_M = 128, GB_K = 64;
constexpr int GB_A_BYTES = GB_M * GB_K * 2;
// N tile widths (multiples of 16 up to 256, the kind::f16 limit at M = 128):
// the host takes the one whose tiles cover nx with the least padding
// (1920 = 8 x 240 exactly, where 256 would pad to 2048).
// Single-SM tiles stage, per 64-wide K range, all four operand tiles (A hi,
// A lo, B hi, B lo) and issue the three split products from them: 12 MMAs
// per 92 KB stage at BN = 240 instead of 4 MMAs per 46 KB, two stages deep.
constexpr int GB_FSTAGES = 2;
template <int BN>
struct GemmTile {
    static_assert(BN % 16 == 0 && BN >= 128 && BN <= 256, "N tile");
    static constexpr int B_BYTES = BN * GB_K * 2;           // a multiple of 1024: SW128 tiles stay aligned
    static constexpr int STAGE = 2 * GB_A_BYTES + 2 * B_BYTES; // A hi, A lo, B hi, B lo
    static constexpr int SMEM = GB_FSTAGES * STAGE + 1024 + 256;
};
constexpr long long GB_WAIT = 4000000000LL; // ~2 s of SM clock per wait

// Per point, the Fresnel phases of the B rows (w) and the A rows (h) as 64-bit
// fixed-point fractions of a cycle (unit 2^-64):  cycles(w) = ax w^2 - bx w + gx
// reduces mod 1 exactly in integer arithmetic (w is an integer, so the
// integer parts of ax and bx drop out), and consecutive rows follow
// P(w + 1) = P(w) + D(w), D(w + 1) = D(w) + 2 ax with no rounding at all.
struct PointCoef {
    unsigned long long ax, bx, gx; // frac(k2 px^2), frac(2 k2 px x), frac(k2 x^2), times 2^64
    unsigned long long ay, by, gy;
    float cr, ci;                  // a_j e^{i phi_j}
};

struct GemmOps {
    const float *pts, *amp, *ph0;
    int n, ny, nx, kp; // kp: K row stride (elements), >= 2n, multiple of 64
    double px, py, lambda;
    PointCoef *coef;
    __half *a_hi, *a_lo, *b_hi, *b_lo;
};

// frac(v) scaled to 2^64.  A double's 53 significant bits sit at or above
// bit 0 of the result for |v| < 2^11 cycles, so the scaling and the
// conversion are exact.
__device__ __forceinline__ unsigned long long frac64(double v)
{
    double f = v - floor(v);
    if (!(f < 1.0)) f = 0.0; // v - floor(v) can round up to 1 for tiny negative v
    return __double2ull_rz(f * 18446744073709551616.0);
}

// 64 threads per CTA: the ~10^4 points spread over every SM (the FP64 work
// per point is a few dozen operations).
constexpr int PREP_THREADS = 64;

__global__ void k_cgh_gemm_prep(GemmOps G)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= G.n) return;
    const double x = G.pts[3 * j], y = G.pts[3 * j + 1], z = G.pts[3 * j + 2];
    const double k2 = 1.0 / (2.0 * G.lambda * z); // cycles per m^2
    PointCoef c;
    c.ax = frac64(k2 * G.px * G.px);
    c.bx = frac64(2.0 * k2 * G.px * x);
    c.gx = frac64(k2 * x * x);
    c.ay = frac64(k2 * G.py * G.py);
    c.by = frac64(2.0 * k2 * G.py * y);
    c.gy = frac64(k2 * y * y);
    // the complex amplitude is stored in FP32: FP32 sincosf (about 1 ulp) suffices
    const float a = G.amp ? G.amp[j] : 1.f;
    float sn = 0.f, cs = 1.f;
    if (G.ph0) sincosf(G.ph0[j], &sn, &cs);
    c.cr = a * cs;
    c.ci = a * sn;
    G.coef[j] = c;
}

// exp(2 pi i P / 2^64): the top 32 bits as a signed fraction of a cycle in
// [-1/2, 1/2), then MUFU sin / cos (about 4e-7 absolute there, below the
// f16 hi + lo representation's 2^-22).
__device__ __forceinline__ float2 cis_fixed(unsigned long long P)
{
    const float rad = (float)(int)(unsigned)(P >> 32) * 1.4629180792671596e-09f; // 2 pi / 2^32
    float s, c;
    __sincosf(rad, &s, &c);
    return make_float2(c, s);
}

// f16 hi + lo of both components (packed conversions)
__device__ __forceinline__ void split2(float2 v, unsigned &hi, unsigned &lo)
{
    const __half2 h = __float22half2_rn(v);
    const float2 b = __half22float2(h);
    const __half2 l = __float22half2_rn(make_float2(v.x - b.x, v.y - b.y));
    hi = *reinterpret_cast<const unsigned *>(&h);
    lo = *reinterpret_cast<const unsigned *>(&l);
}

// grid.x = point j (one per thread), grid.y = block of OPS_ROWS operand rows
// (the nx rows of B, then the ny row pairs of A).  Each thread walks its rows
// with the exact fixed-point recurrence; for each row a warp writes 32
// consecutive points (128 contiguous bytes per f16 plane).
constexpr int OPS_ROWS = 16;

__global__ void k_cgh_gemm_ops(GemmOps G)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (2 * j >= G.kp) return;
    const bool live = j < G.n;
    PointCoef c{};
    if (live) c = G.coef[j];
    const int r0 = blockIdx.y * OPS_ROWS, r1 = min(r0 + OPS_ROWS, G.nx + G.ny);
    // B rows: X[w, j] = exp(2 pi i cycles_x(w))
    const int b1 = min(r1, G.nx);
    if (r0 < b1) {
        const unsigned long long w0 = (unsigned long long)r0;
        unsigned long long P = c.ax * (w0 * w0) - c.bx * w0 + c.gx;
        unsigned long long D = c.ax * (2 * w0 + 1) - c.bx;
        const unsigned long long A2 = c.ax << 1;
        for (int r = r0; r < b1; ++r) {
            unsigned hi = 0u, lo = 0u;
            if (live) split2(cis_fixed(P), hi, lo);
            const size_t o = (size_t)r * G.kp + 2 * j;
            *reinterpret_cast<unsigned *>(G.b_hi + o) = hi;
            *reinterpret_cast<unsigned *>(G.b_lo + o) = lo;
            P += D;
            D += A2;
        }
    }
    // A rows: Y'[h, j] = a_j e^{i phi_j} exp(2 pi i cycles_y(h)); row 2h holds
    // [re, -im] per point, row 2h + 1 [im, re]
    const int a0 = max(r0, G.nx);
    if (a0 < r1) {
        const unsigned long long h0 = (unsigned long long)(a0 - G.nx);
        unsigned long long P = c.ay * (h0 * h0) - c.by * h0 + c.gy;
        unsigned long long D = c.ay * (2 * h0 + 1) - c.by;
        const unsigned long long A2 = c.ay << 1;
        for (int r = a0; r < r1; ++r) {
            unsigned hi = 0u, lo = 0u;
            if (live) {
                const float2 e = cis_fixed(P);
                split2(make_float2(c.cr * e.x - c.ci * e.y, c.cr * e.y + c.ci * e.x), hi, lo);
            }
            const int h = r - G.nx;
            const size_t o0 = (size_t)(2 * h) * G.kp + 2 * j, o1 = o0 + G.kp;
            // the high 16 bits hold the imaginary half
            *reinterpret_cast<unsigned *>(G.a_hi + o0) = hi ^ 0x80000000u;
            *reinterpret_cast<unsigned *>(G.a_lo + o0) = lo ^ 0x80000000u;
            *reinterpret_cast<unsigned *>(G.a_hi + o1) = __byte_perm(hi, 0u, 0x1032);
            *reinterpret_cast<unsigned *>(G.a_lo + o1) = __byte_perm(lo, 0u, 0x1032);
            P += D;
            D += A2;
        }
    }
}

// ------------------------------------------- adjoint (transposed sum)
// g_j = sum_{h,w} conj(X[w, j] Y[h, j]) G[h, w] (unit-weight kernels) as
//   T = G conj(X)          (M = ny, N = points, K = nx: the same GEMM)
//   g_j = sum_h conj(Y[h, j]) T[h, j]   (a per-point reduction over h)
// A holds G scaled by 2^-e (e from max |Re G|, |Im G|: the f16 operands stay
// in [-1, 1]; the scale is undone exactly in the reduction), rows 2h / 2h + 1
// as [re, -im] / [im, re] per column; B row j holds conj(X[., j]) as
// [re, -im] per column, stepped along w with the fixed-point recurrence.

// max over |Re G|, |Im G| into *mx (non-negative floats order as their bits)
__global__ void k_cgh_absmax(const float2 *G, long long count, unsigned *mx)
{
    float m = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
        const float2 v = G[i];
        m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, __float_as_uint(m));
}

// 2^-e with max = m 2^e, m in [0.5, 1); 1 for a zero or non-finite max
__device__ __forceinline__ float adj_scale(unsigned mx)
{
    const float m = __uint_as_float(mx);
    if (!(m > 0.f) || !(m < INFINITY)) return 1.f;
    int e = 0;
    frexpf(m, &e);
    return ldexpf(1.f, -e);
}

// A: grid.x over K columns (kp / 2 of them, the padding written as zeros),
// grid.y over rows h
__global__ void k_cgh_adjt_aops(const float2 *G, int ny, int nx, int kp, const unsigned *mx, __half *a_hi,
                                __half *a_lo)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x, h = blockIdx.y;
    if (w >= kp / 2 || h >= ny) return;
    unsigned hi = 0u, lo = 0u;
    if (w < nx) {
        const float s = adj_scale(*mx);
        const float2 v = G[(size_t)h * nx + w];
        split2(make_float2(v.x * s, v.y * s), hi, lo);
    }
    const size_t o0 = (size_t)(2 * h) * kp + 2 * w, o1 = o0 + kp;
    *reinterpret_cast<unsigned *>(a_hi + o0) = hi ^ 0x80000000u;
    *reinterpret_cast<unsigned *>(a_lo + o0) = lo ^ 0x80000000u;
    *reinterpret_cast<unsigned *>(a_hi + o1) = __byte_perm(hi, 0u, 0x1032);
    *reinterpret_cast<unsigned *>(a_lo + o1) = __byte_perm(lo, 0u, 0x1032);
}

// B: one thread per (point j, 16 columns from 16 blockIdx.y), 64 contiguous
// bytes per f16 plane
__global__ void k_cgh_adjt_bops(GemmOps G)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= G.n) return;
    const int w0 = blockIdx.y * 16;
    const PointCoef c = G.coef[j];
    const unsigned long long u0 = (unsigned long long)w0;
    unsigned long long P = c.ax * (u0 * u0) - c.bx * u0 + c.gx;
    unsigned long long D = c.ax * (2 * u0 + 1) - c.bx;
    const unsigned long long A2 = c.ax << 1;
    unsigned hi[16], lo[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        hi[i] = 0u;
        lo[i] = 0u;
        if (w0 + i < G.nx) {
            const float2 e = cis_fixed(P);
            split2(make_float2(e.x, -e.y), hi[i], lo[i]);
        }
        P += D;
        D += A2;
    }
    uint4 *dh = reinterpret_cast<uint4 *>(G.b_hi + (size_t)j * G.kp + 2 * w0);
    uint4 *dl = reinterpret_cast<uint4 *>(G.b_lo + (size_t)j * G.kp + 2 * w0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        dh[q] = make_uint4(hi[4 * q], hi[4 * q + 1], hi[4 * q + 2], hi[4 * q + 3]);
        dl[q] = make_uint4(lo[4 * q], lo[4 * q + 1], lo[4 * q + 2], lo[4 * q + 3]);
    }
}

// part[b][j] = sum over the rows h of band b of conj(Y[h, j]) T[h, j]
constexpr int ADJT_BAND = 64;
__global__ void k_cgh_adjt_rows(const PointCoef *coef, const float2 *T, int n, int ny, float2 *part)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (j >= n) return;
    const int h0 = b * ADJT_BAND, h1 = min(ny, h0 + ADJT_BAND);
    const PointCoef c = coef[j];
    const unsigned long long u0 = (unsigned long long)h0;
    unsigned long long P = c.ay * (u0 * u0) - c.by * u0 + c.gy;
    unsigned long long D = c.ay * (2 * u0 + 1) - c.by;
    const unsigned long long A2 = c.ay << 1;
    float2 acc = make_float2(0.f, 0.f);
    for (int h = h0; h < h1; ++h) {
        const float2 e = cis_fixed(P), t = T[(size_t)h * n + j];
        acc.x = fmaf(e.x, t.x, fmaf(e.y, t.y, acc.x)); // conj(e) t
        acc.y = fmaf(e.x, t.y, fmaf(-e.y, t.x, acc.y));
        P += D;
        D += A2;
    }
    part[(size_t)b * n + j] = acc;
}

// g_j (+)= 2^e sum_b part[b][j], bands added in a fixed order
__global__ void k_cgh_adjt_sum(const float2 *part, int bands, int n, const unsigned *mx, float2 *g, int accumulate)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float2 s = make_float2(0.f, 0.f);
    for (int b = 0; b < bands; ++b) {
        const float2 v = part[(size_t)b * n + j];
        s.x += v.x;
        s.y += v.y;
    }
    const float inv = 1.f / adj_scale(*mx); // a power of two: exact
    s.x *= inv;
    s.y *= inv;
    if (accumulate) {
        const float2 o = g[j];
        s.x += o.x;
        s.y += o.y;
    }
    g[j] = s;
}

struct GemmParams {
    int m2, n, kblocks; // rows of D (2 ny), columns (nx), K blocks of 64 per segment
    int tiles_n;        // N tiles across D
    int tiles;          // 128 x BN tiles of D
    int total;          // K steps per tile (kblocks: all three split products per step)
    int split;          // K steps a tile's own unit does
    int extra;          // units beyond `tiles` that do the rest [split, total)
    int vec4;           // U is 16-byte aligned and n even: two complex values per atomic
    int chunk;          // K blocks per TMEM accumulation before the f32 register add
    float2 *U;          // added to with atomics (zeroed first unless accumulating)
    int *err;
};

// Work split.  CTA c < tiles does tile c over K blocks [0, split); when there
// are fewer tiles than SMs (1920 x 1080: 136 tiles, 152 SMs) the `extra` CTAs
// do the remaining [split, total) of tiles e, e + extra, e + 2 extra, ... so
// that every SM gets about the same tensor work.  The tile CTAs walk K in
// lockstep (their A / B blocks are shared through L2), and the extra CTAs'
// K range is a small slice of the operands that L2 holds.  Each piece (tile,
// K range) is one accumulation, added into U with atomics when it ends; a
// tile's two pieces add in either order.
// `u` is the CTA (single-SM tiles) or the CTA pair (two-SM tiles).
__device__ __forceinline__ int gemm_pieces(const GemmParams &P, int u)
{
    if (u < P.tiles) return 1;
    const int e = u - P.tiles;
    return e < P.tiles ? (P.tiles - e + P.extra - 1) / P.extra : 0;
}
__device__ __forceinline__ void gemm_piece(const GemmParams &P, int u, int p, int total, int &t, int &k0, int &k1)
{
    if (u < P.tiles) {
        t = u;
        k0 = 0;
        k1 = P.split;
    } else {
        t = u - P.tiles + p * P.extra;
        k0 = P.split;
        k1 = total;
    }
}

// Accumulation within a piece: the MMA warp writes chunks of
// ceil(P.chunk / 3) K steps (each step: the three split products over a
// 64-wide K range) alternately into two TMEM accumulators (BN columns each);
// the 8 epilogue warps add every finished chunk into f32 registers (rounded
// adds) while the next chunk runs, so the tensor pipe's own accumulation
// never spans more than 3 x 64 x 3 = 576 products at the default P.chunk = 8.
constexpr int GB_EPI_WARPS = 8;
constexpr int GB_THREADS = 64 + 32 * GB_EPI_WARPS;
constexpr uint32_t GB_TMEM_COLS = 512; // two accumulators, at columns 0 and 256

// Epilogue warps: warp w drains TMEM lanes [32 (w % 4), +32) of columns
// [128 half, min(BN, 128 half + 128)), half = (w - 2) / 4, in chunks of 16
// (every TMEM load starts on a 16-column boundary).  PAIR keeps two loads in
// flight per wait; at 168 registers per thread that compiles without spills
// for BN = 224 and 240 only (the other widths spill 20-44 bytes paired; 192
// spills 32 bytes either way).
template <bool PAIR>
__device__ __forceinline__ void drain_cols(uint32_t base, int nch, float (&acc)[128])
{
#pragma unroll
    for (int cc = 0; cc < 8; cc += PAIR ? 2 : 1) {
        if (PAIR && cc + 1 < nch) {
            uint32_t r0[16], r1[16];
            tmem_ld_async(base + 16 * cc, r0);
            tmem_ld_async(base + 16 * cc + 16, r1);
            tmem_wait_ld();
            tmem_regs_ready(r0);
            tmem_regs_ready(r1);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                acc[16 * cc + i] += __uint_as_float(r0[i]);
                acc[16 * cc + 16 + i] += __uint_as_float(r1[i]);
            }
        } else if (cc < nch) {
            uint32_t r0[16];
            tmem_ld_async(base + 16 * cc, r0);
            tmem_wait_ld();
            tmem_regs_ready(r0);
#pragma unroll
            for (int i = 0; i < 16; ++i) acc[16 * cc + i] += __uint_as_float(r0[i]);
        }
    }
}

// Add this warp's columns into U.  Lanes 2i / 2i + 1 hold the Re / Im rows of
// one hologram row h: in each 16-column chunk the even lane adds the first 8
// columns and the odd lane the last 8, each forming complex values from its
// own accumulator and its partner's (shuffled).
__device__ __forceinline__ void store_cols(const GemmParams &P, const float (&acc)[128], int nch, bool store,
                                           bool odd, int h, int cbase)
{
#pragma unroll
    for (int cc = 0; cc < 8; ++cc) {
        if (cc >= nch) break; // warp-uniform
        float o[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) o[i] = __shfl_xor_sync(0xffffffffu, acc[16 * cc + i], 1);
        if (!store) continue;
        const int cb = cbase + 16 * cc + (odd ? 8 : 0);
        float2 *dst = P.U + (size_t)h * P.n + cb;
        if (P.vec4 && cb + 8 <= P.n) {
#pragma unroll
            for (int i = 0; i < 8; i += 2) {
                const float4 v = odd ? make_float4(o[8 + i], acc[16 * cc + 8 + i], o[9 + i], acc[16 * cc + 9 + i])
                                     : make_float4(acc[16 * cc + i], o[i], acc[16 * cc + i + 1], o[i + 1]);
                atomicAdd(reinterpret_cast<float4 *>(dst + i), v);
            }
        } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                if (cb + i >= P.n) break;
                const float re = odd ? o[8 + i] : acc[16 * cc + i];
                const float im = odd ? acc[16 * cc + 8 + i] : o[i];
                atomicAdd(dst + i, make_float2(re, im));
            }
        }
    }
}

// 320 threads: ten warps over four SM sub-partitions (three on two of them)
// cap the registers at 168 per thread.
template <int BN>
__global__ void __launch_bounds__(GB_THREADS, 1)
    k_cgh_gemm(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
               const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl, GemmParams P)
{
    using T = GemmTile<BN>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    // stage s: [A hi | A lo | B hi | B lo]
    auto stage = [&](int s) { return smem + s * T::STAGE; };
    uint64_t *full = (uint64_t *)(smem + GB_FSTAGES * T::STAGE);
    uint64_t *empty = full + GB_FSTAGES;
    uint64_t *tfull = empty + GB_FSTAGES; // [2]
    uint64_t *tfree = tfull + 2;          // [2]
    uint32_t *tmem_slot = (uint32_t *)(tfree + 2);
    volatile int *fault = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = P.total; // K steps per tile (kblocks)
    const int np = gemm_pieces(P, blockIdx.x);
    // K steps per TMEM accumulation: P.chunk counts one-product K blocks
    const int chunk = max(1, (P.chunk + 2) / 3);

    if (threadIdx.x == 0) {
        for (int s = 0; s < GB_FSTAGES; ++s) {
            mbar_init(smem_u32(full + s), 1);
            mbar_init(smem_u32(empty + s), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(tfull + b), 1);
            mbar_init(smem_u32(tfree + b), GB_EPI_WARPS);
        }
        *fault = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        tmem_alloc(smem_u32(tmem_slot), GB_TMEM_COLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int i = 0, issued = 0;
            for (int p = 0; p < np && !*fault; ++p) {
                int t, k0, k1;
                gemm_piece(P, blockIdx.x, p, total, t, k0, k1);
                const int m0 = (t / P.tiles_n) * GB_M, n0 = (t % P.tiles_n) * BN;
                for (int kb = k0; kb < k1 && !*fault; ++kb, ++i) {
                    const int s = i % GB_FSTAGES;
                    const uint32_t ph = (uint32_t)(i / GB_FSTAGES) & 1u;
                    if (!mbar_wait(smem_u32(empty + s), ph ^ 1u, GB_WAIT)) {
                        *fault = 1;
                        break;
                    }
                    const int kk = kb * GB_K;
                    uint8_t *st = stage(s);
                    const uint32_t fb = smem_u32(full + s);
                    mbar_expect_tx(fb, T::STAGE);
                    tma_load_2d(smem_u32(st), &tAh, fb, kk, m0);
                    tma_load_2d(smem_u32(st + GB_A_BYTES), &tAl, fb, kk, m0);
                    tma_load_2d(smem_u32(st + 2 * GB_A_BYTES), &tBh, fb, kk, n0);
                    tma_load_2d(smem_u32(st + 2 * GB_A_BYTES + T::B_BYTES), &tBl, fb, kk, n0);
                    issued = i + 1;
                }
            }
            // never leave with copies in flight
            for (int j = issued > GB_FSTAGES ? issued - GB_FSTAGES : 0; j < issued; ++j)
                mbar_wait(smem_u32(full + j % GB_FSTAGES), (uint32_t)(j / GB_FSTAGES) & 1u, GB_WAIT);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_f16_f32(GB_M, BN);
            int c = 0, i = 0; // chunk and stage counters over all pieces
            for (int p = 0; p < np && !*fault; ++p) {
                int t, k0, k1;
                gemm_piece(P, blockIdx.x, p, total, t, k0, k1);
                for (int kb = k0; kb < k1 && !*fault; ++c) {
                    const int b = c & 1;
                    if (c >= 2 && !mbar_wait(smem_u32(tfree + b), (uint32_t)((c >> 1) - 1) & 1u, GB_WAIT)) {
                        *fault = 1;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = tmem + (uint32_t)(b * 256);
                    const int kend = min(k1, kb + chunk);
                    for (int kc = kb; kc < kend; ++kc, ++i) {
                        const int s = i % GB_FSTAGES;
                        if (!mbar_wait(smem_u32(full + s), (uint32_t)(i / GB_FSTAGES) & 1u, GB_WAIT)) {
                            *fault = 1;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t ah = smem_u32(stage(s)), al = ah + GB_A_BYTES;
                        const uint32_t bh = ah + 2 * GB_A_BYTES, bl = bh + T::B_BYTES;
                        // hi.hi, hi.lo, lo.hi of this K range into one accumulator
#pragma unroll
                        for (int k = 0; k < GB_K / 16; ++k)
                            umma_f16(d, sdesc_sw128(ah + 32 * k), sdesc_sw128(bh + 32 * k), idesc,
                                     (kc > kb || k > 0) ? 1u : 0u);
#pragma unroll
                        for (int k = 0; k < GB_K / 16; ++k)
                            umma_f16(d, sdesc_sw128(ah + 32 * k), sdesc_sw128(bl + 32 * k), idesc, 1u);
#pragma unroll
                        for (int k = 0; k < GB_K / 16; ++k)
                            umma_f16(d, sdesc_sw128(al + 32 * k), sdesc_sw128(bh + 32 * k), idesc, 1u);
                        umma_commit(smem_u32(empty + s));
                    }
                    umma_commit(smem_u32(tfull + b));
                    kb = kend;
                }
            }
        }
    } else {
        const int q = warp & 3, half = (warp - 2) >> 2;
        const int nch = max(0, min(128, BN - 128 * half)) / 16;
        bool ok = true;
        int c = 0;
        for (int p = 0; p < np && ok; ++p) {
            int t, k0, k1;
            gemm_piece(P, blockIdx.x, p, total, t, k0, k1);
            float acc[128];
#pragma unroll
            for (int i = 0; i < 128; ++i) acc[i] = 0.f;
            for (int kb = k0; kb < k1; ++c) {
                const int b = c & 1;
                if (!mbar_wait(smem_u32(tfull + b), (uint32_t)(c >> 1) & 1u, GB_WAIT)) {
                    *fault = 1;
                    ok = false;
                }
                if (!ok || *fault) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                drain_cols<BN == 224 || BN == 240>(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * 256 + 128 * half),
                                                   nch, acc);
                tc_fence_before();
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(tfree + b)) : "memory");
                kb = min(k1, kb + chunk);
            }
            const int m0 = (t / P.tiles_n) * GB_M, n0 = (t % P.tiles_n) * BN;
            const int row = m0 + 32 * q + lane; // row of D
            store_cols(P, acc, nch, ok && row < P.m2, row & 1, row >> 1, n0 + 128 * half);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, GB_TMEM_COLS);
    if (threadIdx.x == 0 && *fault) atomicExch(P.err, 1);
}

// ------------------------------------------------- two-SM tiles (CTA pairs)
// The same GEMM with 256 x BN tiles on a cluster of two CTAs (cta_group::2).
// CTA r of the pair loads A rows [128 r, +128) and B rows [BN/2 r, +BN/2) of
// the tile into its own shared memory; the even CTA issues the M = 256 MMAs,
// which read both CTAs' halves, and each CTA's TMEM receives its own 128 rows
// of D.  With all four operand tiles of a K range staged together, each SM
// stages 62 KB per 12 MMAs of 128 x BN per SM, against 92 KB on a single-SM
// tile, and three stages fit instead of two.  Measured on 1920 x 1080 x 10^4:
// 0.27 ms against 0.31 ms single-SM, despite the coarser M padding (2304 vs
// 2176 rows of D); the autotuner picks per shape.
//
// Barriers: full[s] of the even CTA counts both CTAs' TMA bytes (its
// producer posts the expected total; the odd CTA's loads complete on it
// through its cluster address); empty[s] and tfull[b] live in both CTAs and
// receive the MMA commits by multicast; tfree[b] of the even CTA collects the
// 16 epilogue warps of the pair.  Every wait is bounded, and both CTAs meet
// at a cluster barrier before TMEM is released and either exits, so no CTA
// leaves while its peer may still touch its shared memory.
// As the single-SM form, each stage holds all four operand tiles of one K
// range (this CTA's halves): 62 KB at BN = 240, three stages.
constexpr int G2_STAGES = 3;
template <int BN>
struct Gemm2Tile {
    static_assert(BN % 16 == 0 && BN >= 128 && BN <= 256, "N tile");
    static constexpr int BH = BN / 2;                          // B rows per CTA (a multiple of 8)
    static constexpr int B_BYTES = BH * GB_K * 2;              // a multiple of 1024
    static constexpr int STAGE = 2 * GB_A_BYTES + 2 * B_BYTES; // A hi, A lo, B hi, B lo of one CTA
    // + B_BYTES of slack at the end: every B descriptor's reach, even a whole
    // BN-row tile from the last stage, stays inside the allocation
    static constexpr int SMEM = G2_STAGES * STAGE + 1024 + 256 + B_BYTES;
};

template <int BN>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(GB_THREADS, 1)
    k_cgh_gemm2(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl, GemmParams P)
{
    using T = Gemm2Tile<BN>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    auto stage = [&](int s) { return smem + s * T::STAGE; }; // [A hi | A lo | B hi | B lo]
    uint64_t *full = (uint64_t *)(smem + G2_STAGES * T::STAGE);
    uint64_t *empty = full + G2_STAGES;
    uint64_t *tfull = empty + G2_STAGES; // [2]
    uint64_t *tfree = tfull + 2;         // [2]
    uint32_t *tmem_slot = (uint32_t *)(tfree + 2);
    volatile int *fault = (volatile int *)(tmem_slot + 1);

    const uint32_t rank = cluster_ctarank();
    const bool lead = rank == 0;
    const int pair = blockIdx.x >> 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int total = P.total; // kblocks: all three split products per K step
    const int np = gemm_pieces(P, pair);
    const int chunk = max(1, (P.chunk + 2) / 3);

    if (threadIdx.x == 0) {
        for (int s = 0; s < G2_STAGES; ++s) {
            mbar_init(smem_u32(full + s), 1);
            mbar_init(smem_u32(empty + s), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(smem_u32(tfull + b), 1);
            mbar_init(smem_u32(tfree + b), 2 * GB_EPI_WARPS);
        }
        *fault = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        tmem_alloc_pair(smem_u32(tmem_slot), GB_TMEM_COLS);
        tmem_relinquish_pair();
    }
    tc_fence_before();
    cluster_sync(); // both CTAs' barriers initialised and TMEM allocated
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            const uint32_t full_lead = mapa_shared(smem_u32(full), 0);
            int i = 0, issued = 0;
            for (int p = 0; p < np && !*fault; ++p) {
                int t, k0, k1;
                gemm_piece(P, pair, p, total, t, k0, k1);
                const int m0 = (t / P.tiles_n) * (2 * GB_M) + (int)rank * GB_M;
                const int n0 = (t % P.tiles_n) * BN + (int)rank * T::BH;
                for (int kb = k0; kb < k1 && !*fault; ++kb, ++i) {
                    const int s = i % G2_STAGES;
                    const uint32_t ph = (uint32_t)(i / G2_STAGES) & 1u;
                    if (!mbar_wait(smem_u32(empty + s), ph ^ 1u, GB_WAIT)) {
                        *fault = 1;
                        break;
                    }
                    const int kk = kb * GB_K;
                    uint8_t *st = stage(s);
                    const uint32_t fb = full_lead + 8u * s;
                    if (lead) mbar_expect_tx(smem_u32(full + s), 2 * T::STAGE);
                    tma_load_2d_pair(smem_u32(st), &tAh, fb, kk, m0);
                    tma_load_2d_pair(smem_u32(st + GB_A_BYTES), &tAl, fb, kk, m0);
                    tma_load_2d_pair(smem_u32(st + 2 * GB_A_BYTES), &tBh, fb, kk, n0);
                    tma_load_2d_pair(smem_u32(st + 2 * GB_A_BYTES + T::B_BYTES), &tBl, fb, kk, n0);
                    issued = i + 1;
                }
            }
            // the even CTA's full barriers track both CTAs' copies: never
            // leave with any in flight
            if (lead)
                for (int j = issued > G2_STAGES ? issued - G2_STAGES : 0; j < issued; ++j)
                    mbar_wait(smem_u32(full + j % G2_STAGES), (uint32_t)(j / G2_STAGES) & 1u, GB_WAIT);
        }
    } else if (warp == 1) {
        if (lane == 0 && lead) {
            constexpr uint32_t idesc = idesc_f16_f32(2 * GB_M, BN);
            int c = 0, i = 0;
            for (int p = 0; p < np && !*fault; ++p) {
                int t, k0, k1;
                gemm_piece(P, pair, p, total, t, k0, k1);
                for (int kb = k0; kb < k1 && !*fault; ++c) {
                    const int b = c & 1;
                    if (c >= 2 && !mbar_wait(smem_u32(tfree + b), (uint32_t)((c >> 1) - 1) & 1u, GB_WAIT)) {
                        *fault = 1;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = tmem + (uint32_t)(b * 256);
                    const int kend = min(k1, kb + chunk);
                    for (int kc = kb; kc < kend; ++kc, ++i) {
                        const int s = i % G2_STAGES;
                        if (!mbar_wait(smem_u32(full + s), (uint32_t)(i / G2_STAGES) & 1u, GB_WAIT)) {
                            *fault = 1;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t ah = smem_u32(stage(s)), al = ah + GB_A_BYTES;
                        const uint32_t bh = ah + 2 * GB_A_BYTES, bl = bh + T::B_BYTES;
#pragma unroll
                        for (int k = 0; k < GB_K / 16; ++k)
                            umma_f16_pair(d, sdesc_sw128(ah + 32 * k), sdesc_sw128(bh + 32 * k), idesc,
                                          (kc > kb || k > 0) ? 1u : 0u);
#pragma unroll
                        for (int k = 0; k < GB_K / 16; ++k)
                            umma_f16_pair(d, sdesc_sw128(ah + 32 * k), sdesc_sw128(bl + 32 * k), idesc, 1u);
#pragma unroll
                        for (int k = 0; k < GB_K / 16; ++k)
                            umma_f16_pair(d, sdesc_sw128(al + 32 * k), sdesc_sw128(bh + 32 * k), idesc, 1u);
                        umma_commit_pair(smem_u32(empty + s), 3);
                    }
                    umma_commit_pair(smem_u32(tfull + b), 3);
                    kb = kend;
                }
            }
        }
    } else {
        const int q = warp & 3, half = (warp - 2) >> 2;
        const int nch = max(0, min(128, BN - 128 * half)) / 16;
        const uint32_t tfree_lead = mapa_shared(smem_u32(tfree), 0);
        bool ok = true;
        int c = 0;
        for (int p = 0; p < np && ok; ++p) {
            int t, k0, k1;
            gemm_piece(P, pair, p, total, t, k0, k1);
            float acc[128];
#pragma unroll
            for (int i = 0; i < 128; ++i) acc[i] = 0.f;
            for (int kb = k0; kb < k1; ++c) {
                const int b = c & 1;
                if (!mbar_wait(smem_u32(tfull + b), (uint32_t)(c >> 1) & 1u, GB_WAIT)) {
                    *fault = 1;
                    ok = false;
                }
                if (!ok || *fault) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                drain_cols<BN == 224 || BN == 240>(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * 256 + 128 * half),
                                                   nch, acc);
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive_remote(tfree_lead + 8u * b);
                kb = min(k1, kb + chunk);
            }
            const int m0 = (t / P.tiles_n) * (2 * GB_M) + (int)rank * GB_M, n0 = (t % P.tiles_n) * BN;
            const int row = m0 + 32 * q + lane; // row of D
            store_cols(P, acc, nch, ok && row < P.m2, row & 1, row >> 1, n0 + 128 * half);
        }
    }
    __syncwarp();
    tc_fence_before();
    cluster_sync(); // neither CTA releases TMEM or exits while its peer still works
    if (warp == 1) tmem_dealloc_pair(tmem, GB_TMEM_COLS);
    if (threadIdx.x == 0 && *fault) atomicExch(P.err, 1);
}

// ------------------------------------------------------------------ host
namespace {

std::atomic<double> g_tail_weight{1.2};
std::atomic<int> g_pairs{1}; // two-SM tiles unless switched (or autotuned) to single-SM
std::atomic<int> g_chunk{8};
std::mutex g_encode_mu;

int make_map(CUtensorMap *m, void *base, uint64_t rows, uint64_t kp, uint32_t box_rows)
{
    cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
    cuuint32_t box[2] = {(cuuint32_t)GB_K, box_rows};
    cuuint32_t estr[2] = {1, 1};
    PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
    if (int rc = tensor_map_encoder(&enc)) return rc;
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, base, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? OLG_OK : fail(OLG_ERR_CUDA, "cuTensorMapEncodeTiled failed");
}

// N tile width for a hologram nx wide: the fewest padded columns, ties to
// the wider tile.
int pick_bn(int nx)
{
    const int cand[] = {256, 240, 224, 192, 160, 128};
    int best = 256;
    long long pad = 1LL << 40;
    for (int bn : cand) {
        const long long cover = (long long)((nx + bn - 1) / bn) * bn;
        if (cover < pad) {
            pad = cover;
            best = bn;
        }
    }
    return best;
}

constexpr int BN_LIST[] = {256, 240, 224, 192, 160, 128};
int bn_index(int bn)
{
    for (int i = 0; i < 6; ++i)
        if (BN_LIST[i] == bn) return i;
    return 5;
}

// one tile width: both kernels' shared-memory opt-in, and how many CTA pairs
// can be resident at once
template <int BN>
int gemm_setup(int *pairs)
{
    cudaError_t e = cudaFuncSetAttribute(k_cgh_gemm<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, GemmTile<BN>::SMEM);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_cgh_gemm)");
    e = cudaFuncSetAttribute(k_cgh_gemm2<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, Gemm2Tile<BN>::SMEM);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_cgh_gemm2)");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2, 1, 1);
    cfg.blockDim = dim3(GB_THREADS, 1, 1);
    cfg.dynamicSmemBytes = Gemm2Tile<BN>::SMEM;
    e = cudaOccupancyMaxActiveClusters(pairs, k_cgh_gemm2<BN>, &cfg);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveClusters(k_cgh_gemm2)");
    return OLG_OK;
}

struct GemmDevice {
    int nsm = 0;
    int pairs[6] = {};
};

// per context, once: the opt-ins, the SM count and the resident pair counts
int gemm_device(GemmDevice *out)
{
    static std::map<unsigned long long, GemmDevice> cache;
    unsigned long long ctx = 0;
    if (int rc = context_id(&ctx)) return rc;
    std::lock_guard<std::mutex> lk(g_encode_mu);
    auto it = cache.find(ctx);
    if (it == cache.end()) {
        GemmDevice d;
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
        e = cudaDeviceGetAttribute(&d.nsm, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute(SM count)");
        int rc = gemm_setup<256>(&d.pairs[0]);
        if (!rc) rc = gemm_setup<240>(&d.pairs[1]);
        if (!rc) rc = gemm_setup<224>(&d.pairs[2]);
        if (!rc) rc = gemm_setup<192>(&d.pairs[3]);
        if (!rc) rc = gemm_setup<160>(&d.pairs[4]);
        if (!rc) rc = gemm_setup<128>(&d.pairs[5]);
        if (rc) return rc;
        it = cache.emplace(ctx, d).first;
    }
    *out = it->second;
    return OLG_OK;
}

template <int BN>
void launch_gemm(bool pair, int units, const CUtensorMap &a_hi, const CUtensorMap &a_lo, const CUtensorMap &b_hi,
                 const CUtensorMap &b_lo, const GemmParams &P, cudaStream_t st)
{
    if (pair)
        k_cgh_gemm2<BN><<<2 * units, GB_THREADS, Gemm2Tile<BN>::SMEM, st>>>(a_hi, a_lo, b_hi, b_lo, P);
    else
        k_cgh_gemm<BN><<<units, GB_THREADS, GemmTile<BN>::SMEM, st>>>(a_hi, a_lo, b_hi, b_lo, P);
}

size_t gemm_layout(int n, int ny, int nx, int *kp_out, size_t off[5])
{
    const int kp = (int)align_up((size_t)2 * (size_t)(n > 0 ? n : 1), GB_K);
    size_t o = 0;
    off[0] = o; o += align_up((size_t)n * sizeof(PointCoef) + 16, 1024);
    off[1] = o; o += align_up((size_t)2 * ny * kp * 2, 1024); // a_hi
    off[2] = o; o += align_up((size_t)2 * ny * kp * 2, 1024); // a_lo
    off[3] = o; o += align_up((size_t)nx * kp * 2, 1024);     // b_hi
    off[4] = o; o += align_up((size_t)nx * kp * 2, 1024);     // b_lo
    if (kp_out) *kp_out = kp;
    return o;
}

// adjoint workspace: coefficients, A hi/lo (2 ny x kp), B hi/lo (n x kp),
// T (ny x n complex64), per-band partial sums, the max word
size_t adjt_layout(int n, int ny, int nx, int *kp_out, int *bands_out, size_t off[8])
{
    const int kp = (int)align_up((size_t)2 * nx, GB_K);
    const int bands = (ny + ADJT_BAND - 1) / ADJT_BAND;
    const size_t np = (size_t)(n > 0 ? n : 1);
    size_t o = 0;
    off[0] = o; o += align_up(np * sizeof(PointCoef) + 16, 1024);
    off[1] = o; o += align_up((size_t)2 * ny * kp * 2, 1024);
    off[2] = o; o += align_up((size_t)2 * ny * kp * 2, 1024);
    off[3] = o; o += align_up(np * kp * 2, 1024);
    off[4] = o; o += align_up(np * kp * 2, 1024);
    off[5] = o; o += align_up((size_t)ny * np * sizeof(float2), 1024);
    off[6] = o; o += align_up((size_t)bands * np * sizeof(float2), 1024);
    off[7] = o; o += 1024;
    if (kp_out) *kp_out = kp;
    if (bands_out) *bands_out = bands;
    return o;
}

} // namespace

// D = A B^T on the tensor cores into the complex64 field U ((m2 / 2) x n_cols,
// row stride n_cols): A (m2 x kp) and B (n_cols x kp) split-f16 operands,
// K-contiguous, three K segments (hi.hi, hi.lo, lo.hi).  Zeroes U first
// unless accumulating.
int gemm_run(const __half *a_hi, const __half *a_lo, const __half *b_hi, const __half *b_lo, int m2, int n_cols,
             int kp, float2 *U, bool accumulate, int *err, cudaStream_t st)
{
    const int bn = pick_bn(n_cols);
    const bool pair = g_pairs.load(std::memory_order_relaxed) != 0;
    GemmDevice dev{};
    if (int rc = gemm_device(&dev)) return rc;
    const int units_max = pair ? dev.pairs[bn_index(bn)] : dev.nsm; // CTAs or CTA pairs resident at once
    if (units_max < 1) return fail(OLG_ERR_CUDA, "k_cgh_gemm: no resident CTA (pair) fits");
    CUtensorMap mAh, mAl, mBh, mBl;
    if (int rc = make_map(&mAh, (void *)a_hi, (uint64_t)m2, kp, GB_M)) return rc;
    if (int rc = make_map(&mAl, (void *)a_lo, (uint64_t)m2, kp, GB_M)) return rc;
    if (int rc = make_map(&mBh, (void *)b_hi, (uint64_t)n_cols, kp, pair ? bn / 2 : bn)) return rc;
    if (int rc = make_map(&mBl, (void *)b_lo, (uint64_t)n_cols, kp, pair ? bn / 2 : bn)) return rc;
    GemmParams P{};
    P.m2 = m2;
    P.n = n_cols;
    P.kblocks = kp / GB_K;
    P.tiles_n = (n_cols + bn - 1) / bn;
    const int tile_m = pair ? 2 * GB_M : GB_M;
    const long long tiles = (long long)P.tiles_n * ((m2 + tile_m - 1) / tile_m);
    P.tiles = (int)tiles;
    P.U = U;
    P.vec4 = ((uintptr_t)U % 16 == 0 && n_cols % 2 == 0) ? 1 : 0;
    P.chunk = g_chunk.load(std::memory_order_relaxed);
    P.err = err;
    const double tw = g_tail_weight.load(std::memory_order_relaxed);
    // Units (CTAs, or CTA pairs) left over after one per tile take the K
    // tails: with e extra units each holds `per` tails.  A tail K block costs
    // g_tail_weight tile K blocks (its operands are not shared in L2 with
    // other units at the time), so split = total per w / (per w + 1) evens
    // the two kinds of unit; w <= 0 turns the split off.
    const int total = P.kblocks; // K steps: all three split products per step, both forms
    P.total = total;
    P.split = total;
    P.extra = 0;
    if (tiles < units_max && tw > 0.0) {
        const int e = units_max - (int)tiles;
        const int per = ((int)tiles + e - 1) / e;
        const double pw = per * tw;
        const int split = (int)((double)total * pw / (pw + 1.0));
        if (split > 0 && split < total) {
            P.split = split;
            P.extra = std::min(e, (int)tiles);
        }
    }
    if (!accumulate) {
        const cudaError_t e = cudaMemsetAsync(U, 0, sizeof(float2) * (size_t)(m2 / 2) * n_cols, st);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    }
    const int units = (int)tiles + P.extra;
    switch (bn) {
    case 256: launch_gemm<256>(pair, units, mAh, mAl, mBh, mBl, P, st); break;
    case 240: launch_gemm<240>(pair, units, mAh, mAl, mBh, mBl, P, st); break;
    case 224: launch_gemm<224>(pair, units, mAh, mAl, mBh, mBl, P, st); break;
    case 192: launch_gemm<192>(pair, units, mAh, mAl, mBh, mBl, P, st); break;
    case 160: launch_gemm<160>(pair, units, mAh, mAl, mBh, mBl, P, st); break;
    default: launch_gemm<128>(pair, units, mAh, mAl, mBh, mBl, P, st); break;
    }
    count_launch();
    return check_launch(pair ? "k_cgh_gemm2" : "k_cgh_gemm");
}

} // namespace olg

using namespace olg;

extern "C" size_t olg_cgh_gemm_workspace_bytes(int n_points, int ny, int nx)
{
    size_t off[5];
    return gemm_layout(n_points, ny, nx, nullptr, off);
}

extern "C" int olg_cgh_fresnel_gemm_c64(const float *points, const float *amp, const float *phase0, int n_points,
                                        void *U, int ny, int nx, double py, double px, double lambda, int flags,
                                        void *work, size_t work_bytes, olg_stream_t stream)
{
    if ((!points && n_points > 0) || !U) return fail(OLG_ERR_INVALID_ARG, "null pointer");
    if (n_points < 0 || ny <= 0 || nx <= 0 || nx > (1 << 20) || ny > (1 << 20)) return fail(OLG_ERR_INVALID_ARG, "bad sizes");
    if (nx > 4096 || ny > 4096) return fail(OLG_ERR_UNSUPPORTED_SIZE, "hologram side must be <= 4096 (exact w^2 in float)");
    if (!(px > 0) || !(py > 0) || !(lambda > 0)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if ((uintptr_t)U % 8) return fail(OLG_ERR_INVALID_ARG, "U must be 8-byte aligned (complex64)");
    int *err = nullptr;
    if (int rc = device_fault_word(&err)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    int kp = 0;
    size_t off[5];
    const size_t need = gemm_layout(n_points, ny, nx, &kp, off);
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, need, st)) return rc;
    char *base = (char *)sc.ptr;
    GemmOps G{};
    G.pts = points; G.amp = amp; G.ph0 = phase0; G.n = n_points; G.ny = ny; G.nx = nx; G.kp = kp;
    G.px = px; G.py = py; G.lambda = lambda;
    G.coef = (PointCoef *)(base + off[0]);
    G.a_hi = (__half *)(base + off[1]);
    G.a_lo = (__half *)(base + off[2]);
    G.b_hi = (__half *)(base + off[3]);
    G.b_lo = (__half *)(base + off[4]);
    const bool reuse = (flags & OLG_REUSE_OPERANDS) != 0;
    if (reuse && !work) return fail(OLG_ERR_INVALID_ARG, "OLG_REUSE_OPERANDS needs the caller's workspace");
    if (n_points > 0 && !reuse) {
        k_cgh_gemm_prep<<<(n_points + PREP_THREADS - 1) / PREP_THREADS, PREP_THREADS, 0, st>>>(G);
        count_launch();
        if (int rc = check_launch("k_cgh_gemm_prep")) return rc;
    }
    if (!reuse) {
        dim3 og((kp / 2 + 127) / 128, (nx + ny + OPS_ROWS - 1) / OPS_ROWS);
        k_cgh_gemm_ops<<<og, 128, 0, st>>>(G);
        count_launch();
        if (int rc = check_launch("k_cgh_gemm_ops")) return rc;
    }
    return gemm_run(G.a_hi, G.a_lo, G.b_hi, G.b_lo, 2 * ny, nx, kp, (float2 *)U, (flags & OLG_ACCUMULATE) != 0, err,
                    st);
}

// A sequence of holograms from host point clouds: cloud i goes up into device
// slot i % 3 on a copy-in stream, its hologram is formed there on the caller's
// stream (olg_cgh_fresnel_gemm_c64, one workspace for all) and comes down on
// a copy-out stream, so hologram i-1's copy out and cloud i+1's copy in
// overlap hologram i's GEMM.  Ordered on `stream` like `count` single calls.
extern "C" int olg_cgh_fresnel_gemm_host_c64(const float *const *points, const float *const *amp,
                                             const float *const *phase0, const int *n_points, void *const *U,
                                             int count, int ny, int nx, double py, double px, double lambda,
                                             int flags, olg_stream_t stream)
{
    if (count < 0) return fail(OLG_ERR_INVALID_ARG, "negative hologram count");
    if (count == 0) return OLG_OK;
    if (!points || !n_points || !U) return fail(OLG_ERR_INVALID_ARG, "null host arrays");
    if (flags & (OLG_ACCUMULATE | OLG_REUSE_OPERANDS))
        return fail(OLG_ERR_INVALID_ARG, "the host form writes each hologram afresh (no OLG_ACCUMULATE or "
                                         "OLG_REUSE_OPERANDS)");
    if (ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad sizes");
    if (nx > 4096 || ny > 4096) return fail(OLG_ERR_UNSUPPORTED_SIZE, "hologram side must be <= 4096 (exact w^2 in float)");
    if (!(px > 0) || !(py > 0) || !(lambda > 0)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    int n_max = 0;
    for (int i = 0; i < count; ++i) {
        if (n_points[i] < 0) return fail(OLG_ERR_INVALID_ARG, "negative point count");
        if ((!points[i] && n_points[i] > 0) || !U[i]) return fail(OLG_ERR_INVALID_ARG, "null host cloud or hologram");
        n_max = std::max(n_max, n_points[i]);
    }
    cudaStream_t st = (cudaStream_t)stream;
    // per slot: xyz, amplitudes, phases, hologram; then the GEMM workspace
    const size_t pb = align_up(sizeof(float) * 3 * (size_t)n_max + 16, 256);
    const size_t ab = align_up(sizeof(float) * (size_t)n_max + 16, 256);
    const size_t ub = align_up(sizeof(float2) * (size_t)ny * nx, 256);
    const size_t slot = pb + 2 * ab + ub;
    const size_t wb = align_up(olg_cgh_gemm_workspace_bytes(n_max, ny, nx), 256);
    Scratch sc;
    if (int rc = sc.acquire(nullptr, 0, HostPipeline::SLOTS * slot + wb, st)) return rc;
    char *work = (char *)sc.ptr + HostPipeline::SLOTS * slot;
    // on an early return the copy streams may still use the scratch, which
    // is freed on `stream`: let them finish first
    struct Pipe : HostPipeline {
        bool ended = false;
        ~Pipe()
        {
            if (!ended) drain();
            release();
        }
    } H;
    if (int rc = H.init()) return rc;
    if (int rc = H.begin(st)) return rc;
    auto up = [&](void *dst, const void *src, size_t bytes) -> int {
        if (!bytes) return OLG_OK;
        const cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, H.s_in);
        return e == cudaSuccess ? OLG_OK : cuda_fail(e, "cudaMemcpyAsync (cloud in)");
    };
    for (int i = 0; i < count; ++i) {
        char *base = (char *)sc.ptr + (size_t)(i % HostPipeline::SLOTS) * slot;
        float *d_pts = (float *)base, *d_amp = (float *)(base + pb), *d_ph = (float *)(base + pb + ab);
        void *d_U = base + pb + 2 * ab;
        const int n = n_points[i];
        const bool has_amp = amp && amp[i], has_ph = phase0 && phase0[i];
        if (int rc = H.copy_in_begin(i)) return rc;
        if (int rc = up(d_pts, points[i], sizeof(float) * 3 * (size_t)n)) return rc;
        if (has_amp)
            if (int rc = up(d_amp, amp[i], sizeof(float) * (size_t)n)) return rc;
        if (has_ph)
            if (int rc = up(d_ph, phase0[i], sizeof(float) * (size_t)n)) return rc;
        if (int rc = H.copy_in_end(i, st)) return rc;
        if (int rc = olg_cgh_fresnel_gemm_c64(d_pts, has_amp ? d_amp : nullptr, has_ph ? d_ph : nullptr, n, d_U, ny,
                                              nx, py, px, lambda, flags, work, wb, stream))
            return rc;
        if (int rc = H.compute_end(i, st)) return rc;
        const cudaError_t e = cudaMemcpyAsync(U[i], d_U, sizeof(float2) * (size_t)ny * nx, cudaMemcpyDeviceToHost,
                                              H.s_out);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (hologram out)");
        if (int rc = H.copy_out_end(i)) return rc;
    }
    // the scratch is released on `stream` after this wait, behind every copy
    const int rc = H.end(st);
    H.ended = rc == OLG_OK;
    return rc;
}

extern "C" size_t olg_cgh_adjoint_gemm_workspace_bytes(int n_points, int ny, int nx)
{
    if (n_points <= 0 || ny <= 0 || nx <= 0) return 0;
    size_t off[8];
    return adjt_layout(n_points, ny, nx, nullptr, nullptr, off);
}

extern "C" int olg_cgh_fresnel_adjoint_gemm_c64(const float *points, int n_points, const void *G, void *g, int ny,
                                                int nx, double py, double px, double lambda, int flags, void *work,
                                                size_t work_bytes, olg_stream_t stream)
{
    if (n_points < 0 || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad sizes");
    if (nx > 4096 || ny > 4096) return fail(OLG_ERR_UNSUPPORTED_SIZE, "hologram side must be <= 4096");
    if (n_points > 0 && (!points || !G || !g)) return fail(OLG_ERR_INVALID_ARG, "null pointer");
    if (((uintptr_t)G & 7) || ((uintptr_t)g & 7)) return fail(OLG_ERR_INVALID_ARG, "G and g must be 8-byte aligned");
    if (!(px > 0) || !(py > 0) || !(lambda > 0)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if (n_points == 0) return OLG_OK;
    int *err = nullptr;
    if (int rc = device_fault_word(&err)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    int kp = 0, bands = 0;
    size_t off[8];
    const size_t need = adjt_layout(n_points, ny, nx, &kp, &bands, off);
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, need, st)) return rc;
    char *base = (char *)sc.ptr;
    GemmOps O{};
    O.pts = points; O.n = n_points; O.ny = ny; O.nx = nx; O.kp = kp;
    O.px = px; O.py = py; O.lambda = lambda;
    O.coef = (PointCoef *)(base + off[0]);
    O.a_hi = (__half *)(base + off[1]);
    O.a_lo = (__half *)(base + off[2]);
    O.b_hi = (__half *)(base + off[3]);
    O.b_lo = (__half *)(base + off[4]);
    float2 *T = (float2 *)(base + off[5]);
    float2 *part = (float2 *)(base + off[6]);
    unsigned *mx = (unsigned *)(base + off[7]);
    const float2 *Gf = (const float2 *)G;
    k_cgh_gemm_prep<<<(n_points + PREP_THREADS - 1) / PREP_THREADS, PREP_THREADS, 0, st>>>(O);
    count_launch();
    if (int rc = check_launch("k_cgh_gemm_prep")) return rc;
    cudaError_t e = cudaMemsetAsync(mx, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    const long long cnt = (long long)ny * nx;
    const int mb = (int)std::min<long long>((cnt + 255) / 256, 1024); // grid-stride beyond that
    k_cgh_absmax<<<mb, 256, 0, st>>>(Gf, cnt, mx);
    count_launch();
    if (int rc = check_launch("k_cgh_absmax")) return rc;
    k_cgh_adjt_aops<<<dim3((kp / 2 + 127) / 128, ny), 128, 0, st>>>(Gf, ny, nx, kp, mx, O.a_hi, O.a_lo);
    count_launch();
    if (int rc = check_launch("k_cgh_adjt_aops")) return rc;
    k_cgh_adjt_bops<<<dim3((n_points + 127) / 128, kp / 32), 128, 0, st>>>(O);
    count_launch();
    if (int rc = check_launch("k_cgh_adjt_bops")) return rc;
    if (int rc = gemm_run(O.a_hi, O.a_lo, O.b_hi, O.b_lo, 2 * ny, n_points, kp, T, false, err, st)) return rc;
    k_cgh_adjt_rows<<<dim3((n_points + 127) / 128, bands), 128, 0, st>>>(O.coef, T, n_points, ny, part);
    count_launch();
    if (int rc = check_launch("k_cgh_adjt_rows")) return rc;
    k_cgh_adjt_sum<<<(n_points + 255) / 256, 256, 0, st>>>(part, bands, n_points, mx, (float2 *)g,
                                                          (flags & OLG_ACCUMULATE) ? 1 : 0);
    count_launch();
    return check_launch("k_cgh_adjt_sum");
}

extern "C" int olg_cgh_gemm_chunk(int kblocks)
{
    if (kblocks >= 1 && kblocks <= 64) return g_chunk.exchange(kblocks);
    return g_chunk.load();
}

extern "C" int olg_cgh_gemm_pairs(int on)
{
    if (on == 0 || on == 1) return g_pairs.exchange(on);
    return g_pairs.load();
}

extern "C" double olg_cgh_gemm_tail_weight(double w)
{
    if (w >= 0.0 && w <= 16.0) return g_tail_weight.exchange(w);
    return g_tail_weight.load();
}

// Times the GEMM on the caller's hologram shape and point count for each
// tile form (two-SM pairs, single-SM tiles) and a few K-tail weights (the
// work split between tile units and the spare SMs' tail units), and keeps
// the fastest.  Operands are built once (a unit-amplitude cloud spread over
// the hologram at 0.1 m; the choice depends on the shape, not on the values)
// and reused; every timed GEMM starts from a cold L2.
extern "C" int olg_autotune_cgh_gemm(int n_points, int ny, int nx, int reps, olg_stream_t stream)
{
    if (n_points <= 0 || ny <= 0 || nx <= 0 || ny > 4096 || nx > 4096)
        return fail(OLG_ERR_INVALID_ARG, "autotuning needs n_points > 0 and ny, nx in [1, 4096]");
    if (reps < 1) reps = 5;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t wb = olg_cgh_gemm_workspace_bytes(n_points, ny, nx);
    Scratch ws, pts, U, flush;
    if (int rc = ws.acquire(nullptr, 0, wb, st)) return rc;
    if (int rc = pts.acquire(nullptr, 0, sizeof(float) * 3 * (size_t)n_points, st)) return rc;
    if (int rc = U.acquire(nullptr, 0, sizeof(float2) * (size_t)ny * nx, st)) return rc;
    const size_t flush_bytes = (size_t)256 << 20;
    if (int rc = flush.acquire(nullptr, 0, flush_bytes, st)) return rc;
    std::vector<float> h(3 * (size_t)n_points);
    for (int j = 0; j < n_points; ++j) {
        h[3 * j] = (float)(8e-6 * nx * ((j * 0.6180339887) - std::floor(j * 0.6180339887)));
        h[3 * j + 1] = (float)(8e-6 * ny * ((j * 0.7548776662) - std::floor(j * 0.7548776662)));
        h[3 * j + 2] = (float)(0.1 + 1e-3 * ((j * 0.5698402910) - std::floor(j * 0.5698402910)));
    }
    cudaError_t e = cudaMemcpyAsync(pts.ptr, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync (autotune points)");
    const double keep = g_tail_weight.load();
    const int keep_pairs = g_pairs.load();
    auto restore = [&] {
        g_tail_weight.store(keep);
        g_pairs.store(keep_pairs);
    };
    auto run = [&](int flags) {
        return olg_cgh_fresnel_gemm_c64((const float *)pts.ptr, nullptr, nullptr, n_points, U.ptr, ny, nx, 8e-6,
                                        8e-6, 532e-9, flags, ws.ptr, wb, stream);
    };
    if (int rc = run(0)) { // builds the operands
        restore();
        return rc;
    }
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
    // Every (tile form, weight) candidate is timed `reps` times in each of two
    // rounds, the second in reverse order, and keeps its fastest run: the
    // choice then rests on each candidate's best case rather than on when in
    // the sweep it ran.
    const double cand[] = {0.0, 1.0, 1.1, 1.2, 1.3, 1.45, 1.6};
    constexpr int NW = (int)(sizeof(cand) / sizeof(cand[0]));
    float fastest[2][NW];
    for (auto &row : fastest)
        for (float &f : row) f = 1e30f;
    for (int round = 0; round < 2; ++round) {
        for (int k = 0; k < 2 * NW; ++k) {
            const int idx = round == 0 ? k : 2 * NW - 1 - k;
            const int pr = 1 - idx / NW, wi = idx % NW;
            g_pairs.store(pr);
            g_tail_weight.store(cand[wi]);
            for (int r = 0; r < reps; ++r) {
                if ((e = cudaMemsetAsync(flush.ptr, r & 0xff, flush_bytes, st)) != cudaSuccess ||
                    (e = cudaEventRecord(ev.a, st)) != cudaSuccess) {
                    restore();
                    return cuda_fail(e, "autotune timing");
                }
                if (int rc = run(OLG_REUSE_OPERANDS)) {
                    restore();
                    return rc;
                }
                float t = 0.f;
                if ((e = cudaEventRecord(ev.b, st)) != cudaSuccess || (e = cudaEventSynchronize(ev.b)) != cudaSuccess ||
                    (e = cudaEventElapsedTime(&t, ev.a, ev.b)) != cudaSuccess) {
                    restore();
                    return cuda_fail(e, "autotune timing");
                }
                fastest[pr][wi] = std::min(fastest[pr][wi], t);
            }
        }
    }
    double best_w = keep;
    int best_p = keep_pairs;
    float best = 1e30f;
    for (int pr = 1; pr >= 0; --pr)
        for (int wi = 0; wi < NW; ++wi)
            if (fastest[pr][wi] < best) {
                best = fastest[pr][wi];
                best_w = cand[wi];
                best_p = pr;
            }
    g_tail_weight.store(best_w);
    g_pairs.store(best_p);
    return OLG_OK;
}

extern "C" int olg_device_fault_check(int clear)
{
    int *err = nullptr;
    if (int rc = device_fault_word(&err)) return rc;
    int h = 0;
    cudaError_t e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "reading the device fault flag");
    if (clear && h) cudaMemset(err, 0, sizeof(int));
    if (h) return fail(OLG_ERR_CUDA, "a kernel gave up on a bounded wait (tensor-core GEMM or TMA-staged column pass)");
    return OLG_OK;
}
