// cgh.cu -- point-cloud CGH on GB300 (sm_103a): Fresnel form and exact
// spherical waves, one pixel-tile per CTA, points streamed through shared
// memory.
//
// The reference sums every point for every pixel in FP32 (golcgh.h:47-88),
// with the phase pi rho^2 / (lambda z) ~ 1e3..1e4 rad evaluated directly, so
// ~1e-3 rad of it is rounding.  Here the phase of each (tile, point) pair is
// anchored at the tile centre in double-float arithmetic (~44 bits), reduced
// to [-0.5, 0.5] cycles, and each pixel adds a small local expansion in FP32:
//   Fresnel: cycles(w,h) = c0 + ax dw + ay dh + bx dw^2 + by dh^2   (exact: quadratic)
//   exact:   x = (r^2 - r0^2) / r0^2 = ax dw + ay dh + bx dw^2 + by dh^2,
//            cycles = c0 + R (x/2 - x^2/8 + x^3/16),  amplitude = A (1 - x/2)
// with (dw, dh) the pixel offset from the subtile centre (|d| <= 7.5).  The
// series is used while |x| <= 2e-3 for every point of a batch (truncation
// < 1e-7 cycles); otherwise the batch uses the closed form
// R x / (1 + sqrt(1 + x)).  Per term: 2 MUFU (sin, cos) and about 12 other
// instructions (exact form), 9 (Fresnel form), two pixels per paired
// FP32 instruction (fma/add/mul .f32x2).
//
// CTA = 256 threads over a 32 x 32 pixel tile (four 16 x 16 subtiles, each
// with its own anchor), 4 pixels per thread; 128 points per batch.
// Summation is sequential over points (deterministic), in per-batch partial
// sums.
#include <cmath>
#include <cstdio>

#include "common.cuh"

namespace olg {

struct CghParams {
    const float *pts, *amp, *ph0;
    int n, ny, nx;
    float px_hi, px_lo, py_hi, py_lo; // pitches as double-float
    float il_hi, il_lo;               // 1 / lambda
    float l_hi, l_lo;                 // lambda
    float2 *U;
    float *phase_out;
    int accumulate;
};

constexpr int CGH_BATCH = 128;
constexpr float SERIES_XMAX = 2e-3f;

// Per (subtile, point) record, three float4 in shared memory:
//   [c0 ax ay bx] [by h1 h2 h3] [A Ah R -]
// Fresnel: cycles = c0 + ax dw + ay dh + bx dw^2 + by dh^2, amplitude A,
//          stored in the h1 slot (two float4 per record are read).
// exact:   x as above without c0, cycles = c0 + x (h1 + x (h2 + x h3)) with
//          h1 = R/2, h2 = -R/8, h3 = R/16, amplitude A + Ah x (Ah = -A/2; the
//          dropped 3x^2/8 is below 1.5e-6 relative while |x| <= 2e-3).
struct Sub {
    float c0, ax, ay, bx, by, h1, h2, h3, A, Ah, R, pad;
};

template <bool EXACT>
__device__ __forceinline__ Sub prep_sub(const CghParams &P, float x, float y, float z, float a, float ph, float wc,
                                        float hc)
{
    Sub s{};
    const df2 Xc = df_add(df_two_prod(P.px_hi, wc), df2{P.px_lo * wc, 0.f});
    const df2 Yc = df_add(df_two_prod(P.py_hi, hc), df2{P.py_lo * hc, 0.f});
    const df2 Dx = df_add_f(Xc, -x);
    const df2 Dy = df_add_f(Yc, -y);
    const df2 rho2 = df_add(df_mul(Dx, Dx), df_mul(Dy, Dy));
    const float px = P.px_hi, py = P.py_hi;
    const float phc = ph * 0.15915494309189535f; // phi / (2 pi)
    if (!EXACT) {
        // cycles = rho^2 / (2 lambda z) + phi / 2 pi
        const df2 lz2 = df_mul(df2{P.l_hi, P.l_lo}, df2{2.0f * z, 0.f});
        const df2 k2 = df_recip(lz2);
        s.c0 = wrap_cycles(df_frac(df_mul(rho2, k2)) + phc);
        const float k = k2.hi;
        s.ax = 2.0f * Dx.hi * px * k;
        s.ay = 2.0f * Dy.hi * py * k;
        s.bx = px * px * k;
        s.by = py * py * k;
        s.A = a;
    } else {
        const df2 r02 = df_add(rho2, df_two_prod(z, z));
        const df2 r0 = df_sqrt(r02);
        s.c0 = wrap_cycles(df_frac(df_mul(r0, df2{P.il_hi, P.il_lo})) + phc);
        const float inv = 1.0f / r02.hi;
        s.ax = 2.0f * Dx.hi * px * inv;
        s.ay = 2.0f * Dy.hi * py * inv;
        s.bx = px * px * inv;
        s.by = py * py * inv;
        s.R = r0.hi * P.il_hi;
        s.h1 = 0.5f * s.R;
        s.h2 = -0.125f * s.R;
        s.h3 = 0.0625f * s.R;
        s.A = a / r0.hi;
        s.Ah = -0.5f * s.A;
    }
    return s;
}

__device__ __forceinline__ float xbound(const Sub &s)
{
    return fabsf(s.ax) * 7.5f + fabsf(s.ay) * 7.5f + (fabsf(s.bx) + fabsf(s.by)) * 56.25f;
}

// t - round(t) with the rounding done by adding and removing 1.5 * 2^23
// (round to nearest even, exact for |t| < 2^22): plain FP32 adds.
__device__ __forceinline__ float wrap_add(float t)
{
    const float r = __fsub_rn(__fadd_rn(t, 12582912.0f), 12582912.0f);
    return t - r;
}

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

// Two terms at once on the paired FP32 pipe: phases cyc (cycles) and
// amplitudes amp for the pixels of lanes x and y; ba += amp.x e^{2 pi i cyc.x},
// bb += amp.y e^{2 pi i cyc.y}.  Same roundings as the scalar form.
__device__ __forceinline__ void accumulate_pair(float2 &ba, float2 &bb, float2 amp, float2 cyc)
{
    const float2 r = __fadd2_rn(__fadd2_rn(cyc, f2(12582912.0f)), f2(-12582912.0f));
    const float2 a = __fmul2_rn(__ffma2_rn(r, f2(-1.0f), cyc), f2(6.283185307179586f));
    float s0, c0, s1, c1;
    __sincosf(a.x, &s0, &c0);
    __sincosf(a.y, &s1, &c1);
    ba = __ffma2_rn(f2(amp.x), make_float2(c0, s0), ba);
    bb = __ffma2_rn(f2(amp.y), make_float2(c1, s1), bb);
}

// CTA = 256 threads over a 32 x 32 pixel tile: four 16 x 16 subtiles (one
// anchor each), two warps per subtile, each thread one column of 4 pixels
// (rows tq, tq + 4, tq + 8, tq + 12 of its subtile).  The dw terms of x and
// the record loads are shared by the 4 pixels.
template <bool EXACT>
__global__ void __launch_bounds__(256) k_cgh(CghParams P)
{
    __shared__ float4 sp[4][CGH_BATCH][3];
    const int tid = threadIdx.x;
    const int sub = tid >> 6, l = tid & 63;
    const int tx = l & 15, tq = l >> 4;
    const int w0 = blockIdx.x * 32, h0 = blockIdx.y * 32;
    const float dw = (float)tx - 7.5f, dw2 = dw * dw;
    float dh[4], dh2[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        dh[k] = (float)(tq + 4 * k) - 7.5f;
        dh2[k] = dh[k] * dh[k];
    }
    // pixel pairs (i, i + 2) share one paired FP32 instruction per step
    const float2 dhp[2] = {make_float2(dh[0], dh[2]), make_float2(dh[1], dh[3])};
    const float2 dh2p[2] = {make_float2(dh2[0], dh2[2]), make_float2(dh2[1], dh2[3])};
    float2 acc[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = make_float2(0.f, 0.f);

    // preparation: thread t builds point (t mod 128) for subtiles 2 (t / 128) and 2 (t / 128) + 1
    const int pp = tid & (CGH_BATCH - 1), ps = 2 * (tid >> 7);
    for (int base = 0; base < P.n; base += CGH_BATCH) {
        const int j = base + pp;
        float xb = 0.f;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int s = ps + q;
            Sub r{};
            if (j < P.n) {
                const float x = __ldg(P.pts + 3 * j), y = __ldg(P.pts + 3 * j + 1), z = __ldg(P.pts + 3 * j + 2);
                const float a = P.amp ? __ldg(P.amp + j) : 1.0f;
                const float ph = P.ph0 ? __ldg(P.ph0 + j) : 0.0f;
                r = prep_sub<EXACT>(P, x, y, z, a, ph, (float)(w0 + 16 * (s & 1)) + 7.5f,
                                    (float)(h0 + 16 * (s >> 1)) + 7.5f);
                if (EXACT) xb = fmaxf(xb, xbound(r));
            }
            sp[s][pp][0] = make_float4(r.c0, r.ax, r.ay, r.bx);
            sp[s][pp][1] = EXACT ? make_float4(r.by, r.h1, r.h2, r.h3) : make_float4(r.by, r.A, 0.f, 0.f);
            sp[s][pp][2] = make_float4(r.A, r.Ah, r.R, 0.f);
        }
        const int use_closed = EXACT ? __syncthreads_or(xb > SERIES_XMAX) : (__syncthreads(), 0);
        const int cnt = min(CGH_BATCH, P.n - base);
        float2 b[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) b[k] = make_float2(0.f, 0.f);
        const float4 (*rec)[3] = sp[sub];
        if (!EXACT) {
#pragma unroll 2
            for (int k = 0; k < cnt; ++k) {
                const float4 r0 = rec[k][0], r1 = rec[k][1];
                const float u = fmaf(r0.w, dw2, fmaf(r0.y, dw, r0.x));
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    const float2 c = __ffma2_rn(f2(r1.x), dh2p[i], __ffma2_rn(f2(r0.z), dhp[i], f2(u)));
                    accumulate_pair(b[i], b[i + 2], f2(r1.y), c);
                }
            }
        } else if (!use_closed) {
#pragma unroll 2
            for (int k = 0; k < cnt; ++k) {
                const float4 r0 = rec[k][0], r1 = rec[k][1], r2 = rec[k][2];
                const float u = fmaf(r0.w, dw2, r0.y * dw);
#pragma unroll
                for (int i = 0; i < 2; ++i) {
                    const float2 x = __ffma2_rn(f2(r1.x), dh2p[i], __ffma2_rn(f2(r0.z), dhp[i], f2(u)));
                    const float2 cyc =
                        __ffma2_rn(x, __ffma2_rn(x, __ffma2_rn(x, f2(r1.w), f2(r1.z)), f2(r1.y)), f2(r0.x));
                    accumulate_pair(b[i], b[i + 2], __ffma2_rn(f2(r2.y), x, f2(r2.x)), cyc);
                }
            }
        } else {
            for (int k = 0; k < cnt; ++k) {
                const float4 r0 = rec[k][0], r2 = rec[k][2];
                const float4 r1 = rec[k][1];
                const float u = fmaf(r0.w, dw2, r0.y * dw);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float x = fmaf(r1.x, dh2[i], fmaf(r0.z, dh[i], u));
                    const float sq = sqrtf(1.0f + x);
                    const float cyc = fmaf(r2.z, x / (1.0f + sq), r0.x);
                    const float amp = r2.x / sq;
                    const float2 e = cis_cycles(wrap_add(cyc));
                    b[i].x = fmaf(amp, e.x, b[i].x);
                    b[i].y = fmaf(amp, e.y, b[i].y);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            acc[k].x += b[k].x;
            acc[k].y += b[k].y;
        }
        __syncthreads();
    }
    const int w = w0 + 16 * (sub & 1) + tx;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int h = h0 + 16 * (sub >> 1) + tq + 4 * k;
        if (w >= P.nx || h >= P.ny) continue;
        const float2 a = acc[k];
        const size_t i = (size_t)h * P.nx + w;
        if (P.U) {
            float2 v = a;
            if (P.accumulate) {
                const float2 o = P.U[i];
                v.x += o.x;
                v.y += o.y;
            }
            P.U[i] = v;
        }
        if (P.phase_out) P.phase_out[i] = atan2f(a.y, a.x);
    }
}

static int cgh_launch(bool exact, const float *points, const float *amp, const float *phase0, int n, void *U,
                      float *phase_out, int ny, int nx, double py, double px, double lambda, int flags,
                      olg_stream_t stream)
{
    if (!points && n > 0) return fail(OLG_ERR_INVALID_ARG, "null points");
    if (!U && !phase_out) return fail(OLG_ERR_INVALID_ARG, "no output");
    if (n < 0 || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad sizes");
    if (!(px > 0) || !(py > 0) || !(lambda > 0)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if ((flags & OLG_ACCUMULATE) && !U) return fail(OLG_ERR_INVALID_ARG, "accumulate needs U");
    CghParams P{};
    P.pts = points; P.amp = amp; P.ph0 = phase0; P.n = n; P.ny = ny; P.nx = nx;
    DF d = split_df(px); P.px_hi = d.hi; P.px_lo = d.lo;
    d = split_df(py); P.py_hi = d.hi; P.py_lo = d.lo;
    d = split_df(1.0 / lambda); P.il_hi = d.hi; P.il_lo = d.lo;
    d = split_df(lambda); P.l_hi = d.hi; P.l_lo = d.lo;
    P.U = (float2 *)U;
    P.phase_out = phase_out;
    P.accumulate = (flags & OLG_ACCUMULATE) ? 1 : 0;
    dim3 grid((nx + 31) / 32, (ny + 31) / 32);
    cudaStream_t st = (cudaStream_t)stream;
    if (exact) k_cgh<true><<<grid, 256, 0, st>>>(P);
    else k_cgh<false><<<grid, 256, 0, st>>>(P);
    count_launch();
    return check_launch(exact ? "k_cgh<exact>" : "k_cgh<fresnel>");
}

// ------------------------------------------------------------------ adjoint
// Transposed sum g_j = sum_{h,w} conj(K_j(h,w)) G[h,w], K_j the unit-weight
// kernel of the forward sum (no a_j, no phi_j): the adjoint of the linear map
// from the complex point amplitudes c_j = a_j e^{i phi_j} to the hologram.
// Like the reference's gCghReduction (golcgh.h:147-195) it is parallel over
// points.  CTA = 256 threads over 256 points: thread t owns points t and
// t + 128 of its chunk in the two lanes of the paired FP32 pipe, and pixel
// rows 8 (t / 128) .. +7 of each 16 x 16 subtile, so one warp reads one G
// value per step (a shared-memory broadcast) for two terms.  Each CTA walks
// a band of subtiles; per (subtile, point) the phase is anchored at the
// subtile centre in double-float (prep_sub, as the forward), each pixel adds
// the local expansion in FP32.  Per-band partial sums go to scratch and
// k_cgh_adj_reduce adds the bands in a fixed order: deterministic.
constexpr int ADJ_PTS = 256;

struct AdjParams {
    CghParams P;       // points, sizes, pitches, lambda (amp / ph0 unused)
    const float2 *G;   // ny x nx
    float2 *part;      // bands x n partial sums
    float2 *g;         // n
    int bands, nsub_x, nsub;
};

__device__ __forceinline__ float2 ld_sub_g(const AdjParams &A, int s, int i)
{
    const int sy = s / A.nsub_x, sx = s - sy * A.nsub_x;
    const int h = sy * 16 + (i >> 4), w = sx * 16 + (i & 15);
    if (s >= A.nsub || h >= A.P.ny || w >= A.P.nx) return make_float2(0.f, 0.f);
    return __ldg(A.G + (size_t)h * A.P.nx + w);
}

template <bool EXACT>
__global__ void __launch_bounds__(256) k_cgh_adj(AdjParams A)
{
    __shared__ float2 gs[16][17];
    const CghParams &P = A.P;
    const int tid = threadIdx.x;
    const int chunk = blockIdx.x, band = blockIdx.y;
    const int pa = tid & 127, lane = tid >> 7;
    const int ja = chunk * ADJ_PTS + pa, jb = ja + 128;
    const bool va = ja < P.n, vb = jb < P.n;
    float xa = 0.f, ya = 0.f, za = 1.f, xb = 0.f, yb = 0.f, zb = 1.f;
    if (va) { xa = __ldg(P.pts + 3 * ja); ya = __ldg(P.pts + 3 * ja + 1); za = __ldg(P.pts + 3 * ja + 2); }
    if (vb) { xb = __ldg(P.pts + 3 * jb); yb = __ldg(P.pts + 3 * jb + 1); zb = __ldg(P.pts + 3 * jb + 2); }
    // subtiles [s0, s1) of this band
    const int per = (A.nsub + A.bands - 1) / A.bands;
    const int s0 = band * per, s1 = min(A.nsub, s0 + per);
    float2 accr = make_float2(0.f, 0.f), acci = make_float2(0.f, 0.f); // (a, b) lanes
    float2 gnext = s0 < s1 ? ld_sub_g(A, s0, tid) : make_float2(0.f, 0.f);
    for (int s = s0; s < s1; ++s) {
        __syncthreads();
        gs[tid >> 4][tid & 15] = gnext;
        __syncthreads();
        if (s + 1 < s1) gnext = ld_sub_g(A, s + 1, tid);
        const int sy = s / A.nsub_x, sx = s - sy * A.nsub_x;
        const float wc = (float)(sx * 16) + 7.5f, hc = (float)(sy * 16) + 7.5f;
        const Sub ra = prep_sub<EXACT>(P, xa, ya, za, va ? 1.f : 0.f, 0.f, wc, hc);
        const Sub rb = prep_sub<EXACT>(P, xb, yb, zb, vb ? 1.f : 0.f, 0.f, wc, hc);
        const bool closed = EXACT && (xbound(ra) > SERIES_XMAX || xbound(rb) > SERIES_XMAX);
        const float2 ax = make_float2(ra.ax, rb.ax), bx = make_float2(ra.bx, rb.bx);
        for (int r = 0; r < 8; ++r) {
            const int row = lane * 8 + r;
            const float dh = (float)row - 7.5f, dh2 = dh * dh;
            // row part of the expansion: c0 + ay dh + by dh^2 (Fresnel) or ay dh + by dh^2 (exact x)
            const float2 u = make_float2(fmaf(ra.by, dh2, fmaf(ra.ay, dh, EXACT ? 0.f : ra.c0)),
                                         fmaf(rb.by, dh2, fmaf(rb.ay, dh, EXACT ? 0.f : rb.c0)));
#pragma unroll 4
            for (int c = 0; c < 16; ++c) {
                const float dw = (float)c - 7.5f;
                const float2 gv = gs[row][c];
                const float2 t = __ffma2_rn(bx, f2(dw * dw), __ffma2_rn(ax, f2(dw), u));
                float2 cyc, amp;
                if (!EXACT) {
                    cyc = t;
                    amp = make_float2(ra.A, rb.A);
                } else if (!closed) {
                    cyc = __ffma2_rn(t, __ffma2_rn(t, __ffma2_rn(t, make_float2(ra.h3, rb.h3), make_float2(ra.h2, rb.h2)),
                                                     make_float2(ra.h1, rb.h1)),
                                     make_float2(ra.c0, rb.c0));
                    amp = __ffma2_rn(make_float2(ra.Ah, rb.Ah), t, make_float2(ra.A, rb.A));
                } else {
                    const float qa = sqrtf(1.0f + t.x), qb = sqrtf(1.0f + t.y);
                    cyc = make_float2(fmaf(ra.R, t.x / (1.0f + qa), ra.c0), fmaf(rb.R, t.y / (1.0f + qb), rb.c0));
                    amp = make_float2(ra.A / qa, rb.A / qb);
                }
                const float2 rr = __fadd2_rn(__fadd2_rn(cyc, f2(12582912.0f)), f2(-12582912.0f));
                const float2 a = __fmul2_rn(__ffma2_rn(rr, f2(-1.0f), cyc), f2(6.283185307179586f));
                float sa, ca, sb, cb;
                __sincosf(a.x, &sa, &ca);
                __sincosf(a.y, &sb, &cb);
                const float2 cc = __fmul2_rn(amp, make_float2(ca, cb));
                const float2 ss = __fmul2_rn(amp, make_float2(sa, sb));
                // conj(amp e^{i a}) * G
                accr = __ffma2_rn(cc, f2(gv.x), __ffma2_rn(ss, f2(gv.y), accr));
                acci = __ffma2_rn(cc, f2(gv.y), __ffma2_rn(ss, f2(-gv.x), acci));
            }
        }
    }
    // add the two row halves (lanes 0 and 1 hold the same points) in a fixed order
    __shared__ float4 red[128];
    if (lane == 1) red[pa] = make_float4(accr.x, acci.x, accr.y, acci.y);
    __syncthreads();
    if (lane == 0) {
        const float4 o = red[pa];
        float2 *dst = A.part + (size_t)band * P.n;
        if (va) dst[ja] = make_float2(accr.x + o.x, acci.x + o.y);
        if (vb) dst[jb] = make_float2(accr.y + o.z, acci.y + o.w);
    }
}

__global__ void k_cgh_adj_reduce(AdjParams A)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= A.P.n) return;
    float2 s = A.P.accumulate ? A.g[j] : make_float2(0.f, 0.f);
    for (int b = 0; b < A.bands; ++b) {
        const float2 v = A.part[(size_t)b * A.P.n + j];
        s.x += v.x;
        s.y += v.y;
    }
    A.g[j] = s;
}

// bands so that chunks x bands fills about 8 waves of the resident CTAs
static int adj_bands(bool exact, int chunks, int nsub)
{
    int dev = 0, occ = 4;
    const int nsm = sm_count();
    if (cudaGetDevice(&dev) == cudaSuccess) {
        int v = 0;
        const cudaError_t e = exact ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_cgh_adj<true>, 256, 0)
                                    : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_cgh_adj<false>, 256, 0);
        if (e == cudaSuccess && v > 0) occ = v;
    }
    const long target = 8L * nsm * occ;
    long b = target / chunks;
    if (b < 1) b = 1;
    if (b > nsub) b = nsub;
    return (int)b;
}

static size_t adj_workspace(int n, int ny, int nx, bool exact, int *bands_out)
{
    const int nsub = ((ny + 15) / 16) * ((nx + 15) / 16);
    const int chunks = (n + ADJ_PTS - 1) / ADJ_PTS;
    const int bands = adj_bands(exact, chunks > 0 ? chunks : 1, nsub);
    if (bands_out) *bands_out = bands;
    return (size_t)bands * (size_t)(n > 0 ? n : 1) * sizeof(float2);
}

static int cgh_adjoint(bool exact, const float *points, int n, const void *G, void *g, int ny, int nx, double py,
                       double px, double lambda, int flags, void *work, size_t work_bytes, olg_stream_t stream)
{
    if (n < 0 || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad sizes");
    if (n > 0 && (!points || !G || !g)) return fail(OLG_ERR_INVALID_ARG, "null pointer");
    if (((uintptr_t)G & 7) || ((uintptr_t)g & 7)) return fail(OLG_ERR_INVALID_ARG, "G and g must be 8-byte aligned");
    if (!(px > 0) || !(py > 0) || !(lambda > 0)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if (n == 0) return OLG_OK;
    AdjParams A{};
    CghParams &P = A.P;
    P.pts = points; P.n = n; P.ny = ny; P.nx = nx;
    DF d = split_df(px); P.px_hi = d.hi; P.px_lo = d.lo;
    d = split_df(py); P.py_hi = d.hi; P.py_lo = d.lo;
    d = split_df(1.0 / lambda); P.il_hi = d.hi; P.il_lo = d.lo;
    d = split_df(lambda); P.l_hi = d.hi; P.l_lo = d.lo;
    P.accumulate = (flags & OLG_ACCUMULATE) ? 1 : 0;
    A.G = (const float2 *)G;
    A.g = (float2 *)g;
    A.nsub_x = (nx + 15) / 16;
    A.nsub = A.nsub_x * ((ny + 15) / 16);
    const size_t need = adj_workspace(n, ny, nx, exact, &A.bands);
    cudaStream_t st = (cudaStream_t)stream;
    Scratch S;
    if (int rc = S.acquire(work, work_bytes, need, st)) return rc;
    A.part = (float2 *)S.ptr;
    const dim3 grid((n + ADJ_PTS - 1) / ADJ_PTS, A.bands);
    if (exact) k_cgh_adj<true><<<grid, 256, 0, st>>>(A);
    else k_cgh_adj<false><<<grid, 256, 0, st>>>(A);
    count_launch();
    if (int rc = check_launch(exact ? "k_cgh_adj<exact>" : "k_cgh_adj<fresnel>")) return rc;
    k_cgh_adj_reduce<<<(n + 255) / 256, 256, 0, st>>>(A);
    count_launch();
    return check_launch("k_cgh_adj_reduce");
}

} // namespace olg

using namespace olg;

extern "C" size_t olg_cgh_adjoint_workspace_bytes(int n_points, int ny, int nx, int exact)
{
    if (n_points <= 0 || ny <= 0 || nx <= 0) return 0;
    return adj_workspace(n_points, ny, nx, exact != 0, nullptr);
}

extern "C" int olg_cgh_fresnel_adjoint_c64(const float *points, int n_points, const void *G, void *g, int ny, int nx,
                                           double py, double px, double lambda, int flags, void *work,
                                           size_t work_bytes, olg_stream_t stream)
{
    return cgh_adjoint(false, points, n_points, G, g, ny, nx, py, px, lambda, flags, work, work_bytes, stream);
}

extern "C" int olg_cgh_exact_adjoint_c64(const float *points, int n_points, const void *G, void *g, int ny, int nx,
                                         double py, double px, double lambda, int flags, void *work, size_t work_bytes,
                                         olg_stream_t stream)
{
    return cgh_adjoint(true, points, n_points, G, g, ny, nx, py, px, lambda, flags, work, work_bytes, stream);
}

extern "C" int olg_cgh_fresnel_c64(const float *points, const float *amp, const float *phase0, int n_points, void *U,
                                   float *phase_out, int ny, int nx, double py, double px, double lambda, int flags,
                                   olg_stream_t stream)
{
    return cgh_launch(false, points, amp, phase0, n_points, U, phase_out, ny, nx, py, px, lambda, flags, stream);
}

extern "C" int olg_cgh_exact_c64(const float *points, const float *amp, const float *phase0, int n_points, void *U,
                                 int ny, int nx, double py, double px, double lambda, int flags, olg_stream_t stream)
{
    return cgh_launch(true, points, amp, phase0, n_points, U, nullptr, ny, nx, py, px, lambda, flags, stream);
}
