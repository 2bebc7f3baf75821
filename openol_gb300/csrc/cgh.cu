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
//            cycles = c0 + R (x/2 - x^2/8 + x^3/16),  amplitude = A (1 - x/2 + 3x^2/8)
// with (dw, dh) the pixel offset from the tile centre (|d| <= 7.5).  The
// series is used while |x| <= 2e-3 for every point of a batch (truncation
// < 1e-7 cycles); otherwise the batch uses the closed form
// R x / (1 + sqrt(1 + x)).  Per term: 2 MUFU (sin, cos) + ~10 FP32 ops.
//
// CTA = 256 threads over a 16 x 32 pixel tile (two 16 x 16 subtiles, each
// with its own anchor), 2 pixels per thread; 256 points per batch, thread t
// preparing point t's constants for both subtiles.  Summation is sequential
// over points (deterministic), in per-batch partial sums.
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

constexpr int CGH_BATCH = 256;
constexpr float SERIES_XMAX = 2e-3f;

// per (subtile, point) constants
struct Sub {
    float c0, ax, ay, bx, by, R, A, pad;
};

template <bool EXACT>
__device__ __forceinline__ Sub prep_sub(const CghParams &P, float x, float y, float z, float a, float ph, float wc,
                                        float hc)
{
    Sub s;
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
        s.R = 0.f;
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
        s.A = a / r0.hi;
    }
    s.pad = 0.f;
    return s;
}

__device__ __forceinline__ float xbound(const Sub &s)
{
    return fabsf(s.ax) * 7.5f + fabsf(s.ay) * 7.5f + (fabsf(s.bx) + fabsf(s.by)) * 56.25f;
}

template <bool EXACT>
__global__ void __launch_bounds__(256) k_cgh(CghParams P)
{
    __shared__ float4 sp[CGH_BATCH][4]; // [point][sub0 c0..by | sub0 R,A | sub1 ... ]
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int w0 = blockIdx.x * 16, h0 = blockIdx.y * 32;
    const float dw = (float)tx - 7.5f, dh = (float)ty - 7.5f;
    const float dw2 = dw * dw, dh2 = dh * dh;
    const float wc = (float)w0 + 7.5f, hc0 = (float)h0 + 7.5f, hc1 = (float)h0 + 23.5f;
    float2 acc0 = make_float2(0.f, 0.f), acc1 = acc0;

    for (int base = 0; base < P.n; base += CGH_BATCH) {
        const int j = base + tid;
        Sub s0{}, s1{};
        float xb = 0.f;
        if (j < P.n) {
            const float x = __ldg(P.pts + 3 * j), y = __ldg(P.pts + 3 * j + 1), z = __ldg(P.pts + 3 * j + 2);
            const float a = P.amp ? __ldg(P.amp + j) : 1.0f;
            const float ph = P.ph0 ? __ldg(P.ph0 + j) : 0.0f;
            s0 = prep_sub<EXACT>(P, x, y, z, a, ph, wc, hc0);
            s1 = prep_sub<EXACT>(P, x, y, z, a, ph, wc, hc1);
            if (EXACT) xb = fmaxf(xbound(s0), xbound(s1));
        }
        sp[tid][0] = make_float4(s0.c0, s0.ax, s0.ay, s0.bx);
        sp[tid][1] = make_float4(s0.by, s0.R, s0.A, 0.f);
        sp[tid][2] = make_float4(s1.c0, s1.ax, s1.ay, s1.bx);
        sp[tid][3] = make_float4(s1.by, s1.R, s1.A, 0.f);
        const int use_closed = EXACT ? __syncthreads_or(xb > SERIES_XMAX) : (__syncthreads(), 0);
        const int cnt = min(CGH_BATCH, P.n - base);
        float2 b0 = make_float2(0.f, 0.f), b1 = b0;
#pragma unroll 4
        for (int k = 0; k < cnt; ++k) {
            const float4 p0 = sp[k][0], q0 = sp[k][1], p1 = sp[k][2], q1 = sp[k][3];
            if (!EXACT) {
                float c = fmaf(p0.y, dw, fmaf(p0.z, dh, fmaf(p0.w, dw2, fmaf(q0.x, dh2, p0.x))));
                float2 e = cis_cycles(wrap_cycles(c));
                b0.x = fmaf(q0.z, e.x, b0.x);
                b0.y = fmaf(q0.z, e.y, b0.y);
                c = fmaf(p1.y, dw, fmaf(p1.z, dh, fmaf(p1.w, dw2, fmaf(q1.x, dh2, p1.x))));
                e = cis_cycles(wrap_cycles(c));
                b1.x = fmaf(q1.z, e.x, b1.x);
                b1.y = fmaf(q1.z, e.y, b1.y);
            } else {
#pragma unroll
                for (int sidx = 0; sidx < 2; ++sidx) {
                    const float4 p = sidx ? p1 : p0, q = sidx ? q1 : q0;
                    const float x = fmaf(p.y, dw, fmaf(p.z, dh, fmaf(p.w, dw2, q.x * dh2)));
                    float cyc, amp;
                    if (!use_closed) {
                        const float poly = fmaf(x, fmaf(x, 0.0625f, -0.125f), 0.5f);
                        cyc = fmaf(q.y * x, poly, p.x);
                        amp = q.z * fmaf(x, fmaf(x, 0.375f, -0.5f), 1.0f);
                    } else {
                        const float sq = sqrtf(1.0f + x);
                        cyc = fmaf(q.y, x / (1.0f + sq), p.x);
                        amp = q.z / sq;
                    }
                    const float2 e = cis_cycles(wrap_cycles(cyc));
                    float2 &b = sidx ? b1 : b0;
                    b.x = fmaf(amp, e.x, b.x);
                    b.y = fmaf(amp, e.y, b.y);
                }
            }
        }
        acc0.x += b0.x; acc0.y += b0.y;
        acc1.x += b1.x; acc1.y += b1.y;
        __syncthreads();
    }
    const int w = w0 + tx;
#pragma unroll
    for (int sidx = 0; sidx < 2; ++sidx) {
        const int h = h0 + ty + 16 * sidx;
        if (w >= P.nx || h >= P.ny) continue;
        const float2 a = sidx ? acc1 : acc0;
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
    dim3 grid((nx + 15) / 16, (ny + 31) / 32);
    cudaStream_t st = (cudaStream_t)stream;
    if (exact) k_cgh<true><<<grid, 256, 0, st>>>(P);
    else k_cgh<false><<<grid, 256, 0, st>>>(P);
    count_launch();
    return check_launch(exact ? "k_cgh<exact>" : "k_cgh<fresnel>");
}

} // namespace olg

using namespace olg;

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
