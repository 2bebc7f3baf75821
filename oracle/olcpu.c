/*
 * olcpu.c -- FP64 CPU restatement of OpenOL's propagation / CGH / WRP path.
 * TEST INFRASTRUCTURE ONLY (the oracle; see olcpu.h).  Build with
 * -ffp-contract=off: the WRP window test below must round every float32
 * operation separately, on x86 and on Arm alike.
 */
#include "olcpu.h"
#include "olfft.h"

#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

static cplx *cz(long n) { return (cplx *)calloc((size_t)n, sizeof(cplx)); }

/* centred 2x zero padding: olutils.h:155-178 (general zeropadding with
 * out = 2 * in, pad_l = (out - in) / 2) == golutils.h:207-224. */
static cplx *pad2(const cplx *u, long ny, long nx)
{
    const long NY = 2 * ny, NX = 2 * nx, oy = (NY - ny) / 2, ox = (NX - nx) / 2;
    cplx *U = cz(NY * NX);
    for (long h = 0; h < ny; ++h)
        memcpy(U + (h + oy) * NX + ox, u + h * nx, (size_t)nx * sizeof(cplx));
    return U;
}

/* central crop of a 2x padded field: del_zero olutils.h:181-198 ==
 * gdel_zero golutils.h:247-259 == gcut at ((ny2-ny)/2, (nx2-nx)/2) golprop.h:533. */
static void crop2(const cplx *U, long ny, long nx, cplx *out)
{
    const long NY = 2 * ny, NX = 2 * nx, oy = NY / 4, ox = NX / 4;
    for (long h = 0; h < ny; ++h)
        memcpy(out + h * nx, U + (h + oy) * NX + ox, (size_t)nx * sizeof(cplx));
}

/* quadrant swap, fftshift olutils.h:95-117 (even sizes) */
static void fftshift2(cplx *u, long H, long W)
{
    const long hh = H / 2, hw = W / 2;
    for (long h = 0; h < hh; ++h)
        for (long w = 0; w < hw; ++w) {
            long i1 = h * W + w, i2 = (h + hh) * W + (w + hw);
            cplx t = u[i1]; u[i1] = u[i2]; u[i2] = t;
            i1 = h * W + (w + hw); i2 = (h + hh) * W + w;
            t = u[i1]; u[i1] = u[i2]; u[i2] = t;
        }
}

void olc_fft2d(double *u, long ny, long nx, int sign, int nthreads) { olfft_2d(u, ny, nx, sign, nthreads); }

static void fft2(cplx *u, long ny, long nx, int sign) { olfft_2d((double *)u, ny, nx, sign, 0); }

/* ------------------------------------------------------------------ ASM */
void olc_asm_prop(double *ud, long ny, long nx, double dy, double dx, double lambda, double z, int flags)
{
    cplx *u = (cplx *)ud;
    const long NY = 2 * ny, NX = 2 * nx, N = NY * NX;
    const double du = 1.0 / (dx * NX), dv = 1.0 / (dy * NY);
    cplx *U = pad2(u, ny, nx);
    cplx *H = cz(N);
    const double tmp = 1.0 / (lambda * lambda);
    /* AsmTransferF olprop.h:173-189 on the padded grid */
#pragma omp parallel for
    for (long n = 0; n < NY; ++n) {
        const double v = (double)(n - NY / 2) * dv;
        for (long m = 0; m < NX; ++m) {
            const double uu = (double)(m - NX / 2) * du;
            const double w = sqrt(tmp - uu * uu - v * v);
            const double phase = 2 * M_PI * w * z;
            H[n * NX + m] = cos(phase) + I * sin(phase);
        }
    }
    fftshift2(H, NY, NX);
    fft2(U, NY, NX, -1);
    const double sc = (flags & OLC_NO_NORMALIZE) ? 1.0 : 1.0 / (double)N;
    const int cj = flags & OLC_CONJ;
#pragma omp parallel for
    for (long i = 0; i < N; ++i) U[i] *= (cj ? conj(H[i]) : H[i]) * sc;
    fft2(U, NY, NX, +1);
    crop2(U, ny, nx, u);
    free(H);
    free(U);
}

/* ------------------------------------------------------------- Fresnel */
/* FresnelResponse olprop.h:8-24 (optionally band limited, olprop.h:26-50 /
 * golprop.h:202-234), on the padded grid, then fftshift. */
static void fresnel_response(cplx *h, long NY, long NX, double dy, double dx, double lambda, double z,
                             int bandlimit)
{
    const double tmp = 1.0 / (lambda * z);
    const long hh = NY / 2, hw = NX / 2;
    long wlim = 0, hlim = 0;
    if (bandlimit == 1) {
        const double xlim = fabs(lambda * z * 0.5 / dx);
        wlim = hlim = (long)floor(xlim / dx);
    } else if (bandlimit == 2) {
        wlim = (long)floor(fabs(lambda * z * 0.5 / dx) / dx);
        hlim = (long)floor(fabs(lambda * z * 0.5 / dy) / dy);
    }
#pragma omp parallel for
    for (long n = 0; n < NY; ++n) {
        const double y = (double)(n - hh) * dy;
        for (long m = 0; m < NX; ++m) {
            const double x = (double)(m - hw) * dx;
            if (bandlimit && !(labs(m - hw) < wlim && labs(n - hh) < hlim)) {
                h[n * NX + m] = 0;
                continue;
            }
            const double phase = M_PI * (x * x + y * y) * tmp;
            h[n * NX + m] = cos(phase) + I * sin(phase);
        }
    }
    fftshift2(h, NY, NX);
}

void olc_fresnel_prop(double *ud, long ny, long nx, double dy, double dx, double lambda, double z,
                      int bandlimit, int flags)
{
    cplx *u = (cplx *)ud;
    const long NY = 2 * ny, NX = 2 * nx, N = NY * NX;
    cplx *U = pad2(u, ny, nx);
    cplx *h = cz(N);
    fresnel_response(h, NY, NX, dy, dx, lambda, z, bandlimit);
    const int host = flags & OLC_NO_NORMALIZE;
    if (host) fftshift2(U, NY, NX); /* golprop.h:84 */
    fft2(U, NY, NX, -1);
    fft2(h, NY, NX, -1);
    const double sc = host ? 1.0 : 1.0 / ((double)N * (double)N);
    const int cj = flags & OLC_CONJ;
#pragma omp parallel for
    for (long i = 0; i < N; ++i) U[i] *= (cj ? conj(h[i]) : h[i]) * sc;
    fft2(U, NY, NX, +1);
    if (host) fftshift2(U, NY, NX); /* golprop.h:114 */
    crop2(U, ny, nx, u);
    free(h);
    free(U);
}

/* ---------------------------------------------------------------- ARSS */
static long floor_lim(double v)
{
    double f = floor(v);
    if (!(f < 1073741824.0)) f = 1073741824.0; /* +inf / huge: every pixel is inside */
    if (f < -1073741824.0) f = -1073741824.0;
    return (long)f;
}

int olc_arss_windows(long ny, long nx, double dy, double dx, double lambda, double z, double s, int64_t *lims)
{
    (void)ny; (void)nx;
    if (s == 0.0 || s == 1.0) return -1;
    /* golprop.h:849-852 (pre-chirp), :891-892 (h: x only), :928-931 (Cz) */
    lims[0] = floor_lim((lambda * fabs(z) * 0.5 / (s * fabs(s - 1) * dy)) / dy);
    lims[1] = floor_lim((lambda * fabs(z) * 0.5 / (s * fabs(s - 1) * dx)) / dx);
    lims[2] = floor_lim(fabs(lambda * z * 0.5 / (dx * s)) / dx);
    lims[3] = floor_lim((lambda * fabs(z) * 0.5 / (fabs(1 - s) * dy)) / dy);
    lims[4] = floor_lim((lambda * fabs(z) * 0.5 / (fabs(1 - s) * dx)) / dx);
    lims[5] = 0;
    return 0;
}

int olc_arss_prop(const double *srcd, double *dstd, long ny, long nx, double dy, double dx,
                  double lambda, double z, double s, double oy, double ox, int flags)
{
    int64_t L[6];
    if (flags & OLC_NO_WINDOWS) {
        for (int k = 0; k < 6; ++k) L[k] = 1073741824; /* every pixel inside */
    } else if (olc_arss_windows(ny, nx, dy, dx, lambda, z, s, L)) {
        return -1;
    }
    const long hlim_u = L[0], wlim_u = L[1], lim_h = L[2], hlim_c = L[3], wlim_c = L[4];
    const long NY = 2 * ny, NX = 2 * nx, N = NY * NX, n = ny * nx;
    const double tmp = M_PI / (lambda * z);
    const long hny = ny / 2, hnx = nx / 2;
    const int adj = flags & OLC_CONJ;
    cplx *a = cz(n);
    memcpy(a, srcd, (size_t)n * sizeof(cplx));

    /* stage 1: forward gARSSFresnelProp_u golprop.h:817-843 (zero outside its
     * window); adjoint: conj of gARSSFresnelProp_Cz golprop.h:901-922 (identity
     * outside its window) */
#pragma omp parallel for
    for (long h = 0; h < ny; ++h)
        for (long w = 0; w < nx; ++w) {
            const long i = h * nx + w;
            if (!adj) {
                if (labs(w - hnx) >= wlim_u || labs(h - hny) >= hlim_u) { a[i] = 0; continue; }
                const double y1 = (h - hny) * dy, x1 = (w - hnx) * dx;
                double ph = (s * s - s) * x1 * x1 - 2 * s * ox * x1 + (s * s - s) * y1 * y1 - 2 * s * oy * y1;
                ph *= tmp;
                a[i] *= cos(ph) + I * sin(ph);
            } else {
                if (labs(w - hnx) < wlim_c && labs(h - hny) < hlim_c) {
                    const double y2 = (h - hny) * dy, x2 = (w - hnx) * dx;
                    double ph = (1 - s) * x2 * x2 + 2 * ox * x2 + ox * ox + (1 - s) * y2 * y2 + 2 * oy * y2 + oy * oy;
                    ph *= tmp;
                    a[i] *= cos(ph) - I * sin(ph);
                }
            }
        }
    cplx *U = pad2(a, ny, nx);
    fft2(U, NY, NX, -1);
    /* gARSSFresnelProp_h golprop.h:862-884, fftshift, FFT, 1/Np */
    cplx *hb = cz(N);
    const long hh = NY / 2, hw = NX / 2;
#pragma omp parallel for
    for (long h = 0; h < NY; ++h)
        for (long w = 0; w < NX; ++w) {
            if (labs(w - hw) >= lim_h || labs(h - hh) >= lim_h) { hb[h * NX + w] = 0; continue; }
            const double y1 = (h - hh) * dy, x1 = (w - hw) * dx;
            const double ph = (s * x1 * x1 + s * y1 * y1) * tmp;
            hb[h * NX + w] = cos(ph) + I * sin(ph);
        }
    fftshift2(hb, NY, NX);
    fft2(hb, NY, NX, -1);
    const double sc = 1.0 / ((double)N * (double)N);
#pragma omp parallel for
    for (long i = 0; i < N; ++i) U[i] *= (adj ? conj(hb[i]) : hb[i]) * sc;
    fft2(U, NY, NX, +1);
    crop2(U, ny, nx, a);
    /* stage 3: forward Cz (identity outside window); adjoint: conj pre-chirp, zero outside */
#pragma omp parallel for
    for (long h = 0; h < ny; ++h)
        for (long w = 0; w < nx; ++w) {
            const long i = h * nx + w;
            if (!adj) {
                if (labs(w - hnx) < wlim_c && labs(h - hny) < hlim_c) {
                    const double y2 = (h - hny) * dy, x2 = (w - hnx) * dx;
                    double ph = (1 - s) * x2 * x2 + 2 * ox * x2 + ox * ox + (1 - s) * y2 * y2 + 2 * oy * y2 + oy * oy;
                    ph *= tmp;
                    a[i] *= cos(ph) + I * sin(ph);
                }
            } else {
                if (labs(w - hnx) >= wlim_u || labs(h - hny) >= hlim_u) { a[i] = 0; continue; }
                const double y1 = (h - hny) * dy, x1 = (w - hnx) * dx;
                double ph = (s * s - s) * x1 * x1 - 2 * s * ox * x1 + (s * s - s) * y1 * y1 - 2 * s * oy * y1;
                ph *= tmp;
                a[i] *= cos(ph) - I * sin(ph);
            }
        }
    memcpy(dstd, a, (size_t)n * sizeof(cplx));
    free(hb);
    free(U);
    free(a);
    return 0;
}

/* ------------------------------------------------------ shifted ASM / split */
/* band window of shiftedAsmTransferF olprop.h:254-284 for one axis, in double */
static void shifted_band(double d, double o, double z, double lambda, double *c, double *w)
{
    const double s0 = 0.5 / d;
    const double lm = 1 / sqrt(pow(o - 0.5 / d, -2) * z * z + 1.0) / lambda;
    const double lp = 1 / sqrt(pow(o + 0.5 / d, -2) * z * z + 1.0) / lambda;
    if (s0 < o) {
        *c = 0.5 * (lp + lm);
        *w = lp - lm;
    } else if (-s0 <= o && o < s0) {
        *c = 0.5 * (lp - lm);
        *w = lp + lm;
    } else {
        *c = -0.5 * (lp + lm);
        *w = lm - lp;
    }
}

/* the same with PREC_T = float, each operation rounded as that instantiation
 * rounds it: float operands, std::pow(float, int) and the sqrt in double,
 * results stored to float (this file is built with -ffp-contract=off) */
static void shifted_band_f(float d, float o, float z, float lambda, float *c, float *w)
{
    const float s0 = 0.5f / d;
    volatile float tm = o - 0.5f / d, tp = o + 0.5f / d;
    const float lm = (float)(1 / sqrt(pow((double)tm, -2) * z * z + 1.0f) / lambda);
    const float lp = (float)(1 / sqrt(pow((double)tp, -2) * z * z + 1.0f) / lambda);
    volatile float cc, ww;
    if (s0 < o) {
        cc = 0.5f * (lp + lm);
        ww = lp - lm;
    } else if (-s0 <= o && o < s0) {
        cc = 0.5f * (lp - lm);
        ww = lp + lm;
    } else {
        cc = -0.5f * (lp + lm);
        ww = lm - lp;
    }
    *c = cc;
    *w = ww;
}

void olc_shifted_asm_prop(const double *srcd, double *dstd, long ny, long nx, double dy, double dx, double lambda,
                          double z, double oy, double ox, int flags)
{
    const long NY = 2 * ny, NX = 2 * nx, N = NY * NX;
    const double du = 1.0 / (dx * NX), dv = 1.0 / (dy * NY);
    cplx *U = pad2((const cplx *)srcd, ny, nx);
    cplx *H = cz(N);
    double u0 = 0, uw = 0, v0 = 0, vw = 0;
    float u0f = 0, uwf = 0, v0f = 0, vwf = 0, duf = 0, dvf = 0;
    const int band = flags & OLC_BANDLIMIT, f32 = flags & OLC_F32_WINDOW;
    if (band && !f32) {
        shifted_band(du, ox, z, lambda, &u0, &uw);
        shifted_band(dv, oy, z, lambda, &v0, &vw);
    } else if (band) {
        /* shiftedAsmProp olprop.h:313-314: du = 1 / (dx * width2) in PREC_T */
        duf = 1 / ((float)dx * (float)NX);
        dvf = 1 / ((float)dy * (float)NY);
        shifted_band_f(duf, (float)ox, (float)z, (float)lambda, &u0f, &uwf);
        shifted_band_f(dvf, (float)oy, (float)z, (float)lambda, &v0f, &vwf);
    }
    const double tmp = 1.0 / (lambda * lambda);
    /* gshiftedAsmTransferF golprop.h:336-358 / shiftedAsmTransferF olprop.h:286-304 */
#pragma omp parallel for
    for (long n = 0; n < NY; ++n) {
        const double v = (double)(n - NY / 2) * dv;
        for (long m = 0; m < NX; ++m) {
            const double uu = (double)(m - NX / 2) * du;
            if (band && !f32 && !(fabs(uu - u0) * 2 < uw && fabs(v - v0) * 2 < vw)) {
                H[n * NX + m] = 0;
                continue;
            }
            if (band && f32) {
                const float uf = (float)(m - NX / 2) * duf, vf = (float)(n - NY / 2) * dvf;
                if (!(fabsf(uf - u0f) * 2 < uwf && fabsf(vf - v0f) * 2 < vwf)) {
                    H[n * NX + m] = 0;
                    continue;
                }
            }
            const double w = sqrt(tmp - uu * uu - v * v);
            const double phase = 2 * M_PI * (w * z + ox * uu + oy * v);
            H[n * NX + m] = cos(phase) + I * sin(phase);
        }
    }
    fftshift2(H, NY, NX);
    fft2(U, NY, NX, -1);
    const double sc = (flags & OLC_NO_NORMALIZE) ? 1.0 : 1.0 / (double)N;
    const int cj = flags & OLC_CONJ;
#pragma omp parallel for
    for (long i = 0; i < N; ++i) U[i] *= (cj ? conj(H[i]) : H[i]) * sc;
    fft2(U, NY, NX, +1);
    crop2(U, ny, nx, (cplx *)dstd);
    free(H);
    free(U);
}

int olc_split_prop(const double *srcd, double *dstd, long ny, long nx, double dy, double dx, double lambda, double z,
                   int mode, int blocks_y, int blocks_x, int flags)
{
    if (blocks_y <= 0 || blocks_x <= 0 || (mode != 0 && mode != 1)) return -1;
    const long bh = ny / blocks_y, bw = nx / blocks_x, nb = bh * bw;
    const cplx *src = (const cplx *)srcd;
    cplx *dst = (cplx *)dstd;
    if (!(flags & OLC_ACCUMULATE)) memset(dst, 0, sizeof(cplx) * (size_t)(ny * nx));
    cplx *a = cz(nb), *b = cz(nb);
    for (long gn = 0; gn < blocks_y; ++gn)
        for (long gm = 0; gm < blocks_x; ++gm) {
            for (long h = 0; h < bh; ++h)
                memcpy(a + h * bw, src + (gn * bh + h) * nx + gm * bw, sizeof(cplx) * (size_t)bw);
            for (long dn = 0; dn < blocks_y; ++dn)
                for (long dm = 0; dm < blocks_x; ++dm) {
                    /* golprop.h:795-796: an int times a float pitch, in float */
                    const double oy = (double)((float)((gn - dn) * bh) * (float)dy);
                    const double ox = (double)((float)((gm - dm) * bw) * (float)dx);
                    if (mode == 0)
                        olc_shifted_asm_prop((const double *)a, (double *)b, bh, bw, dy, dx, lambda, z, oy, ox,
                                             flags & (OLC_CONJ | OLC_NO_NORMALIZE | OLC_BANDLIMIT | OLC_F32_WINDOW));
                    else
                        olc_arss_prop((const double *)a, (double *)b, bh, bw, dy, dx, lambda, z, 1.0, oy, ox,
                                      (flags & OLC_CONJ) | OLC_NO_WINDOWS);
                    for (long h = 0; h < bh; ++h)
                        for (long w = 0; w < bw; ++w) dst[(dn * bh + h) * nx + dm * bw + w] += b[h * bw + w];
                }
        }
    free(a);
    free(b);
    return 0;
}

/* -------------------------------------------------------------- tilted */
/* bilinear olutils.h:213-233: the four neighbours when the cell is inside,
 * the nearest sample on the last row / column, 0 outside. */
static cplx tilt_bilinear(const cplx *src, double dsty, double dstx, long ny, long nx)
{
    const int64_t ms = (int64_t)floor(dstx), ns = (int64_t)floor(dsty);
    if (0 <= ms && ms < nx - 1 && 0 <= ns && ns < ny - 1) {
        const double s = dstx - ms, t = dsty - ns;
        const cplx u1 = (1 - s) * src[ms + ns * nx] + s * src[(ms + 1) + ns * nx];
        const cplx u2 = (1 - s) * src[ms + (ns + 1) * nx] + s * src[(ms + 1) + (ns + 1) * nx];
        return (1 - t) * u1 + t * u2;
    }
    if (0 <= ms && ms < nx && 0 <= ns && ns < ny) return src[ms + ns * nx];
    return 0;
}

/* bicubic olutils.h:290-321: 4 x 4 window, kernel of the radial distance,
 * a = -1, taps outside the grid dropped, 0 when (floor x, floor y) is outside. */
static cplx tilt_bicubic(const cplx *src, double dsty, double dstx, long ny, long nx)
{
    const double a = -1;
    const int64_t ms = (int64_t)floor(dstx), ns = (int64_t)floor(dsty);
    if (!(0 <= ms && ms < nx && 0 <= ns && ns < ny)) return 0;
    cplx avg = 0;
    for (int64_t j = 0; j < 4; j++)
        for (int64_t i = 0; i < 4; i++) {
            const int64_t m = ms - 1 + i, n = ns - 1 + j;
            if (!(0 <= m && m < nx && 0 <= n && n < ny)) continue;
            const double d = sqrt((m - dstx) * (m - dstx) + (n - dsty) * (n - dsty));
            double k;
            if (0 <= d && d < 1) k = 1 - (a + 3) * d * d + (a + 2) * d * d * d;
            else if (1 <= d && d < 2) k = -4 * a + 8 * a * d - 5 * a * d * d + a * d * d * d;
            else k = 0;
            avg += k * src[m + n * nx];
        }
    return avg;
}

/* Fresnel response with an optional linear phase exp(-2 pi i x c), fftshift,
 * FFT, 1/N, fftshift: the spectrum TiltedSourceProp (olprop.h:481-494,
 * c = a13 f0) and TiltedReferenceProp (olprop.h:546-552, none) use. */
static void tilt_fresnel_spectrum(cplx *H, long NY, long NX, double dy, double dx, double lambda, double z, double a13,
                                  double f0)
{
    const double tmp = 1 / (lambda * z);
    const long hh = NY / 2, hw = NX / 2, N = NY * NX;
#pragma omp parallel for
    for (long n = 0; n < NY; ++n) {
        const double y = (double)(n - hh) * dy;
        for (long m = 0; m < NX; ++m) {
            const double x = (double)(m - hw) * dx;
            const double phase = M_PI * (x * x + y * y) * tmp;
            cplx h = cos(phase) + I * sin(phase);
            if (f0 != 0) {
                const double w = (double)(m - NX / 2) * dx;
                const double p2 = -2 * M_PI * w * a13 * f0;
                h *= cos(p2) + I * sin(p2);
            }
            H[n * NX + m] = h;
        }
    }
    fftshift2(H, NY, NX);
    fft2(H, NY, NX, -1);
    for (long i = 0; i < N; ++i) H[i] *= 1.0 / (double)N;
    fftshift2(H, NY, NX);
}

/* TiltedSourceProp olprop.h:414-521 (reference == 0) and TiltedReferenceProp
 * olprop.h:523-600 (reference != 0), with PREC_T = double, in place on u
 * (ny x nx).  Centred spectrum of the 2x padded field (1/N), then for every
 * output frequency (fpx, fpy, fpz) the rotated source frequency
 * fsx = a11 fpx + a13 fpz [- a13 f0], fsy = fpy, sampled by bilinear or bicubic
 * interpolation and weighted by the Jacobian a11 - a13 fpx / fpz; the
 * transfer function (ASM, or the FFT of the Fresnel response) multiplies the
 * resampled spectrum (source form) or the spectrum before resampling
 * (reference form); fftshift, inverse FFT, crop, 1/N. */
void olc_tilted_prop(double *ud, long ny, long nx, double dy, double dx, double lambda, double z, double angle,
                     int interp, int mode, int reference)
{
    cplx *u = (cplx *)ud;
    const long NY = 2 * ny, NX = 2 * nx, N = NY * NX;
    const double du = 1 / (dx * NX), dv = 1 / (dy * NY);
    const double fsqr = 1 / (lambda * lambda);
    cplx *U = pad2(u, ny, nx);
    fft2(U, NY, NX, -1);
    fftshift2(U, NY, NX);
    for (long i = 0; i < N; ++i) U[i] *= 1.0 / (double)N;
    const double ang = reference ? angle : -angle;
    const double a11 = cos(ang), a12 = 0, a13 = -sin(ang);
    const double a21 = 0, a22 = 1, a23 = 0;
    const double f0 = 1 / lambda;
    cplx *H = cz(N);
    if (mode == 0) {
        const double tmp = 1 / (lambda * lambda);
        /* reference form: AsmTransferF olprop.h:173-189; source form: its
         * frequency shifted by a13 f0 (olprop.h:468-479) */
#pragma omp parallel for
        for (long n = 0; n < NY; ++n) {
            const double v = (double)(n - NY / 2) * dv;
            for (long m = 0; m < NX; ++m) {
                const double uu = reference ? (double)(m - NX / 2) * du : (double)(m - NX / 2) * du + a13 * f0;
                const double w = sqrt(tmp - uu * uu - v * v);
                const double phase = 2 * M_PI * w * z;
                H[n * NX + m] = cos(phase) + I * sin(phase);
            }
        }
    } else {
        tilt_fresnel_spectrum(H, NY, NX, dy, dx, lambda, z, a13, reference ? 0.0 : f0);
    }
    if (reference)
        for (long i = 0; i < N; ++i) U[i] = U[i] * H[i];
    cplx *Up = cz(N);
#pragma omp parallel for
    for (long n = 0; n < NY; ++n)
        for (long m = 0; m < NX; ++m) {
            const double fpx = (m - NX / 2) * du;
            const double fpy = (n - NY / 2) * dv;
            const double fpz = sqrt(fsqr - fpx * fpx - fpy * fpy);
            const double fsx = reference ? a11 * fpx + a12 * fpy + a13 * fpz
                                         : a11 * fpx + a12 * fpy + a13 * fpz - a13 * f0;
            const double fsy = a21 * fpx + a22 * fpy + a23 * fpz;
            const double y = fsy / dv + NY / 2, x = fsx / du + NX / 2;
            cplx v = interp == 1 ? tilt_bicubic(U, y, x, NY, NX) : tilt_bilinear(U, y, x, NY, NX);
            const double J = (a11 * a22 - a12 * a21) + (a12 * a23 - a13 * a22) * fpx / fpz +
                             (a13 * a21 - a11 * a23) * fpy / fpz;
            v *= J;
            Up[m + n * NX] = v;
        }
    if (!reference)
        for (long i = 0; i < N; ++i) Up[i] = Up[i] * H[i];
    fftshift2(Up, NY, NX);
    fft2(Up, NY, NX, +1);
    crop2(Up, ny, nx, u);
    for (long i = 0; i < ny * nx; ++i) u[i] *= 1.0 / (double)N;
    free(Up);
    free(H);
    free(U);
}

/* ------------------------------------------------------------- AUTO checks */
int olc_asm_prop_check(long ny, long nx, double dy, double dx, double lambda, double z)
{
    const long nx2 = 2 * nx, ny2 = 2 * ny;
    const double du = 1 / (dx * nx2), dv = 1 / (dy * ny2);
    const double umax = du * nx2 / 2, vmax = dv * ny2 / 2;
    const double t = sqrt(1 / (lambda * lambda) - umax * umax - vmax * vmax);
    const double zmax_u = t / (2 * umax * du), zmax_v = t / (2 * vmax * dv);
    return !(zmax_u < fabs(z) || zmax_v < fabs(z));
}

int olc_fresnel_prop_check(long ny, long nx, double dy, double dx, double lambda, double z)
{
    const double xmax = dx * (2 * nx) / 2, ymax = dy * (2 * ny) / 2;
    const double zmin_x = 2 * xmax * dx / lambda, zmin_y = 2 * ymax * dy / lambda;
    return !(zmin_x > fabs(z) || zmin_y > fabs(z));
}

/* ----------------------------------------------------------------- CGH */
void olc_cgh_fresnel(const double *pts, const double *amp, const double *phase0, long n,
                     double *Ud, double *phase_out, long ny, long nx, double py, double px,
                     double lambda, int flags)
{
    cplx *U = (cplx *)Ud;
#pragma omp parallel for schedule(dynamic, 1)
    for (long h = 0; h < ny; ++h)
        for (long w = 0; w < nx; ++w) {
            cplx acc = 0;
            for (long j = 0; j < n; ++j) {
                const double dx = px * w - pts[3 * j], dy = py * h - pts[3 * j + 1], dz = pts[3 * j + 2];
                double theta = 2 * M_PI * (dx * dx + dy * dy) / (2 * dz * lambda);
                if (phase0) theta += phase0[j];
                const double a = amp ? amp[j] : 1.0;
                acc += a * (cos(theta) + I * sin(theta));
            }
            const long i = h * nx + w;
            if (U) U[i] = (flags & OLC_ACCUMULATE) ? U[i] + acc : acc;
            if (phase_out) phase_out[i] = atan2(cimag(acc), creal(acc));
        }
}

void olc_cgh_exact(const double *pts, const double *amp, const double *phase0, long n,
                   double *Ud, long ny, long nx, double py, double px, double lambda, int flags)
{
    cplx *U = (cplx *)Ud;
    const double k = 2 * M_PI / lambda;
#pragma omp parallel for schedule(dynamic, 1)
    for (long h = 0; h < ny; ++h)
        for (long w = 0; w < nx; ++w) {
            cplx acc = 0;
            for (long j = 0; j < n; ++j) {
                const double dx = px * w - pts[3 * j], dy = py * h - pts[3 * j + 1], z = pts[3 * j + 2];
                const double r = sqrt(dx * dx + dy * dy + z * z);
                double theta = k * r;
                if (phase0) theta += phase0[j];
                const double a = (amp ? amp[j] : 1.0) / r;
                acc += a * (cos(theta) + I * sin(theta));
            }
            const long i = h * nx + w;
            U[i] = (flags & OLC_ACCUMULATE) ? U[i] + acc : acc;
        }
}

void olc_cgh_fresnel_adjoint(const double *pts, long n, const double *Gd, double *gd, long ny, long nx,
                             double py, double px, double lambda)
{
    const cplx *G = (const cplx *)Gd;
    cplx *g = (cplx *)gd;
#pragma omp parallel for schedule(dynamic, 4)
    for (long j = 0; j < n; ++j) {
        cplx acc = 0;
        for (long h = 0; h < ny; ++h)
            for (long w = 0; w < nx; ++w) {
                const double dx = px * w - pts[3 * j], dy = py * h - pts[3 * j + 1], dz = pts[3 * j + 2];
                const double theta = 2 * M_PI * (dx * dx + dy * dy) / (2 * dz * lambda);
                acc += (cos(theta) - I * sin(theta)) * G[h * nx + w];
            }
        g[j] = acc;
    }
}

void olc_cgh_exact_adjoint(const double *pts, long n, const double *Gd, double *gd, long ny, long nx,
                           double py, double px, double lambda)
{
    const cplx *G = (const cplx *)Gd;
    cplx *g = (cplx *)gd;
    const double k = 2 * M_PI / lambda;
#pragma omp parallel for schedule(dynamic, 4)
    for (long j = 0; j < n; ++j) {
        cplx acc = 0;
        for (long h = 0; h < ny; ++h)
            for (long w = 0; w < nx; ++w) {
                const double dx = px * w - pts[3 * j], dy = py * h - pts[3 * j + 1], z = pts[3 * j + 2];
                const double r = sqrt(dx * dx + dy * dy + z * z);
                acc += (cos(k * r) - I * sin(k * r)) / r * G[h * nx + w];
            }
        g[j] = acc;
    }
}

/* ----------------------------------------------------------------- WRP */
/* W_j: WRPStep1Pre golcgh.h:291-299; D_j = W_j * sqrt(2): WRPStep1Pre_D
 * golcgh.h:392-401.  Evaluated in double from the float inputs, rounded to
 * float once (W), and D = fl(W * sqrtf(2)). */
static float wrp_radius_one(float z, float plimit, float lambda, float plane_z, int window)
{
    const double q = (double)plimit / (double)lambda;
    const double c = 1.0 / sqrt(4.0 * q * q - 1.0);
    const float W = (float)(c * fabs((double)z - (double)plane_z));
    if (window == 0) return W;
    volatile float r2 = sqrtf(2.0f);
    volatile float D = W * r2;
    return D;
}

void olc_wrp_radius(const float *pts, long n, float *W, float plimit, float lambda, float plane_z, int window)
{
    for (long j = 0; j < n; ++j) W[j] = wrp_radius_one(pts[3 * j + 2], plimit, lambda, plane_z, window);
}

/* float32 window membership, each operation rounded (golcgh.h:311-316 circle,
 * golcgh.h:416-419 square) */
static int wrp_inside(float p, long w, long h, float x, float y, float R, int window)
{
    volatile float pw = p * (float)w;
    volatile float ph = p * (float)h;
    volatile float dx = pw - x;
    volatile float dy = ph - y;
    if (window == 0) {
        volatile float dx2 = dx * dx;
        volatile float dy2 = dy * dy;
        volatile float t = dx2 + dy2;
        volatile float R2 = R * R;
        return t < R2;
    }
    volatile float ax = fabsf(dx) * 2.0f;
    volatile float ay = fabsf(dy) * 2.0f;
    return (ax <= R) && (ay <= R);
}

void olc_wrp_step1(const float *pts, long n, double *Ud, long ny, long nx, float p, float lambda,
                   float plane_z, float plimit, int window)
{
    cplx *U = (cplx *)Ud;
    float *R = (float *)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
    olc_wrp_radius(pts, n, R, plimit, lambda, plane_z, window);
    memset(U, 0, (size_t)(ny * nx) * sizeof(cplx));
    /* scatter form: each point visits its own bounding box (the same terms the
     * reference's per-pixel loop over all points adds) */
#pragma omp parallel
    {
        cplx *acc = cz(ny * nx);
#pragma omp for schedule(dynamic, 16)
        for (long j = 0; j < n; ++j) {
            const float x = pts[3 * j], y = pts[3 * j + 1];
            const double dz = (double)pts[3 * j + 2] - (double)plane_z;
            const double Rd = R[j];
            const double reach = (window == 0 ? Rd : 0.5 * Rd) / (double)p + 2.0;
            long w0 = (long)floor(x / (double)p - reach), w1 = (long)ceil(x / (double)p + reach);
            long h0 = (long)floor(y / (double)p - reach), h1 = (long)ceil(y / (double)p + reach);
            if (w0 < 0) w0 = 0;
            if (h0 < 0) h0 = 0;
            if (w1 > nx - 1) w1 = nx - 1;
            if (h1 > ny - 1) h1 = ny - 1;
            const double k = M_PI / ((double)lambda * dz), inv = 1.0 / fabs(dz);
            for (long h = h0; h <= h1; ++h)
                for (long w = w0; w <= w1; ++w) {
                    if (!wrp_inside(p, w, h, x, y, R[j], window)) continue;
                    const double ddx = (double)p * w - x, ddy = (double)p * h - y;
                    const double th = k * (ddx * ddx + ddy * ddy);
                    acc[h * nx + w] += inv * (cos(th) + I * sin(th));
                }
        }
#pragma omp critical
        for (long i = 0; i < ny * nx; ++i) U[i] += acc[i];
        free(acc);
    }
    free(R);
}

/* ---------------------------------------------------------- quantisers */
static void to_u8(const double *v, uint8_t *img, long n, double mn, double mx)
{
    for (long i = 0; i < n; ++i) img[i] = (mx == mn) ? 0 : (uint8_t)round((255 * (v[i] - mn)) / (mx - mn));
}

void olc_complex2img(const double *ud, uint8_t *img, long ny, long nx, int mode)
{
    const cplx *u = (const cplx *)ud;
    const long n = ny * nx;
    double *v = (double *)malloc((size_t)n * sizeof(double));
    for (long i = 0; i < n; ++i) {
        const double re = creal(u[i]), im = cimag(u[i]);
        v[i] = mode == 1 ? re : mode == 2 ? im : mode == 3 ? sqrt(re * re + im * im) : atan2(im, re);
    }
    double mn, mx;
    if (mode == 0) {
        mn = -M_PI;
        mx = M_PI;
    } else {
        mn = mx = v[0];
        for (long i = 0; i < n; ++i) {
            if (v[i] > mx) mx = v[i];
            if (v[i] < mn) mn = v[i];
        }
    }
    to_u8(v, img, n, mn, mx);
    free(v);
}

void olc_quant8bit(const double *real, uint8_t *img, long ny, long nx)
{
    const long n = ny * nx;
    double mx = real[0], mn = real[0];
    for (long i = 0; i < n; ++i) {
        if (real[i] > mx) mx = real[i];
        else if (real[i] < mn) mn = real[i];
    }
    for (long i = 0; i < n; ++i) img[i] = (mx == mn) ? 0 : (uint8_t)round((real[i] - mn) / (mx - mn) * 255);
}

void olc_binarize(const double *ud, uint8_t *img, long ny, long nx)
{
    for (long i = 0; i < ny * nx; ++i) img[i] = ud[2 * i] >= 0.0 ? 255 : 0;
}
