/*
 * olfft.c -- project-written mixed-radix DFT for the CPU oracle.
 * TEST INFRASTRUCTURE ONLY (see olfft.h).  Recursive decimation in time:
 * N = p * m, the p interleaved sub-sequences are transformed recursively into
 * contiguous blocks of m, then combined with twiddles w_N^(r k) and a length-p
 * DFT.  Radix 4 and 2 are peeled first, then odd factors in increasing order.
 */
#include "olfft.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

typedef struct {
    long n;
    int nf;
    long f[64];
    cplx *tw; /* tw[k] = exp(-2 pi i k / n) */
} plan_t;

static void plan_init(plan_t *p, long n)
{
    p->n = n;
    p->nf = 0;
    long m = n;
    while (m % 4 == 0 && m > 4) { p->f[p->nf++] = 4; m /= 4; }
    while (m % 2 == 0 && m > 2) { p->f[p->nf++] = 2; m /= 2; }
    for (long q = 3; q * q <= m; q += 2)
        while (m % q == 0 && m > q) { p->f[p->nf++] = q; m /= q; }
    if (m > 1) p->f[p->nf++] = m;
    p->tw = (cplx *)malloc((size_t)n * sizeof(cplx));
    for (long k = 0; k < n; ++k) {
        double a = -2.0 * M_PI * (double)k / (double)n;
        p->tw[k] = cos(a) + I * sin(a);
    }
}

static void plan_free(plan_t *p) { free(p->tw); }

static inline cplx twid(const plan_t *P, long idx, int sign)
{
    cplx w = P->tw[idx % P->n];
    return sign > 0 ? conj(w) : w;
}

/* DFT of in[0], in[is], ..., in[(n-1) is] into contiguous out[0..n-1]. */
static void rec(const cplx *in, cplx *out, long n, long is, const long *f,
                const plan_t *P, int sign, cplx *tmp)
{
    if (n == 1) { out[0] = in[0]; return; }
    const long p = f[0], m = n / p;
    for (long r = 0; r < p; ++r)
        rec(in + r * is, out + r * m, m, is * p, f + 1, P, sign, tmp);
    const long tws = P->n / n;
    if (p == 2) {
        for (long k = 0; k < m; ++k) {
            cplx a = out[k], b = out[m + k] * twid(P, k * tws, sign);
            out[k] = a + b;
            out[m + k] = a - b;
        }
    } else if (p == 4) {
        const cplx jrot = sign < 0 ? -I : I; /* exp(sign * 2 pi i / 4) */
        for (long k = 0; k < m; ++k) {
            cplx a0 = out[k];
            cplx a1 = out[m + k] * twid(P, k * tws, sign);
            cplx a2 = out[2 * m + k] * twid(P, 2 * k * tws, sign);
            cplx a3 = out[3 * m + k] * twid(P, 3 * k * tws, sign);
            cplx s02 = a0 + a2, d02 = a0 - a2, s13 = a1 + a3, d13 = (a1 - a3) * jrot;
            out[k] = s02 + s13;
            out[m + k] = d02 + d13;
            out[2 * m + k] = s02 - s13;
            out[3 * m + k] = d02 - d13;
        }
    } else {
        for (long k = 0; k < m; ++k) {
            for (long r = 0; r < p; ++r)
                tmp[r] = out[r * m + k] * twid(P, r * k * tws, sign);
            for (long q = 0; q < p; ++q) {
                cplx s = 0;
                for (long r = 0; r < p; ++r)
                    s += tmp[r] * twid(P, ((r * q) % p) * (P->n / p), sign);
                out[q * m + k] = s;
            }
        }
    }
}

static long max_factor(const plan_t *P)
{
    long mf = 1;
    for (int i = 0; i < P->nf; ++i)
        if (P->f[i] > mf) mf = P->f[i];
    return mf;
}

void olfft_1d(double *x, long n, int sign)
{
    if (n <= 1) return;
    plan_t P;
    plan_init(&P, n);
    cplx *buf = (cplx *)malloc((size_t)n * sizeof(cplx));
    cplx *tmp = (cplx *)malloc((size_t)max_factor(&P) * sizeof(cplx));
    memcpy(buf, x, (size_t)n * sizeof(cplx));
    rec(buf, (cplx *)x, n, 1, P.f, &P, sign, tmp);
    free(tmp);
    free(buf);
    plan_free(&P);
}

void olfft_2d(double *xd, long ny, long nx, int sign, int nthreads)
{
    cplx *x = (cplx *)xd;
    plan_t Px, Py;
    plan_init(&Px, nx);
    plan_init(&Py, ny);
    const long mfx = max_factor(&Px), mfy = max_factor(&Py);
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        cplx *a = (cplx *)malloc((size_t)(nx > ny ? nx : ny) * sizeof(cplx));
        cplx *tmp = (cplx *)malloc((size_t)(mfx > mfy ? mfx : mfy) * sizeof(cplx));
        if (nx > 1) {
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
            for (long h = 0; h < ny; ++h) {
                memcpy(a, x + h * nx, (size_t)nx * sizeof(cplx));
                rec(a, x + h * nx, nx, 1, Px.f, &Px, sign, tmp);
            }
        }
        if (ny > 1) {
            cplx *b = (cplx *)malloc((size_t)ny * sizeof(cplx));
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
            for (long w = 0; w < nx; ++w) {
                for (long h = 0; h < ny; ++h) a[h] = x[h * nx + w];
                rec(a, b, ny, 1, Py.f, &Py, sign, tmp);
                for (long h = 0; h < ny; ++h) x[h * nx + w] = b[h];
            }
            free(b);
        }
        free(tmp);
        free(a);
    }
    plan_free(&Px);
    plan_free(&Py);
}

void olfft_2d_f(float *xf, long ny, long nx, int sign, int nthreads)
{
    const long n = ny * nx;
    double *x = (double *)malloc((size_t)n * 2 * sizeof(double));
    for (long i = 0; i < 2 * n; ++i) x[i] = xf[i];
    olfft_2d(x, ny, nx, sign, nthreads);
    for (long i = 0; i < 2 * n; ++i) xf[i] = (float)x[i];
    free(x);
}
