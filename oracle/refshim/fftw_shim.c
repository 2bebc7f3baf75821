/*
 * fftw_shim.c -- implements the FFTW3 subset declared in fftw3.h on top of the
 * project-written DFT (../olfft.c).  TEST INFRASTRUCTURE ONLY.
 */
#include "fftw3.h"
#include "../olfft.h"

#include <stdlib.h>
#include <string.h>

struct ol_fftw_plan_s {
    int n0, n1, sign, is_float;
    void *in, *out;
};

static int g_threads = 0, g_threads_f = 0;

int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { g_threads = n; }
int fftwf_init_threads(void) { return 1; }
void fftwf_plan_with_nthreads(int n) { g_threads_f = n; }

static struct ol_fftw_plan_s *mk(int n0, int n1, void *in, void *out, int sign, int is_float)
{
    struct ol_fftw_plan_s *p = (struct ol_fftw_plan_s *)calloc(1, sizeof(*p));
    p->n0 = n0; p->n1 = n1; p->sign = sign; p->is_float = is_float; p->in = in; p->out = out;
    return p;
}

fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags)
{
    (void)flags;
    return mk(n0, n1, in, out, sign, 0);
}

fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags)
{
    (void)flags;
    return mk(n0, n1, in, out, sign, 1);
}

static void run(const struct ol_fftw_plan_s *p)
{
    const size_t n = (size_t)p->n0 * (size_t)p->n1;
    if (p->is_float) {
        if (p->out != p->in) memmove(p->out, p->in, n * 2 * sizeof(float));
        olfft_2d_f((float *)p->out, p->n0, p->n1, p->sign, g_threads_f);
    } else {
        if (p->out != p->in) memmove(p->out, p->in, n * 2 * sizeof(double));
        olfft_2d((double *)p->out, p->n0, p->n1, p->sign, g_threads);
    }
}

void fftw_execute(const fftw_plan p) { run(p); }
void fftwf_execute(const fftwf_plan p) { run(p); }
void fftw_destroy_plan(fftw_plan p) { free(p); }
void fftwf_destroy_plan(fftwf_plan p) { free(p); }
