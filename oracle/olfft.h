/*
 * olfft.h -- project-written mixed-radix DFT for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the discrete Fourier transform that the
 * CPU oracle (olcpu.c) and the FFTW shim (refshim/fftw_shim.c, which lets the
 * reference's own olutils.h fft/ifft at olutils.h:19-66 compile without FFTW)
 * both use.  Nothing in the GPU product links it.
 *
 * Convention (same as FFTW and cuFFT): unnormalised,
 *   X[k] = sum_n x[n] exp(sign * 2*pi*i * n*k / N),  sign = -1 forward, +1 backward.
 * Data are interleaved complex (re, im) pairs, row-major for 2-D.
 * Any length is supported: radix 2/3/4/5 butterflies, generic O(p^2) for
 * other prime factors.  Twiddles are computed in double from exact integer
 * index products reduced modulo N, so each twiddle is correct to ~1 ulp.
 */
#ifndef OLFFT_H
#define OLFFT_H
#ifdef __cplusplus
extern "C" {
#endif

/* 1-D in-place transform of n complex doubles. */
void olfft_1d(double *x, long n, int sign);
/* 2-D in-place transform of an ny x nx row-major complex double array.
 * nthreads <= 0 uses the OpenMP default. */
void olfft_2d(double *x, long ny, long nx, int sign, int nthreads);
/* Single-precision variants (computed in double internally, stored as float). */
void olfft_2d_f(float *x, long ny, long nx, int sign, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
