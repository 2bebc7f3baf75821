/*
 * fftw3.h -- minimal FFTW3 API shim for compiling the reference's CPU headers.
 * TEST INFRASTRUCTURE ONLY.  FFTW 3.3.10 (which the reference expects, README.md
 * install steps) is not installed in this image; this header declares exactly
 * the FFTW surface that olutils.h:19-66 calls, and fftw_shim.c implements it on
 * top of the project-written DFT in ../olfft.c.  Semantics follow FFTW's public
 * documentation: unnormalised transforms, FFTW_FORWARD = -1, FFTW_BACKWARD = +1,
 * in-place allowed, the plan binds the array pointers given at planning time.
 */
#ifndef OL_FFTW3_SHIM_H
#define OL_FFTW3_SHIM_H
#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct ol_fftw_plan_s *fftw_plan;
typedef struct ol_fftw_plan_s *fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

int fftwf_init_threads(void);
void fftwf_plan_with_nthreads(int nthreads);
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);

#ifdef __cplusplus
}
#endif
#endif
