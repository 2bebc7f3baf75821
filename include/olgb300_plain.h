/*
 * olgb300_plain.h -- "plain form" GPU baselines exported by libolgb300.so for
 * measurement only: the reference's own GPU structure re-expressed on this
 * GPU, so that the fused kernels can be timed against it on the same device.
 */
#ifndef OLGB300_PLAIN_H
#define OLGB300_PLAIN_H
#include "olgb300.h"
#ifdef __cplusplus
extern "C" {
#endif

/* ASM the way golprop.h:507-534 chains it: pad kernel, cuFFT forward, 1/Np,
 * FP32 transfer function (golprop.h:307-322), fftshift, multiply, cuFFT
 * inverse, crop.  cuFFT plan and padded buffers are cached per size. */
int olg_plain_asm_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                           double z, olg_stream_t stream);

/* Fresnel the way golprop.h:167-198 chains it: pad, cuFFT forward, 1/Np,
 * FP32 sampled response (golprop.h:9-30), fftshift, cuFFT forward, 1/Np,
 * multiply, cuFFT inverse, crop.  Same cached plan and buffers. */
int olg_plain_fresnel_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                               double z, olg_stream_t stream);

/* ARSS the way golprop.h:941-988 chains it: FP32 windowed pre-chirp into
 * u_dst, pad, FFT, 1/Np, windowed chirp, fftshift, FFT, 1/Np, multiply,
 * IFFT, crop, FP32 windowed post-chirp.  u_src != u_dst. */
int olg_plain_arss_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx, double lambda,
                            double z, double s, double oy, double ox, olg_stream_t stream);

/* Fresnel-form CGH the way gCghShared (golcgh.h:47-88) computes it: one
 * thread per pixel, points staged in shared memory, FP32 phase with
 * full-precision sin/cos.  Unit amplitudes. */
int olg_plain_cgh_fresnel_c64(const float *points, int n_points, void *U, int ny, int nx, double p, double lambda,
                              olg_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
