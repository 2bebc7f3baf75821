/*
 * olcpu.h -- FP64 CPU restatement of OpenOL's propagation / CGH / WRP path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: the parity tests, smoke() and
 * bench.py's cpu_baseline leg call it as the checker.  The GPU product never
 * links or calls it.
 *
 * Every routine restates a reference function (file:line given beside each
 * declaration, paths relative to the reference project) in double precision,
 * with the reference's own conventions: centred 2x zero padding, fftshift'ed
 * transfer functions, unnormalised FFTs, the 1/Np factors where the reference
 * applies them, windows computed with floor() exactly as written there.
 * Complex data are interleaved (re, im) doubles, row-major.
 */
#ifndef OLCPU_H
#define OLCPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* flags (same bit values as the GPU C-ABI in include/olgb300.h) */
#define OLC_CONJ 0x1         /* adjoint: conjugate transfer function / swap+conjugate chirps */
#define OLC_NO_NORMALIZE 0x2 /* host-pointer overload convention: no 1/Np factors */
#define OLC_ACCUMULATE 0x4   /* U += result instead of U = result */
#define OLC_F32_WINDOW 0x10  /* with OLC_BANDLIMIT: decide the window in float, as PREC_T = float does */
#define OLC_BANDLIMIT 0x40   /* shifted ASM: the host overload's band window (olprop.h:251-305) */
#define OLC_NO_WINDOWS 0x80  /* olc_arss_prop: no windows -- the shifted Fresnel propagation */

/* Unnormalised 2-D DFT, sign -1 forward / +1 backward (FFTW/cuFFT convention). */
void olc_fft2d(double *u, long ny, long nx, int sign, int nthreads);

/* Angular spectrum method, olprop.h:227-248 (AsmProp) with AsmTransferF
 * olprop.h:173-189; device convention of golprop.h:507-534 (1/Np applied).
 * OLC_NO_NORMALIZE gives the host-pointer overload golprop.h:458-504.
 * OLC_CONJ conjugates H (the adjoint operator). In place, u is ny x nx. */
void olc_asm_prop(double *u, long ny, long nx, double dy, double dx, double lambda, double z, int flags);

/* Fresnel propagation by convolution with the sampled impulse response.
 * bandlimit = 0: FresnelProp olprop.h:125-148 / gFresnelProp golprop.h:167-198.
 * bandlimit = 1: gFresnelPropBandLimit golprop.h:202-302 (one limit, from x, on both axes).
 * bandlimit = 2: CPU FresnelPropBandLimit olprop.h:26-50,150-170 (x and y limits).
 * OLC_NO_NORMALIZE: host-pointer overload golprop.h:70-124 (fftshift of the padded
 * field before the FFT and after the IFFT, no 1/Np).  OLC_CONJ: adjoint. */
void olc_fresnel_prop(double *u, long ny, long nx, double dy, double dx, double lambda, double z,
                      int bandlimit, int flags);

/* ARSS Fresnel propagation, golprop.h:816-995 (the reference has no CPU ARSS).
 * src and dst are ny x nx and may alias.  Returns 0, or -1 for s in {0, 1}
 * (the reference's window limits divide by s*|s-1| and |1-s|).
 * OLC_CONJ applies the exact adjoint of that linear map.  OLC_NO_WINDOWS
 * drops every window (any s): gshiftedFresnelProp golprop.h:606-752. */
int olc_arss_prop(const double *src, double *dst, long ny, long nx, double dy, double dx,
                  double lambda, double z, double s, double oy, double ox, int flags);

/* Shifted angular spectrum method, gshiftedAsmProp golprop.h:537-575 with
 * gshiftedAsmTransferF golprop.h:335-420: H = exp(2 pi i (w z + ox u + oy v)),
 * 1/Np (none with OLC_NO_NORMALIZE).  OLC_BANDLIMIT: H = 0 outside the band
 * window of shiftedAsmTransferF olprop.h:251-305 (the host overload
 * shiftedAsmProp olprop.h:307-327 also scales by a further 1/Np, which this
 * function leaves to the caller).  OLC_CONJ: adjoint.  src, dst ny x nx. */
void olc_shifted_asm_prop(const double *src, double *dst, long ny, long nx, double dy, double dx, double lambda,
                          double z, double oy, double ox, int flags);

/* Split propagation, gsplitProp golprop.h:772-813 / splitAsmProp
 * olprop.h:618-654: dst = sum over (source, destination) block pairs of the
 * shifted propagation (mode 0 ASM with the given flags, mode 1 shifted
 * Fresnel with s = 1) of the source block into the destination block, with
 * offsets (src - dst) * block size * pitch formed in float as the reference
 * does.  dst must not alias src. */
int olc_split_prop(const double *src, double *dst, long ny, long nx, double dy, double dx, double lambda, double z,
                   int mode, int blocks_y, int blocks_x, int flags);

/* Tilted-plane propagation, TiltedSourceProp olprop.h:414-521 (reference == 0:
 * the destination plane is rotated by `angle` about y as seen from the source)
 * and TiltedReferenceProp olprop.h:523-600 (reference != 0: rotation `angle`),
 * in PREC_T = double.  interp 0 bilinear, 1 bicubic (a = -1); mode 0 ASM,
 * 1 Fresnel.  In place on u (ny x nx). */
void olc_tilted_prop(double *u, long ny, long nx, double dy, double dx, double lambda, double z, double angle,
                     int interp, int mode, int reference);

/* ARSS window limits as the reference computes them: lims[0..5] =
 * {hlim_u, wlim_u, lim_h, hlim_cz, wlim_cz, unused}. */
int olc_arss_windows(long ny, long nx, double dy, double dx, double lambda, double z, double s, int64_t *lims);

/* AUTO method selection, AsmPropCheck olprop.h:209-225 / FresnelPropCheck
 * olprop.h:109-123, evaluated in double.  Returns 1 when the check passes. */
int olc_asm_prop_check(long ny, long nx, double dy, double dx, double lambda, double z);
int olc_fresnel_prop_check(long ny, long nx, double dy, double dx, double lambda, double z);

/* Point-cloud CGH, Fresnel form: _CghFresnel olcgh.h:297-313 (complex output)
 * and olcgh.h:276-295 (phase output), gCgh/gCghShared golcgh.h:5-145.
 * pts: N x (x, y, z).  amp / phase0 (nullable) extend the reference's unit
 * amplitude to a_j * exp(i phi_j).  U (nullable) ny x nx complex;
 * phase_out (nullable) receives atan2(Im U, Re U).  OLC_ACCUMULATE gives the
 * += semantics of gCghReduction golcgh.h:147-195. */
void olc_cgh_fresnel(const double *pts, const double *amp, const double *phase0, long n,
                     double *U, double *phase_out, long ny, long nx, double py, double px,
                     double lambda, int flags);

/* Exact spherical-wave CGH: U = sum_j a_j exp(i (k r_j + phi_j)) / r_j,
 * r_j = sqrt((px w - x_j)^2 + (py h - y_j)^2 + z_j^2), k = 2 pi / lambda
 * (the kernel left commented out at golcgh.h:218,323; no reference code runs it). */
void olc_cgh_exact(const double *pts, const double *amp, const double *phase0, long n,
                   double *U, long ny, long nx, double py, double px, double lambda, int flags);

/* Adjoints (transposed sums): g_j = sum_{h,w} conj(K_j(h,w)) G[h,w] where K_j
 * is the unit-weight kernel of the forward routine.  g is n complex. */
void olc_cgh_fresnel_adjoint(const double *pts, long n, const double *G, double *g, long ny, long nx,
                             double py, double px, double lambda);
void olc_cgh_exact_adjoint(const double *pts, long n, const double *G, double *g, long ny, long nx,
                           double py, double px, double lambda);

/* WRP step 1, golcgh.h:291-378 (window = 0, circle) and golcgh.h:392-491
 * (window = 1, square).  Inputs are the reference's float32 values.  The
 * window radius W_j and the membership test follow the reference expression
 * evaluated in float32 with each operation rounded (no FMA contraction);
 * the phase pi rho^2 / (lambda dz) and 1/|dz| are evaluated in double.
 * plimit is the pitch used for W_j (the p_limit overloads), pass p otherwise.
 * U is ny x nx, overwritten. */
void olc_wrp_step1(const float *pts, long n, double *U, long ny, long nx, float p, float lambda,
                   float plane_z, float plimit, int window);
/* W_j (window = 0) or D_j (window = 1) as float, golcgh.h:291-299 / 392-401. */
void olc_wrp_radius(const float *pts, long n, float *W, float plimit, float lambda, float plane_z, int window);

/* 8-bit quantisers: complex2img(MODE) olimg.h:348-391 (mode: 0 PHASE, 1 REAL,
 * 2 IMAG, 3 AMP, the reference's MODE enum olimg.h:268) and quant8bit
 * olimg.h:178-203.  A constant image (max == min) maps to 0. */
void olc_complex2img(const double *u, uint8_t *img, long ny, long nx, int mode);
void olc_quant8bit(const double *real, uint8_t *img, long ny, long nx);
/* Binarised 8-bit hologram (project rule; the reference has none): 255 where
 * Re(U) >= 0, else 0. */
void olc_binarize(const double *u, uint8_t *img, long ny, long nx);

#ifdef __cplusplus
}
#endif
#endif
