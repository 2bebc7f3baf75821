// propmr.cuh -- host entry points of the mixed-radix passes (propmr.cu),
// called by the propagation dispatch in prop.cu for lengths that are not
// powers of two.
#pragma once
#include "propdev.cuh"

namespace olg {

// radices for N = 2^a 3^b 5^c (false otherwise)
bool mr_plan(int N, MrPlan *pl);
// a plan exists and one CTA can hold a sequence of length N
bool mr_length_ok(int N);
// fill P's plans, twiddle tables and tile sizes for its non-power-of-two axes
int mr_prepare(PropParams &P);
int mr_rows_pass(const PropParams &P, bool inverse, cudaStream_t st);
int mr_cols_pass(const PropParams &P, cudaStream_t st);
int mr_chirp_axis(const ChirpAxis &A, cudaStream_t st);

// Tilted-plane propagation, the part between the row passes (propmr.cu).
// Frequencies (fpx, fpy) = ((m - NX/2) du, (n - NY/2) dv) on the centred grid;
// the source frequency sampled for output frequency (n, m) is
//   fsx = a11 fpx + a13 fpz - a13f0,  fsy = fpy,  fpz = sqrt(fsqr - fpx^2 - fpy^2)
// (a13f0 = 0 for the reference form), weighted by J = J0 + Jb fpx / fpz.
struct TiltArgs {
    int ny, nx, NY, NX;
    int reference;               // 1: transfer function before resampling; 0: after
    int interp;                  // 0 bilinear, 1 bicubic (a = -1)
    int fresnel;                 // transfer function Hx[kx] Hy[ky] (else ASM)
    double du, dv, fsqr, a11, a13, a13f0, z;
    float J0, Jb, invN;
    // FP32 form of the sampling position (see k_tilt_resample):
    //   x = NX/2 + m' + round(c1 m') + Ki + [frac(c1 m') + Kf - a13 g / du],
    //   c1 = a11 - 1 (split hi + lo), K = Ki + Kf = a13 f0 / du (reference form, else 0),
    //   g / du = (m'^2 du + n'^2 dv^2 / du) / (f0 + fpz)
    float c1_hi, c1_lo, Kf, a13f, duf, dvf, dv2du, f0f, f0sq;
    int Ki;
    // double-float constants of the source form's ASM phase z sqrt(f0^2 - (fpx + a13 f0)^2 - fpy^2)
    float du_hi, du_lo, dv_hi, dv_lo, c_hi, c_lo, f0sq_hi, f0sq_lo, z_hi, z_lo;
    PropParams tf;               // reference form: tf_at() of the unrotated grid
    const float2 *Hx, *Hy;       // Fresnel spectra, natural order (Hx carries 1/N)
    float2 *C;                   // centred spectrum, NY x NX
    float2 *D;                   // resampled spectrum, natural order, NY x NX; its
                                 // first ny rows are the row-pass scratch (ny x NX)
};
// column FFTs of the row spectra (D) -> C, resampling C -> D, inverse column
// FFTs D -> D's first ny rows (x 1/N)
int tilt_middle(const TiltArgs &T, cudaStream_t st);
// tuned column FFTs of the tilted path for power-of-two heights 256..8192 (tilt.cu)
int tilt_cols_pow2(const TiltArgs &T, bool inverse, cudaStream_t st);
// Column FFTs between a half-padded row spectrum (ny x NX) and a full padded
// spectrum (NY x NX elements, stored by column tiles; private to spec.cu)
// (spec.cu).  Forward: out = FFT_col(in) [x T] [+ out]; inverse:
// out = central ny rows of IFFT_col(in [x T]).  T = tf_at(P) when tf != 0.
struct SpecArgs {
    int ny, NY, NX;
    const float2 *in;
    float2 *out;
    int tf, accumulate;
    PropParams P;
};
bool spec_cols_ok(int NY);
int spec_cols(const SpecArgs &A, bool inverse, cudaStream_t st);
// device address of the FFT_MAX-point twiddle table of the tuned passes
// (prop.cu; uploaded on first use on this device), or nullptr
const float2 *twiddle_table();

} // namespace olg
