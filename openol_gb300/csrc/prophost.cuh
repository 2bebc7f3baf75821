// prophost.cuh -- host-side interfaces shared by the propagation translation
// units: pass dispatch (prop_rows_fwd.cu, prop_rows_inv.cu, prop_cols.cu,
// prop_aux.cu; mixed-radix passes in propmr.cu), the scratch layout and
// per-method set-up (prop.cu), the launch-variant table (autotune.cu) and
// the twiddle-table registry (prop.cu).
#pragma once
#include <atomic>

#include <cuda_runtime.h>

#include "common.cuh"
#include "propdev.cuh"
#include "propmr.cuh"

namespace olg {

// Twiddle tables.  Every translation unit that instantiates pass kernels has
// its own copy (no relocatable device code) and registers an uploader at load
// time; ensure_twiddles() fills every copy once per CUDA context.
int register_twiddle_uploader(int (*fn)(const float2 *tw, const float4 *tw4));
int ensure_twiddles();

// selected launch variant per pass kind (0 rows fwd, 1 cols, 2 rows inv) and
// log2 of the FFT length; atomic so that a set or an autotune on one host
// thread races no launch on another (autotune.cu)
extern std::atomic<int> g_variant[3][14];

// power-of-two passes, one translation unit each
int rows_fwd_pass_pow2(const PropParams &P, cudaStream_t st); // prop_rows_fwd.cu
int rows_inv_pass_pow2(const PropParams &P, cudaStream_t st); // prop_rows_inv.cu
int cols_pass_pow2(const PropParams &P, cudaStream_t st);     // prop_cols.cu
// the persistent TMA-staged column pass, padded heights 2048..8192 (prop_cols_tma.cu)
int cols_pass_tma(const PropParams &P, cudaStream_t st);
int chirp_axis_pow2(const ChirpAxis &A, cudaStream_t st);     // prop_aux.cu
// forward pass 3 (OP_SEED) and adjoint pass 1 of one plane, fused; padded
// widths 256..8192 (prop_aux.cu)
int rows_seed_pass(const PropParams &P, cudaStream_t st);
// any supported length (mixed-radix passes for the others); prop.cu
int rows_pass(const PropParams &P, bool inverse, cudaStream_t st);
int cols_pass(const PropParams &P, cudaStream_t st);
int chirp_axis(const ChirpAxis &A, cudaStream_t st);

// Propagation scratch: the half-padded spectrum S (ny x 2nx), the 1-D chirp
// spectra Hx (2nx), Hy (2ny) and the per-axis pre/post chirp tables.
struct Layout {
    float2 *S, *Hx, *Hy, *tax, *tay, *tbx, *tby;
};
size_t layout_bytes(int ny, int nx, Layout *L, char *base);
// A field axis n is supported when the padded length 2n is a power of two in
// [32, 8192] (the tuned passes) or 2^a 3^b 5^c with n >= 8 that one CTA holds
// (mixed radix, up to 7680).
bool axis_ok(int n);
int validate(const void *a, const void *b, int ny, int nx);
PropParams base_params(const void *in, void *out, int ny, int nx, const Layout &L);
int run_passes(const PropParams &P, cudaStream_t st);
// 1 when every t of the NY x NX ASM frequency grid is <= 1/64 (PropParams::tf_series)
int asm_series_ok(double NY, double NX, double dv, double du, double lambda);
long floor_lim(double v);
void set_quad(float &hi, float &lo, double v);
// frac(v) in [-0.5, 0.5]
float frac_host(double v);
ChirpAxis chirp_axis_params(int L, int n, double d, double lambda, double z, double s_factor, int lim, double scale,
                            float2 *H);

// Parameters of one propagation: the three passes plus the per-axis chirp
// jobs (none for ASM; spectra for Fresnel; spectra and pre/post tables for ARSS).
struct PropSetup {
    PropParams P;
    ChirpAxis ax, ay;
    bool chirps = false;
};
int check_phys(double dy, double dx, double lambda, double z, bool nonzero_z);
int setup_asm(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z, int flags,
              const Layout &L, PropSetup *S);
int setup_shifted_asm(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z,
                      double oy, double ox, int flags, const Layout &L, PropSetup *S);
int setup_fresnel(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z,
                  int bandlimit, int flags, const Layout &L, PropSetup *S);
int setup_arss(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx, double lambda, double z,
               double s, double oy, double ox, int flags, const Layout &L, PropSetup *S, bool windows = true);
int run_setup(const PropSetup &S, cudaStream_t st);

} // namespace olg
