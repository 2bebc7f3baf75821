/*
 * olgb300.h -- C-ABI of libolgb300.so, the GB300 (sm_103a) engine behind the
 * OpenOL propagation / hologram calls.
 *
 * The reference (somamake/openol) is a header-only C++ template library; its
 * callers instantiate ol::gAsmProp, ol::gFresnelProp, ol::ARSSFresnelProp,
 * ol::Prop, ol::gCgh, ol::WRPMethod ... directly.  Each entry point below is
 * what those templates reduce to once the template and RAII layers are peeled
 * off: raw device pointers (thrust::complex<float> == float2 == 8 bytes
 * interleaved re/im, row-major), sizes, physical parameters, a CUDA stream.
 * The drop-in C++ headers in include/openol_gb300/ and the Python mirror in
 * openol_gb300/ both call these functions; each comment names the reference
 * function (file:line in the reference project) that the entry point replaces.
 *
 * Conventions
 *  - Return value: OLG_OK (0) or a negative OLG_ERR_* code; never exits,
 *    never throws.  olg_last_error() gives a message for the calling thread.
 *  - Asynchronous on `stream` (a cudaStream_t; NULL = legacy default stream).
 *  - `work`/`work_bytes`: optional caller-provided device scratch of at least
 *    the size reported by the matching *_workspace_bytes() query.  With
 *    work == NULL the library takes stream-ordered scratch on `stream` from
 *    its own CUDA memory pool per device, which keeps up to 8 GiB of freed
 *    scratch mapped between calls (the device's default pool is not used).
 *  - In-place operation is allowed wherever an input and an output pointer
 *    have the same shape (u_in == u_out).
 *  - Sizes: each axis n (ny or nx) is a power of two in [16, 4096] (tuned
 *    passes, padded 32 .. 8192), or has a padded length 2n = 2^a 3^b 5^c up
 *    to 7680 with n >= 8 (mixed-radix passes; e.g. 3840 x 2160).  Other
 *    sizes return OLG_ERR_UNSUPPORTED_SIZE.
 */
#ifndef OLGB300_H
#define OLGB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OLG_OK 0
#define OLG_ERR_INVALID_ARG (-1)
#define OLG_ERR_UNSUPPORTED_SIZE (-2)
#define OLG_ERR_CUDA (-3)
#define OLG_ERR_WORKSPACE (-4)
#define OLG_ERR_NOMEM (-5)

/* flags */
#define OLG_CONJ 0x1         /* adjoint operator (conjugate transfer function / chirps) */
#define OLG_NO_NORMALIZE 0x2 /* host-pointer overload convention: no 1/Np factors */
#define OLG_ACCUMULATE 0x4   /* out += result (gCghReduction semantics) */
#define OLG_VERBOSE 0x8      /* print the chosen method like the reference's printf */
#define OLG_CHECK_F32 0x10   /* evaluate the AUTO checks (olg_prop_c64) / the shifted band window in float (PREC_T=float) */
#define OLG_REUSE_OPERANDS 0x20 /* olg_cgh_fresnel_gemm_c64: operands already in `work` from a call with the same points */
#define OLG_BANDLIMIT 0x40   /* shifted ASM: the band window of the host overload (olprop.h:251-305) */

/* propagation modes, ol::PROPMODE (oldefine.h:7-9) */
#define OLG_ASM 0
#define OLG_FRESNEL 1
#define OLG_AUTO 2

/* complex2img modes, ol::MODE (olimg.h:268) */
#define OLG_PHASE 0
#define OLG_REAL 1
#define OLG_IMAG 2
#define OLG_AMP 3

/* WRP windows */
#define OLG_WINDOW_CIRCLE 0 /* WRPStep1   golcgh.h:291-378 */
#define OLG_WINDOW_SQUARE 1 /* WRPStep1_D golcgh.h:392-491 */

/* tilted propagation interpolation, ol::INTERPOLATION (olprop.h:408-410) */
#define OLG_BILINEAR 0
#define OLG_BICUBIC 1

/* objset modes, ol::OBJSET_MODE (olobject.h:192-194) */
#define OLG_OBJSET_ZMIN 0
#define OLG_OBJSET_ZMIDDLE 1

typedef void *olg_stream_t;

/* ---------------------------------------------------------------- library */
int olg_version(void);
const char *olg_status_string(int status);
/* Message of the last failing call on this host thread ("" if none). */
const char *olg_last_error(void);
/* Number of kernels this library has launched so far in this process. */
unsigned long long olg_launch_count(void);
/* Device address of page-locked (pinned) host memory.  Passed as u_in /
 * u_out of olg_asm_prop_c64, it lets pass 1 read the input and pass 3 write
 * the output over the host link (NVLink-C2C on GB300) with no staging copies.
 * OLG_ERR_INVALID_ARG if `host` is not page-locked memory mapped for the
 * current device. */
int olg_host_device_pointer(const void *host, void **dev);
/* Budget of every bounded device-side wait of the persistent batch kernel
 * and launches after this call, in SM clock cycles (default 4e9, about 2 s):
 * a wait that runs out records an error and the kernel returns instead of
 * hanging.  Sets the budget when cycles > 0; returns the previous value. */
long long olg_wait_budget_cycles(long long cycles);
/* Host-side fault injection for tests: the next n scratch allocations from
 * the library's pool fail with OLG_ERR_NOMEM before touching the device, as
 * an exhausted device would.  Returns the previous count. */
int olg_inject_alloc_failures(int n);

/* ------------------------------------------------------------ propagation */
/* Device scratch for one propagation of an ny x nx field (any method). */
size_t olg_prop_workspace_bytes(int ny, int nx);

/* Angular spectrum method.  Replaces ol::gAsmProp (device overload,
 * golprop.h:507-534): u_out = crop(IFFT(H * FFT(pad(u_in)) / Np)).
 * OLG_NO_NORMALIZE reproduces the host-pointer overload (golprop.h:458-504,
 * no 1/Np); OLG_CONJ applies the adjoint (conj H). */
int olg_asm_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                     double z, int flags, void *work, size_t work_bytes, olg_stream_t stream);

/* Fresnel propagation (convolution with the sampled impulse response).
 * Replaces ol::gFresnelProp (device overload golprop.h:167-198; host overload
 * golprop.h:70-124 with OLG_NO_NORMALIZE) and, with bandlimit = 1,
 * ol::gFresnelPropBandLimit (golprop.h:202-302). */
int olg_fresnel_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx,
                         double lambda, double z, int bandlimit, int flags, void *work, size_t work_bytes,
                         olg_stream_t stream);

/* ARSS scaled Fresnel propagation.  Replaces ol::ARSSFresnelProp
 * (golprop.h:941-995): pre-chirp with window, pad, FFT/Np, x FFT(chirp_s)/Np,
 * IFFT, crop, post-chirp inside its window.  s in {0, 1} is rejected
 * (OLG_ERR_INVALID_ARG): the reference's window limits divide by s|s-1|. */
int olg_arss_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx, double lambda,
                      double z, double s, double oy, double ox, int flags, void *work, size_t work_bytes,
                      olg_stream_t stream);

/* Shifted angular spectrum method: the destination plane is offset by
 * (oy, ox).  Replaces ol::gshiftedAsmProp (golprop.h:335-420, 537-575):
 * T = exp(2 pi i (w z + ox u + oy v)), 1/Np.  OLG_BANDLIMIT adds the band
 * window of the host overload ol::shiftedAsmProp (olprop.h:251-327), which
 * also scales by a further 1/Np (apply it, or not, on the caller's side);
 * with OLG_CHECK_F32 the window is decided in float, as that overload's
 * PREC_T = float instantiation decides it.  OLG_NO_NORMALIZE drops the 1/Np,
 * OLG_CONJ gives the adjoint. */
int olg_shifted_asm_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                             double z, double oy, double ox, int flags, void *work, size_t work_bytes,
                             olg_stream_t stream);

/* Shifted (scaled) Fresnel propagation.  Replaces ol::gshiftedFresnelProp
 * (golprop.h:606-752): the ARSS chirps without windows; any finite s. */
int olg_shifted_fresnel_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx,
                                 double lambda, double z, double s, double oy, double ox, int flags, void *work,
                                 size_t work_bytes, olg_stream_t stream);

/* ol::shiftedProp (golprop.h:755-768): OLG_ASM -> shifted ASM, OLG_FRESNEL ->
 * shifted Fresnel with s = 1; any other mode is OLG_ERR_INVALID_ARG (the
 * reference prints "error" and exits). */
int olg_shifted_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx, double lambda,
                         double z, double oy, double ox, int propmode, int flags, void *work, size_t work_bytes,
                         olg_stream_t stream);

/* Split propagation.  Replaces ol::gsplitProp (golprop.h:772-813) and
 * ol::splitAsmProp (olprop.h:618-654) on device fields: the ny x nx field
 * is cut into blocks_y x blocks_x blocks (each block side a supported size), and every
 * (source, destination) block pair adds olg_shifted_prop_c64 of the source
 * block, offset by the blocks' distance, into the destination block.  u_out
 * must not overlap u_in; it is zeroed first unless OLG_ACCUMULATE.  Flags
 * pass on to the shifted propagations: OLG_BANDLIMIT | OLG_CHECK_F32 gives
 * splitAsmProp's per-block window (its only instantiation is PREC_T = float);
 * each block then carries its further 1/Np_block on the caller's side.
 * Scratch: olg_split_prop_workspace_bytes, reused for every pair. */
size_t olg_split_prop_workspace_bytes(int ny, int nx, int blocks_y, int blocks_x);
int olg_split_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda, double z,
                       int propmode, int blocks_y, int blocks_x, int flags, void *work, size_t work_bytes,
                       olg_stream_t stream);

/* Tilted-plane propagation.  Replaces ol::TiltedSourceProp (olprop.h:414-521,
 * reference == 0: the destination plane is rotated by `angle` radians about
 * the y axis as seen from the source) and ol::TiltedReferenceProp
 * (olprop.h:523-600, reference != 0: propagate, then resample for a plane
 * rotated by `angle`).  interp OLG_BILINEAR / OLG_BICUBIC (radial kernel,
 * a = -1), propmode OLG_ASM / OLG_FRESNEL.  Normalisation as the reference
 * (1/Np after the forward and after the inverse FFT; the Fresnel spectrum
 * carries one more).  Every frequency of the 2x padded grid must propagate
 * (no evanescent sample), else OLG_ERR_INVALID_ARG.  u_out may equal u_in.
 * Scratch: olg_tilted_workspace_bytes (two padded spectra). */
size_t olg_tilted_workspace_bytes(int ny, int nx);
int olg_tilted_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                        double z, double angle, int interp, int propmode, int reference, void *work,
                        size_t work_bytes, olg_stream_t stream);

/* Angular spectrum method that allocates nothing -- no counterpart in the
 * reference.  Same computation and flags as olg_asm_prop_c64, but its scratch
 * is a 17 MiB array compiled into the library, so it never calls cudaMalloc,
 * cudaMallocAsync or any other allocator.  It is meant for callers that must
 * not allocate device memory while they run: a holographic display loop with
 * a fixed per-frame budget (an allocation can synchronise the device and miss
 * a frame), or a plugin inside a host application that owns all GPU memory.
 * Limits: ny and nx powers of two in [16, 4096] (mixed-radix sizes, which
 * olg_asm_prop_c64 accepts, return OLG_ERR_UNSUPPORTED_SIZE: their twiddle
 * tables are allocated on first use) and ny * nx <= 1048576 (e.g. 1024 x 1024
 * or 256 x 4096); larger fields return OLG_ERR_WORKSPACE.  The first call in
 * each CUDA context (per device, and again after a device reset) looks up the
 * array's device address and uploads the FFT twiddle table; make that first
 * call before any stream capture.  All calls on a device share the one array:
 * calls that overlap on the GPU (e.g. on two streams) race and corrupt each
 * other's results, so serialise them. */
int olg_asm_prop_noalloc_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                             double z, int flags, olg_stream_t stream);

/* Launch-shape autotuner of the three propagation passes (project-written;
 * the reference has none).  Each pass has a few launch variants per FFT
 * length (threads per CTA, elements per CTA, registers); olg_autotune_prop
 * times every valid one on the device for an ny x nx field (real kernels,
 * real shapes; synchronises `stream`) and keeps the fastest for the rest of
 * the process.  kind: 0 row forward pass, 1 column pass, 2 row inverse pass;
 * n: FFT length (2 nx or 2 ny).  Untuned lengths use variant 0. */
int olg_autotune_prop(int ny, int nx, int reps, olg_stream_t stream);
int olg_prop_variant_count(void);
int olg_prop_get_variant(int kind, int n);
int olg_prop_set_variant(int kind, int n, int idx);

/* AUTO method selection, ol::AsmPropCheck (olprop.h:209-225) and
 * ol::FresnelPropCheck (olprop.h:109-123); single_precision != 0 evaluates
 * them in float like the reference's PREC_T=float instantiation.  1 = pass. */
int olg_asm_prop_check(int ny, int nx, double dy, double dx, double lambda, double z, int single_precision);
int olg_fresnel_prop_check(int ny, int nx, double dy, double dx, double lambda, double z, int single_precision);

/* Dispatcher.  Replaces ol::Prop (device overload, golprop.h:578-604):
 * mode OLG_ASM / OLG_FRESNEL / OLG_AUTO; AUTO picks ASM, else Fresnel, else
 * band-limited Fresnel.  *chosen (nullable) receives 0 ASM, 1 Fresnel,
 * 2 band-limited Fresnel.  In place on u. */
int olg_prop_c64(void *u, int ny, int nx, double dy, double dx, double lambda, double z, int mode, int flags,
                 int *chosen, void *work, size_t work_bytes, olg_stream_t stream);

/* ------------------------------------------------------ batched launch */
/* Many propagations of different sizes, methods, distances and wavelengths
 * in ONE persistent launch (the reference runs them one by one, each through
 * its own chain of kernels and cuFFT calls).  Sizes: ny, nx powers of two in
 * [256, 4096].  olg_batch_plan_create uploads the descriptors and takes all
 * scratch (cudaMalloc; synchronous); olg_batch_execute then only resets
 * counters and launches on `stream`, so it can be captured in a CUDA graph
 * and replayed.  Fields of at least olg_batch_direct_pixels() pixels (default
 * 2048 x 2048; each fills the GPU alone) run after the persistent kernel
 * through the single-field passes; the persistent kernel takes the rest.
 * olg_batch_execute_serial runs every field one after another through the
 * single-field passes (the baseline). */
#define OLG_BATCH_ASM 0
#define OLG_BATCH_FRESNEL 1
#define OLG_BATCH_ARSS 2
#define OLG_BATCH_FRESNEL_BANDLIMIT 3
typedef struct olg_field {
    const void *in;  /* ny x nx complex64 device field (in == out allowed) */
    void *out;
    int ny, nx;
    int method;      /* OLG_BATCH_* */
    int flags;       /* OLG_CONJ, OLG_NO_NORMALIZE (ASM / Fresnel) */
    double dy, dx, lambda, z;
    double s, oy, ox; /* ARSS only */
} olg_field;
typedef struct olg_batch_plan_s *olg_batch_plan;
int olg_batch_plan_create(const olg_field *fields, int n_fields, olg_batch_plan *plan);
int olg_batch_execute(olg_batch_plan plan, olg_stream_t stream);
int olg_batch_execute_serial(olg_batch_plan plan, olg_stream_t stream);
/* The plan's fields from host buffers and back (the reference's host-field
 * calls copy in and out around every propagation): host_in[i] (ny x nx
 * complex64) is copied into field i's `in`, the plan runs, and field i's `out`
 * is copied into host_out[i].  The copies in, the propagations and the copies
 * out are pipelined over two copy streams owned by the plan and `stream`:
 * the persistent kernel's fields arrive first and it starts at once, each
 * large field's passes start when that field has arrived, and each result
 * leaves when it is computed.  Ordered on `stream` like olg_batch_execute
 * (synchronize it before reading host_out).  Pinned host buffers give
 * asynchronous copies; pageable ones work but copy synchronously. */
int olg_batch_execute_host(olg_batch_plan plan, const void *const *host_in, void *const *host_out,
                           olg_stream_t stream);
/* Synchronous: OLG_ERR_CUDA if an item of the last execution gave up on its bounded wait. */
int olg_batch_check(olg_batch_plan plan);
/* For tests of the bounded waits (no counterpart in the reference): raises by
 * `delta` the number of finished units that the items of `field` wait for at
 * `stage` (0 set-up jobs, 1 pass-1 units, 2 pass-2 units), so that those
 * waits can never be satisfied and run out of their budget
 * (olg_wait_budget_cycles); the kernel then skips those items, records the
 * error for olg_batch_check and returns.  Synchronous. */
int olg_batch_plan_raise_target(olg_batch_plan plan, int field, int stage, int delta);
int olg_batch_plan_items(olg_batch_plan plan);
/* Fields of this plan that run through the single-field passes. */
int olg_batch_plan_direct_fields(olg_batch_plan plan);
/* Sets the size (ny * nx) from which plans created afterwards run a field
 * through the single-field passes (pixels > 0); returns the previous value
 * (pixels <= 0: only returns the current one). */
long long olg_batch_direct_pixels(long long pixels);
int olg_batch_plan_destroy(olg_batch_plan plan);

/* Single-field propagation plans (the cached-plan form of olg_asm_prop_c64,
 * olg_fresnel_prop_c64 and olg_arss_prop_c64): the field described by an
 * olg_field (its `in` / `out` are ignored; method OLG_BATCH_*, sizes as the
 * single calls accept, mixed radix included) is checked, its scratch
 * allocated and, for Fresnel and ARSS, its chirp spectra computed once, at
 * creation (cudaMalloc and a synchronisation).  Each execution then binds
 * device fields (16-byte aligned, in == out allowed) and runs the three
 * passes on `stream`, with the results of the matching single call.  The
 * executions of one plan share its scratch: order them (one stream, or
 * synchronised between streams). */
typedef struct olg_prop_plan_s *olg_prop_plan;
int olg_prop_plan_create(const olg_field *field, olg_prop_plan *plan);
int olg_prop_plan_execute(olg_prop_plan plan, const void *in, void *out, olg_stream_t stream);
/* A sequence of `count` host fields through one plan (host_out[i] = the
 * propagation of host_in[i]; page-locked host memory for asynchronous
 * copies).  Field i is copied into device slot i % 3 on a copy stream owned
 * by the plan, propagated in place there on `stream` and copied back on a
 * second copy stream, so field i+1's copy in and field i-1's copy out overlap
 * field i's passes.  Ordered on `stream` like `count` calls of
 * olg_prop_plan_execute: synchronise `stream` before reading host_out.  The
 * slots (3 fields) are allocated on first use and freed with the plan. */
int olg_prop_plan_execute_host(olg_prop_plan plan, const void *const *host_in, void *const *host_out, int count,
                               olg_stream_t stream);
int olg_prop_plan_destroy(olg_prop_plan plan);

/* -------------------------------------------------- phase optimisation */
/* Multi-plane phase-only hologram optimisation (the reference has none; it
 * builds on its ASM, golprop.h:507-534).  phi: ny x nx float (radians);
 * targets: n_planes x ny x nx float intensities; z: n_planes host doubles.
 * Loss L = sum_p mean((|ASM_{z_p}(e^{i phi})|^2 - t_p)^2).  The gradient is
 * formed with the hand-written adjoint (conjugate transfer function), each
 * plane's field recomputed rather than stored.  For padded heights
 * 256..8192 the planes share the forward spectrum of e^{i phi} and sum
 * their adjoint spectra: per plane one inverse and one forward column
 * transform and one row pass; otherwise 2 propagations per plane.
 * loss (nullable) is a device double receiving L. */
size_t olg_phase_opt_workspace_bytes(int ny, int nx);
int olg_phase_loss_grad(const float *phi, const float *targets, const double *z, int n_planes, int ny, int nx,
                        double dy, double dx, double lambda, float *grad, double *loss, void *work,
                        size_t work_bytes, olg_stream_t stream);
/* One Adam step (bias-corrected, step >= 1) on phi with state m, v. */
int olg_phase_adam_step(float *phi, float *m, float *v, const float *targets, const double *z, int n_planes, int ny,
                        int nx, double dy, double dx, double lambda, double lr, double beta1, double beta2, double eps,
                        int step, double *loss, void *work, size_t work_bytes, olg_stream_t stream);

/* ------------------------------------------------------------------- CGH */
/* Points are AoS float32 triples (x, y, z) in metres, ol::Vect3<float>
 * (olclass.h:45-52) as held by ol::gObject (golclass.h:58-71).  Pixel (w, h)
 * sits at (px*w, py*h) (corner origin, golcgh.h:75-76).  amp / phase0 are
 * optional per-point float arrays (NULL = 1 and 0). */

/* Fresnel-form CGH, U[h,w] = sum_j a_j exp(i(pi rho^2 / (lambda z_j) + phi_j)).
 * Replaces ol::gCgh / gCghShared (golcgh.h:47-145) and, with OLG_ACCUMULATE,
 * ol::gCghReduction (golcgh.h:147-195).  phase_out (nullable, float ny x nx)
 * receives atan2(Im U, Re U) like the phase kernels golcgh.h:5-45; U may be
 * NULL when only the phase is wanted. */
int olg_cgh_fresnel_c64(const float *points, const float *amp, const float *phase0, int n_points, void *U,
                        float *phase_out, int ny, int nx, double py, double px, double lambda, int flags,
                        olg_stream_t stream);

/* Exact spherical-wave CGH, U = sum_j a_j exp(i(k r_j + phi_j)) / r_j
 * (the kernel commented out at golcgh.h:218,323).  FP32 terms with the phase
 * range reduced per pixel tile in double-float arithmetic. */
int olg_cgh_exact_c64(const float *points, const float *amp, const float *phase0, int n_points, void *U,
                      int ny, int nx, double py, double px, double lambda, int flags, olg_stream_t stream);

/* Adjoints of the two CGH sums (the transposed sum; hand-written kernels
 * with no counterpart in the reference, which has only the forward sums).
 * With K_j(h,w) the unit-weight kernel of the forward routine (no a_j, no
 * phi_j) and G an ny x nx complex64 field,
 *   g_j = sum_{h,w} conj(K_j(h,w)) G[h,w]        (n_points complex64),
 * the adjoint of the linear map from complex point amplitudes a_j e^{i phi_j}
 * to the hologram: the gradient of a real loss of U with respect to the
 * amplitudes is g evaluated at G = dL/dU*.  Parallel over points, as the
 * reference's gCghReduction (golcgh.h:147-195) is; per-band partial sums are
 * added in a fixed order, so results are deterministic.  OLG_ACCUMULATE
 * adds into g.  Scratch: olg_cgh_adjoint_workspace_bytes (work == NULL:
 * stream-ordered pool). */
size_t olg_cgh_adjoint_workspace_bytes(int n_points, int ny, int nx, int exact);
/* The Fresnel adjoint above on the tensor cores: T = G conj(X) as the same
 * split-FP16 tcgen05 GEMM as olg_cgh_fresnel_gemm_c64 (M = ny, N = n_points,
 * K = nx; G scaled by a power of two so its f16 operands stay in [-1, 1]),
 * then g_j = sum_h conj(Y[h, j]) T[h, j] summed over row bands in a fixed
 * order (deterministic).  Same arguments and flags as
 * olg_cgh_fresnel_adjoint_c64; nx, ny <= 4096.  Scratch:
 * olg_cgh_adjoint_gemm_workspace_bytes (work == NULL: stream-ordered pool),
 * about (2 ny + n_points) x 2 nx x 4 + ny x n_points x 8 bytes (275 MB for
 * 1080 x 1920 and 10^4 points): it holds T, so it grows with ny x n_points,
 * where the direct adjoint's grows with n_points alone. */
size_t olg_cgh_adjoint_gemm_workspace_bytes(int n_points, int ny, int nx);
int olg_cgh_fresnel_adjoint_gemm_c64(const float *points, int n_points, const void *G, void *g, int ny, int nx,
                                     double py, double px, double lambda, int flags, void *work, size_t work_bytes,
                                     olg_stream_t stream);
int olg_cgh_fresnel_adjoint_c64(const float *points, int n_points, const void *G, void *g, int ny, int nx, double py,
                                double px, double lambda, int flags, void *work, size_t work_bytes,
                                olg_stream_t stream);
int olg_cgh_exact_adjoint_c64(const float *points, int n_points, const void *G, void *g, int ny, int nx, double py,
                              double px, double lambda, int flags, void *work, size_t work_bytes, olg_stream_t stream);

/* Fresnel-form CGH (same sum as olg_cgh_fresnel_c64, amplitudes/phases
 * included) as a split-FP16 complex GEMM on the tcgen05 tensor cores:
 * U = Y' X^T with X[w,j], Y'[h,j] the separable per-point chirps, each f16
 * hi + lo, three f16 products accumulated in f32.  nx, ny <= 4096.
 * Scratch: olg_cgh_gemm_workspace_bytes() (work == NULL: stream-ordered pool).
 * A bounded wait that expires inside the kernel is reported by
 * olg_device_fault_check(). */
size_t olg_cgh_gemm_workspace_bytes(int n_points, int ny, int nx);
int olg_cgh_fresnel_gemm_c64(const float *points, const float *amp, const float *phase0, int n_points, void *U,
                             int ny, int nx, double py, double px, double lambda, int flags, void *work,
                             size_t work_bytes, olg_stream_t stream);
/* A sequence of `count` holograms from host point clouds (the host-buffer
 * form of olg_cgh_fresnel_gemm_c64, as ol::Cgh takes host objects,
 * olcgh.h:351-379): U[i] (ny x nx complex64, host) = the hologram of
 * points[i] (n_points[i] x 3 floats, host), with amp[i] / phase0[i] (host;
 * the arrays or their entries may be NULL: unit amplitude, zero phase).
 * Cloud i goes up into a device slot on a copy stream, its hologram is formed
 * on `stream` and comes down on a second copy stream, so hologram i-1's copy
 * out and cloud i+1's copy in overlap hologram i's GEMM (page-locked host
 * memory for asynchronous copies).  Ordered on `stream` like `count` single
 * calls: synchronise `stream` before reading U.  Scratch from the
 * stream-ordered pool: three slots of clouds and holograms plus one GEMM
 * workspace.  OLG_ACCUMULATE and OLG_REUSE_OPERANDS are rejected. */
int olg_cgh_fresnel_gemm_host_c64(const float *const *points, const float *const *amp, const float *const *phase0,
                                  const int *n_points, void *const *U, int count, int ny, int nx, double py,
                                  double px, double lambda, int flags, olg_stream_t stream);
/* Tuning hook of the GEMM's work split (no counterpart in the reference):
 * when a hologram has fewer output tiles than the GPU has tile units (SMs, or
 * SM pairs), the spare units take the last part of every tile's K range, and
 * w is the cost of one of their K blocks relative to a tile unit's (default
 * 1.2; 0 turns the split off).  Sets w when 0 <= w <= 16 and returns the
 * previous value. */
double olg_cgh_gemm_tail_weight(double w);
/* Accumulation length of the GEMM (no counterpart in the reference), in K
 * blocks of 64 of one split product: ceil(kblocks / 3) K steps, each the
 * three split products over a 64-wide K range, are summed in the tensor
 * core's f32 accumulator before each partial sum is added into f32 registers
 * (default 8: 3 steps, 576 products).  Longer chunks hand accumulators to the epilogue less often; shorter
 * ones keep the tensor-core sums shorter.  Sets it for 1 <= kblocks <= 64
 * and returns the previous value; other values only return it. */
int olg_cgh_gemm_chunk(int kblocks);
/* Tile form of the GEMM (no counterpart in the reference): 1 = 256 x BN tiles
 * on pairs of SMs (a two-CTA cluster sharing each MMA; the default), 0 =
 * 128 x BN tiles on single SMs.  Sets the form when on is 0 or 1 and returns
 * the previous one; any other value only returns the current one. */
int olg_cgh_gemm_pairs(int on);
/* Autotuner of the tile form and that split (project-written; the reference
 * has none): times the GEMM for an n_points x ny x nx hologram in both forms
 * at a few tail weights (0, 1.0 .. 1.6; operands built once and reused, L2
 * flushed before every timed GEMM; synchronises `stream`) and keeps the
 * fastest for the rest of the process. */
int olg_autotune_cgh_gemm(int n_points, int ny, int nx, int reps, olg_stream_t stream);
/* Synchronises the device and reports (OLG_ERR_CUDA) whether a kernel of this
 * library with mbarrier waits (the tensor-core GEMM, the TMA-staged column
 * pass) gave up on a bounded wait; clear != 0 resets the flag. */
int olg_device_fault_check(int clear);

/* ------------------------------------------------------------------- WRP */
/* plane_z of ol::WRPMethod (golcgh.h:561-581, window = circle) and
 * ol::WRPMethod_D (golcgh.h:519-559, window = square), float arithmetic as
 * there; plimit <= 0 means plimit = p. */
float olg_wrp_plane_z(int window, int ny, int nx, float p, float plimit, float lambda, float zmin, float s);

/* WRP step 1.  Replaces ol::WRPStep1 (golcgh.h:369-389, circle window) and
 * ol::WRPStep1_D (golcgh.h:470-491, square window): U (ny x nx) is
 * overwritten with sum_j [inside window_j] exp(i pi rho^2 / (lambda dz_j)) / |dz_j|,
 * dz_j = z_j - plane_z.  Window radii and membership follow the reference's
 * float32 expressions; plimit <= 0 means plimit = p. */
int olg_wrp_step1_c64(const float *points, int n_points, void *U, int ny, int nx, float p, float lambda,
                      float plane_z, float plimit, int window, olg_stream_t stream);

/* Whole WRP method: step 1 onto the plane at olg_wrp_plane_z(), then
 * ol::WRPStep2 (golcgh.h:494-517): propagate by plane_z with `propmode`
 * (AUTO falls back to ASM, not band-limited Fresnel, as there).
 * Replaces ol::WRPMethod / ol::WRPMethod_D.  *plane_z_out is nullable. */
int olg_wrp_method_c64(const float *points, int n_points, void *U, int ny, int nx, float p, float lambda,
                       float zmin, float s, float plimit, int window, int propmode, int flags,
                       float *plane_z_out, olg_stream_t stream);

/* ------------------------------------------------------------ quantisers */
/* ol::complex2img(u, img, ny, nx, MODE) (olimg.h:348-391): per-pixel value
 * (phase / real / imag / amplitude), min-max (phase: -pi..pi) normalised to
 * round(255 (v - min) / (max - min)); a constant image maps to 0. */
int olg_complex2img_u8(const void *u, uint8_t *img, int ny, int nx, int mode, olg_stream_t stream);
/* Binarised 8-bit hologram (project rule): 255 where Re(U) >= 0, else 0. */
int olg_binarize_u8(const void *u, uint8_t *img, int ny, int nx, olg_stream_t stream);

/* ------------------------------------------- point clouds and image files */
/* Device point clouds are n records of float (x, y, z), as ol::gObject<float>. */

/* ol::objinfo (olobject.h:163-174) on the device: minmax_out (host, 6 floats)
 * = {xmin, ymin, zmin, xmax, ymax, zmax}.  Synchronises `stream`. */
int olg_obj_minmax_f32(const float *points, int n, float *minmax_out, olg_stream_t stream);

/* ol::objset on the device, in place.  y_range < 0: the one-range form
 * (olobject.h:196-230): scale = x_range / max(x extent, y extent); otherwise
 * the two-range form (olobject.h:232-264): the smaller of x_range / x extent
 * and y_range / y extent.  Then offset (host, 3 floats) minus the scaled
 * centre in x, y and the scaled zmin (OLG_OBJSET_ZMIN) or z centre
 * (OLG_OBJSET_ZMIDDLE), and p = p * scale + offset, rounded as the
 * reference's float code rounds it.  OLG_VERBOSE prints the extents as the
 * one-range form does.  Reads the extents back (synchronises `stream`). */
int olg_objset_f32(float *points, int n, float x_range, float y_range, const float *offset, int mode, int flags,
                   olg_stream_t stream);

/* ol::objsort (olobject.h:176-181) on the device, in place: records ordered
 * by z, largest first; equal z keep their order (the reference's std::sort
 * leaves it unspecified).  Scratch: olg_objsort_workspace_bytes(n). */
size_t olg_objsort_workspace_bytes(int n);
int olg_objsort_f32(float *points, int n, void *work, size_t work_bytes, olg_stream_t stream);

/* ol::objread (olobject.h:9-91), host: a .3d (int32 records) or .3df (float
 * records) file of a 4-byte count and n (x, y, z) records into `points`
 * (host, 3 * capacity floats).  points == NULL: only *n_out is set. */
int olg_objread(const char *path, float *points, int capacity, int *n_out);
/* ol::objread(path, offset, scale) (olobject.h:93-161), host: int32 records,
 * p = xint * scale + offset in float. */
int olg_objread_scaled(const char *path, const float *offset, float scale, float *points, int capacity,
                       int *n_out);

/* ol::bmpwrite (olimg.h:136-165) and ol::bmpread (olimg.h:55-99), host: an
 * 8-bit grey BMP (256-entry palette), rows in memory order, each followed by
 * nx % 4 zero bytes as the reference writes them (a standard row padding only
 * when nx % 4 is 0 or 2). */
int olg_bmpwrite_u8(const char *fname, const uint8_t *img, int ny, int nx);
int olg_bmpread_u8(const char *fname, uint8_t *img, int ny, int nx);

#ifdef __cplusplus
}
#endif
#endif
