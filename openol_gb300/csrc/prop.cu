// prop.cu -- fused ASM / Fresnel / ARSS propagation on GB300 (sm_103a):
// scratch layout, per-method set-up, the single-field entry points, the
// AUTO dispatcher and the tilted-plane glue.  The pass kernels are in
// propk.cuh, instantiated in prop_rows_fwd.cu, prop_rows_inv.cu,
// prop_cols.cu and prop_aux.cu; the batched launch in batch.cu, the phase
// optimiser in phase.cu, the autotuner in autotune.cu.
//
// The reference runs each propagation as ~8 full-size elementwise kernels
// plus 2-3 cuFFT calls over a 2x zero-padded grid (golprop.h:507-534 for ASM,
// 167-198 Fresnel, 941-995 ARSS), synchronising after every step.  Here one
// propagation of an ny x nx field (padded NY = 2ny, NX = 2nx) is three passes
// over HBM, with the padding, transfer function / chirp products and the
// crop folded into the FFT passes:
//
//   pass 1 (k_rows_fwd): the ny non-zero rows: load (x pre-chirp), zero-pad to
//          NX in shared memory, row FFT, store to scratch S (ny x NX).
//   pass 2 (k_cols):     tiles of C adjacent columns of S: load the ny rows
//          into the centre of an NY-long column (zeros around), column FFT,
//          x T(ky, kx), inverse column FFT, keep the central ny rows, store
//          back in place.
//   pass 3 (k_rows_inv): rows of S: inverse row FFT, keep the central nx
//          columns (x post-chirp), store the ny x nx result.
//
// Algorithmic HBM traffic per propagation: 8n + 16n + 16n + 16n + 16n + 8n =
// 80 n bytes (n = ny * nx), against ~71 n complex64 reads/writes in the
// reference's chain.  Transfer functions are evaluated in registers (ASM) or
// from two 1-D spectra of the separable chirp (Fresnel, ARSS): the 2-D FFT of
// the sampled chirp exp(i pi (x^2 + y^2) / (lambda z)) is the outer product of
// two 1-D FFTs, which k_chirp computes per call (exactly the DFT of the sampled
// response the reference builds, golprop.h:184-187, olprop.h:133-137).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "propk.cuh"

namespace olg {

namespace {
std::mutex g_tw_mu;
std::set<unsigned long long> g_tw_ready; // contexts whose tables hold the twiddles
std::vector<int (*)(const float2 *, const float4 *)> &tw_uploaders()
{
    static std::vector<int (*)(const float2 *, const float4 *)> v;
    return v;
}
} // namespace

int register_twiddle_uploader(int (*fn)(const float2 *, const float4 *))
{
    std::lock_guard<std::mutex> lk(g_tw_mu);
    tw_uploaders().push_back(fn);
    return 1;
}

int ensure_twiddles()
{
    unsigned long long ctx = 0;
    if (int rc = context_id(&ctx)) return rc;
    std::lock_guard<std::mutex> lk(g_tw_mu);
    if (g_tw_ready.count(ctx)) return OLG_OK;
    std::vector<float2> t(FFT_MAX);
    for (int m = 0; m < FFT_MAX; ++m) {
        const double a = -2.0 * M_PI * (double)m / (double)FFT_MAX;
        t[m] = make_float2((float)cos(a), (float)sin(a));
    }
    std::vector<float4> t4(FFT_MAX);
    for (int m = 0; m < FFT_MAX; ++m) t4[m] = make_float4(t[m].x, t[m].x, t[m].y, t[m].y);
    for (auto fn : tw_uploaders())
        if (int rc = fn(t.data(), t4.data())) return rc;
    g_tw_ready.insert(ctx);
    return OLG_OK;
}

// SMs of the current device (cached per device; 152 on GB300)
int sm_count()
{
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        cache[dev] = n;
    }
    return cache[dev];
}

// lengths that are not powers of two take the mixed-radix passes (propmr.cu)
int rows_pass(const PropParams &P, bool inverse, cudaStream_t st)
{
    if (!is_pow2(P.NX)) return mr_rows_pass(P, inverse, st);
    return inverse ? rows_inv_pass_pow2(P, st) : rows_fwd_pass_pow2(P, st);
}
int cols_pass(const PropParams &P, cudaStream_t st)
{
    if (!is_pow2(P.NY)) return mr_cols_pass(P, st);
    return cols_pass_pow2(P, st);
}
int chirp_axis(const ChirpAxis &A, cudaStream_t st)
{
    if (!is_pow2(A.L)) return mr_chirp_axis(A, st);
    return chirp_axis_pow2(A, st);
}

size_t layout_bytes(int ny, int nx, Layout *L, char *base)
{
    size_t off = 0;
    auto take = [&](size_t elems) {
        char *p = base ? base + off : nullptr;
        off += align_up(elems * sizeof(float2), 256);
        return (float2 *)p;
    };
    Layout l;
    l.S = take((size_t)ny * 2 * nx);
    l.Hx = take(2 * (size_t)nx);
    l.Hy = take(2 * (size_t)ny);
    l.tax = take(nx);
    l.tay = take(ny);
    l.tbx = take(nx);
    l.tby = take(ny);
    if (L) *L = l;
    return off;
}

// A field axis n is supported when the padded length 2n is a power of two in
// [32, 8192] (the tuned passes) or 2^a 3^b 5^c with n >= 8 that one CTA holds
// (mixed radix, up to 7680).
bool axis_ok(int n) { return is_pow2(n) ? (n >= 16 && 2 * n <= FFT_MAX) : (n >= 8 && mr_length_ok(2 * n)); }

int validate(const void *a, const void *b, int ny, int nx)
{
    if (!a || !b) return fail(OLG_ERR_INVALID_ARG, "null field pointer");
    if (((uintptr_t)a & 15) || ((uintptr_t)b & 15)) return fail(OLG_ERR_INVALID_ARG, "field pointers must be 16-byte aligned");
    if (!axis_ok(ny) || !axis_ok(nx))
        return fail(OLG_ERR_UNSUPPORTED_SIZE,
                    "ny, nx must be powers of two in [16, 4096] or have 2n = 2^a 3^b 5^c <= 7680 (n >= 8)");
    return OLG_OK;
}

PropParams base_params(const void *in, void *out, int ny, int nx, const Layout &L)
{
    PropParams P{};
    P.ny = ny; P.nx = nx; P.NY = 2 * ny; P.NX = 2 * nx;
    P.in = (const float2 *)in;
    P.out = (float2 *)out;
    P.S = L.S;
    P.Hx = L.Hx; P.Hy = L.Hy;
    P.pre_mode = OP_NONE; P.post_mode = OP_NONE;
    P.in_ld = nx;
    P.out_ld = nx;
    return P;
}

int run_passes(const PropParams &P, cudaStream_t st)
{
    if (int rc = rows_pass(P, false, st)) return rc;
    if (int rc = cols_pass(P, st)) return rc;
    return rows_pass(P, true, st);
}

long floor_lim(double v)
{
    double f = std::floor(v);
    if (!(f < 1073741824.0)) f = 1073741824.0;
    if (f < -1073741824.0) f = -1073741824.0;
    return (long)f;
}

void set_quad(float &hi, float &lo, double v)
{
    DF d = split_df(v);
    hi = d.hi;
    lo = d.lo;
}

// frac(v) in [-0.5, 0.5]
float frac_host(double v) { return (float)(v - std::nearbyint(v)); }

ChirpAxis chirp_axis_params(int L, int n, double d, double lambda, double z, double s_factor, int lim, double scale,
                            float2 *H)
{
    ChirpAxis A{};
    A.L = L;
    A.n = n;
    set_quad(A.kap_hi, A.kap_lo, s_factor * d * d / (2.0 * lambda * z));
    A.lim = lim;
    A.scale = (float)scale;
    A.conj_spec = 0;
    A.H = H;
    A.alim = A.blim = -1;
    return A;
}

} // namespace olg

using namespace olg;

extern "C" size_t olg_prop_workspace_bytes(int ny, int nx)
{
    if (ny <= 0 || nx <= 0) return 0;
    return layout_bytes(ny, nx, nullptr, nullptr);
}

namespace olg {

int check_phys(double dy, double dx, double lambda, double z, bool nonzero_z)
{
    if (!(dy > 0) || !(dx > 0) || !(lambda > 0) || !std::isfinite(z) || (nonzero_z && z == 0.0))
        return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    return OLG_OK;
}

// Whether every t = lambda^2 (u^2 + v^2) of an NY x NX frequency grid (steps
// du, dv; |u| <= NX du / 2, |v| <= NY dv / 2) is <= 1/64, where the ASM
// transfer function's phase remainder is taken from its series.
int asm_series_ok(double NY, double NX, double dv, double du, double lambda)
{
    const double um = 0.5 * NX * du, vm = 0.5 * NY * dv;
    return lambda * lambda * (um * um + vm * vm) <= 1.0 / 64.0 ? 1 : 0;
}

int setup_asm(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z, int flags,
              const Layout &L, PropSetup *S)
{
    if (int rc = check_phys(dy, dx, lambda, z, false)) return rc;
    PropParams P = base_params(in, out, ny, nx, L);
    if (int rc = mr_prepare(P)) return rc;
    const double NX = 2.0 * nx, NY = 2.0 * ny;
    const double du = 1.0 / (dx * NX), dv = 1.0 / (dy * NY);
    const double zl = z / lambda;
    P.method = M_ASM;
    P.conj = (flags & OLG_CONJ) ? 1 : 0;
    P.scale = (flags & OLG_NO_NORMALIZE) ? 1.0f : (float)(1.0 / (NX * NY));
    P.c0 = frac_host(zl);
    set_quad(P.ax_hi, P.ax_lo, z * lambda * du * du / 2.0);
    set_quad(P.ay_hi, P.ay_lo, z * lambda * dv * dv / 2.0);
    P.tx = (float)(lambda * lambda * du * du);
    P.ty = (float)(lambda * lambda * dv * dv);
    P.zl = (float)zl;
    P.tf_series = asm_series_ok(NY, NX, dv, du, lambda);
    S->P = P;
    S->chirps = false;
    return OLG_OK;
}

// Shifted ASM (golprop.h:335-420, 536-576): T gains the phase ox u + oy v,
// an integer multiple of (lx, ly) = (ox du, oy dv) cycles per frequency index.
// OLG_BANDLIMIT adds the band window of the host overload (olprop.h:251-300):
// T = 0 unless |u - u0| 2 < uw and |v - v0| 2 < vw, decided here in double
// for every frequency index exactly as that code decides it.
// T = double decides in double; T = float mirrors the PREC_T = float
// instantiation operation by operation (float operands, std::pow(float, int)
// and the sqrt in double, results stored to float; this file is compiled with
// -ffp-contract=off).  Adjacent split blocks sit exactly on a branch boundary
// (offset == 0.5 / du), so the precision decides which branch is taken.
template <typename T>
static void shifted_window(double pitch, int L, double o_, double z_, double lambda_, int *lo, int *hi)
{
    const T d = (T)1 / ((T)pitch * (T)L);
    const T o = (T)o_, z = (T)z_, lambda = (T)lambda_;
    const T s0 = (T)0.5 / d;
    const T tm = o - (T)0.5 / d, tp = o + (T)0.5 / d;
    const T lm = (T)(1 / std::sqrt(std::pow((double)tm, -2.0) * z * z + 1.0) / lambda);
    const T lp = (T)(1 / std::sqrt(std::pow((double)tp, -2.0) * z * z + 1.0) / lambda);
    T c, w;
    if (s0 < o) {
        c = (T)0.5 * (lp + lm);
        w = lp - lm;
    } else if (-s0 <= o && o < s0) {
        c = (T)0.5 * (lp - lm);
        w = lp + lm;
    } else {
        c = (T)-0.5 * (lp + lm);
        w = lm - lp;
    }
    *lo = 1;
    *hi = 0;
    bool any = false;
    for (int m = 0; m < L; ++m) {
        const int f = m - L / 2;
        const T u = (T)f * d;
        if (std::fabs(u - c) * 2 < w) {
            if (!any) *lo = f;
            *hi = f;
            any = true;
        }
    }
}

int setup_shifted_asm(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z,
                      double oy, double ox, int flags, const Layout &L, PropSetup *S)
{
    if (!std::isfinite(oy) || !std::isfinite(ox)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if (int rc = setup_asm(in, out, ny, nx, dy, dx, lambda, z, flags, L, S)) return rc;
    PropParams &P = S->P;
    const double du = 1.0 / (dx * 2.0 * nx), dv = 1.0 / (dy * 2.0 * ny);
    P.shift = 1;
    set_quad(P.lx_hi, P.lx_lo, ox * du);
    set_quad(P.ly_hi, P.ly_lo, oy * dv);
    if (flags & OLG_BANDLIMIT) {
        P.band = 1;
        if (flags & OLG_CHECK_F32) {
            shifted_window<float>(dx, 2 * nx, ox, z, lambda, &P.fx_lo, &P.fx_hi);
            shifted_window<float>(dy, 2 * ny, oy, z, lambda, &P.fy_lo, &P.fy_hi);
        } else {
            shifted_window<double>(dx, 2 * nx, ox, z, lambda, &P.fx_lo, &P.fx_hi);
            shifted_window<double>(dy, 2 * ny, oy, z, lambda, &P.fy_lo, &P.fy_hi);
        }
    }
    return OLG_OK;
}

int setup_fresnel(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z,
                  int bandlimit, int flags, const Layout &L, PropSetup *S)
{
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (bandlimit < 0 || bandlimit > 2) return fail(OLG_ERR_INVALID_ARG, "bandlimit must be 0, 1 or 2");
    PropParams P = base_params(in, out, ny, nx, L);
    if (int rc = mr_prepare(P)) return rc;
    const int NX = 2 * nx, NY = 2 * ny;
    const double np = (double)NX * (double)NY;
    const double sc1 = (flags & OLG_NO_NORMALIZE) ? 1.0 : 1.0 / np;
    int limx = -1, limy = -1;
    if (bandlimit == 1) { // golprop.h:227-233: one limit, from x, on both axes
        limx = limy = (int)floor_lim(std::fabs(lambda * z * 0.5 / dx) / dx);
    } else if (bandlimit == 2) { // olprop.h:34-39
        limx = (int)floor_lim(std::fabs(lambda * z * 0.5 / dx) / dx);
        limy = (int)floor_lim(std::fabs(lambda * z * 0.5 / dy) / dy);
    }
    S->ax = chirp_axis_params(NX, nx, dx, lambda, z, 1.0, limx, sc1, L.Hx);
    S->ay = chirp_axis_params(NY, ny, dy, lambda, z, 1.0, limy, sc1, L.Hy);
    S->chirps = true;
    P.method = M_CHIRP;
    P.conj = (flags & OLG_CONJ) ? 1 : 0;
    P.scale = 1.0f;
    S->P = P;
    return OLG_OK;
}

// windows == false: the shifted Fresnel propagation (golprop.h:606-752), the
// same three chirps without any window.
int setup_arss(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx, double lambda, double z,
               double s, double oy, double ox, int flags, const Layout &L, PropSetup *S, bool windows)
{
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (!std::isfinite(s) || !std::isfinite(oy) || !std::isfinite(ox))
        return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if (windows && (s == 0.0 || s == 1.0))
        return fail(OLG_ERR_INVALID_ARG, "ARSS is undefined for s = 0 or s = 1 (window limits divide by s|s-1|)");
    PropParams P = base_params(u_src, u_dst, ny, nx, L);
    if (int rc = mr_prepare(P)) return rc;
    const int NX = 2 * nx, NY = 2 * ny;
    const double np = (double)NX * (double)NY;
    // windows, golprop.h:849-852, 891-892, 928-931 (-1: none).  A computed
    // limit <= 0 is an empty window (the reference's |m| >= lim then holds for
    // every m; s < 0 makes the pre-chirp limits negative), so limits are
    // clamped at 0 and never reach the "none" value.
    int hlim_u = -1, wlim_u = -1, lim_h = -1, hlim_c = -1, wlim_c = -1;
    if (windows) {
        auto win = [](long v) { return (int)std::max(v, 0L); };
        hlim_u = win(floor_lim((lambda * std::fabs(z) * 0.5 / (s * std::fabs(s - 1) * dy)) / dy));
        wlim_u = win(floor_lim((lambda * std::fabs(z) * 0.5 / (s * std::fabs(s - 1) * dx)) / dx));
        lim_h = win(floor_lim(std::fabs(lambda * z * 0.5 / (dx * s)) / dx));
        hlim_c = win(floor_lim((lambda * std::fabs(z) * 0.5 / (std::fabs(1 - s) * dy)) / dy));
        wlim_c = win(floor_lim((lambda * std::fabs(z) * 0.5 / (std::fabs(1 - s) * dx)) / dx));
    }
    const bool adj = (flags & OLG_CONJ) != 0;
    const double lz2 = 2.0 * lambda * z;
    ChirpAxis ax = chirp_axis_params(NX, nx, dx, lambda, z, s, lim_h, 1.0 / np, L.Hx);
    ChirpAxis ay = chirp_axis_params(NY, ny, dy, lambda, z, s, lim_h, 1.0 / np, L.Hy);
    // pre-chirp (golprop.h:830-841) and post-chirp (golprop.h:910-920) coefficients, cycles
    struct Q {
        double a2, a1, a0;
    };
    const Q prex{(s * s - s) * dx * dx / lz2, -2.0 * s * ox * dx / lz2, 0.0};
    const Q prey{(s * s - s) * dy * dy / lz2, -2.0 * s * oy * dy / lz2, 0.0};
    const Q postx{(1 - s) * dx * dx / lz2, 2.0 * ox * dx / lz2, (ox * ox + oy * oy) / lz2};
    const Q posty{(1 - s) * dy * dy / lz2, 2.0 * oy * dy / lz2, 0.0};
    auto fill = [&](ChirpAxis &A, float2 *ta, float2 *tb, const Q &qa, int alim, int aconj, const Q &qb, int blim,
                    int bconj) {
        A.ta = ta;
        A.tb = tb;
        set_quad(A.a2_hi, A.a2_lo, qa.a2);
        set_quad(A.a1_hi, A.a1_lo, qa.a1);
        A.a0 = frac_host(qa.a0);
        A.alim = alim;
        A.aconj = aconj;
        set_quad(A.b2_hi, A.b2_lo, qb.a2);
        set_quad(A.b1_hi, A.b1_lo, qb.a1);
        A.b0 = frac_host(qb.a0);
        A.blim = blim;
        A.bconj = bconj;
    };
    if (!adj) {
        // pass 1: pre-chirp, zero outside its window; pass 3: post-chirp inside its window
        fill(ax, L.tax, L.tbx, prex, wlim_u, 0, postx, -1, 0);
        fill(ay, L.tay, L.tby, prey, hlim_u, 0, posty, -1, 0);
        P.pre_mode = OP_TABLE;
        P.post_mode = windows ? OP_TABLE_IN_WINDOW : OP_TABLE;
        P.post_hlim = hlim_c;
        P.post_wlim = wlim_c;
    } else {
        // adjoint: conj(post-chirp) inside the Cz window first, conj(pre-chirp) with its window last
        fill(ax, L.tax, L.tbx, postx, -1, 1, prex, wlim_u, 1);
        fill(ay, L.tay, L.tby, posty, -1, 1, prey, hlim_u, 1);
        P.pre_mode = windows ? OP_TABLE_IN_WINDOW : OP_TABLE;
        P.pre_hlim = hlim_c;
        P.pre_wlim = wlim_c;
        P.post_mode = OP_TABLE;
    }
    P.prex = L.tax;
    P.prey = L.tay;
    P.postx = L.tbx;
    P.posty = L.tby;
    P.method = M_CHIRP;
    P.conj = adj ? 1 : 0;
    P.scale = 1.0f;
    S->P = P;
    S->ax = ax;
    S->ay = ay;
    S->chirps = true;
    return OLG_OK;
}

int run_setup(const PropSetup &S, cudaStream_t st)
{
    if (S.chirps) {
        if (int rc = chirp_axis(S.ax, st)) return rc;
        if (int rc = chirp_axis(S.ay, st)) return rc;
    }
    return run_passes(S.P, st);
}

} // namespace olg

extern "C" int olg_asm_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                                double z, int flags, void *work, size_t work_bytes, olg_stream_t stream)
{
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, false)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_asm(u_in, u_out, ny, nx, dy, dx, lambda, z, flags, L, &S)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_fresnel_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                                    double z, int bandlimit, int flags, void *work, size_t work_bytes,
                                    olg_stream_t stream)
{
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (bandlimit < 0 || bandlimit > 2) return fail(OLG_ERR_INVALID_ARG, "bandlimit must be 0, 1 or 2");
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_fresnel(u_in, u_out, ny, nx, dy, dx, lambda, z, bandlimit, flags, L, &S)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_arss_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx, double lambda,
                                 double z, double s, double oy, double ox, int flags, void *work, size_t work_bytes,
                                 olg_stream_t stream)
{
    if (int rc = validate(u_src, u_dst, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (!std::isfinite(s)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if (s == 0.0 || s == 1.0)
        return fail(OLG_ERR_INVALID_ARG, "ARSS is undefined for s = 0 or s = 1 (window limits divide by s|s-1|)");
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_arss(u_src, u_dst, ny, nx, dy, dx, lambda, z, s, oy, ox, flags, L, &S)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_shifted_asm_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx,
                                        double lambda, double z, double oy, double ox, int flags, void *work,
                                        size_t work_bytes, olg_stream_t stream)
{
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, false)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_shifted_asm(u_in, u_out, ny, nx, dy, dx, lambda, z, oy, ox, flags, L, &S)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_shifted_fresnel_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx,
                                            double lambda, double z, double s, double oy, double ox, int flags,
                                            void *work, size_t work_bytes, olg_stream_t stream)
{
    if (int rc = validate(u_src, u_dst, ny, nx)) return rc;
    if (int rc = check_phys(dy, dx, lambda, z, true)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_arss(u_src, u_dst, ny, nx, dy, dx, lambda, z, s, oy, ox, flags, L, &S, false)) return rc;
    return run_setup(S, st);
}

extern "C" int olg_shifted_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx,
                                    double lambda, double z, double oy, double ox, int propmode, int flags, void *work,
                                    size_t work_bytes, olg_stream_t stream)
{
    if (propmode == OLG_ASM)
        return olg_shifted_asm_prop_c64(u_src, u_dst, ny, nx, dy, dx, lambda, z, oy, ox, flags, work, work_bytes,
                                        stream);
    if (propmode == OLG_FRESNEL)
        return olg_shifted_fresnel_prop_c64(u_src, u_dst, ny, nx, dy, dx, lambda, z, 1.0, oy, ox, flags, work,
                                            work_bytes, stream);
    return fail(OLG_ERR_INVALID_ARG, "shifted propagation takes OLG_ASM or OLG_FRESNEL");
}

extern "C" size_t olg_split_prop_workspace_bytes(int ny, int nx, int blocks_y, int blocks_x)
{
    if (ny <= 0 || nx <= 0 || blocks_y <= 0 || blocks_x <= 0) return 0;
    return layout_bytes(ny / blocks_y, nx / blocks_x, nullptr, nullptr);
}

// Split propagation (golprop.h:772-813, olprop.h:618-654): the field is cut
// into blocks_y x blocks_x blocks; every (source block, destination block)
// pair adds a shifted propagation of the source block, offset by the blocks'
// distance, into the destination block.  Blocks are read and written in place
// through row strides; u_out must not overlap u_in.
extern "C" int olg_split_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                                  double z, int propmode, int blocks_y, int blocks_x, int flags, void *work,
                                  size_t work_bytes, olg_stream_t stream)
{
    if (!u_in || !u_out || blocks_y <= 0 || blocks_x <= 0 || ny % blocks_y || nx % blocks_x)
        return fail(OLG_ERR_INVALID_ARG, "blocks must divide the field");
    const int bh = ny / blocks_y, bw = nx / blocks_x;
    if (int rc = validate(u_in, u_out, bh, bw)) return rc;
    if (propmode != OLG_ASM && propmode != OLG_FRESNEL)
        return fail(OLG_ERR_INVALID_ARG, "split propagation takes OLG_ASM or OLG_FRESNEL");
    const size_t bytes = (size_t)ny * nx * sizeof(float2);
    const char *a = (const char *)u_in, *b = (const char *)u_out;
    if (a < b + bytes && b < a + bytes) return fail(OLG_ERR_INVALID_ARG, "u_out must not overlap u_in");
    if (int rc = check_phys(dy, dx, lambda, z, propmode == OLG_FRESNEL)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, layout_bytes(bh, bw, nullptr, nullptr), st)) return rc;
    Layout L;
    layout_bytes(bh, bw, &L, (char *)sc.ptr);
    if (!(flags & OLG_ACCUMULATE)) {
        const cudaError_t e = cudaMemsetAsync(u_out, 0, bytes, st);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    }
    const int pflags = flags & (OLG_CONJ | OLG_NO_NORMALIZE | OLG_BANDLIMIT | OLG_CHECK_F32);
    for (int gn = 0; gn < blocks_y; ++gn)
        for (int gm = 0; gm < blocks_x; ++gm) {
            const float2 *src = (const float2 *)u_in + (size_t)gn * bh * nx + (size_t)gm * bw;
            for (int dn = 0; dn < blocks_y; ++dn)
                for (int dm = 0; dm < blocks_x; ++dm) {
                    float2 *dst = (float2 *)u_out + (size_t)dn * bh * nx + (size_t)dm * bw;
                    // offsets as the reference forms them: an int times a float pitch, in float
                    const double oy = (double)((float)((gn - dn) * bh) * (float)dy);
                    const double ox = (double)((float)((gm - dm) * bw) * (float)dx);
                    PropSetup S;
                    int rc = propmode == OLG_ASM
                                 ? setup_shifted_asm(src, dst, bh, bw, dy, dx, lambda, z, oy, ox, pflags, L, &S)
                                 : setup_arss(src, dst, bh, bw, dy, dx, lambda, z, 1.0, oy, ox, pflags, L, &S, false);
                    if (rc) return rc;
                    S.P.in_ld = nx;
                    S.P.out_ld = nx;
                    S.P.accumulate = 1;
                    if ((rc = run_setup(S, st))) return rc;
                }
        }
    return OLG_OK;
}

// ------------------------------------------------------------- tilted
namespace olg {

const float2 *twiddle_table()
{
    static std::mutex mu;
    static std::map<unsigned long long, const float2 *> cache; // per context
    unsigned long long ctx = 0;
    if (context_id(&ctx) != OLG_OK) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(ctx);
    if (it != cache.end()) return it->second;
    if (ensure_twiddles() != OLG_OK) return nullptr;
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tw) != cudaSuccess) return nullptr;
    cache.emplace(ctx, (const float2 *)p);
    return (const float2 *)p;
}

namespace {

struct TiltLayout {
    float2 *C, *D, *Hx, *Hy;
};

size_t tilt_layout(int ny, int nx, TiltLayout *L, char *base)
{
    size_t off = 0;
    auto take = [&](size_t elems) {
        char *p = base ? base + off : nullptr;
        off += align_up(elems * sizeof(float2), 256);
        return (float2 *)p;
    };
    const size_t full = (size_t)4 * ny * nx;
    TiltLayout l;
    l.C = take(full);
    l.D = take(full);
    l.Hx = take(2 * (size_t)nx);
    l.Hy = take(2 * (size_t)ny);
    if (L) *L = l;
    return off;
}

} // namespace
} // namespace olg

extern "C" size_t olg_tilted_workspace_bytes(int ny, int nx)
{
    if (ny <= 0 || nx <= 0) return 0;
    return tilt_layout(ny, nx, nullptr, nullptr);
}

// Tilted-plane propagation (olprop.h:414-600).  reference == 0:
// TiltedSourceProp, the destination plane rotated by `angle` about the y axis
// as seen from the source; the spectrum is resampled on the rotated grid and
// then propagated.  reference != 0: TiltedReferenceProp, propagated first and
// then resampled for a plane rotated by `angle`.  Every frequency of the 2x
// padded grid must propagate (no evanescent sample), as the reference's
// square roots require.  u_out may equal u_in.
extern "C" int olg_tilted_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda,
                                   double z, double angle, int interp, int propmode, int reference, void *work,
                                   size_t work_bytes, olg_stream_t stream)
{
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    if (propmode != OLG_ASM && propmode != OLG_FRESNEL)
        return fail(OLG_ERR_INVALID_ARG, "tilted propagation takes OLG_ASM or OLG_FRESNEL");
    if (interp != OLG_BILINEAR && interp != OLG_BICUBIC)
        return fail(OLG_ERR_INVALID_ARG, "interp must be OLG_BILINEAR or OLG_BICUBIC");
    if (int rc = check_phys(dy, dx, lambda, z, propmode == OLG_FRESNEL)) return rc;
    if (!std::isfinite(angle)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    const int NY = 2 * ny, NX = 2 * nx;
    const double N = (double)NY * (double)NX;
    const double du = 1 / (dx * NX), dv = 1 / (dy * NY);
    const double fsqr = 1 / (lambda * lambda), f0 = 1 / lambda;
    const double ang = reference ? angle : -angle;
    const double a11 = std::cos(ang), a13 = -std::sin(ang);
    const double a13f0 = reference ? 0.0 : a13 * f0;
    // the largest |fpx|, |fpy| (and |fpx + a13 f0| for the shifted ASM) sit on the grid's corners
    for (int cm = 0; cm < 2; ++cm)
        for (int cn = 0; cn < 2; ++cn) {
            const double fpx = (double)((cm ? NX - 1 : 0) - NX / 2) * du, fpy = (double)((cn ? NY - 1 : 0) - NY / 2) * dv;
            const double uu = fpx + a13f0;
            if (!(fsqr - fpx * fpx - fpy * fpy > 0) ||
                (!reference && propmode == OLG_ASM && !(fsqr - uu * uu - fpy * fpy >= 0)))
                return fail(OLG_ERR_INVALID_ARG, "tilted propagation: the padded grid reaches evanescent frequencies");
        }
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, tilt_layout(ny, nx, nullptr, nullptr), st)) return rc;
    TiltLayout TL;
    tilt_layout(ny, nx, &TL, (char *)sc.ptr);
    Layout L{};
    L.S = TL.D;
    PropParams P = base_params(u_in, u_out, ny, nx, L);
    if (int rc = mr_prepare(P)) return rc;

    TiltArgs T{};
    T.ny = ny; T.nx = nx; T.NY = NY; T.NX = NX;
    T.reference = reference ? 1 : 0;
    T.interp = interp;
    T.fresnel = propmode == OLG_FRESNEL ? 1 : 0;
    T.du = du; T.dv = dv; T.fsqr = fsqr; T.a11 = a11; T.a13 = a13; T.a13f0 = a13f0; T.z = z;
    T.J0 = (float)a11;
    T.Jb = (float)(-a13);
    T.invN = (float)(1.0 / N);
    {
        // a11 - 1 = -2 sin^2(ang / 2), without cancellation
        const double sh = std::sin(ang / 2);
        set_quad(T.c1_hi, T.c1_lo, -2.0 * sh * sh);
        const double K = reference ? a13 * f0 / du : 0.0;
        const double Ki = std::nearbyint(K);
        T.Ki = (int)Ki;
        T.Kf = (float)(K - Ki);
        T.a13f = (float)a13;
        T.duf = (float)du;
        T.dvf = (float)dv;
        T.dv2du = (float)(dv * dv / du);
        T.f0f = (float)f0;
        T.f0sq = (float)(f0 * f0);
        set_quad(T.du_hi, T.du_lo, du);
        set_quad(T.dv_hi, T.dv_lo, dv);
        set_quad(T.c_hi, T.c_lo, a13 * f0);
        set_quad(T.f0sq_hi, T.f0sq_lo, fsqr);
        set_quad(T.z_hi, T.z_lo, z);
    }
    T.Hx = TL.Hx; T.Hy = TL.Hy;
    T.C = TL.C; T.D = TL.D;
    PropParams &tf = T.tf;
    tf.ny = ny; tf.nx = nx; tf.NY = NY; tf.NX = NX;
    tf.scale = 1.0f;
    if (propmode == OLG_FRESNEL) {
        tf.method = M_CHIRP;
        tf.Hx = TL.Hx;
        tf.Hy = TL.Hy;
    } else {
        const double zl = z / lambda;
        tf.method = M_ASM;
        tf.c0 = frac_host(zl);
        set_quad(tf.ax_hi, tf.ax_lo, z * lambda * du * du / 2.0);
        set_quad(tf.ay_hi, tf.ay_lo, z * lambda * dv * dv / 2.0);
        tf.tx = (float)(lambda * lambda * du * du);
        tf.ty = (float)(lambda * lambda * dv * dv);
        tf.zl = (float)zl;
    }

    if (int rc = rows_pass(P, false, st)) return rc;
    if (propmode == OLG_FRESNEL) {
        // the Fresnel response's spectrum, fftshift'ed, 1/N (on x), with the
        // source form's linear phase exp(-2 pi i x a13 f0) along x
        ChirpAxis ax = chirp_axis_params(NX, nx, dx, lambda, z, 1.0, -1, 1.0 / N, TL.Hx);
        if (!reference) set_quad(ax.lin_hi, ax.lin_lo, -a13 * f0 * dx);
        ChirpAxis ay = chirp_axis_params(NY, ny, dy, lambda, z, 1.0, -1, 1.0, TL.Hy);
        if (int rc = chirp_axis(ax, st)) return rc;
        if (int rc = chirp_axis(ay, st)) return rc;
    }
    if (int rc = tilt_middle(T, st)) return rc;
    return rows_pass(P, true, st);
}

// ---------------------------------------------------------------- AUTO checks
// AsmPropCheck olprop.h:209-225 and FresnelPropCheck olprop.h:109-123 in the
// caller's precision.  This file is compiled with -ffp-contract=off so the
// float versions round each operation like the reference's float build.
template <typename T>
static int asm_check_t(int ny, int nx, T dy, T dx, T lambda, T z)
{
    const int64_t nx2 = 2 * (int64_t)nx, ny2 = 2 * (int64_t)ny;
    const T du = 1 / (dx * nx2);
    const T dv = 1 / (dy * ny2);
    const T umax = du * nx2 / 2;
    const T vmax = dv * ny2 / 2;
    const T tmpsqrt = std::sqrt(1 / (lambda * lambda) - umax * umax - vmax * vmax);
    const T zmax_u = tmpsqrt / (2 * umax * du);
    const T zmax_v = tmpsqrt / (2 * vmax * dv);
    return (zmax_u < std::abs(z) || zmax_v < std::abs(z)) ? 0 : 1;
}
template <typename T>
static int fresnel_check_t(int ny, int nx, T dy, T dx, T lambda, T z)
{
    const size_t nx2 = 2 * (size_t)nx, ny2 = 2 * (size_t)ny;
    const T xmax = dx * nx2 / 2;
    const T ymax = dy * ny2 / 2;
    const T zmin_x = 2 * xmax * dx / lambda;
    const T zmin_y = 2 * ymax * dy / lambda;
    return (zmin_x > std::abs(z) || zmin_y > std::abs(z)) ? 0 : 1;
}

extern "C" int olg_asm_prop_check(int ny, int nx, double dy, double dx, double lambda, double z, int single_precision)
{
    if (single_precision) return asm_check_t<float>(ny, nx, (float)dy, (float)dx, (float)lambda, (float)z);
    return asm_check_t<double>(ny, nx, dy, dx, lambda, z);
}

extern "C" int olg_fresnel_prop_check(int ny, int nx, double dy, double dx, double lambda, double z, int single_precision)
{
    if (single_precision) return fresnel_check_t<float>(ny, nx, (float)dy, (float)dx, (float)lambda, (float)z);
    return fresnel_check_t<double>(ny, nx, dy, dx, lambda, z);
}

extern "C" int olg_prop_c64(void *u, int ny, int nx, double dy, double dx, double lambda, double z, int mode, int flags,
                            int *chosen, void *work, size_t work_bytes, olg_stream_t stream)
{
    const bool verbose = (flags & OLG_VERBOSE) != 0;
    const int f = flags & (OLG_CONJ | OLG_NO_NORMALIZE);
    const int sp = (flags & OLG_CHECK_F32) ? 1 : 0;
    int pick;
    if (mode == OLG_FRESNEL) pick = 1;
    else if (mode == OLG_ASM) pick = 0;
    else if (mode == OLG_AUTO) {
        if (olg_asm_prop_check(ny, nx, dy, dx, lambda, z, sp)) pick = 0;
        else if (!olg_fresnel_prop_check(ny, nx, dy, dx, lambda, z, sp)) pick = 2;
        else pick = 1;
    } else {
        return fail(OLG_ERR_INVALID_ARG, "invalid PROPMODE");
    }
    if (chosen) *chosen = pick;
    if (verbose) {
        if (pick == 0) printf("AsmProp\n");
        else if (pick == 1) printf("FresnelProp\n");
        else printf("warning!!\neither AsmProp or FresnelProp does not meet the condition.\n");
    }
    if (pick == 0) return olg_asm_prop_c64(u, u, ny, nx, dy, dx, lambda, z, f, work, work_bytes, stream);
    return olg_fresnel_prop_c64(u, u, ny, nx, dy, dx, lambda, z, pick == 2 ? 1 : 0, f, work, work_bytes, stream);
}

