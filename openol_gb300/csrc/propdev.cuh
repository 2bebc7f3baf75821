// propdev.cuh -- device-side definitions shared by the propagation
// translation units (prop.cu: power-of-two passes, batch, phase optimisation;
// propmr.cu: mixed-radix passes): parameters, the pass prologue/epilogue
// operations, the ASM transfer function and the chirp tables.
#pragma once
#include "common.cuh"

namespace olg {

// Programmatic dependent launch: a pass lets the next one launch as soon as all
// of its CTAs are running, and waits for the previous grid's completion (and
// memory) before touching any field data.  Both are no-ops when the launch
// carries no programmatic-serialisation attribute.
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Mixed-radix stage plan of one FFT length: nst radices in order (product n),
// 5 bits each in `radices` (stage i: (radices >> 5 i) & 31), so that device code
// reads them with shifts (an indexed array in a kernel parameter would be
// copied to local memory).
struct MrPlan {
    int n, nst;
    unsigned long long radices;
};

enum : int { M_ASM = 0, M_CHIRP = 1 };
// pre/post operation modes
enum : int { OP_NONE = 0, OP_TABLE = 1, OP_TABLE_IN_WINDOW = 2, OP_SEED = 3 };

struct PropParams {
    int ny, nx, NY, NX;
    int method;     // M_ASM: T computed in registers; M_CHIRP: T = Hx[kx] * Hy[ky]
    int conj;       // conjugate T (adjoint)
    float scale;    // folded into T
    // ASM transfer function constants (cycles)
    float c0;               // frac(z / lambda)
    float ax_hi, ax_lo;     // z lambda du^2 / 2
    float ay_hi, ay_lo;     // z lambda dv^2 / 2
    float tx, ty;           // lambda^2 du^2, lambda^2 dv^2
    float zl;               // z / lambda
    // every t = lambda^2 (u^2 + v^2) of the grid is <= 1/64: g by its series
    int tf_series;
    // chirp spectra (M_CHIRP)
    const float2 *Hx, *Hy;
    // pass-1 and pass-3 elementwise operations
    int pre_mode, post_mode;
    const float2 *prex, *prey, *postx, *posty;
    int pre_hlim, pre_wlim, post_hlim, post_wlim;
    int accumulate;
    const float2 *in;
    float2 *out;
    float2 *S;
    // phase-only input (pass 1 reads phi and forms exp(i phi)) when non-null
    const float *in_phase;
    // OP_SEED (pass 3): out = seed_scale (|v|^2 - target) v, loss += sum (|v|^2 - target)^2
    const float *target;
    float seed_scale;
    double *loss;
    // tables written earlier in the same launch (batched persistent kernel):
    // read them through L2 (ld.global.cg), never the non-coherent path
    int coherent;
    // row strides (elements) of in / in_phase and of out (sub-blocks of a larger field)
    long in_ld, out_ld;
    // mixed-radix passes (lengths that are not powers of two): stage plans,
    // tables exp(-2 pi i m / N), rows per pass-1/3 CTA and columns per pass-2 CTA
    MrPlan mrx, mry;
    const float2 *twx, *twy;
    int mr_rows, mr_cols;
    // shifted ASM: extra phase ox u + oy v = lx fx + ly fy cycles; optional band
    // window fx in [fx_lo, fx_hi], fy in [fy_lo, fy_hi] (T = 0 outside)
    int shift, band;
    float lx_hi, lx_lo, ly_hi, ly_lo;
    int fx_lo, fx_hi, fy_lo, fy_hi;
};

__device__ __forceinline__ float2 apply_op(float2 v, int mode, const float2 *tx, const float2 *ty, int h, int w,
                                           int ny, int nx, int hlim, int wlim)
{
    if (mode == OP_NONE) return v;
    if (mode == OP_TABLE_IN_WINDOW) {
        if (!(abs(w - nx / 2) < wlim && abs(h - ny / 2) < hlim)) return v;
    }
    return cmul(v, cmul(__ldg(tx + w), __ldg(ty + h)));
}

__device__ __forceinline__ float2 ld_tab(const float2 *p, int coherent) { return coherent ? __ldcg(p) : __ldg(p); }

__device__ __forceinline__ float2 apply_op_c(float2 v, int mode, const float2 *tx, const float2 *ty, int h, int w,
                                             int ny, int nx, int hlim, int wlim, int coherent)
{
    if (mode == OP_NONE) return v;
    if (mode == OP_TABLE_IN_WINDOW) {
        if (!(abs(w - nx / 2) < wlim && abs(h - ny / 2) < hlim)) return v;
    }
    return cmul(v, cmul(ld_tab(tx + w, coherent), ld_tab(ty + h, coherent)));
}

// ASM transfer function exp(2 pi i z w) at (fx, fy), cycles evaluated as
//   frac(z/lambda) - ax fx^2 - ay fy^2 - (z/lambda) t^2 / (2 (1 + sqrt(1-t))^2)
// with t = lambda^2 (u^2 + v^2): the exact expansion of z sqrt(1/lambda^2 - u^2 - v^2).
// The two quadratic terms are reduced exactly (frac_mul); the remainder is
// a few cycles at most, so FP32 keeps ~1e-6 rad of phase.  t > 1 gives NaN,
// as sqrt of a negative argument does in the reference (golprop.h:318).
__device__ __forceinline__ float2 asm_tf(const PropParams &P, int fx, int fy)
{
    const float fx2 = (float)(fx * fx), fy2 = (float)(fy * fy);
    const float t = P.tx * fx2 + P.ty * fy2;
    // s enters only through q = t / (1 + s), so its relative error reaches the
    // phase scaled by t / (1 + s) ~ 1e-2: the approximate square root (about
    // 1 ulp) moves the phase by < 1e-6 cycles at z / lambda ~ 3e5, where the
    // correctly rounded sqrtf costs a multi-instruction sequence per element.
    // A negative argument (evanescent t > 1) still gives NaN.
    float g;
    if (P.tf_series) {
        // g = (1 - sqrt(1 - t))^2 / 2 by the binomial series of sqrt(1 - t):
        // g = t^2/8 + t^3/16 + 5 t^4/128 + 7 t^5/256 + 21 t^6/1024 + ...;
        // for t <= 1/64 the first omitted term is < 2e-8 of g, below the
        // float rounding of the sum.
        const float t2 = t * t;
        g = t2 * fmaf(t, fmaf(t, fmaf(t, 0.02734375f, 0.0390625f), 0.0625f), 0.125f);
    } else {
        float s;
        asm("sqrt.approx.f32 %0, %1;" : "=f"(s) : "f"(1.0f - t));
        const float q = __fdividef(t, 1.0f + s); // 1 + s in [1, 2]: the fast divide is within 2 ulp
        g = 0.5f * q * q;
    }
    float cyc = P.c0 - frac_mul(P.ax_hi, P.ax_lo, fx2) - frac_mul(P.ay_hi, P.ay_lo, fy2) - P.zl * g;
    if (P.shift) {
        if (P.band && (fx < P.fx_lo || fx > P.fx_hi || fy < P.fy_lo || fy > P.fy_hi)) return make_float2(0.f, 0.f);
        cyc += frac_mul(P.lx_hi, P.lx_lo, (float)fx) + frac_mul(P.ly_hi, P.ly_lo, (float)fy);
    }
    cyc = wrap_cycles(cyc);
    if (P.conj) cyc = -cyc;
    return cscale(cis_cycles(cyc), P.scale);
}

__device__ __forceinline__ float2 tf_at(const PropParams &P, int ky, int kx, int NY)
{
    if (P.method == M_ASM) {
        const int fx = kx < P.NX / 2 ? kx : kx - P.NX;
        const int fy = ky < NY / 2 ? ky : ky - NY;
        return asm_tf(P, fx, fy);
    }
    float2 T = cmul(ld_tab(P.Hx + kx, P.coherent), ld_tab(P.Hy + ky, P.coherent));
    return P.conj ? cconj(T) : T;
}

__device__ __forceinline__ float2 load_in(const PropParams &P, int h, int w)
{
    float2 x;
    if (P.in_phase) {
        const float ph = __ldg(P.in_phase + (size_t)h * P.in_ld + w);
        sincosf(ph, &x.y, &x.x);
    } else {
        x = __ldg(P.in + (size_t)h * P.in_ld + w);
    }
    return apply_op_c(x, P.pre_mode, P.prex, P.prey, h, w, P.ny, P.nx, P.pre_hlim, P.pre_wlim, P.coherent);
}

__device__ __forceinline__ void store_out(const PropParams &P, int h, int w, float2 a, float &lsum)
{
    const size_t o = (size_t)h * P.out_ld + w;
    if (P.post_mode == OP_SEED) {
        const float r2 = a.x * a.x + a.y * a.y - __ldg(P.target + (size_t)h * P.nx + w);
        lsum = fmaf(r2, r2, lsum);
        a = cscale(a, P.seed_scale * r2);
    } else {
        a = apply_op_c(a, P.post_mode, P.postx, P.posty, h, w, P.ny, P.nx, P.post_hlim, P.post_wlim, P.coherent);
    }
    if (P.accumulate) {
        const float2 v = P.out[o];
        a.x += v.x;
        a.y += v.y;
    }
    P.out[o] = a;
}

__device__ __forceinline__ void loss_reduce(float lsum, double *loss, int tid, int nt)
{
    __shared__ float red[32];
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((tid & 31) == 0) red[tid >> 5] = lsum;
    __syncthreads();
    if (tid < 32) {
        float v = tid < nt / 32 ? red[tid] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (tid == 0) atomicAdd(loss, (double)v);
    }
}

struct ChirpAxis {
    int L, n;                  // padded length, field length along this axis
    float kap_hi, kap_lo;      // chirp cycles per index^2
    int lim;                   // chirp window (< 0: none)
    float scale;               // applied to the spectrum
    int conj_spec;             // conjugate the spectrum
    float2 *H;                 // out: L
    // elementwise tables (nullable)
    float2 *ta, *tb;           // out: n each
    float a2_hi, a2_lo, a1_hi, a1_lo, a0; int alim; int aconj;
    float b2_hi, b2_lo, b1_hi, b1_lo, b0; int blim; int bconj;
    float lin_hi, lin_lo;      // linear chirp term, cycles per index (0: none)
};

// One sample of the chirp: exp(2 pi i (kap m^2 + lin m)), 0 outside the window.
__device__ __forceinline__ float2 chirp_sample(const ChirpAxis &A, int m)
{
    if (A.lim >= 0 && abs(m) >= A.lim) return make_float2(0.f, 0.f);
    const float q = frac_mul(A.kap_hi, A.kap_lo, (float)m * (float)m);
    if (A.lin_hi == 0.f && A.lin_lo == 0.f) return cis_cycles(q);
    return cis_cycles(wrap_cycles(q + frac_mul(A.lin_hi, A.lin_lo, (float)m)));
}


// The ARSS pre/post tables of one axis (no FFT): ta, tb of length n.
__device__ __forceinline__ void chirp_tables(const ChirpAxis &A, int tid, int nt)
{
    for (int m = tid; m < A.n; m += nt) {
        const int mp = m - A.n / 2;
        const float fm = (float)mp, fm2 = (float)(mp * mp);
        if (A.ta) {
            float2 v = make_float2(0.f, 0.f);
            if (A.alim < 0 || abs(mp) < A.alim) {
                const float cyc = frac_mul(A.a2_hi, A.a2_lo, fm2) + frac_mul(A.a1_hi, A.a1_lo, fm) + A.a0;
                v = cis_cycles(wrap_cycles(cyc));
                if (A.aconj) v = cconj(v);
            }
            A.ta[m] = v;
        }
        if (A.tb) {
            float2 v = make_float2(0.f, 0.f);
            if (A.blim < 0 || abs(mp) < A.blim) {
                const float cyc = frac_mul(A.b2_hi, A.b2_lo, fm2) + frac_mul(A.b1_hi, A.b1_lo, fm) + A.b0;
                v = cis_cycles(wrap_cycles(cyc));
                if (A.bconj) v = cconj(v);
            }
            A.tb[m] = v;
        }
    }
}

} // namespace olg
