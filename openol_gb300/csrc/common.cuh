// common.cuh -- shared helpers for the libolgb300 kernels (sm_103a).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/olgb300.h"

namespace olg {

// ------------------------------------------------------------------ host side
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *where);
int fail(int status, const std::string &msg);
void count_launch(unsigned n = 1);

// Check the last launch; returns OLG_OK or OLG_ERR_CUDA with a message.
int check_launch(const char *what);

// Identifier of the calling thread's current CUDA context (the runtime's
// primary context of the current device, made current if none is).  Ids are
// unique over the process: a context destroyed by cudaDeviceReset and created
// again gets a new one.  Host-side caches of device state (uploaded tables,
// symbol addresses, allocations, function attributes) are keyed on it, so a
// re-created context never inherits pointers or "already done" flags that
// belonged to its predecessor.
int context_id(unsigned long long *id);

// Budget of one bounded device-side wait, in SM clock cycles (default 4e9,
// about 2 s at 2 GHz); olg_wait_budget_cycles sets it.
long long wait_budget_cycles();
// SMs of the current device (cached per device; prop.cu)
int sm_count();

// Copies of a sequence of host items pipelined against their computation:
// item i's inputs go up on the copy-in stream, its computation runs on the
// caller's stream and its result comes down on the copy-out stream, and
// device slot i % 3 holds item i.  So item i+1's copy in and item i-1's copy
// out overlap item i's computation.  Both copy streams first wait for the
// caller's stream, and the caller's stream ends waiting for the last copy
// out, so the whole sequence is ordered on the caller's stream like one call.
// Per item: copy_in_begin (then the copies in on s_in), copy_in_end (then
// the computation on the caller's stream), compute_end (then the copies out
// on s_out), copy_out_end.
struct HostPipeline {
    static constexpr int SLOTS = 3;
    cudaStream_t s_in = nullptr, s_out = nullptr;
    cudaEvent_t entry = nullptr, last = nullptr;
    cudaEvent_t in[SLOTS]{}, done[SLOTS]{}, out[SLOTS]{};
    int init(); // idempotent
    void release();
    int begin(cudaStream_t st);
    int copy_in_begin(int i);
    int copy_in_end(int i, cudaStream_t st);
    int compute_end(int i, cudaStream_t st);
    int copy_out_end(int i);
    int end(cudaStream_t st);
    void drain(); // waits on the host for both copy streams (error paths)
};

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against libcuda).
int tensor_map_encoder(PFN_cuTensorMapEncodeTiled_v12000 *out);

// Device word, one per CUDA context, that kernels with bounded waits set
// when a wait runs out; olg_device_fault_check reads and clears it.
int device_fault_word(int **out);

// Stream-ordered scratch: caller memory when given, else cudaMallocAsync.
struct Scratch {
    void *ptr = nullptr;
    size_t bytes = 0;
    bool owned = false;
    cudaStream_t stream = nullptr;
    int acquire(void *work, size_t work_bytes, size_t need, cudaStream_t s);
    ~Scratch();
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

inline bool is_pow2(long v) { return v > 0 && (v & (v - 1)) == 0; }

// Double-float constant: value = hi + lo, |lo| <= ulp(hi)/2.
struct DF {
    float hi, lo;
};
inline DF split_df(double v)
{
    DF r;
    r.hi = (float)v;
    r.lo = (float)(v - (double)r.hi);
    return r;
}

// ---------------------------------------------------------------- device side
// frac(c * m) in cycles, wrapped to [-0.5, 0.5], for c = c.hi + c.lo and an
// exactly representable float m (|m| <= 2^24).  The product c.hi * m is split
// exactly with an FMA, its integer part removed exactly, and the rounding
// error terms added back at small magnitude.
// Round to an integer by adding and removing 1.5 * 2^23: round to nearest
// even, exact for |x| < 2^22; beyond that an integer near x (callers only use
// the result modulo 1, and every caller wraps its final sum again).  Plain
// FP32 adds, cheaper than a rounding instruction.
__device__ __forceinline__ float round_int(float x) { return __fsub_rn(__fadd_rn(x, 12582912.0f), 12582912.0f); }

__device__ __forceinline__ float frac_mul(float chi, float clo, float m)
{
    const float p = __fmul_rn(chi, m); // never contracted into an FMA
    const float e = __fmaf_rn(chi, m, -p);
    const float r = p - round_int(p);
    float t = r + (e + clo * m);
    return t - round_int(t);
}

__device__ __forceinline__ float wrap_cycles(float t) { return t - round_int(t); }

// exp(2 pi i t) for t in cycles (|t| <= ~1 after wrapping).
__device__ __forceinline__ float2 cis_cycles(float t)
{
    float s, c;
    __sincosf(6.283185307179586f * t, &s, &c);
    return make_float2(c, s);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// ---- double-float arithmetic (pairs of floats, ~44 bits) for range reduction
struct df2 {
    float hi, lo;
};
__device__ __forceinline__ df2 df_two_sum(float a, float b)
{
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
__device__ __forceinline__ df2 df_fast_two_sum(float a, float b)
{
    float s = a + b;
    float e = b - (s - a);
    return {s, e};
}
__device__ __forceinline__ df2 df_two_prod(float a, float b)
{
    float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ df2 df_add(df2 a, df2 b)
{
    df2 s = df_two_sum(a.hi, b.hi);
    df2 t = df_two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = df_fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df2 df_add_f(df2 a, float b)
{
    df2 s = df_two_sum(a.hi, b);
    s.lo += a.lo;
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df2 df_mul(df2 a, df2 b)
{
    df2 p = df_two_prod(a.hi, b.hi);
    p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
    return df_fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df2 df_sqrt(df2 a)
{
    // one Newton step on the float square root: r = s + (a - s^2) / (2 s)
    float s = sqrtf(a.hi);
    df2 s2 = df_two_prod(s, s);
    float d = ((a.hi - s2.hi) - s2.lo + a.lo) / (2.0f * s);
    return df_fast_two_sum(s, d);
}
__device__ __forceinline__ df2 df_recip(df2 a)
{
    // r = 1/a.hi corrected once: r' = r + r (1 - a r)
    float r = 1.0f / a.hi;
    df2 ar = df_mul(a, {r, 0.0f});
    float e = (1.0f - ar.hi) - ar.lo;
    return df_fast_two_sum(r, r * e);
}
// fractional part in [-0.5, 0.5] of a double-float
__device__ __forceinline__ float df_frac(df2 a)
{
    float r = a.hi - rintf(a.hi);
    float t = r + a.lo;
    return t - rintf(t);
}

} // namespace olg
