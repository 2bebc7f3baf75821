// fftp.cuh -- paired-sequence FFT building blocks (sm_100 and later).
//
// Two complex sequences advance in lockstep, held as planar pairs:
//   cpair { re = (re_a, re_b), im = (im_a, im_b) }.
// Every real operation of a butterfly is then one paired FP32 instruction
// (add / mul / fma .f32x2): both sequences share the butterfly's index, so
// twiddles are shared too, and a radix-16 butterfly costs half the issue
// slots of the scalar form.  Shared memory holds one float4
// (re_a, re_b, im_a, im_b) per element pair, with the same one-slot-per-16
// padding as fft.cuh, which keeps both the row and the column-tile layouts
// free of bank conflicts for 128-bit accesses.
//
// Twiddles come from a table of float4 (c, c, s, s) with
// c + i s = exp(-2 pi i m / FFT_MAX).
#pragma once
#include "fft2.cuh"

namespace olg {

struct cpair {
    float2 re, im;
};

__device__ __forceinline__ float2 pp(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b (one fused multiply-add by -1: rounds exactly like a subtraction)
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, pp(-1.f), a); }
__device__ __forceinline__ float2 pneg(float2 a) { return __fmul2_rn(a, pp(-1.f)); }
__device__ __forceinline__ cpair cp_add(const cpair &a, const cpair &b) { return {padd(a.re, b.re), padd(a.im, b.im)}; }
__device__ __forceinline__ cpair cp_sub(const cpair &a, const cpair &b) { return {psub(a.re, b.re), psub(a.im, b.im)}; }
__device__ __forceinline__ cpair cp_zero() { return {pp(0.f), pp(0.f)}; }

// pack two complex values (sequence a, sequence b) / unpack lane 0 or 1
__device__ __forceinline__ cpair cp_pack(float2 a, float2 b) { return {make_float2(a.x, b.x), make_float2(a.y, b.y)}; }
__device__ __forceinline__ float2 cp_lane0(const cpair &v) { return make_float2(v.re.x, v.im.x); }
__device__ __forceinline__ float2 cp_lane1(const cpair &v) { return make_float2(v.re.y, v.im.y); }
__device__ __forceinline__ cpair cp_ld(const float4 *p)
{
    const float4 f = *p;
    return {make_float2(f.x, f.y), make_float2(f.z, f.w)};
}
__device__ __forceinline__ void cp_st(float4 *p, const cpair &v) { *p = make_float4(v.re.x, v.re.y, v.im.x, v.im.y); }

// v * (DIR i)
template <int DIR>
__device__ __forceinline__ cpair cp_mul_di(const cpair &v)
{
    return DIR < 0 ? cpair{v.im, pneg(v.re)} : cpair{pneg(v.im), v.re};
}

// v * (c + i s) with (c, s) the same for both lanes
__device__ __forceinline__ cpair cp_rot(const cpair &v, float2 C, float2 S, float2 NS)
{
    return {__ffma2_rn(v.im, NS, __fmul2_rn(v.re, C)), __ffma2_rn(v.re, S, __fmul2_rn(v.im, C))};
}

// a twiddle broadcast to both lanes: (c, c), (s, s) and (-s, -s); loaded
// from table entry m it is exp(-2 pi i m / FFT_MAX) for DIR < 0, else its
// conjugate
struct cptw {
    float2 C, S, NS;
};

template <int DIR>
__device__ __forceinline__ cptw cp_tw_load(const float4 *__restrict__ tw, int m)
{
    const float4 w = __ldg(tw + m);
    const float2 S = make_float2(w.z, w.w), NS = pneg(S);
    return DIR < 0 ? cptw{make_float2(w.x, w.y), S, NS} : cptw{make_float2(w.x, w.y), NS, S};
}

// a b for two broadcast twiddles (paired ops; the lanes stay equal)
__device__ __forceinline__ cptw cp_tw_mul(const cptw &a, const cptw &b)
{
    const float2 C = __ffma2_rn(a.S, b.NS, __fmul2_rn(a.C, b.C));
    const float2 S = __ffma2_rn(a.S, b.C, __fmul2_rn(a.C, b.S));
    return {C, S, pneg(S)};
}

__device__ __forceinline__ cpair cp_rot(const cpair &v, const cptw &w) { return cp_rot(v, w.C, w.S, w.NS); }

// v[r] *= w^r for r = 1 .. R-1 with w = table[m] (conjugated for DIR > 0):
// w, w^2, w^4, w^8 from the table, the other powers as products of those,
// as twiddle_powers does for the scalar form.
template <int R, int DIR>
__device__ __forceinline__ void cp_twiddle_powers(cpair (&v)[R], const float4 *__restrict__ tw, int m)
{
    static_assert(R == 2 || R == 4 || R == 8 || R == 16, "radix 2, 4, 8 or 16");
    const cptw w1 = cp_tw_load<DIR>(tw, m);
    v[1] = cp_rot(v[1], w1);
    if constexpr (R >= 4) {
        const cptw w2 = cp_tw_load<DIR>(tw, 2 * m), w3 = cp_tw_mul(w2, w1);
        v[2] = cp_rot(v[2], w2);
        v[3] = cp_rot(v[3], w3);
        if constexpr (R >= 8) {
            const cptw w4 = cp_tw_load<DIR>(tw, 4 * m);
            const cptw w5 = cp_tw_mul(w4, w1), w6 = cp_tw_mul(w4, w2), w7 = cp_tw_mul(w4, w3);
            v[4] = cp_rot(v[4], w4);
            v[5] = cp_rot(v[5], w5);
            v[6] = cp_rot(v[6], w6);
            v[7] = cp_rot(v[7], w7);
            if constexpr (R == 16) {
                const cptw w8 = cp_tw_load<DIR>(tw, 8 * m);
                v[8] = cp_rot(v[8], w8);
                v[9] = cp_rot(cp_rot(v[9], w8), w1);
                v[10] = cp_rot(cp_rot(v[10], w8), w2);
                v[11] = cp_rot(cp_rot(v[11], w8), w3);
                v[12] = cp_rot(cp_rot(v[12], w8), w4);
                v[13] = cp_rot(cp_rot(v[13], w8), w5);
                v[14] = cp_rot(cp_rot(v[14], w8), w6);
                v[15] = cp_rot(cp_rot(v[15], w8), w7);
            }
        }
    }
}

template <int DIR>
__device__ __forceinline__ void cp_dft4(cpair &a, cpair &b, cpair &c, cpair &d)
{
    const cpair s02 = cp_add(a, c), d02 = cp_sub(a, c), s13 = cp_add(b, d), t = cp_sub(b, d);
    a = cp_add(s02, s13);
    c = cp_sub(s02, s13);
    // d13 = t * (DIR i); b = d02 + d13, d = d02 - d13
    if (DIR < 0) {
        b = {padd(d02.re, t.im), psub(d02.im, t.re)};
        d = {psub(d02.re, t.im), padd(d02.im, t.re)};
    } else {
        b = {psub(d02.re, t.im), padd(d02.im, t.re)};
        d = {padd(d02.re, t.im), psub(d02.im, t.re)};
    }
}

// multiply by the compile-time twiddle exp(DIR 2 pi i e / 16)
template <int DIR, int E>
__device__ __forceinline__ cpair cp_w16(const cpair &a)
{
    constexpr float C1 = 0.92387953251128674f, S1 = 0.38268343236508977f, H = 0.70710678118654752f;
    constexpr int e = E & 15;
    if constexpr (e == 0) return a;
    else if constexpr (e == 4) return cp_mul_di<DIR>(a);
    else {
        float c, s;
        if constexpr (e == 1) { c = C1; s = S1; }
        else if constexpr (e == 2) { c = H; s = H; }
        else if constexpr (e == 3) { c = S1; s = C1; }
        else if constexpr (e == 6) { c = -H; s = H; }
        else if constexpr (e == 9) { c = -C1; s = -S1; }
        else { static_assert(e == 1, "unused twiddle"); }
        s = DIR < 0 ? -s : s;
        return cp_rot(a, pp(c), pp(s), pp(-s));
    }
}

template <int R, int DIR>
__device__ __forceinline__ void cp_dft(cpair (&v)[R])
{
    if constexpr (R == 2) {
        const cpair a = v[0];
        v[0] = cp_add(a, v[1]);
        v[1] = cp_sub(a, v[1]);
    } else if constexpr (R == 4) {
        cp_dft4<DIR>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 8) {
        cp_dft4<DIR>(v[0], v[2], v[4], v[6]);
        cp_dft4<DIR>(v[1], v[3], v[5], v[7]);
        v[3] = cp_w16<DIR, 2>(v[3]);
        v[5] = cp_w16<DIR, 4>(v[5]);
        v[7] = cp_w16<DIR, 6>(v[7]);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            const cpair a = v[2 * k1], b = v[2 * k1 + 1];
            v[2 * k1] = cp_add(a, b);
            v[2 * k1 + 1] = cp_sub(a, b);
        }
    } else {
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) cp_dft4<DIR>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
        v[5] = cp_w16<DIR, 1>(v[5]);
        v[9] = cp_w16<DIR, 2>(v[9]);
        v[13] = cp_w16<DIR, 3>(v[13]);
        v[6] = cp_w16<DIR, 2>(v[6]);
        v[10] = cp_w16<DIR, 4>(v[10]);
        v[14] = cp_w16<DIR, 6>(v[14]);
        v[7] = cp_w16<DIR, 3>(v[7]);
        v[11] = cp_w16<DIR, 6>(v[11]);
        v[15] = cp_w16<DIR, 9>(v[15]);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) cp_dft4<DIR>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    }
}

// radix-16 DFT with inputs only at r in [4, 12) (the rest zero)
template <int DIR>
__device__ __forceinline__ void cp_dft16_in_mid(cpair (&v)[16])
{
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) {
        const cpair a = v[n2 + 4], b = v[n2 + 8];
        const cpair ia = cp_mul_di<DIR>(a);
        const cpair s = cp_add(b, ia);
        v[n2] = cp_add(a, b);
        v[n2 + 4] = cp_sub(ia, b);
        v[n2 + 8] = cp_sub(b, a);
        v[n2 + 12] = {pneg(s.re), pneg(s.im)};
    }
    v[5] = cp_w16<DIR, 1>(v[5]);
    v[9] = cp_w16<DIR, 2>(v[9]);
    v[13] = cp_w16<DIR, 3>(v[13]);
    v[6] = cp_w16<DIR, 2>(v[6]);
    v[10] = cp_w16<DIR, 4>(v[10]);
    v[14] = cp_w16<DIR, 6>(v[14]);
    v[7] = cp_w16<DIR, 3>(v[7]);
    v[11] = cp_w16<DIR, 6>(v[11]);
    v[15] = cp_w16<DIR, 9>(v[15]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) cp_dft4<DIR>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
}

// radix-16 DFT forming only the outputs k in [4, 12), left at v[outpos<16>(k)]
template <int DIR>
__device__ __forceinline__ void cp_dft16_out_mid(cpair (&v)[16])
{
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) cp_dft4<DIR>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
    v[5] = cp_w16<DIR, 1>(v[5]);
    v[9] = cp_w16<DIR, 2>(v[9]);
    v[13] = cp_w16<DIR, 3>(v[13]);
    v[6] = cp_w16<DIR, 2>(v[6]);
    v[10] = cp_w16<DIR, 4>(v[10]);
    v[14] = cp_w16<DIR, 6>(v[14]);
    v[7] = cp_w16<DIR, 3>(v[7]);
    v[11] = cp_w16<DIR, 6>(v[11]);
    v[15] = cp_w16<DIR, 9>(v[15]);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        const cpair a = v[4 * k1], b = v[4 * k1 + 1], c = v[4 * k1 + 2], d = v[4 * k1 + 3];
        const cpair s02 = cp_add(a, c), d02 = cp_sub(a, c), s13 = cp_add(b, d), t = cp_sub(b, d);
        v[4 * k1 + 2] = cp_sub(s02, s13);
        v[4 * k1 + 1] = DIR < 0 ? cpair{padd(d02.re, t.im), psub(d02.im, t.re)}
                                : cpair{psub(d02.re, t.im), padd(d02.im, t.re)};
    }
}

// last-stage twiddles (Ns = N/16): v[r] *= w^(r j), w = exp(DIR 2 pi i / N)
template <int N, int DIR>
__device__ __forceinline__ void cp_last_twiddle(cpair (&v)[16], int j, const float4 *__restrict__ tw)
{
    constexpr int STEP = FFT_MAX / N;
    cp_twiddle_powers<16, DIR>(v, tw, j * STEP);
}

template <int N, int NSP, bool COLS>
__device__ __forceinline__ int cp_saddr(int q, int i, int ss)
{
    if constexpr (COLS) return pidx(i) * NSP + q;
    else return q * ss + pidx(i);
}

// One Stockham stage over NSP sequence pairs (radix R, NS = radices applied).
template <int N, int R, int NS, int DIR, int NT, bool COLS, int NSP>
__device__ __forceinline__ void cp_fft_stage(float4 *s, int ss, const float4 *__restrict__ tw, int tid)
{
    constexpr int B = N / R;
    constexpr int BT = NSP * B;
    static_assert(BT % NT == 0 || NT % BT == 0, "threads and butterflies must divide one another");
    constexpr int BPT = BT >= NT ? BT / NT : 1;
    constexpr bool GUARD = BT < NT;
    cpair v[BPT][R];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT;
        if (GUARD && b >= BT) continue;
        const int q = COLS ? (b % NSP) : (b / B);
        const int j = COLS ? (b / NSP) : (b % B);
        const int a0 = cp_saddr<N, NSP, COLS>(q, j, ss);
        constexpr int LS = pstride<B>() * (COLS ? NSP : 1);
#pragma unroll
        for (int r = 0; r < R; ++r) v[t][r] = cp_ld(s + a0 + r * LS);
        if constexpr (NS > 1) {
            const int k = j & (NS - 1);
            constexpr int STEP = FFT_MAX / (NS * R);
            cp_twiddle_powers<R, DIR>(v[t], tw, k * STEP);
        }
        cp_dft<R, DIR>(v[t]);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT;
        if (GUARD && b >= BT) continue;
        const int q = COLS ? (b % NSP) : (b / B);
        const int j = COLS ? (b / NSP) : (b % B);
        const int k = j & (NS - 1);
        const int base = (j / NS) * NS * R + k;
        const int a0 = cp_saddr<N, NSP, COLS>(q, base, ss);
        static_assert(NS % 16 == 0, "middle stages start at NS = 16");
        constexpr int SS = pstride<NS>() * (COLS ? NSP : 1);
#pragma unroll
        for (int r = 0; r < R; ++r) cp_st(s + a0 + r * SS, v[t][outpos<R>(r)]);
    }
    __syncthreads();
}

// Middle stages from Ns = 16 up to Ns = N/16 (none when N == 256).
template <int N, int NS, int DIR, int NT, bool COLS, int NSP>
struct CpMidRun {
    static __device__ __forceinline__ void run(float4 *s, int ss, const float4 *__restrict__ tw, int tid)
    {
        constexpr int REM = N / 16 / NS;
        constexpr int R = REM >= 16 ? 16 : REM;
        cp_fft_stage<N, R, NS, DIR, NT, COLS, NSP>(s, ss, tw, tid);
        CpMidRun<N, NS * R, DIR, NT, COLS, NSP>::run(s, ss, tw, tid);
    }
};
template <int N, int DIR, int NT, bool COLS, int NSP>
struct CpMidRun<N, N / 16, DIR, NT, COLS, NSP> {
    static __device__ __forceinline__ void run(float4 *, int, const float4 *__restrict__, int) {}
};

template <int N, int DIR, int NT, bool COLS, int NSP>
__device__ __forceinline__ void cp_mid_stages(float4 *s, int ss, const float4 *__restrict__ tw, int tid)
{
    if constexpr (N > 256) CpMidRun<N, 16, DIR, NT, COLS, NSP>::run(s, ss, tw, tid);
}

// largest butterflies-per-thread over the middle stages (register budget check)
template <int N, int NT, int NSP>
__host__ __device__ constexpr int cp_mid_bpt()
{
    int m = 0;
    for (int ns = 16; ns < N / 16;) {
        const int rem = N / 16 / ns, r = rem >= 16 ? 16 : rem;
        const int bt = NSP * (N / r), bpt = bt >= NT ? bt / NT : 1;
        if (bpt * r > m) m = bpt * r;
        ns *= r;
    }
    return m;
}

} // namespace olg
