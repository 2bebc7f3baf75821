// fft.cuh -- in-shared-memory Stockham FFT building blocks (sm_103a).
//
// A CTA transforms NSEQ sequences of length N (a power of two, 64..8192) that
// live in shared memory.  Two layouts:
//   rows (COLS = false): element i of sequence q at s[q * SS + pidx(i)],
//   cols (COLS = true) : element i of sequence q at s[pidx(i) * NSEQ + q]
//                        (q = column of a tile of NSEQ adjacent columns).
// pidx(i) = i + i/16 inserts one pad slot per 16 elements, which makes every
// Stockham stage's strided writes land in distinct banks for both layouts.
//
// Stages run in place: every thread reads the R inputs of its butterflies
// into registers, the CTA synchronises, then writes the R outputs.  Radix 16
// stages first, one radix 2/4/8 stage last.  Twiddles come from a table
// exp(-2 pi i m / FFT_MAX) in global memory (L1-resident).
#pragma once
#include "common.cuh"

namespace olg {

constexpr int FFT_MAX = 8192;

__host__ __device__ constexpr int padded_len(int n) { return n + (n >> 4); }
__device__ __forceinline__ int pidx(int i) { return i + (i >> 4); }
// pidx is affine along the index sets the transforms walk, so addresses can be
// formed as one base plus compile-time offsets:
//   pidx(j + r M) = pidx(j) + r pstride<M>()   (M a multiple of 16)
//   pidx(16 j + k) = 17 j + k                  (0 <= k < 16)
template <int M>
__host__ __device__ constexpr int pstride()
{
    static_assert(M % 16 == 0 && M > 0, "pidx is affine only on multiples of 16");
    return M + M / 16;
}

template <int DIR>
__device__ __forceinline__ float2 twid(const float2 *__restrict__ table, int m)
{
    const float2 w = __ldg(table + m);
    return DIR < 0 ? w : make_float2(w.x, -w.y);
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// a * (DIR * i)
template <int DIR>
__device__ __forceinline__ float2 mul_di(float2 a)
{
    return DIR < 0 ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
}

// v[r] *= w^r for r = 1 .. R-1 with w = table[m] (conjugated for DIR > 0).
// Only w, w^2, w^4 and w^8 are read from the table; the other powers are
// products of those, at most three roundings deep (~2e-7 relative).  Four
// loads in flight instead of R - 1 keep ~20 fewer registers live across the
// butterfly.  Needs (R - 1) m < FFT_MAX, as the direct lookups do.
template <int R, int DIR>
__device__ __forceinline__ void twiddle_powers(float2 (&v)[R], const float2 *__restrict__ table, int m)
{
    static_assert(R == 2 || R == 4 || R == 8 || R == 16, "radix 2, 4, 8 or 16");
    const float2 w1 = twid<DIR>(table, m);
    v[1] = cmul(v[1], w1);
    if constexpr (R >= 4) {
        const float2 w2 = twid<DIR>(table, 2 * m), w3 = cmul(w2, w1);
        v[2] = cmul(v[2], w2);
        v[3] = cmul(v[3], w3);
        if constexpr (R >= 8) {
            const float2 w4 = twid<DIR>(table, 4 * m);
            const float2 w5 = cmul(w4, w1), w6 = cmul(w4, w2), w7 = cmul(w4, w3);
            v[4] = cmul(v[4], w4);
            v[5] = cmul(v[5], w5);
            v[6] = cmul(v[6], w6);
            v[7] = cmul(v[7], w7);
            if constexpr (R == 16) {
                const float2 w8 = twid<DIR>(table, 8 * m);
                v[8] = cmul(v[8], w8);
                v[9] = cmul(cmul(v[9], w8), w1);
                v[10] = cmul(cmul(v[10], w8), w2);
                v[11] = cmul(cmul(v[11], w8), w3);
                v[12] = cmul(cmul(v[12], w8), w4);
                v[13] = cmul(cmul(v[13], w8), w5);
                v[14] = cmul(cmul(v[14], w8), w6);
                v[15] = cmul(cmul(v[15], w8), w7);
            }
        }
    }
}

template <int DIR>
__device__ __forceinline__ void dft4(float2 &a, float2 &b, float2 &c, float2 &d)
{
    const float2 s02 = cadd(a, c), d02 = csub(a, c), s13 = cadd(b, d), d13 = mul_di<DIR>(csub(b, d));
    a = cadd(s02, s13);
    b = cadd(d02, d13);
    c = csub(s02, s13);
    d = csub(d02, d13);
}

// multiply by a compile-time twiddle exp(DIR * 2 pi i e / 16)
template <int DIR, int E>
__device__ __forceinline__ float2 w16(float2 a)
{
    constexpr float C1 = 0.92387953251128674f, S1 = 0.38268343236508977f, H = 0.70710678118654752f;
    constexpr int e = E & 15;
    if constexpr (e == 0) return a;
    float c, s;
    if constexpr (e == 1) { c = C1; s = S1; }
    else if constexpr (e == 2) { c = H; s = H; }
    else if constexpr (e == 3) { c = S1; s = C1; }
    else if constexpr (e == 4) { c = 0.f; s = 1.f; }
    else if constexpr (e == 6) { c = -H; s = H; }
    else if constexpr (e == 9) { c = -C1; s = -S1; }
    else { static_assert(e == 1, "unused twiddle"); }
    s = DIR < 0 ? -s : s;
    return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
}

// Radix-R DFT in registers.  Output X[k] is left at v[outpos<R>(k)].
template <int R>
__device__ __host__ constexpr int outpos(int k)
{
    return R == 16 ? 4 * (k & 3) + (k >> 2) : R == 8 ? 2 * (k & 3) + (k >> 2) : k;
}

template <int R, int DIR>
__device__ __forceinline__ void dft(float2 (&v)[R])
{
    if constexpr (R == 2) {
        const float2 a = v[0];
        v[0] = cadd(a, v[1]);
        v[1] = csub(a, v[1]);
    } else if constexpr (R == 4) {
        dft4<DIR>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 8) {
        // n = n2 + 2 n1, k = k1 + 4 k2
        dft4<DIR>(v[0], v[2], v[4], v[6]);
        dft4<DIR>(v[1], v[3], v[5], v[7]);
        v[3] = w16<DIR, 2>(v[3]);
        v[5] = w16<DIR, 4>(v[5]);
        v[7] = w16<DIR, 6>(v[7]);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) {
            const float2 a = v[2 * k1], b = v[2 * k1 + 1];
            v[2 * k1] = cadd(a, b);
            v[2 * k1 + 1] = csub(a, b);
        }
    } else {
        // R == 16: n = n2 + 4 n1, k = k1 + 4 k2
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) dft4<DIR>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
        v[5] = w16<DIR, 1>(v[5]);
        v[9] = w16<DIR, 2>(v[9]);
        v[13] = w16<DIR, 3>(v[13]);
        v[6] = w16<DIR, 2>(v[6]);
        v[10] = w16<DIR, 4>(v[10]);
        v[14] = w16<DIR, 6>(v[14]);
        v[7] = w16<DIR, 3>(v[7]);
        v[11] = w16<DIR, 6>(v[11]);
        v[15] = w16<DIR, 9>(v[15]);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) dft4<DIR>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    }
}

template <int N, int NSEQ, bool COLS>
__device__ __forceinline__ int saddr(int q, int i, int ss)
{
    if constexpr (COLS) return pidx(i) * NSEQ + q;
    else return q * ss + pidx(i);
}

// One Stockham stage: radix R, NS = product of the radices already applied.
// NT threads share the NSEQ * N / R butterflies; when NT exceeds them the
// extra threads only take part in the barriers.
template <int N, int R, int NS, int DIR, int NT, bool COLS, int NSEQ>
__device__ __forceinline__ void fft_stage(float2 *s, int ss, const float2 *__restrict__ tw, int tid)
{
    constexpr int B = N / R;
    constexpr int BT = NSEQ * B;
    static_assert(BT % NT == 0 || NT % BT == 0, "threads and butterflies must divide one another");
    constexpr int BPT = BT >= NT ? BT / NT : 1;
    constexpr bool GUARD = BT < NT;
    float2 v[BPT][R];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT;
        if (GUARD && b >= BT) continue;
        const int q = COLS ? (b % NSEQ) : (b / B);
        const int j = COLS ? (b / NSEQ) : (b % B);
        if constexpr (B % 16 == 0) {
            const int a0 = saddr<N, NSEQ, COLS>(q, j, ss);
            constexpr int LS = pstride<B>() * (COLS ? NSEQ : 1);
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = s[a0 + r * LS];
        } else { // short transforms (N < 256)
#pragma unroll
            for (int r = 0; r < R; ++r) v[t][r] = s[saddr<N, NSEQ, COLS>(q, j + r * B, ss)];
        }
        if constexpr (NS > 1) {
            const int k = j & (NS - 1);
            constexpr int STEP = FFT_MAX / (NS * R);
            twiddle_powers<R, DIR>(v[t], tw, k * STEP);
        }
        dft<R, DIR>(v[t]);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT;
        if (GUARD && b >= BT) continue;
        const int q = COLS ? (b % NSEQ) : (b / B);
        const int j = COLS ? (b / NSEQ) : (b % B);
        const int k = j & (NS - 1);
        const int base = (j / NS) * NS * R + k;
        if constexpr (NS % 16 == 0 || (NS == 1 && R == 16)) {
            // NS == 1 with radix 16: base = 16 j, offsets r < 16 stay in one 16-block
            const int a0 = saddr<N, NSEQ, COLS>(q, base, ss);
            constexpr int SS = (NS == 1 ? 1 : pstride<(NS % 16 == 0 ? NS : 16)>()) * (COLS ? NSEQ : 1);
#pragma unroll
            for (int r = 0; r < R; ++r) s[a0 + r * SS] = v[t][outpos<R>(r)];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) s[saddr<N, NSEQ, COLS>(q, base + r * NS, ss)] = v[t][outpos<R>(r)];
        }
    }
    __syncthreads();
}

template <int N, int NS, int DIR, int NT, bool COLS, int NSEQ>
struct FFTRun {
    static __device__ __forceinline__ void run(float2 *s, int ss, const float2 *__restrict__ tw, int tid)
    {
        constexpr int REM = N / NS;
        constexpr int R = REM >= 16 ? 16 : REM;
        fft_stage<N, R, NS, DIR, NT, COLS, NSEQ>(s, ss, tw, tid);
        FFTRun<N, NS * R, DIR, NT, COLS, NSEQ>::run(s, ss, tw, tid);
    }
};
template <int N, int DIR, int NT, bool COLS, int NSEQ>
struct FFTRun<N, N, DIR, NT, COLS, NSEQ> {
    static __device__ __forceinline__ void run(float2 *, int, const float2 *__restrict__, int) {}
};

// Transform all NSEQ sequences in place.  DIR = -1 forward, +1 inverse
// (unnormalised).  Must be called by all NT threads of the CTA; the caller
// must __syncthreads() between filling `s` and this call.
template <int N, int DIR, int NT, bool COLS, int NSEQ>
__device__ __forceinline__ void smem_fft(float2 *s, int ss, const float2 *__restrict__ tw, int tid)
{
    FFTRun<N, 1, DIR, NT, COLS, NSEQ>::run(s, ss, tw, tid);
}

} // namespace olg
