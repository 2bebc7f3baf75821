// fftmr.cuh -- mixed-radix in-shared-memory Stockham FFT with a run-time
// stage plan (sm_103a).
//
// Lengths N = 2^a 3^b 5^c that are not powers of two run through here: the
// reference's default field 3840 x 2160 pads to 7680 x 4320.  The plan is a
// list of radices from {16, 8, 4, 2, 5, 3} (powers of two first); every
// stage is the same in-place Stockham step as fft.cuh (read all R inputs
// into registers, barrier, write the R outputs), with twiddles
// exp(-2 pi i m / N) from a per-length table.  Layouts as fft.cuh: rows
// (q * ss + pidx(i)) or column tiles (pidx(i) * nseq + q).
#pragma once
#include "fft.cuh"
#include "fft2.cuh"
#include "propdev.cuh"

namespace olg {

// X[k] = sum_n x[n] w^(n k), w = exp(DIR 2 pi i / 3): natural output order
template <int DIR>
__device__ __forceinline__ void dft3(float2 (&v)[3])
{
    constexpr float S3 = 0.86602540378443865f; // sin(2 pi / 3)
    const float2 s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    const float2 a = v[0];
    const float2 t = make_float2(a.x - 0.5f * s.x, a.y - 0.5f * s.y);
    // (DIR i) sin(2 pi / 3) d
    const float2 id = DIR < 0 ? make_float2(S3 * d.y, -S3 * d.x) : make_float2(-S3 * d.y, S3 * d.x);
    v[0] = cadd(a, s);
    v[1] = cadd(t, id);
    v[2] = csub(t, id);
}

template <int DIR>
__device__ __forceinline__ void dft5(float2 (&v)[5])
{
    constexpr float C1 = 0.30901699437494742f, C2 = -0.80901699437494742f; // cos(2 pi / 5), cos(4 pi / 5)
    constexpr float S1 = 0.95105651629515357f, S2 = 0.58778525229247313f;  // sin(2 pi / 5), sin(4 pi / 5)
    const float2 a = v[0];
    const float2 s1 = cadd(v[1], v[4]), d1 = csub(v[1], v[4]), s2 = cadd(v[2], v[3]), d2 = csub(v[2], v[3]);
    const float2 r1 = make_float2(a.x + C1 * s1.x + C2 * s2.x, a.y + C1 * s1.y + C2 * s2.y);
    const float2 r2 = make_float2(a.x + C2 * s1.x + C1 * s2.x, a.y + C2 * s1.y + C1 * s2.y);
    const float2 q1 = make_float2(S1 * d1.x + S2 * d2.x, S1 * d1.y + S2 * d2.y);
    const float2 q2 = make_float2(S2 * d1.x - S1 * d2.x, S2 * d1.y - S1 * d2.y);
    // (DIR i) q
    const float2 i1 = DIR < 0 ? make_float2(q1.y, -q1.x) : make_float2(-q1.y, q1.x);
    const float2 i2 = DIR < 0 ? make_float2(q2.y, -q2.x) : make_float2(-q2.y, q2.x);
    v[0] = cadd(a, cadd(s1, s2));
    v[1] = cadd(r1, i1);
    v[4] = csub(r1, i1);
    v[2] = cadd(r2, i2);
    v[3] = csub(r2, i2);
}

// exp(DIR 2 pi i p / n) from (cos, sin) of 2 pi p / n
template <int DIR>
__device__ __forceinline__ float2 mr_w(float c, float s)
{
    return make_float2(c, DIR < 0 ? -s : s);
}

// Composite radices of the compile-time plans, Cooley-Tukey over a radix-3 or
// radix-2 outer split with the inner DFTs in registers; natural output order.
// DFT6: n = 2m + e, X[k] = A[k mod 3] + w6^k B[k mod 3] (A, B the DFT3s of the
// even and odd samples; w6^(k+3) = -w6^k).
template <int DIR>
__device__ __forceinline__ void dft6(float2 (&v)[6])
{
    float2 a[3] = {v[0], v[2], v[4]}, b[3] = {v[1], v[3], v[5]};
    dft3<DIR>(a);
    dft3<DIR>(b);
    const float2 b1 = cmul(b[1], mr_w<DIR>(0.5f, 0.86602540378443865f));
    const float2 b2 = cmul(b[2], mr_w<DIR>(-0.5f, 0.86602540378443865f));
    v[0] = cadd(a[0], b[0]);
    v[3] = csub(a[0], b[0]);
    v[1] = cadd(a[1], b1);
    v[4] = csub(a[1], b1);
    v[2] = cadd(a[2], b2);
    v[5] = csub(a[2], b2);
}

// DFT9: n = 3m + e, X[k + 3j] = DFT3 over e of w9^(e k) Y_e[k], Y_e the DFT3
// of samples e, e + 3, e + 6.
template <int DIR>
__device__ __forceinline__ void dft9(float2 (&v)[9])
{
    float2 y[3][3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        float2 t[3] = {v[e], v[e + 3], v[e + 6]};
        dft3<DIR>(t);
        y[e][0] = t[0];
        y[e][1] = t[1];
        y[e][2] = t[2];
    }
    const float2 w1 = mr_w<DIR>(0.76604444311897804f, 0.64278760968653933f);  // w9
    const float2 w2 = mr_w<DIR>(0.17364817766693035f, 0.98480775301220806f);  // w9^2
    const float2 w4 = mr_w<DIR>(-0.93969262078590838f, 0.34202014332566873f); // w9^4
    y[1][1] = cmul(y[1][1], w1);
    y[1][2] = cmul(y[1][2], w2);
    y[2][1] = cmul(y[2][1], w2);
    y[2][2] = cmul(y[2][2], w4);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float2 z[3] = {y[0][k], y[1][k], y[2][k]};
        dft3<DIR>(z);
        v[k] = z[0];
        v[k + 3] = z[1];
        v[k + 6] = z[2];
    }
}

// DFT15: n = 3m + e, X[k + 5j] = DFT3 over e of w15^(e k) Y_e[k], Y_e the DFT5
// of samples e, e + 3, ..., e + 12.
template <int DIR>
__device__ __forceinline__ void dft15(float2 (&v)[15])
{
    float2 y[3][5];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        float2 t[5] = {v[e], v[e + 3], v[e + 6], v[e + 9], v[e + 12]};
        dft5<DIR>(t);
#pragma unroll
        for (int k = 0; k < 5; ++k) y[e][k] = t[k];
    }
    y[1][1] = cmul(y[1][1], mr_w<DIR>(0.91354545764260087f, 0.40673664307580021f));  // w15
    y[1][2] = cmul(y[1][2], mr_w<DIR>(0.66913060635885824f, 0.74314482547739424f));  // w15^2
    y[1][3] = cmul(y[1][3], mr_w<DIR>(0.30901699437494742f, 0.95105651629515357f));  // w15^3
    y[1][4] = cmul(y[1][4], mr_w<DIR>(-0.10452846326765347f, 0.99452189536827329f)); // w15^4
    y[2][1] = cmul(y[2][1], mr_w<DIR>(0.66913060635885824f, 0.74314482547739424f));  // w15^2
    y[2][2] = cmul(y[2][2], mr_w<DIR>(-0.10452846326765347f, 0.99452189536827329f)); // w15^4
    y[2][3] = cmul(y[2][3], mr_w<DIR>(-0.80901699437494742f, 0.58778525229247313f)); // w15^6
    y[2][4] = cmul(y[2][4], mr_w<DIR>(-0.97814760073380569f, -0.20791169081775934f)); // w15^8
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        float2 z[3] = {y[0][k], y[1][k], y[2][k]};
        dft3<DIR>(z);
        v[k] = z[0];
        v[k + 5] = z[1];
        v[k + 10] = z[2];
    }
}

template <int R, int DIR>
__device__ __forceinline__ void mr_dft(float2 (&v)[R])
{
    if constexpr (R == 3) dft3<DIR>(v);
    else if constexpr (R == 5) dft5<DIR>(v);
    else if constexpr (R == 6) dft6<DIR>(v);
    else if constexpr (R == 9) dft9<DIR>(v);
    else if constexpr (R == 15) dft15<DIR>(v);
    else dft<R, DIR>(v);
}

// twiddle m of the per-length table (forward), conjugated for DIR > 0
template <int DIR>
__device__ __forceinline__ float2 mr_twid(const float2 *__restrict__ tw, int m)
{
    const float2 w = __ldg(tw + m);
    return DIR < 0 ? w : make_float2(w.x, -w.y);
}

// complex values a thread holds in one stage; a radix-R stage covers at most
// NT * (MR_VALS / R) butterflies, and the host sizes nseq (mr_nseq) so that
// every stage of the plan stays within that.
constexpr int MR_VALS = 16;

// One radix-R stage over nseq sequences of length N (NS = radices already
// applied).
template <int R, int DIR, int NT, bool COLS>
__device__ __forceinline__ void mr_stage(float2 *s, int ss, int nseq, int N, int NS, const float2 *__restrict__ tw,
                                         int tid)
{
    constexpr int BMAX = MR_VALS / R;
    const int B = N / R, BT = nseq * B, L = NS * R, step = N / L;
    float2 v[BMAX][R];
#pragma unroll
    for (int t = 0; t < BMAX; ++t) {
        const int b = tid + t * NT;
        if (b >= BT) continue;
        const int q = COLS ? b % nseq : b / B;
        const int j = COLS ? b / nseq : b % B;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = j + r * B;
            v[t][r] = s[COLS ? pidx(i) * nseq + q : q * ss + pidx(i)];
        }
        if (NS > 1) {
            const int k = j % NS;
#pragma unroll
            for (int r = 1; r < R; ++r) v[t][r] = cmul(v[t][r], mr_twid<DIR>(tw, r * k * step));
        }
        mr_dft<R, DIR>(v[t]);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < BMAX; ++t) {
        const int b = tid + t * NT;
        if (b >= BT) continue;
        const int q = COLS ? b % nseq : b / B;
        const int j = COLS ? b / nseq : b % B;
        const int k = j % NS, base = (j / NS) * L + k;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = base + r * NS;
            s[COLS ? pidx(i) * nseq + q : q * ss + pidx(i)] = v[t][outpos<R>(r)];
        }
    }
    __syncthreads();
}

// The whole transform of nseq sequences in place (unnormalised); all NT
// threads of the CTA call it after a barrier that follows the loads.
template <int DIR, int NT, bool COLS>
__device__ __forceinline__ void mr_fft(float2 *s, int ss, int nseq, const MrPlan &pl, const float2 *__restrict__ tw,
                                       int tid)
{
    int NS = 1;
    for (int i = 0; i < pl.nst; ++i) {
        const int R = (int)((pl.radices >> (5 * i)) & 31);
        switch (R) {
        case 16: mr_stage<16, DIR, NT, COLS>(s, ss, nseq, pl.n, NS, tw, tid); break;
        case 8: mr_stage<8, DIR, NT, COLS>(s, ss, nseq, pl.n, NS, tw, tid); break;
        case 4: mr_stage<4, DIR, NT, COLS>(s, ss, nseq, pl.n, NS, tw, tid); break;
        case 2: mr_stage<2, DIR, NT, COLS>(s, ss, nseq, pl.n, NS, tw, tid); break;
        case 5: mr_stage<5, DIR, NT, COLS>(s, ss, nseq, pl.n, NS, tw, tid); break;
        default: mr_stage<3, DIR, NT, COLS>(s, ss, nseq, pl.n, NS, tw, tid); break;
        }
        NS *= R;
    }
}

// ------------------------------------------------- compile-time stage plans
// The same Stockham transform for a few lengths with the plan, the sequence
// count and the thread count known at compile time: those of the reference's
// default field (3840 x 2160, padded 7680 x 4320) and of 1920 x 1080,
// 2560 x 1440 and 1280 x 720 fields.  The index arithmetic (divisions by B,
// NS and the sequence count) then folds into multiplications and shifts and
// each thread's values stay in registers; the plans use the composite radices
// 6, 9 and 15 as well, and radix-2^k stages form their twiddles as powers.
// Results agree with the run-time plan's to float rounding, not bit for bit.
template <int... Rs>
struct MrRadices {};
// `full`: the whole plan (the inverse transforms run it in shared memory),
// radix 16 first and the composite radices 6, 9 and 15 in place of pairs of
// 2, 3 and 5, so that 7680 takes four stages and 4320 four instead of six.
// The lengths are those of 3840 x 2160, 1920 x 1080, 2560 x 1440 and
// 1280 x 720 fields.
// `fwd`: the plan after its leading radix 16, which the forward transforms
// apply zero-pruned, straight from global memory.  Listed for the lengths it
// serves; every stage keeps each thread within 16 values.
template <int N>
struct MrFixedPlan {
    static constexpr bool ok = false;
};
template <> struct MrFixedPlan<7680> {
    static constexpr bool ok = true;
    using full = MrRadices<16, 16, 15, 2>;
    using fwd = MrRadices<16, 15, 2>;
};
template <> struct MrFixedPlan<4320> {
    static constexpr bool ok = true;
    using full = MrRadices<16, 6, 5, 9>;
    using fwd = MrRadices<6, 5, 9>;
};
template <> struct MrFixedPlan<3840> {
    static constexpr bool ok = true;
    using full = MrRadices<16, 16, 15>;
    using fwd = MrRadices<16, 15>;
};
template <> struct MrFixedPlan<5120> {
    static constexpr bool ok = true;
    using full = MrRadices<16, 16, 4, 5>;
    using fwd = MrRadices<16, 4, 5>;
};
template <> struct MrFixedPlan<2880> {
    static constexpr bool ok = true;
    using full = MrRadices<16, 4, 5, 9>;
    using fwd = MrRadices<4, 5, 9>;
};
template <> struct MrFixedPlan<2560> {
    static constexpr bool ok = true;
    using full = MrRadices<16, 16, 2, 5>;
    using fwd = MrRadices<16, 2, 5>;
};
template <> struct MrFixedPlan<1440> {
    static constexpr bool ok = true;
    using full = MrRadices<16, 6, 15>;
    using fwd = MrRadices<6, 15>;
};
template <> struct MrFixedPlan<2160> {
    static constexpr bool ok = true;
    using full = MrRadices<16, 15, 9>;
    using fwd = MrRadices<15, 9>;
};

// One in-place Stockham stage (as mr_stage) with compile-time sizes.  TFE:
// the stage is the forward transform's last and multiplies each output, a
// final frequency ky, by the transfer function of its column as it stores.
template <int N, int R, int NS, int DIR, int NT, bool COLS, int NSEQ, bool TFE>
__device__ __forceinline__ void mrc_stage(float2 *s, int ss, const float2 *__restrict__ tw, int tid,
                                          const PropParams *P, int c0)
{
    constexpr int B = N / R, BT = NSEQ * B, L = NS * R, step = N / L;
    constexpr int BPT = (BT + NT - 1) / NT;
    float2 v[BPT][R];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT;
        if (BT % NT != 0 && b >= BT) continue;
        const int q = COLS ? b % NSEQ : b / B;
        const int j = COLS ? b / NSEQ : b % B;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = j + r * B;
            v[t][r] = s[COLS ? pidx(i) * NSEQ + q : q * ss + pidx(i)];
        }
        if constexpr (NS > 1) {
            const int k = j % NS;
            if constexpr (R == 2 || R == 4 || R == 8 || R == 16) {
                twiddle_powers<R, DIR>(v[t], tw, k * step); // w^r from log2(R) table loads
            } else {
#pragma unroll
                for (int r = 1; r < R; ++r) v[t][r] = cmul(v[t][r], mr_twid<DIR>(tw, r * k * step));
            }
        }
        mr_dft<R, DIR>(v[t]);
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT;
        if (BT % NT != 0 && b >= BT) continue;
        const int q = COLS ? b % NSEQ : b / B;
        const int j = COLS ? b / NSEQ : b % B;
        const int k = j % NS, base = (j / NS) * L + k;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = base + r * NS;
            float2 x = v[t][outpos<R>(r)];
            if constexpr (TFE) {
                const int kx = c0 + q;
                if (kx < P->NX) x = cmul(x, tf_at(*P, i, kx, N));
            }
            s[COLS ? pidx(i) * NSEQ + q : q * ss + pidx(i)] = x;
        }
    }
    __syncthreads();
}

template <int N, int NS, int DIR, int NT, bool COLS, int NSEQ, bool TFE, int... Rs>
struct MrcRun {
    static __device__ __forceinline__ void run(float2 *, int, const float2 *__restrict__, int, const PropParams *,
                                               int)
    {
    }
};
template <int N, int NS, int DIR, int NT, bool COLS, int NSEQ, bool TFE, int R, int... Rest>
struct MrcRun<N, NS, DIR, NT, COLS, NSEQ, TFE, R, Rest...> {
    static __device__ __forceinline__ void run(float2 *s, int ss, const float2 *__restrict__ tw, int tid,
                                               const PropParams *P, int c0)
    {
        mrc_stage<N, R, NS, DIR, NT, COLS, NSEQ, TFE && sizeof...(Rest) == 0>(s, ss, tw, tid, P, c0);
        MrcRun<N, NS * R, DIR, NT, COLS, NSEQ, TFE, Rest...>::run(s, ss, tw, tid, P, c0);
    }
};
// The same stage out of place, from `src` to `dst` (a second shared buffer):
// each butterfly is read, transformed and written at once, and one barrier
// ends the stage instead of two.
template <int N, int R, int NS, int DIR, int NT, bool COLS, int NSEQ, bool TFE>
__device__ __forceinline__ void mrc_stage_pp(const float2 *src, float2 *dst, int ss, const float2 *__restrict__ tw,
                                             int tid, const PropParams *P, int c0)
{
    constexpr int B = N / R, BT = NSEQ * B, L = NS * R, step = N / L;
    constexpr int BPT = (BT + NT - 1) / NT;
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT;
        if (BT % NT != 0 && b >= BT) continue;
        const int q = COLS ? b % NSEQ : b / B;
        const int j = COLS ? b / NSEQ : b % B;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = j + r * B;
            v[r] = src[COLS ? pidx(i) * NSEQ + q : q * ss + pidx(i)];
        }
        const int k = j % NS;
        if constexpr (NS > 1) {
            if constexpr (R == 2 || R == 4 || R == 8 || R == 16) {
                twiddle_powers<R, DIR>(v, tw, k * step);
            } else {
#pragma unroll
                for (int r = 1; r < R; ++r) v[r] = cmul(v[r], mr_twid<DIR>(tw, r * k * step));
            }
        }
        mr_dft<R, DIR>(v);
        const int base = (j / NS) * L + k;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int i = base + r * NS;
            float2 x = v[outpos<R>(r)];
            if constexpr (TFE) {
                const int kx = c0 + q;
                if (kx < P->NX) x = cmul(x, tf_at(*P, i, kx, N));
            }
            dst[COLS ? pidx(i) * NSEQ + q : q * ss + pidx(i)] = x;
        }
    }
    __syncthreads();
}

template <int N, int NS, int DIR, int NT, bool COLS, int NSEQ, bool TFE, bool SRC_B, int... Rs>
struct MrcRunPP {
    static __device__ __forceinline__ void run(float2 *, float2 *, int, const float2 *__restrict__, int,
                                               const PropParams *, int)
    {
    }
};
template <int N, int NS, int DIR, int NT, bool COLS, int NSEQ, bool TFE, bool SRC_B, int R, int... Rest>
struct MrcRunPP<N, NS, DIR, NT, COLS, NSEQ, TFE, SRC_B, R, Rest...> {
    static __device__ __forceinline__ void run(float2 *a, float2 *b, int ss, const float2 *__restrict__ tw, int tid,
                                               const PropParams *P, int c0)
    {
        mrc_stage_pp<N, R, NS, DIR, NT, COLS, NSEQ, TFE && sizeof...(Rest) == 0>(SRC_B ? b : a, SRC_B ? a : b, ss, tw,
                                                                                 tid, P, c0);
        MrcRunPP<N, NS * R, DIR, NT, COLS, NSEQ, TFE, !SRC_B, Rest...>::run(a, b, ss, tw, tid, P, c0);
    }
};
// Stages Rs... from NS0 on, alternating between buffers a and b, starting
// from a (SRC_B false) or b; the result is in b after an odd count.
template <int N, int NS0, int DIR, int NT, bool COLS, int NSEQ, bool TFE, bool SRC_B, int... Rs>
__device__ __forceinline__ void mrc_stages_pp(MrRadices<Rs...>, float2 *a, float2 *b, int ss,
                                              const float2 *__restrict__ tw, int tid, const PropParams *P = nullptr,
                                              int c0 = 0)
{
    MrcRunPP<N, NS0, DIR, NT, COLS, NSEQ, TFE, SRC_B, Rs...>::run(a, b, ss, tw, tid, P, c0);
}
template <int... Rs>
__host__ __device__ constexpr int mr_count(MrRadices<Rs...>) { return (int)sizeof...(Rs); }

// Stages Rs... from NS0 on (all NT threads, after a barrier).
template <int N, int NS0, int DIR, int NT, bool COLS, int NSEQ, bool TFE, int... Rs>
__device__ __forceinline__ void mrc_stages(MrRadices<Rs...>, float2 *s, int ss, const float2 *__restrict__ tw,
                                           int tid, const PropParams *P = nullptr, int c0 = 0)
{
    MrcRun<N, NS0, DIR, NT, COLS, NSEQ, TFE, Rs...>::run(s, ss, tw, tid, P, c0);
}

} // namespace olg
