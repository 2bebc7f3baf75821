// propmr.cu -- the three propagation passes and the chirp spectra for FFT
// lengths that are not powers of two (N = 2^a 3^b 5^c), with the mixed-radix
// FFT of fftmr.cuh.  Same dataflow as the power-of-two passes in prop.cu
// (zero padding, transfer function and crop folded into the passes,
// S = ny x NX scratch): pass 1 row FFTs of the ny stored rows, pass 2 column
// tiles (FFT, x T, inverse FFT, central rows), pass 3 inverse row FFTs with
// the crop and the pass-3 operations.  Rows and columns choose their path
// independently, so a power-of-two width with a mixed-radix height works.
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "fftmr.cuh"
#include "propmr.cuh"

namespace olg {

constexpr int MR_NT = 512;

__global__ void __launch_bounds__(MR_NT, 1) k_rows_fwd_mr(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    const MrPlan &pl = P.mrx;
    const int N = pl.n, nseq = P.mr_rows, SS = padded_len(N), tid = threadIdx.x;
    const int r0 = blockIdx.x * nseq, off = (N - P.nx) / 2;
    for (int e = tid; e < nseq * N; e += MR_NT) {
        const int q = e / N, i = e % N, h = r0 + q, w = i - off;
        float2 v = make_float2(0.f, 0.f);
        if (h < P.ny && w >= 0 && w < P.nx) v = load_in(P, h, w);
        sm[q * SS + pidx(i)] = v;
    }
    __syncthreads();
    mr_fft<-1, MR_NT, false>(sm, SS, nseq, pl, P.twx, tid);
    for (int e = tid; e < nseq * N; e += MR_NT) {
        const int q = e / N, i = e % N, h = r0 + q;
        if (h < P.ny) __stcg(P.S + (size_t)h * N + i, sm[q * SS + pidx(i)]);
    }
}

__global__ void __launch_bounds__(MR_NT, 1) k_cols_mr(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    const MrPlan &pl = P.mry;
    const int N = pl.n, C = P.mr_cols, NX = P.NX, tid = threadIdx.x;
    const int c0 = blockIdx.x * C, off = (N - P.ny) / 2;
    for (int e = tid; e < N * C; e += MR_NT) {
        const int i = e / C, c = e % C, kx = c0 + c, h = i - off;
        float2 v = make_float2(0.f, 0.f);
        if (kx < NX && h >= 0 && h < P.ny) v = __ldcg(P.S + (size_t)h * NX + kx);
        sm[pidx(i) * C + c] = v;
    }
    __syncthreads();
    mr_fft<-1, MR_NT, true>(sm, 0, C, pl, P.twy, tid);
    for (int e = tid; e < N * C; e += MR_NT) {
        const int ky = e / C, c = e % C, kx = c0 + c;
        if (kx < NX) {
            float2 &x = sm[pidx(ky) * C + c];
            x = cmul(x, tf_at(P, ky, kx, N));
        }
    }
    __syncthreads();
    mr_fft<+1, MR_NT, true>(sm, 0, C, pl, P.twy, tid);
    for (int e = tid; e < P.ny * C; e += MR_NT) {
        const int h = e / C, c = e % C, kx = c0 + c;
        if (kx < NX) __stcg(P.S + (size_t)h * NX + kx, sm[pidx(h + off) * C + c]);
    }
}

__global__ void __launch_bounds__(MR_NT, 1) k_rows_inv_mr(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    const MrPlan &pl = P.mrx;
    const int N = pl.n, nseq = P.mr_rows, SS = padded_len(N), tid = threadIdx.x;
    const int r0 = blockIdx.x * nseq, off = (N - P.nx) / 2;
    for (int e = tid; e < nseq * N; e += MR_NT) {
        const int q = e / N, i = e % N, h = r0 + q;
        sm[q * SS + pidx(i)] = h < P.ny ? __ldcg(P.S + (size_t)h * N + i) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    mr_fft<+1, MR_NT, false>(sm, SS, nseq, pl, P.twx, tid);
    float lsum = 0.f;
    for (int e = tid; e < nseq * P.nx; e += MR_NT) {
        const int q = e / P.nx, w = e % P.nx, h = r0 + q;
        if (h < P.ny) store_out(P, h, w, sm[q * SS + pidx(w + off)], lsum);
    }
    if (P.post_mode == OP_SEED) loss_reduce(lsum, P.loss, tid, MR_NT);
}

// The three passes again for the lengths with a compile-time plan (fftmr.cuh
// MrFixedPlan: 3840 x 2160, 2560 x 1440, 1920 x 1080 and 1280 x 720 fields),
// NSEQ rows or columns per CTA of NT threads.  As in the tuned
// power-of-two passes, the forward transforms start with a radix-16 stage
// that reads the stored half of the padded input straight from global memory
// (the padding is never formed), and the column pass multiplies by the
// transfer function as its last forward stage stores.  The inverse transforms
// run the whole plan in shared memory and store the central half: an inverse
// ending in a crop-pruned radix-16 stage written straight to global memory
// (as in the power-of-two passes) measured slower here, ASM 3840 x 2160 in
// 0.77 ms against 0.70 ms, its twiddled radix-16 butterflies leaving half of
// the threads idle at these lengths.
template <int N, int NT, int NSEQ>
__global__ void __launch_bounds__(NT, 1) k_rows_fwd_mrc(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    constexpr int SS = padded_len(N), B = N / 16, BT = NSEQ * B, BPT = (BT + NT - 1) / NT;
    const int tid = threadIdx.x, r0 = blockIdx.x * NSEQ;
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT;
        if (BT % NT != 0 && b >= BT) continue;
        const int q = b / B, j = b % B, h = r0 + q;
        float2 v[16];
#pragma unroll
        for (int r = 4; r < 12; ++r) v[r] = h < P.ny ? load_in(P, h, j + (r - 4) * B) : make_float2(0.f, 0.f);
        dft16_in_mid<-1>(v);
#pragma unroll
        for (int r = 0; r < 16; ++r) sm[q * SS + pidx(16 * j + r)] = v[outpos<16>(r)];
    }
    __syncthreads();
    mrc_stages<N, 16, -1, NT, false, NSEQ, false>(typename MrFixedPlan<N>::fwd{}, sm, SS, P.twx, tid);
    for (int e = tid; e < NSEQ * N; e += NT) {
        const int q = e / N, i = e % N, h = r0 + q;
        if (h < P.ny) __stcg(P.S + (size_t)h * N + i, sm[q * SS + pidx(i)]);
    }
}

// Two shared buffers of the column tile (2 C padded_len(N) complex values):
// the stages alternate between them with one barrier each.
template <int N, int NT, int C>
__global__ void __launch_bounds__(NT, 1) k_cols_mrc(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    using Plan = MrFixedPlan<N>;
    constexpr int B = N / 16, BT = C * B, BPT = (BT + NT - 1) / NT;
    float2 *sa = sm, *sb = sm + C * padded_len(N);
    const int NX = P.NX, tid = threadIdx.x, c0 = blockIdx.x * C;
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT;
        if (BT % NT != 0 && b >= BT) continue;
        const int c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 4; r < 12; ++r)
            v[r] = kx < NX ? __ldcg(P.S + (size_t)(j + (r - 4) * B) * NX + kx) : make_float2(0.f, 0.f);
        dft16_in_mid<-1>(v);
#pragma unroll
        for (int r = 0; r < 16; ++r) sa[pidx(16 * j + r) * C + c] = v[outpos<16>(r)];
    }
    __syncthreads();
    // forward: a -> b -> ... (the transfer function in the last stage)
    mrc_stages_pp<N, 16, -1, NT, true, C, true, false>(typename Plan::fwd{}, sa, sb, 0, P.twy, tid, &P, c0);
    // the spectrum is in b after an odd count of forward stages
    constexpr bool FWD_IN_B = mr_count(typename Plan::fwd{}) % 2 == 1;
    mrc_stages_pp<N, 1, +1, NT, true, C, false, FWD_IN_B>(typename Plan::full{}, sa, sb, 0, P.twy, tid);
    constexpr bool INV_IN_B = FWD_IN_B != (mr_count(typename Plan::full{}) % 2 == 1);
    const float2 *res = INV_IN_B ? sb : sa;
    constexpr int OFF = N / 4;
    for (int e = tid; e < (N / 2) * C; e += NT) {
        const int h = e / C, c = e % C, kx = c0 + c;
        if (kx < NX) __stcg(P.S + (size_t)h * NX + kx, res[pidx(h + OFF) * C + c]);
    }
}

template <int N, int NT, int NSEQ>
__global__ void __launch_bounds__(NT, 1) k_rows_inv_mrc(PropParams P)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    constexpr int SS = padded_len(N);
    const int tid = threadIdx.x, r0 = blockIdx.x * NSEQ;
    for (int e = tid; e < NSEQ * N; e += NT) {
        const int q = e / N, i = e % N, h = r0 + q;
        sm[q * SS + pidx(i)] = h < P.ny ? __ldcg(P.S + (size_t)h * N + i) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    mrc_stages<N, 1, +1, NT, false, NSEQ, false>(typename MrFixedPlan<N>::full{}, sm, SS, P.twx, tid);
    constexpr int OFF = N / 4, NXS = N / 2;
    float lsum = 0.f;
    for (int e = tid; e < NSEQ * NXS; e += NT) {
        const int q = e / NXS, w = e % NXS, h = r0 + q;
        if (h < P.ny) store_out(P, h, w, sm[q * SS + pidx(w + OFF)], lsum);
    }
    if (P.post_mode == OP_SEED) loss_reduce(lsum, P.loss, tid, NT);
}

// The chirp spectrum of one axis with a compile-time plan (blockIdx.x == 0),
// and its elementwise tables (blockIdx.x == 1), as k_chirp_mr.
template <int N>
__global__ void __launch_bounds__(1024, 1) k_chirp_mrc(ChirpAxis A, const float2 *tw)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    const int tid = threadIdx.x;
    if (blockIdx.x == 0) {
        for (int j = tid; j < N; j += 1024) {
            const int m = j < N / 2 ? j : j - N;
            sm[pidx(j)] = chirp_sample(A, m);
        }
        __syncthreads();
        mrc_stages<N, 1, -1, 1024, false, 1, false>(typename MrFixedPlan<N>::full{}, sm, padded_len(N), tw, tid);
        for (int j = tid; j < N; j += 1024) {
            const float2 v = cscale(sm[pidx(j)], A.scale);
            A.H[j] = A.conj_spec ? cconj(v) : v;
        }
    } else {
        chirp_tables(A, tid, 1024);
    }
}

// Chirp spectrum of one axis (blockIdx.x == 0) and its elementwise tables
// (blockIdx.x == 1); as the power-of-two chirp kernel in prop.cu.
__global__ void __launch_bounds__(MR_NT, 1) k_chirp_mr(ChirpAxis A, MrPlan pl, const float2 *tw)
{
    pdl_enter();
    extern __shared__ float2 sm[];
    const int N = A.L, tid = threadIdx.x;
    if (blockIdx.x == 0) {
        for (int j = tid; j < N; j += MR_NT) {
            const int m = j < N / 2 ? j : j - N;
            sm[pidx(j)] = chirp_sample(A, m);
        }
        __syncthreads();
        mr_fft<-1, MR_NT, false>(sm, padded_len(N), 1, pl, tw, tid);
        for (int j = tid; j < N; j += MR_NT) {
            const float2 v = cscale(sm[pidx(j)], A.scale);
            A.H[j] = A.conj_spec ? cconj(v) : v;
        }
    } else {
        chirp_tables(A, tid, MR_NT);
    }
}

// ------------------------------------------------------------------ tilted
// Column FFTs of the ny stored row spectra (D rows 0..ny-1, centred zero
// padding to NY) and the centred spectrum C[(ky + NY/2) % NY][(kx + NX/2) % NX]
// = F[ky][kx] / N (x the unrotated transfer function, reference form).
__global__ void __launch_bounds__(MR_NT, 1) k_tilt_cols_fwd(TiltArgs T, MrPlan pl, const float2 *tw, int C)
{
    extern __shared__ float2 sm[];
    const int N = T.NY, NX = T.NX, tid = threadIdx.x;
    const int c0 = blockIdx.x * C, off = (N - T.ny) / 2;
    for (int e = tid; e < N * C; e += MR_NT) {
        const int i = e / C, c = e % C, kx = c0 + c, h = i - off;
        float2 v = make_float2(0.f, 0.f);
        if (kx < NX && h >= 0 && h < T.ny) v = T.D[(size_t)h * NX + kx];
        sm[pidx(i) * C + c] = v;
    }
    __syncthreads();
    mr_fft<-1, MR_NT, true>(sm, 0, C, pl, tw, tid);
    for (int e = tid; e < N * C; e += MR_NT) {
        const int ky = e / C, c = e % C, kx = c0 + c;
        if (kx >= NX) continue;
        float2 v = cscale(sm[pidx(ky) * C + c], T.invN);
        if (T.reference) v = cmul(v, tf_at(T.tf, ky, kx, N));
        const int n = ky < N / 2 ? ky + N / 2 : ky - N / 2, m = kx < NX / 2 ? kx + NX / 2 : kx - NX / 2;
        T.C[(size_t)n * NX + m] = v;
    }
}

// radial bicubic kernel, a = -1 (olutils.h:290-321)
__device__ __forceinline__ float tilt_cubic(float d)
{
    constexpr float a = -1.f;
    if (d < 1.f) return 1.f - (a + 3.f) * d * d + (a + 2.f) * d * d * d;
    if (d < 2.f) return -4.f * a + 8.f * a * d - 5.f * a * d * d + a * d * d * d;
    return 0.f;
}

// One resampled sample per thread: output frequency (n, m) of the centred
// grid, stored at its natural-order position in D.
//
// Sampling position.  The reference forms x = fsx / du + NX/2 and y = fsy / dv
// + NY/2 in double; the interpolation is continuous in (x, y) except where
// the cell crosses the grid's edges (x or y near 0, N - 1 or N: inside /
// nearest sample / outside), and in the bilinear rule's last column, whose
// nearest sample takes row floor(y) as is.  So the position is formed in FP32 as
//   x = NX/2 + m' + (a11 - 1) m' + K - a13 g / du,   g = f0 - fpz = (fpx^2 + fpy^2) / (f0 + fpz),
// with (a11 - 1) m' split exactly into an integer and a fraction, and y = n
// (the reference's y is n to within an ulp); near an x edge, on the first and
// last rows and in that last column the coordinate is recomputed in FP64
// operation by operation as the reference forms it (each rounding explicit),
// so those cases are decided on the reference's numbers.
// Weights, the Jacobian and all products are FP32.
__device__ __forceinline__ double tilt_x_exact(const TiltArgs &T, double fpx, double fpy)
{
    const double fpz = __dsqrt_rn(__dsub_rn(__dsub_rn(T.fsqr, __dmul_rn(fpx, fpx)), __dmul_rn(fpy, fpy)));
    double fsx = __dadd_rn(__dmul_rn(T.a11, fpx), __dmul_rn(T.a13, fpz));
    if (!T.reference) fsx = __dsub_rn(fsx, T.a13f0);
    return __dadd_rn(__ddiv_rn(fsx, T.du), (double)(T.NX / 2));
}

__global__ void __launch_bounds__(256) k_tilt_resample(TiltArgs T)
{
    const int NX = T.NX, NY = T.NY;
    const int n = blockIdx.y, m = blockIdx.x * 256 + threadIdx.x;
    if (m >= NX) return;
    const int mp = m - NX / 2, np = n - NY / 2;
    const float mpf = (float)mp, npf = (float)np;
    const float fpxf = mpf * T.duf, fpyf = npf * T.dvf;
    const float fpzf = sqrtf(T.f0sq - fpxf * fpxf - fpyf * fpyf);
    // (a11 - 1) m' = I + F exactly enough: integer I, |F| <= 1/2
    const float p = __fmul_rn(T.c1_hi, mpf);
    const float e = __fmaf_rn(T.c1_hi, mpf, -p);
    const float i1 = round_int(p);
    const float t1 = (p - i1) + (e + T.c1_lo * mpf);
    const float i2 = round_int(t1);
    const float gdu = (mpf * mpf * T.duf + npf * npf * T.dv2du) / (T.f0f + fpzf);
    int xi = NX / 2 + mp + T.Ki + (int)i1 + (int)i2;
    float d = (t1 - i2) + T.Kf - T.a13f * gdu;
    const float xa = (float)xi + d;
    if (fabsf(xa) < 0.01f || fabsf(xa - (float)(NX - 1)) < 0.01f || fabsf(xa - (float)NX) < 0.01f) {
        const double x = tilt_x_exact(T, __dmul_rn((double)mp, T.du), __dmul_rn((double)np, T.dv));
        const double xf = floor(x);
        if (!(xf >= -4.0 && xf <= (double)NX + 4.0)) {
            xi = -8; // far outside: zero
            d = 0.f;
        } else {
            xi = (int)xf;
            d = (float)(x - xf);
        }
    }
    const float fx = floorf(d);
    const int ms = xi + (int)fx;
    const float s = d - fx;
    // y = n, except where its last bits decide a case: the first and last rows,
    // and (bilinear) the last column, whose nearest-sample rule takes row floor(y)
    int ns = n;
    float t = 0.f;
    if (n == 0 || n == NY - 1 || (T.interp == 0 && ms == NX - 1)) {
        const double y = __dadd_rn(__ddiv_rn(__dmul_rn((double)np, T.dv), T.dv), (double)(NY / 2));
        const double yf = floor(y);
        ns = (int)yf;
        t = (float)(y - yf);
    }
    const float2 *C = T.C;
    float2 v = make_float2(0.f, 0.f);
    if (T.interp == 0) {
        if (ms >= 0 && ms < NX - 1 && ns >= 0 && ns < NY - 1) {
            const float2 *q = C + (size_t)ns * NX + ms;
            const float2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + NX), dd = __ldg(q + NX + 1);
            const float2 u1 = make_float2((1.f - s) * a.x + s * b.x, (1.f - s) * a.y + s * b.y);
            const float2 u2 = make_float2((1.f - s) * c.x + s * dd.x, (1.f - s) * c.y + s * dd.y);
            v = make_float2((1.f - t) * u1.x + t * u2.x, (1.f - t) * u1.y + t * u2.y);
        } else if (ms >= 0 && ms < NX && ns >= 0 && ns < NY) {
            v = __ldg(C + (size_t)ns * NX + ms);
        }
    } else if (ms >= 0 && ms < NX && ns >= 0 && ns < NY) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int nn = ns - 1 + j;
            if (nn < 0 || nn >= NY) continue;
            const float dyv = (float)(j - 1) - t;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int mm = ms - 1 + i;
                if (mm < 0 || mm >= NX) continue;
                const float dxv = (float)(i - 1) - s;
                const float k = tilt_cubic(sqrtf(dxv * dxv + dyv * dyv));
                const float2 q = __ldg(C + (size_t)nn * NX + mm);
                v.x = fmaf(k, q.x, v.x);
                v.y = fmaf(k, q.y, v.y);
            }
        }
    }
    const float J = T.J0 + T.Jb * fpxf / fpzf;
    v = cscale(v, J);
    const int ky = n < NY / 2 ? n + NY / 2 : n - NY / 2, kx = m < NX / 2 ? m + NX / 2 : m - NX / 2;
    if (!T.reference) {
        float2 H;
        if (T.fresnel) {
            H = cmul(__ldg(T.Hx + kx), __ldg(T.Hy + ky));
        } else {
            // exp(2 pi i z w), w = sqrt(f0^2 - (fpx + a13 f0)^2 - fpy^2), in double-float
            // (~44 bits: z w ~ 1e5 cycles keeps ~1e-8 cycles; FP64 runs at a small
            // fraction of the FP32 rate on this GPU)
            const df2 u = df_add(df_mul(df2{T.du_hi, T.du_lo}, df2{mpf, 0.f}), df2{T.c_hi, T.c_lo});
            const df2 v = df_mul(df2{T.dv_hi, T.dv_lo}, df2{npf, 0.f});
            const df2 u2 = df_mul(u, u), v2 = df_mul(v, v);
            const df2 w2 = df_add(df2{T.f0sq_hi, T.f0sq_lo}, df_add(df2{-u2.hi, -u2.lo}, df2{-v2.hi, -v2.lo}));
            const df2 w = df_sqrt(w2);
            H = cis_cycles(df_frac(df_mul(w, df2{T.z_hi, T.z_lo})));
        }
        v = cmul(v, H);
    }
    T.D[(size_t)ky * NX + kx] = v;
}

// Inverse column FFTs of the resampled spectrum; the central ny rows, x 1/N,
// go to D's first ny rows (the scratch the inverse row pass reads).  A CTA
// reads its whole column tile before writing back into the same columns.
__global__ void __launch_bounds__(MR_NT, 1) k_tilt_cols_inv(TiltArgs T, MrPlan pl, const float2 *tw, int C)
{
    extern __shared__ float2 sm[];
    const int N = T.NY, NX = T.NX, tid = threadIdx.x;
    const int c0 = blockIdx.x * C, off = (N - T.ny) / 2;
    for (int e = tid; e < N * C; e += MR_NT) {
        const int i = e / C, c = e % C, kx = c0 + c;
        sm[pidx(i) * C + c] = kx < NX ? T.D[(size_t)i * NX + kx] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    mr_fft<+1, MR_NT, true>(sm, 0, C, pl, tw, tid);
    for (int e = tid; e < T.ny * C; e += MR_NT) {
        const int h = e / C, c = e % C, kx = c0 + c;
        if (kx < NX) T.D[(size_t)h * NX + kx] = cscale(sm[pidx(h + off) * C + c], T.invN);
    }
}

namespace {

std::mutex g_mr_mu;
std::map<std::pair<unsigned long long, int>, float2 *> g_mr_tw; // (context, N) -> exp(-2 pi i m / N)

int mr_table(int N, const float2 **out)
{
    unsigned long long ctx = 0;
    if (int rc = context_id(&ctx)) return rc;
    cudaError_t e = cudaSuccess;
    std::lock_guard<std::mutex> lk(g_mr_mu);
    auto it = g_mr_tw.find({ctx, N});
    if (it == g_mr_tw.end()) {
        std::vector<float2> t(N);
        for (int m = 0; m < N; ++m) {
            const double a = -2.0 * M_PI * (double)m / (double)N;
            t[m] = make_float2((float)std::cos(a), (float)std::sin(a));
        }
        float2 *d = nullptr;
        e = cudaMalloc(&d, sizeof(float2) * N);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (twiddle table)");
        e = cudaMemcpy(d, t.data(), sizeof(float2) * N, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(d);
            return cuda_fail(e, "twiddle table upload");
        }
        it = g_mr_tw.emplace(std::make_pair(ctx, N), d).first;
    }
    *out = it->second;
    return OLG_OK;
}

template <typename K>
int mr_smem(K kern, int bytes)
{
    if (bytes <= 48 * 1024) return OLG_OK;
    const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, "cudaFuncSetAttribute");
}

int mr_launch(void (*kern)(PropParams), int grid, int smem, cudaStream_t st, const PropParams &P, const char *what)
{
    if (int rc = mr_smem(kern, smem)) return rc;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(MR_NT);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, P);
    if (e != cudaSuccess) return cuda_fail(e, what);
    count_launch();
    return check_launch(what);
}

// Sequences per CTA: the largest nseq for which every stage's nseq * N / R
// butterflies fit in MR_NT threads x (MR_VALS / R) each, within 160 KiB of
// shared memory (0: the length does not fit one CTA).
int mr_nseq(const MrPlan &pl)
{
    int best = 1 << 30;
    for (int i = 0; i < pl.nst; ++i) {
        const int R = (int)((pl.radices >> (5 * i)) & 31);
        const int cap = MR_NT * (MR_VALS / R) * R / pl.n;
        best = cap < best ? cap : best;
    }
    const int smem_cap = (160 * 1024) / (padded_len(pl.n) * (int)sizeof(float2));
    return best < smem_cap ? best : smem_cap;
}

} // namespace

bool mr_plan(int N, MrPlan *pl)
{
    if (N < 2 || N > FFT_MAX) return false;
    int m = N, k = 0;
    unsigned long long code = 0;
    auto add = [&](int R) {
        code |= (unsigned long long)R << (5 * k);
        ++k;
        m /= R;
    };
    while (m % 16 == 0 && k < 12) add(16);
    if (m % 8 == 0 && k < 12) add(8);
    if (m % 4 == 0 && k < 12) add(4);
    if (m % 2 == 0 && k < 12) add(2);
    while (m % 5 == 0 && k < 12) add(5);
    while (m % 3 == 0 && k < 12) add(3);
    if (m != 1) return false;
    pl->n = N;
    pl->nst = k;
    pl->radices = code;
    return true;
}

bool mr_length_ok(int N)
{
    MrPlan pl;
    return mr_plan(N, &pl) && mr_nseq(pl) >= 1;
}

int mr_prepare(PropParams &P)
{
    if (!is_pow2(P.NX)) {
        if (!mr_plan(P.NX, &P.mrx) || mr_nseq(P.mrx) < 1)
            return fail(OLG_ERR_UNSUPPORTED_SIZE, "width: 2 nx must be a power of two or 2^a 3^b 5^c <= 7680");
        if (int rc = mr_table(P.NX, &P.twx)) return rc;
        P.mr_rows = mr_nseq(P.mrx);
    }
    if (!is_pow2(P.NY)) {
        if (!mr_plan(P.NY, &P.mry) || mr_nseq(P.mry) < 1)
            return fail(OLG_ERR_UNSUPPORTED_SIZE, "height: 2 ny must be a power of two or 2^a 3^b 5^c <= 7680");
        if (int rc = mr_table(P.NY, &P.twy)) return rc;
        P.mr_cols = mr_nseq(P.mry);
    }
    return OLG_OK;
}

// Launch shapes of the compile-time plans: {N, threads, rows or columns per CTA}.
template <int N, int NT, int NSEQ, typename K>
int mrc_launch(K kern, int count, cudaStream_t st, const PropParams &P, const char *what, int buffers = 1)
{
    const int smem = buffers * NSEQ * padded_len(N) * (int)sizeof(float2);
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    }
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((count + NSEQ - 1) / NSEQ);
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, P);
    if (e != cudaSuccess) return cuda_fail(e, what);
    count_launch();
    return check_launch(what);
}

template <int N, int NT, int NSEQ>
int mrc_rows(const PropParams &P, bool inverse, cudaStream_t st)
{
    return inverse ? mrc_launch<N, NT, NSEQ>(k_rows_inv_mrc<N, NT, NSEQ>, P.ny, st, P, "k_rows_inv_mrc")
                   : mrc_launch<N, NT, NSEQ>(k_rows_fwd_mrc<N, NT, NSEQ>, P.ny, st, P, "k_rows_fwd_mrc");
}

template <int N, int NT, int C>
int mrc_cols(const PropParams &P, cudaStream_t st)
{
    return mrc_launch<N, NT, C>(k_cols_mrc<N, NT, C>, P.NX, st, P, "k_cols_mrc", 2);
}

int mr_rows_pass(const PropParams &P, bool inverse, cudaStream_t st)
{
    switch (P.NX) {
    case 7680: return mrc_rows<7680, 1024, 2>(P, inverse, st);
    case 5120: return mrc_rows<5120, 1024, 3>(P, inverse, st);
    case 3840: return mrc_rows<3840, 1024, 4>(P, inverse, st);
    case 2560: return mrc_rows<2560, 1024, 6>(P, inverse, st);
    default: break;
    }
    const int grid = (P.ny + P.mr_rows - 1) / P.mr_rows;
    const int smem = P.mr_rows * padded_len(P.NX) * (int)sizeof(float2);
    return inverse ? mr_launch(k_rows_inv_mr, grid, smem, st, P, "k_rows_inv_mr")
                   : mr_launch(k_rows_fwd_mr, grid, smem, st, P, "k_rows_fwd_mr");
}

int mr_cols_pass(const PropParams &P, cudaStream_t st)
{
    switch (P.NY) {
    case 4320: return mrc_cols<4320, 1024, 2>(P, st);
    case 2880: return mrc_cols<2880, 1024, 4>(P, st);
    case 2160: return mrc_cols<2160, 1024, 4>(P, st);
    case 1440: return mrc_cols<1440, 1024, 8>(P, st);
    default: break;
    }
    const int grid = (P.NX + P.mr_cols - 1) / P.mr_cols;
    const int smem = P.mr_cols * padded_len(P.NY) * (int)sizeof(float2);
    return mr_launch(k_cols_mr, grid, smem, st, P, "k_cols_mr");
}

int mr_chirp_axis(const ChirpAxis &A, cudaStream_t st)
{
    MrPlan pl;
    if (!mr_plan(A.L, &pl) || mr_nseq(pl) < 1)
        return fail(OLG_ERR_UNSUPPORTED_SIZE, "chirp length must be a power of two or 2^a 3^b 5^c <= 7680");
    const float2 *tw = nullptr;
    if (int rc = mr_table(A.L, &tw)) return rc;
    const int smem = padded_len(A.L) * (int)sizeof(float2);
    const int grid = (A.ta || A.tb) ? 2 : 1;
    auto fixed = [&](auto kern) -> int {
        if (int rc = mr_smem(kern, smem)) return rc;
        kern<<<grid, 1024, smem, st>>>(A, tw);
        count_launch();
        return check_launch("k_chirp_mrc");
    };
    switch (A.L) {
    case 7680: return fixed(k_chirp_mrc<7680>);
    case 5120: return fixed(k_chirp_mrc<5120>);
    case 4320: return fixed(k_chirp_mrc<4320>);
    case 3840: return fixed(k_chirp_mrc<3840>);
    case 2880: return fixed(k_chirp_mrc<2880>);
    case 2560: return fixed(k_chirp_mrc<2560>);
    case 2160: return fixed(k_chirp_mrc<2160>);
    case 1440: return fixed(k_chirp_mrc<1440>);
    default: break;
    }
    if (int rc = mr_smem(k_chirp_mr, smem)) return rc;
    k_chirp_mr<<<grid, MR_NT, smem, st>>>(A, pl, tw);
    count_launch();
    return check_launch("k_chirp_mr");
}

int tilt_middle(const TiltArgs &T, cudaStream_t st)
{
    if (is_pow2(T.NY) && T.NY >= 256) {
        if (int rc = tilt_cols_pow2(T, false, st)) return rc;
        k_tilt_resample<<<dim3((T.NX + 255) / 256, T.NY), 256, 0, st>>>(T);
        count_launch();
        if (int rc = check_launch("k_tilt_resample")) return rc;
        return tilt_cols_pow2(T, true, st);
    }
    MrPlan pl;
    if (!mr_plan(T.NY, &pl) || mr_nseq(pl) < 1)
        return fail(OLG_ERR_UNSUPPORTED_SIZE, "height: 2 ny must be a power of two or 2^a 3^b 5^c <= 7680");
    const float2 *tw = nullptr;
    if (int rc = mr_table(T.NY, &tw)) return rc;
    const int C = mr_nseq(pl);
    const int smem = C * padded_len(T.NY) * (int)sizeof(float2);
    if (int rc = mr_smem(k_tilt_cols_fwd, smem)) return rc;
    if (int rc = mr_smem(k_tilt_cols_inv, smem)) return rc;
    const int gc = (T.NX + C - 1) / C;
    k_tilt_cols_fwd<<<gc, MR_NT, smem, st>>>(T, pl, tw, C);
    count_launch();
    if (int rc = check_launch("k_tilt_cols_fwd")) return rc;
    k_tilt_resample<<<dim3((T.NX + 255) / 256, T.NY), 256, 0, st>>>(T);
    count_launch();
    if (int rc = check_launch("k_tilt_resample")) return rc;
    k_tilt_cols_inv<<<gc, MR_NT, smem, st>>>(T, pl, tw, C);
    count_launch();
    return check_launch("k_tilt_cols_inv");
}

} // namespace olg
