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
            float2 c = make_float2(0.f, 0.f);
            if (A.lim < 0 || abs(m) < A.lim) c = cis_cycles(frac_mul(A.kap_hi, A.kap_lo, (float)m * (float)m));
            sm[pidx(j)] = c;
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

namespace {

std::mutex g_mr_mu;
std::map<std::pair<int, int>, float2 *> g_mr_tw; // (device, N) -> exp(-2 pi i m / N)

int mr_table(int N, const float2 **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lk(g_mr_mu);
    auto it = g_mr_tw.find({dev, N});
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
        if (e != cudaSuccess) return cuda_fail(e, "twiddle table upload");
        it = g_mr_tw.emplace(std::make_pair(dev, N), d).first;
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

int mr_rows_pass(const PropParams &P, bool inverse, cudaStream_t st)
{
    const int grid = (P.ny + P.mr_rows - 1) / P.mr_rows;
    const int smem = P.mr_rows * padded_len(P.NX) * (int)sizeof(float2);
    return inverse ? mr_launch(k_rows_inv_mr, grid, smem, st, P, "k_rows_inv_mr")
                   : mr_launch(k_rows_fwd_mr, grid, smem, st, P, "k_rows_fwd_mr");
}

int mr_cols_pass(const PropParams &P, cudaStream_t st)
{
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
    if (int rc = mr_smem(k_chirp_mr, smem)) return rc;
    k_chirp_mr<<<(A.ta || A.tb) ? 2 : 1, MR_NT, smem, st>>>(A, pl, tw);
    count_launch();
    return check_launch("k_chirp_mr");
}

} // namespace olg
