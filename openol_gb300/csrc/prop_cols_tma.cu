// prop_cols_tma.cu -- persistent, TMA-staged column pass of the fused
// propagation (pass 2) for padded heights N = 2048, 4096, 8192.
//
// The column pass reads C adjacent columns of the ny stored rows of the
// half-padded spectrum S, transforms them (zero-padded forward FFT, x T,
// crop-pruned inverse FFT) and writes the central ny rows back.  In the
// one-shot shapes every CTA starts with a burst of strided global loads and
// one 128-register CTA per SM has nothing to overlap them with.  Here one CTA
// per SM walks the column tiles; while a tile's transforms run, the next
// tile's ny x C block of S streams into a shared staging buffer with
// cp.async.bulk.tensor.2d (boxes of C columns x 256 rows, completed on an
// mbarrier), and the first radix-16 stage reads it from shared memory.
//
// Shared memory: staging ny x C x 8 B = 64 KB, the transform buffer
// padded_len(N) x C x 8 B = 139 KB, one mbarrier.  Waits are bounded: on
// expiry the kernel records the device fault word (olg_device_fault_check),
// waits (bounded) for its own copy in flight and returns.
#include <algorithm>
#include <cstdio>

#include "propk.cuh"
#include "tc.cuh"

namespace olg {

constexpr int CT_NT = 512;
constexpr int CT_BOX_ROWS = 256;

template <int N>
struct ColTmaCfg {
    static constexpr int C = 16384 / N; // 8 at 2048, 4 at 4096, 2 at 8192
    static constexpr int NYS = N / 2;   // stored rows of S (ny)
    static constexpr int STG_BYTES = NYS * C * 8;
    static constexpr int FFT_BYTES = padded_len(N) * C * 8;
    static constexpr int SMEM = STG_BYTES + FFT_BYTES + 64;
};

// One column tile: the forward first stage from the staged rows, then (the
// staging buffer being free) the copy of the next tile is issued, then the
// rest of the pass.  Not inlined, so that the persistent loop's few live
// values are saved once per tile and the transforms keep the whole register
// budget of the one-shot kernel.
template <int N>
__device__ __noinline__ void cols_tile_tma(const PropParams &P, const CUtensorMap *mS, float2 *stg, float2 *sm,
                                           int tile, int next, uint32_t bar)
{
    using Cf = ColTmaCfg<N>;
    constexpr int C = Cf::C, B = N / 16, NT = CT_NT;
    constexpr int BPT = C * B / NT;
    const int tid = threadIdx.x;
    const int NX = P.NX, c0 = tile * C;
    // forward first stage from the staged ny rows (the rest is zero padding)
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C;
        float2 v[16];
#pragma unroll
        for (int r = 4; r < 12; ++r) v[r] = stg[(j + (r - 4) * B) * C + c];
        dft16_in_mid<-1>(v);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[17 * C * j + c + k * C] = v[outpos<16>(k)];
    }
    __syncthreads();
    // the staging buffer is free: fetch the next tile behind this one's transforms
    if (next >= 0 && tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(bar, Cf::STG_BYTES);
#pragma unroll 1
        for (int b = 0; b < Cf::NYS / CT_BOX_ROWS; ++b)
            tma_load_2d(smem_u32(stg + b * CT_BOX_ROWS * C), mS, bar, next * C, b * CT_BOX_ROWS);
    }
    mid_stages<N, -1, NT, true, C>(sm, 0, g_tw, tid);
    // forward last stage -> x T(ky, kx) -> inverse first stage, in registers
    float2 vv[BPT][16];
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C;
#pragma unroll
        for (int r = 0; r < 16; ++r) vv[t][r] = sm[pidx(j) * C + c + r * (pstride<B>() * C)];
    }
    __syncthreads();
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        last_twiddle<N, -1>(vv[t], j, g_tw);
        dft<16, -1>(vv[t]);
        float2 w[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) w[k] = kx < NX ? cmul(vv[t][outpos<16>(k)], tf_at(P, j + k * B, kx, N)) : vv[t][outpos<16>(k)];
        dft<16, +1>(w);
#pragma unroll
        for (int k = 0; k < 16; ++k) sm[17 * C * j + c + k * C] = w[outpos<16>(k)];
    }
    __syncthreads();
    mid_stages<N, +1, NT, true, C>(sm, 0, g_tw, tid);
    // inverse last stage: only the central ny rows, back in place
#pragma unroll
    for (int t = 0; t < BPT; ++t) {
        const int b = tid + t * NT, c = b % C, j = b / C, kx = c0 + c;
        float2 v[16];
#pragma unroll
        for (int r = 0; r < 16; ++r) v[r] = sm[pidx(j) * C + c + r * (pstride<B>() * C)];
        last_twiddle<N, +1>(v, j, g_tw);
        dft16_out_mid<+1>(v);
        if (kx < NX) {
#pragma unroll
            for (int k = 4; k < 12; ++k) __stcg(P.S + (size_t)(j + (k - 4) * B) * NX + kx, v[outpos<16>(k)]);
        }
    }
    __syncthreads(); // the next tile's first stage overwrites sm
}

template <int N>
__global__ void __launch_bounds__(CT_NT, 1)
    k_cols_tma(const __grid_constant__ PropParams P, const __grid_constant__ CUtensorMap mS, int *fault, long long budget)
{
    using Cf = ColTmaCfg<N>;
    constexpr int C = Cf::C;
    static_assert((C * (N / 16)) % CT_NT == 0, "threads must divide the butterflies");
    extern __shared__ __align__(1024) unsigned char smraw[];
    float2 *stg = reinterpret_cast<float2 *>(smraw);
    float2 *sm = reinterpret_cast<float2 *>(smraw + Cf::STG_BYTES);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(smraw + Cf::STG_BYTES + Cf::FFT_BYTES);
    const uint32_t bar = smem_u32(mbar);
    const int ntiles = P.NX / C;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    pdl_enter(); // S is written by pass 1
    int tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < ntiles) {
        mbar_expect_tx(bar, Cf::STG_BYTES);
#pragma unroll 1
        for (int b = 0; b < Cf::NYS / CT_BOX_ROWS; ++b)
            tma_load_2d(smem_u32(stg + b * CT_BOX_ROWS * C), &mS, bar, tile * C, b * CT_BOX_ROWS);
    }
    uint32_t phase = 0;
    bool ok = true;
#pragma unroll 1
    for (; tile < ntiles; tile += gridDim.x) {
        ok = __syncthreads_and(mbar_wait(bar, phase, budget));
        if (!ok) break;
        phase ^= 1;
        const int next = tile + (int)gridDim.x < ntiles ? tile + (int)gridDim.x : -1;
        cols_tile_tma<N>(P, &mS, stg, sm, tile, next, bar);
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(fault, 1);
        // the staging copy of this tile may still be in flight: let it land
        // (bounded) before the CTA's shared memory is released
        mbar_wait(bar, phase, budget);
    }
}

namespace {

template <int N>
int launch_cols_tma_n(const PropParams &P, cudaStream_t st)
{
    using Cf = ColTmaCfg<N>;
    if (P.NY != N || P.ny != Cf::NYS || P.NX % Cf::C != 0)
        return fail(OLG_ERR_INVALID_ARG, "TMA column pass: shape not covered");
    // the staged tile is ny rows x C columns of S (ny x NX complex64, row pitch NX)
    if (((uintptr_t)P.S & 15) || (P.NX * 8) % 16)
        return fail(OLG_ERR_INVALID_ARG, "TMA column pass: S must be 16-byte aligned with a 16-byte row pitch");
    PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
    if (int rc = tensor_map_encoder(&enc)) return rc;
    CUtensorMap map;
    cuuint64_t dims[2] = {(cuuint64_t)P.NX, (cuuint64_t)P.ny};
    cuuint64_t strides[1] = {(cuuint64_t)P.NX * 8};
    cuuint32_t box[2] = {(cuuint32_t)Cf::C, (cuuint32_t)CT_BOX_ROWS};
    cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, (void *)P.S, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(OLG_ERR_CUDA, "cuTensorMapEncodeTiled (S) failed");
    int *fault = nullptr;
    if (int rc = device_fault_word(&fault)) return rc;
    if (int rc = prep_smem(k_cols_tma<N>, Cf::SMEM)) return rc;
    const int ntiles = P.NX / Cf::C;
    const int grid = std::min(ntiles, sm_count());
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(CT_NT);
    cfg.dynamicSmemBytes = (size_t)Cf::SMEM;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const long long budget = wait_budget_cycles();
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k_cols_tma<N>, P, map, fault, budget);
    if (e != cudaSuccess) return cuda_fail(e, "k_cols_tma");
    count_launch();
    return check_launch("k_cols_tma");
}

} // namespace

int cols_pass_tma(const PropParams &P, cudaStream_t st)
{
    switch (P.NY) {
    case 2048: return launch_cols_tma_n<2048>(P, st);
    case 4096: return launch_cols_tma_n<4096>(P, st);
    case 8192: return launch_cols_tma_n<8192>(P, st);
    default: return fail(OLG_ERR_UNSUPPORTED_SIZE, "TMA column pass: padded heights 2048..8192");
    }
}

} // namespace olg
