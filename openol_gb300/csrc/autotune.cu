// autotune.cu -- the launch-variant table of the propagation passes and the
// project-written autotuner that fills it (olg_autotune_prop).
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
std::atomic<int> g_variant[3][14];
} // namespace olg

using namespace olg;

// ------------------------------------------------------------- autotuner
namespace olg {
namespace {

#define OLG_N_SWITCH(n, EXPR)                                                                                           \
    switch (n) {                                                                                                       \
    case 256: { constexpr int NN = 256; EXPR; }                                                                        \
    case 512: { constexpr int NN = 512; EXPR; }                                                                        \
    case 1024: { constexpr int NN = 1024; EXPR; }                                                                      \
    case 2048: { constexpr int NN = 2048; EXPR; }                                                                      \
    case 4096: { constexpr int NN = 4096; EXPR; }                                                                      \
    case 8192: { constexpr int NN = 8192; EXPR; }                                                                      \
    default: return false;                                                                                             \
    }

bool variant_valid(int kind, int n, int i)
{
    if (kind == 1) { OLG_N_SWITCH(n, return col_variant_valid<NN>(i)) }
    OLG_N_SWITCH(n, return row_variant_valid<NN>(i))
}

int log2i(int n)
{
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

} // namespace
} // namespace olg

extern "C" int olg_prop_variant_count(void) { return N_ROW_VARIANTS > N_COL_VARIANTS ? N_ROW_VARIANTS : N_COL_VARIANTS; }

extern "C" int olg_prop_get_variant(int kind, int n)
{
    if (kind < 0 || kind > 2 || !is_pow2(n) || n < 256 || n > FFT_MAX) return -1;
    return g_variant[kind][log2i(n)];
}

extern "C" int olg_prop_set_variant(int kind, int n, int idx)
{
    if (kind < 0 || kind > 2 || !is_pow2(n) || n < 256 || n > FFT_MAX) return fail(OLG_ERR_INVALID_ARG, "bad pass kind or length");
    if (!variant_valid(kind, n, idx)) return fail(OLG_ERR_INVALID_ARG, "launch variant not valid for this length");
    g_variant[kind][log2i(n)] = idx;
    return OLG_OK;
}

// Times every valid launch variant of the three passes on an ny x nx ASM
// propagation (the real kernels on the real shapes) and keeps the fastest.
extern "C" int olg_autotune_prop(int ny, int nx, int reps, olg_stream_t stream)
{
    if (!is_pow2(nx) || !is_pow2(ny) || nx < 128 || ny < 128 || 2 * nx > FFT_MAX || 2 * ny > FFT_MAX)
        return fail(OLG_ERR_UNSUPPORTED_SIZE, "autotuning covers fields with ny, nx powers of two in [128, 4096]");
    if (reps < 1) reps = 5;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch buf, sc;
    if (int rc = buf.acquire(nullptr, 0, (size_t)ny * nx * sizeof(float2), st)) return rc;
    if (int rc = sc.acquire(nullptr, 0, layout_bytes(ny, nx, nullptr, nullptr), st)) return rc;
    cudaError_t e = cudaMemsetAsync(buf.ptr, 0, (size_t)ny * nx * sizeof(float2), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    Layout L;
    layout_bytes(ny, nx, &L, (char *)sc.ptr);
    PropSetup S;
    if (int rc = setup_asm(buf.ptr, buf.ptr, ny, nx, 8e-6, 8e-6, 532e-9, 0.05, 0, L, &S)) return rc;
    // events released on every return path
    struct Events {
        cudaEvent_t a = nullptr, b = nullptr;
        ~Events()
        {
            if (a) cudaEventDestroy(a);
            if (b) cudaEventDestroy(b);
        }
    } ev;
    if ((e = cudaEventCreate(&ev.a)) != cudaSuccess || (e = cudaEventCreate(&ev.b)) != cudaSuccess)
        return cuda_fail(e, "cudaEventCreate");
    // Coordinate descent over the three passes, timing whole propagations:
    // a pass's speed depends on its neighbours (L2 contents, dependent-launch
    // overlap), so passes are not timed alone.
    const int lens[3] = {2 * nx, 2 * ny, 2 * nx};
    int lns[3];
    for (int k = 0; k < 3; ++k) lns[k] = log2i(lens[k]);
    // Each timed propagation starts from a cold L2 (a 256 MiB write first),
    // like a propagation of a field that was not just touched.
    const size_t flush_bytes = (size_t)256 << 20;
    Scratch flush;
    if (int rc = flush.acquire(nullptr, 0, flush_bytes, st)) return rc;
    auto time_prop = [&](float *ms) -> int {
        int rc = run_passes(S.P, st);
        *ms = 0.f;
        for (int r = 0; r < reps && !rc; ++r) {
            cudaError_t te = cudaMemsetAsync(flush.ptr, r & 0xff, flush_bytes, st);
            if (te != cudaSuccess) return cuda_fail(te, "cudaMemsetAsync (L2 flush)");
            if ((te = cudaEventRecord(ev.a, st)) != cudaSuccess) return cuda_fail(te, "cudaEventRecord");
            rc = run_passes(S.P, st);
            if (rc) break;
            if ((te = cudaEventRecord(ev.b, st)) != cudaSuccess) return cuda_fail(te, "cudaEventRecord");
            if ((te = cudaEventSynchronize(ev.b)) != cudaSuccess) return cuda_fail(te, "cudaEventSynchronize");
            float t = 0.f;
            if ((te = cudaEventElapsedTime(&t, ev.a, ev.b)) != cudaSuccess) return cuda_fail(te, "cudaEventElapsedTime");
            *ms += t;
        }
        return rc;
    };
    for (int round = 0; round < 2; ++round) {
        for (int kind = 0; kind < 3; ++kind) {
            const int n = lens[kind], ln = lns[kind];
            float best = 1e30f;
            int best_i = g_variant[kind][ln];
            for (int i = 0; i < olg_prop_variant_count(); ++i) {
                if (!variant_valid(kind, n, i)) continue;
                g_variant[kind][ln] = i;
                float ms = 0.f;
                if (int rc = time_prop(&ms)) {
                    g_variant[kind][ln] = best_i; // keep the last good choice
                    return rc;
                }
                if (ms < best) {
                    best = ms;
                    best_i = i;
                }
            }
            g_variant[kind][ln] = best_i;
        }
    }
    return OLG_OK;
}

