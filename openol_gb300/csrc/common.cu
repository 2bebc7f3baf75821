// common.cu -- library-wide host helpers: status strings, per-thread error
// messages, launch counter, stream-ordered scratch.
#include <atomic>
#include <cstdio>
#include <map>
#include <mutex>
#include <string>

#include <cuda.h>

#include "common.cuh"

namespace olg {

static thread_local std::string t_err;
static std::atomic<unsigned long long> g_launches{0};
static std::atomic<long long> g_wait_budget{4000000000LL};
static std::atomic<int> g_fail_allocs{0};

long long wait_budget_cycles() { return g_wait_budget.load(std::memory_order_relaxed); }

void set_error(const std::string &msg) { t_err = msg; }

int fail(int status, const std::string &msg)
{
    t_err = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char *where)
{
    t_err = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? OLG_ERR_NOMEM : OLG_ERR_CUDA;
}

int check_launch(const char *what)
{
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? OLG_OK : cuda_fail(e, what);
}

void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {
using PFN_ctx_current = CUresult (*)(CUcontext *);
using PFN_ctx_id = CUresult (*)(CUcontext, unsigned long long *);
std::once_flag g_ctx_once;
PFN_ctx_current g_ctx_current = nullptr;
PFN_ctx_id g_ctx_id = nullptr;

void load_ctx_entry_points()
{
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_ctx_current = (PFN_ctx_current)fn;
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_ctx_id = (PFN_ctx_id)fn;
}
} // namespace

namespace {
std::mutex g_encode_mu;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::map<unsigned long long, int *> g_fault_word; // per context
} // namespace

int tensor_map_encoder(PFN_cuTensorMapEncodeTiled_v12000 *out)
{
    std::lock_guard<std::mutex> lk(g_encode_mu);
    if (!g_encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        const cudaError_t e =
            cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || !fn || q != cudaDriverEntryPointSuccess)
            return fail(OLG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    *out = g_encode;
    return OLG_OK;
}

int device_fault_word(int **out)
{
    unsigned long long ctx = 0;
    if (int rc = context_id(&ctx)) return rc;
    std::lock_guard<std::mutex> lk(g_encode_mu);
    auto it = g_fault_word.find(ctx);
    if (it == g_fault_word.end()) {
        int *f = nullptr;
        cudaError_t e = cudaMalloc(&f, sizeof(int));
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc (fault word)");
        e = cudaMemset(f, 0, sizeof(int));
        if (e != cudaSuccess) {
            cudaFree(f);
            return cuda_fail(e, "cudaMemset (fault word)");
        }
        it = g_fault_word.emplace(ctx, f).first;
    }
    *out = it->second;
    return OLG_OK;
}

int context_id(unsigned long long *id)
{
    std::call_once(g_ctx_once, load_ctx_entry_points);
    if (!g_ctx_current || !g_ctx_id) return fail(OLG_ERR_CUDA, "cuCtxGetCurrent / cuCtxGetId unavailable");
    CUcontext c = nullptr;
    if (g_ctx_current(&c) != CUDA_SUCCESS) return fail(OLG_ERR_CUDA, "cuCtxGetCurrent failed");
    if (!c) {
        // no context current on this thread yet: let the runtime make the
        // current device's primary context current
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaSetDevice(dev);
        if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
        if (g_ctx_current(&c) != CUDA_SUCCESS || !c) return fail(OLG_ERR_CUDA, "no current CUDA context");
    }
    if (g_ctx_id(c, id) != CUDA_SUCCESS) return fail(OLG_ERR_CUDA, "cuCtxGetId failed");
    return OLG_OK;
}

// The library's own stream-ordered pool per device.  It keeps up to 8 GiB of
// freed scratch mapped between calls: the default pool returns everything at
// each synchronisation, and re-mapping a few hundred MB per call (the WRP pair
// lists) cost more than the kernels that use it.  Leaves the device's default
// pool untouched.
// Pools are keyed on the context (a reset device gets a new pool).
static cudaMemPool_t scratch_pool()
{
    static std::mutex mu;
    static std::map<unsigned long long, cudaMemPool_t> pools;
    int dev = 0;
    unsigned long long ctx = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || context_id(&ctx) != OLG_OK) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    auto it = pools.find(ctx);
    if (it != pools.end()) return it->second;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) == cudaSuccess) {
        unsigned long long keep = 8ull << 30;
        cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    } else if (cudaDeviceGetDefaultMemPool(&p, dev) != cudaSuccess) {
        return nullptr;
    }
    pools.emplace(ctx, p);
    return p;
}

int Scratch::acquire(void *work, size_t work_bytes, size_t need, cudaStream_t s)
{
    stream = s;
    if (work) {
        if (work_bytes < need) return fail(OLG_ERR_WORKSPACE, "workspace smaller than required");
        if ((uintptr_t)work & 255) return fail(OLG_ERR_WORKSPACE, "workspace must be 256-byte aligned");
        ptr = work;
        bytes = work_bytes;
        owned = false;
        return OLG_OK;
    }
    // host-side fault injection (olg_inject_alloc_failures): fail this
    // allocation as an out-of-memory would, before touching the device
    for (int k = g_fail_allocs.load(); k > 0;)
        if (g_fail_allocs.compare_exchange_weak(k, k - 1)) {
            ptr = nullptr;
            return fail(OLG_ERR_NOMEM, "injected allocation failure (olg_inject_alloc_failures)");
        }
    cudaMemPool_t pool = scratch_pool();
    if (!pool) return fail(OLG_ERR_CUDA, std::string("no scratch memory pool: ") + t_err);
    cudaError_t e = cudaMallocFromPoolAsync(&ptr, need, pool, s);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return cuda_fail(e, "cudaMallocFromPoolAsync (scratch)");
    }
    bytes = need;
    owned = true;
    return OLG_OK;
}

Scratch::~Scratch()
{
    if (owned && ptr) cudaFreeAsync(ptr, stream);
}

} // namespace olg

extern "C" int olg_version(void) { return 100; }

extern "C" const char *olg_status_string(int status)
{
    switch (status) {
    case OLG_OK: return "ok";
    case OLG_ERR_INVALID_ARG: return "invalid argument";
    case OLG_ERR_UNSUPPORTED_SIZE: return "unsupported size";
    case OLG_ERR_CUDA: return "CUDA error";
    case OLG_ERR_WORKSPACE: return "workspace too small or misaligned";
    case OLG_ERR_NOMEM: return "out of device memory";
    default: return "unknown status";
    }
}

extern "C" const char *olg_last_error(void) { return olg::t_err.c_str(); }

extern "C" unsigned long long olg_launch_count(void) { return olg::g_launches.load(); }

extern "C" long long olg_wait_budget_cycles(long long cycles)
{
    if (cycles > 0) return olg::g_wait_budget.exchange(cycles);
    return olg::g_wait_budget.load();
}

namespace olg {

int HostPipeline::init()
{
    if (s_in) return OLG_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&s_in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s_out, cudaStreamNonBlocking);
    cudaEvent_t *all[2 + 3 * SLOTS] = {&entry, &last};
    for (int k = 0; k < SLOTS; ++k) {
        all[2 + k] = &in[k];
        all[2 + SLOTS + k] = &done[k];
        all[2 + 2 * SLOTS + k] = &out[k];
    }
    for (cudaEvent_t *v : all)
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(v, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        release();
        return cuda_fail(e, "creating the host copy pipeline");
    }
    return OLG_OK;
}

// Streams and events are released once the work queued on them has
// completed, so this is safe right after the last enqueue.
void HostPipeline::release()
{
    cudaEvent_t *all[2 + 3 * SLOTS] = {&entry, &last};
    for (int k = 0; k < SLOTS; ++k) {
        all[2 + k] = &in[k];
        all[2 + SLOTS + k] = &done[k];
        all[2 + 2 * SLOTS + k] = &out[k];
    }
    for (cudaEvent_t *v : all)
        if (*v) {
            cudaEventDestroy(*v);
            *v = nullptr;
        }
    if (s_in) cudaStreamDestroy(s_in);
    if (s_out) cudaStreamDestroy(s_out);
    s_in = s_out = nullptr;
}

namespace {
int ck(cudaError_t e, const char *what) { return e == cudaSuccess ? OLG_OK : cuda_fail(e, what); }
} // namespace

int HostPipeline::begin(cudaStream_t st)
{
    if (int rc = ck(cudaEventRecord(entry, st), "cudaEventRecord (pipeline entry)")) return rc;
    if (int rc = ck(cudaStreamWaitEvent(s_in, entry, 0), "cudaStreamWaitEvent")) return rc;
    return ck(cudaStreamWaitEvent(s_out, entry, 0), "cudaStreamWaitEvent");
}

// slot i % 3 is free once item i - 3 has been copied out of it
int HostPipeline::copy_in_begin(int i)
{
    if (i < SLOTS) return OLG_OK;
    return ck(cudaStreamWaitEvent(s_in, out[i % SLOTS], 0), "cudaStreamWaitEvent (slot free)");
}

int HostPipeline::copy_in_end(int i, cudaStream_t st)
{
    if (int rc = ck(cudaEventRecord(in[i % SLOTS], s_in), "cudaEventRecord (copied in)")) return rc;
    return ck(cudaStreamWaitEvent(st, in[i % SLOTS], 0), "cudaStreamWaitEvent (copied in)");
}

int HostPipeline::compute_end(int i, cudaStream_t st)
{
    if (int rc = ck(cudaEventRecord(done[i % SLOTS], st), "cudaEventRecord (computed)")) return rc;
    return ck(cudaStreamWaitEvent(s_out, done[i % SLOTS], 0), "cudaStreamWaitEvent (computed)");
}

int HostPipeline::copy_out_end(int i)
{
    return ck(cudaEventRecord(out[i % SLOTS], s_out), "cudaEventRecord (copied out)");
}

void HostPipeline::drain()
{
    if (s_in) cudaStreamSynchronize(s_in);
    if (s_out) cudaStreamSynchronize(s_out);
}

// The caller's stream waited for every copy in before the computation that
// used it, so waiting for the last copy out orders everything.
int HostPipeline::end(cudaStream_t st)
{
    if (int rc = ck(cudaEventRecord(last, s_out), "cudaEventRecord (pipeline end)")) return rc;
    return ck(cudaStreamWaitEvent(st, last, 0), "cudaStreamWaitEvent (pipeline end)");
}

} // namespace olg

extern "C" int olg_inject_alloc_failures(int n)
{
    return olg::g_fail_allocs.exchange(n > 0 ? n : 0);
}

extern "C" int olg_host_device_pointer(const void *host, void **dev)
{
    if (!host || !dev) return olg::fail(OLG_ERR_INVALID_ARG, "null pointer");
    *dev = nullptr;
    cudaPointerAttributes a{};
    const cudaError_t e = cudaPointerGetAttributes(&a, host);
    if (e != cudaSuccess) return olg::cuda_fail(e, "cudaPointerGetAttributes");
    if (a.type != cudaMemoryTypeHost || !a.devicePointer)
        return olg::fail(OLG_ERR_INVALID_ARG, "not page-locked host memory mapped for the device");
    *dev = a.devicePointer;
    return OLG_OK;
}
