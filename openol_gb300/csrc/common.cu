// common.cu -- library-wide host helpers: status strings, per-thread error
// messages, launch counter, stream-ordered scratch.
#include <atomic>
#include <cstdio>
#include <string>

#include <mutex>

#include "common.cuh"

namespace olg {

static thread_local std::string t_err;
static std::atomic<unsigned long long> g_launches{0};

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

// The library's own stream-ordered pool per device.  It keeps up to 8 GiB of
// freed scratch mapped between calls: the default pool returns everything at
// each synchronisation, and re-mapping a few hundred MB per call (the WRP pair
// lists) cost more than the kernels that use it.  Leaves the device's default
// pool untouched.
static cudaMemPool_t scratch_pool()
{
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[dev]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        if (cudaMemPoolCreate(&p, &props) == cudaSuccess) {
            unsigned long long keep = 8ull << 30;
            cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
            pools[dev] = p;
        } else if (cudaDeviceGetDefaultMemPool(&p, dev) == cudaSuccess) {
            pools[dev] = p;
        }
    }
    return pools[dev];
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
    cudaError_t e = cudaMallocFromPoolAsync(&ptr, need, scratch_pool(), s);
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
