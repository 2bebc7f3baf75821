// noalloc.cu -- the ASM propagation entry point that allocates nothing
// (olg_asm_prop_noalloc_c64): its scratch is an array compiled into the library.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "common.cuh"
#include "prophost.cuh"

using namespace olg;

// ------------------------------------------------------- no-allocation entry
// Scratch for olg_asm_prop_noalloc_c64, owned by the library module itself:
// 17 MiB per device, enough for any field with ny * nx <= 1,048,576
// (1024 x 1024, 512 x 2048, ...).  Every device that loads the library keeps
// this array until the process exits.
namespace {
constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)17 << 20;
constexpr long NOALLOC_MAX_PIXELS = 1L << 20;
std::mutex g_noalloc_mu;
std::map<unsigned long long, void *> g_noalloc_ptr; // per context
} // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch in the current context.  The name
// g_noalloc_scratch in host code is only a host-side handle for the symbol,
// so the address is looked up with the device current, once per context (a
// device reset gives a new context, and the array may then sit elsewhere),
// and cached; kernels receive this pointer like any caller-provided workspace.
static int noalloc_scratch(void **out)
{
    unsigned long long ctx = 0;
    if (int rc = context_id(&ctx)) return rc;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    auto it = g_noalloc_ptr.find(ctx);
    if (it == g_noalloc_ptr.end()) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        it = g_noalloc_ptr.emplace(ctx, p).first;
    }
    *out = it->second;
    return OLG_OK;
}

extern "C" int olg_asm_prop_noalloc_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx,
                                        double lambda, double z, int flags, olg_stream_t stream)
{
    if (int rc = validate(u_in, u_out, ny, nx)) return rc;
    // mixed-radix lengths allocate their twiddle table on first use
    if (!is_pow2(ny) || !is_pow2(nx))
        return fail(OLG_ERR_UNSUPPORTED_SIZE, "olg_asm_prop_noalloc_c64 takes power-of-two ny, nx in [16, 4096]");
    if ((long)ny * (long)nx > NOALLOC_MAX_PIXELS)
        return fail(OLG_ERR_WORKSPACE, "olg_asm_prop_noalloc_c64: ny * nx must be <= 1048576; use "
                                       "olg_asm_prop_c64 with a workspace for larger fields");
    if (layout_bytes(ny, nx, nullptr, nullptr) > NOALLOC_SCRATCH_BYTES)
        return fail(OLG_ERR_WORKSPACE, "olg_asm_prop_noalloc_c64: this shape's scratch exceeds the 17 MiB static "
                                       "array; use olg_asm_prop_c64 with a workspace");
    void *scratch = nullptr;
    if (int rc = noalloc_scratch(&scratch)) return rc;
    // Pass 1 writes every element of the scratch spectrum before passes 2 and 3
    // read it, so the previous call's contents never leak into this one and
    // nothing needs clearing.
    return olg_asm_prop_c64(u_in, u_out, ny, nx, dy, dx, lambda, z, flags, scratch, NOALLOC_SCRATCH_BYTES, stream);
}
