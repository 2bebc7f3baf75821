// quant.cu -- 8-bit hologram quantisers on GB300 (sm_103a).
//
// complex2img (olimg.h:348-391): per-pixel value (phase, real, imaginary or
// amplitude), min-max normalisation (phase: fixed -pi..pi), round to 0..255.
// Values are computed in FP32 from the complex64 field; a pixel can differ by
// one level from the FP64 reference only where 255 (v - min) / (max - min)
// lies within FP32 rounding of a .5 boundary.
#include <cmath>

#include "common.cuh"

namespace olg {

__device__ __forceinline__ float q_value(float2 u, int mode)
{
    switch (mode) {
    case OLG_REAL: return u.x;
    case OLG_IMAG: return u.y;
    case OLG_AMP: return sqrtf(u.x * u.x + u.y * u.y);
    default: return atan2f(u.y, u.x);
    }
}

// order-preserving float <-> int mapping for atomic min / max
__device__ __forceinline__ int f2o(float f)
{
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float o2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__global__ void k_q_init(int *mm)
{
    mm[0] = 0x7fffffff;
    mm[1] = (int)0x80000000;
}

__global__ void k_q_minmax(const float2 *u, long n, int mode, int *mm)
{
    float mn = INFINITY, mx = -INFINITY;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float v = q_value(u[i], mode);
        mn = fminf(mn, v);
        mx = fmaxf(mx, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mm, f2o(mn));
        atomicMax(mm + 1, f2o(mx));
    }
}

__global__ void k_q_apply(const float2 *u, uint8_t *img, long n, int mode, const int *mm)
{
    float mn, mx;
    if (mode == OLG_PHASE) {
        mn = -3.14159265358979323846f;
        mx = 3.14159265358979323846f;
    } else {
        mn = o2f(mm[0]);
        mx = o2f(mm[1]);
    }
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float v = q_value(u[i], mode);
        img[i] = (mx == mn) ? 0 : (uint8_t)roundf((255.0f * (v - mn)) / (mx - mn));
    }
}

__global__ void k_binarize(const float2 *u, uint8_t *img, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        img[i] = u[i].x >= 0.0f ? 255 : 0;
}

static int grid_for(long n)
{
    long g = (n + 255) / 256;
    const long cap = 16L * sm_count(); // grid-stride beyond sixteen CTAs per SM
    return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

} // namespace olg

using namespace olg;

extern "C" int olg_complex2img_u8(const void *u, uint8_t *img, int ny, int nx, int mode, olg_stream_t stream)
{
    if (!u || !img || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad arguments");
    if (mode < OLG_PHASE || mode > OLG_AMP) return fail(OLG_ERR_INVALID_ARG, "bad MODE");
    cudaStream_t st = (cudaStream_t)stream;
    const long n = (long)ny * nx;
    Scratch sc;
    if (int rc = sc.acquire(nullptr, 0, 256, st)) return rc;
    int *mm = (int *)sc.ptr;
    if (mode != OLG_PHASE) {
        k_q_init<<<1, 1, 0, st>>>(mm);
        k_q_minmax<<<grid_for(n), 256, 0, st>>>((const float2 *)u, n, mode, mm);
        count_launch(2);
        if (int rc = check_launch("k_q_minmax")) return rc;
    }
    k_q_apply<<<grid_for(n), 256, 0, st>>>((const float2 *)u, img, n, mode, mm);
    count_launch();
    return check_launch("k_q_apply");
}

extern "C" int olg_binarize_u8(const void *u, uint8_t *img, int ny, int nx, olg_stream_t stream)
{
    if (!u || !img || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad arguments");
    const long n = (long)ny * nx;
    k_binarize<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((const float2 *)u, img, n);
    count_launch();
    return check_launch("k_binarize");
}
