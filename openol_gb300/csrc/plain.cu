// plain.cu -- "plain form" GPU baselines, measured beside the fused kernels.
//
// These restate the reference's own GPU structure on this GPU, so that the
// fused kernels are compared against the straightforward form:
//  * ASM as golprop.h:507-534 does it: zero-pad kernel, cuFFT C2C forward,
//    1/Np scale, transfer function in FP32 (golprop.h:307-322), fftshift,
//    multiply, cuFFT inverse, crop -- one kernel per step (cuFFT plan and
//    buffers cached per size rather than created per call).
//  * Fresnel as golprop.h:167-198: pad, FFT, 1/Np, the sampled response
//    (FP32, golprop.h:9-30), fftshift, FFT, 1/Np, multiply, IFFT, crop.
//  * ARSS as golprop.h:941-988: windowed pre-chirp, pad, FFT, 1/Np, windowed
//    chirp, fftshift, FFT, 1/Np, multiply, IFFT, crop, windowed post-chirp.
//  * Fresnel-form CGH as gCghShared (golcgh.h:47-88): one thread per pixel,
//    points staged through shared memory, FP32 phase, full-precision sin/cos.
// Not used by any product path.
#include <cufft.h>

#include <cmath>
#include <map>
#include <mutex>

#include "common.cuh"
#include "../../include/olgb300_plain.h"

namespace olg {
namespace plain {

__global__ void k_pad(const float2 *in, float2 *out, int ny, int nx)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x, h = blockIdx.y * blockDim.y + threadIdx.y;
    const int NX = 2 * nx, NY = 2 * ny;
    if (w >= NX || h >= NY) return;
    const int oy = ny / 2, ox = nx / 2;
    float2 v = make_float2(0.f, 0.f);
    if (h >= oy && h < oy + ny && w >= ox && w < ox + nx) v = in[(size_t)(h - oy) * nx + (w - ox)];
    out[(size_t)h * NX + w] = v;
}

__global__ void k_scale(float2 *u, long n, float s)
{
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) u[i] = make_float2(u[i].x * s, u[i].y * s);
}

__global__ void k_asm_tf(float2 *H, int NY, int NX, float dv, float du, float lambda, float z)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x, h = blockIdx.y * blockDim.y + threadIdx.y;
    if (w >= NX || h >= NY) return;
    const float u = (w - NX / 2) * du, v = (h - NY / 2) * dv;
    const float ww = sqrtf(1.0f / (lambda * lambda) - u * u - v * v);
    const float ph = 2.0f * 3.14159265358979f * ww * z;
    H[(size_t)h * NX + w] = make_float2(cosf(ph), sinf(ph));
}

__global__ void k_fftshift(float2 *u, int NY, int NX)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x, h = blockIdx.y * blockDim.y + threadIdx.y;
    const int hx = NX / 2, hy = NY / 2;
    if (w >= hx || h >= hy) return;
    size_t a = (size_t)h * NX + w, b = (size_t)(h + hy) * NX + (w + hx);
    float2 t = u[a]; u[a] = u[b]; u[b] = t;
    a = (size_t)h * NX + (w + hx); b = (size_t)(h + hy) * NX + w;
    t = u[a]; u[a] = u[b]; u[b] = t;
}

__global__ void k_mult(float2 *a, const float2 *b, long n)
{
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) a[i] = cmul(a[i], b[i]);
}

__global__ void k_crop(const float2 *in, float2 *out, int ny, int nx)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x, h = blockIdx.y * blockDim.y + threadIdx.y;
    if (w >= nx || h >= ny) return;
    out[(size_t)h * nx + w] = in[(size_t)(h + ny / 2) * (2 * nx) + (w + nx / 2)];
}

__global__ void k_fresnel_h(float2 *h, int NY, int NX, float dy, float dx, float lambda, float z, float s, int lim)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x, hh = blockIdx.y * blockDim.y + threadIdx.y;
    if (w >= NX || hh >= NY) return;
    const int cy = NY / 2, cx = NX / 2;
    float2 v = make_float2(0.f, 0.f);
    if (lim < 0 || (abs(w - cx) < lim && abs(hh - cy) < lim)) {
        const float y = (hh - cy) * dy, x = (w - cx) * dx;
        const float ph = 3.14159265358979f / (lambda * z) * s * (x * x + y * y);
        v = make_float2(cosf(ph), sinf(ph));
    }
    h[(size_t)hh * NX + w] = v;
}

// ARSS pre-chirp (mode 0: zero outside its window) and post-chirp (mode 1:
// identity outside its window), in FP32 like golprop.h:817-843 / 901-922
__global__ void k_arss_chirp(const float2 *in, float2 *out, int ny, int nx, float dy, float dx, float lambda, float z,
                             float s, float oy, float ox, int hlim, int wlim, int mode)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x, h = blockIdx.y * blockDim.y + threadIdx.y;
    if (w >= nx || h >= ny) return;
    const size_t i = (size_t)h * nx + w;
    const bool inside = abs(w - nx / 2) < wlim && abs(h - ny / 2) < hlim;
    if (!inside) {
        out[i] = mode == 0 ? make_float2(0.f, 0.f) : in[i];
        return;
    }
    const float tmp = 3.14159265358979f / (lambda * z);
    const float y = (h - ny / 2) * dy, x = (w - nx / 2) * dx;
    float ph = mode == 0 ? (s * s - s) * (x * x + y * y) - 2 * s * (ox * x + oy * y)
                         : (1 - s) * (x * x + y * y) + 2 * (ox * x + oy * y) + ox * ox + oy * oy;
    ph *= tmp;
    out[i] = cmul(in[i], make_float2(cosf(ph), sinf(ph)));
}

__global__ void k_cgh_shared(const float *pts, int n, float2 *U, int ny, int nx, float p, float lambda)
{
    const int w = blockIdx.x * blockDim.x + threadIdx.x, h = blockIdx.y * blockDim.y + threadIdx.y;
    __shared__ float3 buf[256];
    float2 acc = make_float2(0.f, 0.f);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int b = 0; b < n; b += 256) {
        if (b + tid < n) buf[tid] = make_float3(pts[3 * (b + tid)], pts[3 * (b + tid) + 1], pts[3 * (b + tid) + 2]);
        __syncthreads();
        const int m = min(256, n - b);
        for (int j = 0; j < m; ++j) {
            const float dx = p * w - buf[j].x, dy = p * h - buf[j].y, dz = buf[j].z;
            const float th = 2.0f * 3.14159265f * (dx * dx + dy * dy) / (2.0f * dz * lambda);
            float s, c;
            sincosf(th, &s, &c);
            acc.x += c;
            acc.y += s;
        }
        __syncthreads();
    }
    if (w < nx && h < ny) U[(size_t)h * nx + w] = acc;
}

struct Plan {
    cufftHandle h = 0;
    float2 *b1 = nullptr, *b2 = nullptr;
};
std::mutex g_mu;
std::map<std::pair<unsigned long long, std::pair<int, int>>, Plan> g_plans; // (context, (ny, nx))

int get_plan(int ny, int nx, Plan **out)
{
    unsigned long long ctx = 0;
    if (int rc = context_id(&ctx)) return rc;
    std::lock_guard<std::mutex> lk(g_mu);
    auto key = std::make_pair(ctx, std::make_pair(ny, nx));
    auto it = g_plans.find(key);
    if (it == g_plans.end()) {
        Plan p;
        if (cufftPlan2d(&p.h, 2 * ny, 2 * nx, CUFFT_C2C) != CUFFT_SUCCESS) return fail(OLG_ERR_CUDA, "cufftPlan2d");
        const size_t bytes = (size_t)4 * ny * nx * sizeof(float2);
        cudaError_t e = cudaMalloc(&p.b1, bytes);
        if (e == cudaSuccess) e = cudaMalloc(&p.b2, bytes);
        if (e != cudaSuccess) {
            cudaFree(p.b1);
            cufftDestroy(p.h);
            return cuda_fail(e, "cudaMalloc (plain buffers)");
        }
        it = g_plans.emplace(key, p).first;
    }
    *out = &it->second;
    return OLG_OK;
}

// plain Fresnel / ARSS: the convolution form with the response's spectrum
// formed per call, as golprop.h:167-198 and 941-988 do
static int plain_conv(const void *u_in, void *u_out, int ny, int nx, double dy, double dx, double lambda, double z,
                      bool arss, double s, double oy, double ox, cudaStream_t st)
{
    Plan *P = nullptr;
    if (int rc = get_plan(ny, nx, &P)) return rc;
    if (cufftSetStream(P->h, st) != CUFFT_SUCCESS) return fail(OLG_ERR_CUDA, "cufftSetStream");
    const int NY = 2 * ny, NX = 2 * nx;
    const long Np = (long)NY * NX;
    dim3 blk(16, 16), g2((NX + 15) / 16, (NY + 15) / 16), g1((nx + 15) / 16, (ny + 15) / 16),
        gs((NX / 2 + 15) / 16, (NY / 2 + 15) / 16);
    const int lin = (int)((Np + 255) / 256);
    const float inv = (float)(1.0 / (double)Np);
    const float *src = (const float *)u_in;
    int launches = 0;
    int hlim_u = 0, wlim_u = 0, lim_h = -1, hlim_c = 0, wlim_c = 0;
    if (arss) {
        hlim_u = (int)std::floor(lambda * std::fabs(z) * 0.5 / (s * std::fabs(s - 1) * dy) / dy);
        wlim_u = (int)std::floor(lambda * std::fabs(z) * 0.5 / (s * std::fabs(s - 1) * dx) / dx);
        lim_h = (int)std::floor(std::fabs(lambda * z * 0.5 / (dx * s)) / dx);
        hlim_c = (int)std::floor(lambda * std::fabs(z) * 0.5 / (std::fabs(1 - s) * dy) / dy);
        wlim_c = (int)std::floor(lambda * std::fabs(z) * 0.5 / (std::fabs(1 - s) * dx) / dx);
        // the pre-chirp goes to the output field first (udst in the reference)
        k_arss_chirp<<<g1, blk, 0, st>>>((const float2 *)u_in, (float2 *)u_out, ny, nx, (float)dy, (float)dx,
                                         (float)lambda, (float)z, (float)s, (float)oy, (float)ox, hlim_u, wlim_u, 0);
        ++launches;
        src = (const float *)u_out;
    }
    k_pad<<<g2, blk, 0, st>>>((const float2 *)src, P->b1, ny, nx);
    if (cufftExecC2C(P->h, (cufftComplex *)P->b1, (cufftComplex *)P->b1, CUFFT_FORWARD) != CUFFT_SUCCESS)
        return fail(OLG_ERR_CUDA, "cufftExecC2C");
    k_scale<<<lin, 256, 0, st>>>(P->b1, Np, inv);
    k_fresnel_h<<<g2, blk, 0, st>>>(P->b2, NY, NX, (float)dy, (float)dx, (float)lambda, (float)z,
                                    arss ? (float)s : 1.0f, lim_h);
    k_fftshift<<<gs, blk, 0, st>>>(P->b2, NY, NX);
    if (cufftExecC2C(P->h, (cufftComplex *)P->b2, (cufftComplex *)P->b2, CUFFT_FORWARD) != CUFFT_SUCCESS)
        return fail(OLG_ERR_CUDA, "cufftExecC2C");
    k_scale<<<lin, 256, 0, st>>>(P->b2, Np, inv);
    k_mult<<<lin, 256, 0, st>>>(P->b1, P->b2, Np);
    if (cufftExecC2C(P->h, (cufftComplex *)P->b1, (cufftComplex *)P->b1, CUFFT_INVERSE) != CUFFT_SUCCESS)
        return fail(OLG_ERR_CUDA, "cufftExecC2C");
    k_crop<<<g1, blk, 0, st>>>(P->b1, (float2 *)u_out, ny, nx);
    launches += 7;
    if (arss) {
        k_arss_chirp<<<g1, blk, 0, st>>>((const float2 *)u_out, (float2 *)u_out, ny, nx, (float)dy, (float)dx,
                                         (float)lambda, (float)z, (float)s, (float)oy, (float)ox, hlim_c, wlim_c, 1);
        ++launches;
    }
    count_launch(launches);
    return check_launch("plain convolution propagation");
}

} // namespace plain
} // namespace olg

using namespace olg;
using namespace olg::plain;

extern "C" int olg_plain_asm_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx,
                                      double lambda, double z, olg_stream_t stream)
{
    if (!u_in || !u_out || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad arguments");
    Plan *P = nullptr;
    if (int rc = get_plan(ny, nx, &P)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (cufftSetStream(P->h, st) != CUFFT_SUCCESS) return fail(OLG_ERR_CUDA, "cufftSetStream");
    const int NY = 2 * ny, NX = 2 * nx;
    const long Np = (long)NY * NX;
    dim3 blk(16, 16), g2((NX + 15) / 16, (NY + 15) / 16), g1((nx + 15) / 16, (ny + 15) / 16),
        gs((NX / 2 + 15) / 16, (NY / 2 + 15) / 16);
    const int lin = (int)((Np + 255) / 256);
    k_pad<<<g2, blk, 0, st>>>((const float2 *)u_in, P->b1, ny, nx);
    if (cufftExecC2C(P->h, (cufftComplex *)P->b1, (cufftComplex *)P->b1, CUFFT_FORWARD) != CUFFT_SUCCESS)
        return fail(OLG_ERR_CUDA, "cufftExecC2C");
    k_scale<<<lin, 256, 0, st>>>(P->b1, Np, (float)(1.0 / (double)Np));
    k_asm_tf<<<g2, blk, 0, st>>>(P->b2, NY, NX, (float)(1.0 / (dy * NY)), (float)(1.0 / (dx * NX)), (float)lambda,
                                 (float)z);
    k_fftshift<<<gs, blk, 0, st>>>(P->b2, NY, NX);
    k_mult<<<lin, 256, 0, st>>>(P->b1, P->b2, Np);
    if (cufftExecC2C(P->h, (cufftComplex *)P->b1, (cufftComplex *)P->b1, CUFFT_INVERSE) != CUFFT_SUCCESS)
        return fail(OLG_ERR_CUDA, "cufftExecC2C");
    k_crop<<<g1, blk, 0, st>>>(P->b1, (float2 *)u_out, ny, nx);
    count_launch(6);
    return check_launch("plain asm");
}

extern "C" int olg_plain_cgh_fresnel_c64(const float *points, int n_points, void *U, int ny, int nx, double p,
                                         double lambda, olg_stream_t stream)
{
    if (!points || !U || ny <= 0 || nx <= 0 || n_points < 0) return fail(OLG_ERR_INVALID_ARG, "bad arguments");
    dim3 blk(16, 16), g((nx + 15) / 16, (ny + 15) / 16);
    k_cgh_shared<<<g, blk, 0, (cudaStream_t)stream>>>(points, n_points, (float2 *)U, ny, nx, (float)p, (float)lambda);
    count_launch();
    return check_launch("plain cgh");
}

extern "C" int olg_plain_fresnel_prop_c64(const void *u_in, void *u_out, int ny, int nx, double dy, double dx,
                                          double lambda, double z, olg_stream_t stream)
{
    if (!u_in || !u_out || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad arguments");
    return plain_conv(u_in, u_out, ny, nx, dy, dx, lambda, z, false, 1.0, 0.0, 0.0, (cudaStream_t)stream);
}

extern "C" int olg_plain_arss_prop_c64(const void *u_src, void *u_dst, int ny, int nx, double dy, double dx,
                                       double lambda, double z, double s, double oy, double ox, olg_stream_t stream)
{
    if (!u_src || !u_dst || ny <= 0 || nx <= 0 || s == 0.0 || s == 1.0) return fail(OLG_ERR_INVALID_ARG, "bad arguments");
    if (u_src == u_dst) return fail(OLG_ERR_INVALID_ARG, "plain ARSS writes its pre-chirp into u_dst: u_src != u_dst");
    return plain_conv(u_src, u_dst, ny, nx, dy, dx, lambda, z, true, s, oy, ox, (cudaStream_t)stream);
}
