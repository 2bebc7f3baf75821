/*
 * olcgh.h (drop-in) -- the reference's CPU point-cloud CGH templates
 * (include/olcgh.h: ol::Cgh and the CPU ol::WRPStep1) for host point clouds
 * and host holograms, with the same names and signatures, computed on the
 * GPU by libolgb300.so (include/olgb300.h).
 *
 * Precision: the reference sums in PREC_T (double for its accuracy checks).
 * Here the points are rounded to float32 (ol::Vect3<float>, the GPU path's
 * point type) and the hologram is summed in FP32 with double-float phase
 * anchors (direct kernel) or as a split-FP16 tensor-core GEMM from 1024
 * points up; both keep relative L2 within 1e-5 of the FP64 sum on float32
 * points.  The result is widened to the caller's COMPLEX_T / PHASE_T.
 *
 * Each call copies the points in and the hologram out, and returns with the
 * device synchronised; errors throw std::runtime_error.
 */
#ifndef OLGB300_OLCGH_H
#define OLGB300_OLCGH_H
#include <cmath>
#include <complex>
#include <memory>
#include <stdexcept>
#include <type_traits>
#include <vector>

#include "../olgb300.h"
#include "golclass.h"
#include "olclass.h"
#include "olprop.h"

namespace ol {
namespace olgb {
constexpr int kHostTensorMinPoints = 1024;

// float32 AoS device copy of a host point cloud of any Vect3<_Tp>
template <typename _Tp>
cuda::unique_ptr<float[]> points_to_device(Object<_Tp> &obj)
{
    const size_t n = (size_t)obj.size;
    auto d = cuda::make_unique<float[]>(3 * (n ? n : 1));
    std::vector<float> h(3 * n);
    for (size_t j = 0; j < n; ++j) {
        h[3 * j] = (float)obj[(int)j].x;
        h[3 * j + 1] = (float)obj[(int)j].y;
        h[3 * j + 2] = (float)obj[(int)j].z;
    }
    if (n) CHECK_CUDA_ERROR(cudaMemcpy(d.get(), h.data(), 3 * n * sizeof(float), cudaMemcpyHostToDevice));
    return d;
}

// Fresnel-form hologram of a host cloud into a device complex64 buffer
// (U != nullptr) and/or a device float phase buffer (phase != nullptr)
template <typename _Tp>
void host_cgh(Object<_Tp> &obj, void *U, float *phase, int ny, int nx, double py, double px, double lambda)
{
    auto pts = points_to_device(obj);
    if (!phase && obj.size >= kHostTensorMinPoints && ny <= 4096 && nx <= 4096)
        check(olg_cgh_fresnel_gemm_c64(pts.get(), nullptr, nullptr, obj.size, U, ny, nx, py, px, lambda, 0, nullptr, 0,
                                       nullptr),
              "Cgh");
    else
        check(olg_cgh_fresnel_c64(pts.get(), nullptr, nullptr, obj.size, U, phase, ny, nx, py, px, lambda, 0, nullptr),
              "Cgh");
    sync("Cgh");
}

template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void cgh_complex(Object<_Tp> &obj, std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T py, PREC_T px,
                 PREC_T lambda)
{
    const size_t n = (size_t)ny * (size_t)nx;
    auto d = cuda::make_unique<std::complex<float>[]>(n);
    host_cgh(obj, d.get(), nullptr, ny, nx, py, px, lambda);
    if (!u) u = std::make_unique<std::complex<COMPLEX_T>[]>(n);
    to_host(u.get(), d.get(), n);
}

template <typename _Tp, typename PHASE_T, typename PREC_T>
void cgh_phase(Object<_Tp> &obj, std::unique_ptr<PHASE_T[]> &phase, int ny, int nx, PREC_T py, PREC_T px,
               PREC_T lambda)
{
    const size_t n = (size_t)ny * (size_t)nx;
    auto d = cuda::make_unique<float[]>(n);
    host_cgh(obj, nullptr, d.get(), ny, nx, py, px, lambda);
    std::vector<float> h(n);
    CHECK_CUDA_ERROR(cudaMemcpy(h.data(), d.get(), n * sizeof(float), cudaMemcpyDeviceToHost));
    if (!phase) phase = std::make_unique<PHASE_T[]>(n);
    for (size_t i = 0; i < n; ++i) phase[i] = (PHASE_T)h[i];
}
} // namespace olgb

// phase output, one pitch: ol::Cgh olcgh.h:351-359 (_CghFresnel olcgh.h:276-295).
// normalized = true names _CghFresnelNormalized, which the reference leaves
// commented out (olcgh.h:111-130); it throws here.
template <typename _Tp, typename PHASE_T, typename PREC_T>
void Cgh(Object<_Tp> &obj, std::unique_ptr<PHASE_T[]> &phase, int ny, int nx, PREC_T p, PREC_T lambda,
         bool normalized = false)
{
    if (normalized) throw std::runtime_error("Cgh: the normalized form has no implementation in the reference");
    olgb::cgh_phase(obj, phase, ny, nx, p, p, lambda);
}

// phase output, pitches py, px: olcgh.h:361-366
template <typename _Tp, typename PHASE_T, typename PREC_T>
void Cgh(Object<_Tp> &obj, std::unique_ptr<PHASE_T[]> &phase, int ny, int nx, PREC_T py, PREC_T px, PREC_T lambda)
{
    olgb::cgh_phase(obj, phase, ny, nx, py, px, lambda);
}

// complex output, one pitch: olcgh.h:368-373 (_CghFresnel olcgh.h:297-313)
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void Cgh(Object<_Tp> &obj, std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T p, PREC_T lambda)
{
    olgb::cgh_complex(obj, u, ny, nx, p, p, lambda);
}

// complex output, pitches py, px: olcgh.h:375-379
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void Cgh(Object<_Tp> &obj, std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T py, PREC_T px,
         PREC_T lambda)
{
    olgb::cgh_complex(obj, u, ny, nx, py, px, lambda);
}

// The CPU ol::WRPStep1, olcgh.h:381-398: despite its name it is the full
// Fresnel sum with dz = z_j (no window, no plane; d is unused there too), so
// it is the one-pitch complex Cgh.
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void WRPStep1(Object<_Tp> &obj, std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T p, PREC_T lambda,
              PREC_T d)
{
    (void)d;
    olgb::cgh_complex(obj, u, ny, nx, p, p, lambda);
}
} // namespace ol
#endif
