/*
 * golprop.h (drop-in) -- the reference's GPU propagation templates
 * (include/golprop.h) with the same names and signatures, forwarding to
 * libolgb300.so (include/olgb300.h).  Like the reference wrappers, each call
 * returns with the device synchronised; errors throw std::runtime_error (the
 * reference's CHECK_CUDA_ERROR behaviour) instead of passing silently.
 * Fields are complex64 (thrust::complex<float>).  AsmPropCheck /
 * FresnelPropCheck live in olprop.h, as in the reference; Prop evaluates them
 * through olg_asm_prop_check / olg_fresnel_prop_check in PREC_T precision.
 */
#ifndef OLGB300_GOLPROP_H
#define OLGB300_GOLPROP_H
#include <thrust/complex.h>

#include <complex>
#include <cstdio>
#include <string>
#include <type_traits>

#include "../olgb300.h"
#include "golclass.h"
#include "oldefine.h"
#include "olprop.h"

namespace ol {

// device overload, golprop.h:507-534
template <typename COMPLEX_T, typename PREC_T>
void gAsmProp(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T dy, PREC_T dx, PREC_T lambda,
              PREC_T d)
{
    olgb::complex64_only<COMPLEX_T>();
    olgb::check(olg_asm_prop_c64(u.get(), u.get(), ny, nx, dy, dx, lambda, d, 0, nullptr, 0, nullptr), "gAsmProp");
    olgb::sync("gAsmProp");
}

// host overload (no 1/Np), golprop.h:458-504
template <typename COMPLEX_T, typename PREC_T>
void gAsmProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T dy, PREC_T dx, PREC_T lambda,
              PREC_T d)
{
    olgb::host_field(u, ny, nx, [&](void *p) {
        olgb::check(olg_asm_prop_c64(p, p, ny, nx, dy, dx, lambda, d, OLG_NO_NORMALIZE, nullptr, 0, nullptr), "gAsmProp");
    });
}

// device overload, golprop.h:167-198
template <typename COMPLEX_T, typename PREC_T>
void gFresnelProp(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T dy, PREC_T dx,
                  PREC_T lambda, PREC_T d)
{
    olgb::complex64_only<COMPLEX_T>();
    olgb::check(olg_fresnel_prop_c64(u.get(), u.get(), ny, nx, dy, dx, lambda, d, 0, 0, nullptr, 0, nullptr),
                "gFresnelProp");
    olgb::sync("gFresnelProp");
}

// host overload, golprop.h:70-124
template <typename COMPLEX_T, typename PREC_T>
void gFresnelProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T dy, PREC_T dx, PREC_T lambda,
                  PREC_T d)
{
    olgb::host_field(u, ny, nx, [&](void *p) {
        olgb::check(olg_fresnel_prop_c64(p, p, ny, nx, dy, dx, lambda, d, 0, OLG_NO_NORMALIZE, nullptr, 0, nullptr),
                    "gFresnelProp");
    });
}

// golprop.h:278-302
template <typename COMPLEX_T, typename PREC_T>
void gFresnelPropBandLimit(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T dy, PREC_T dx,
                           PREC_T lambda, PREC_T d)
{
    olgb::complex64_only<COMPLEX_T>();
    olgb::check(olg_fresnel_prop_c64(u.get(), u.get(), ny, nx, dy, dx, lambda, d, 1, 0, nullptr, 0, nullptr),
                "gFresnelPropBandLimit");
    olgb::sync("gFresnelPropBandLimit");
}

// golprop.h:941-988
template <typename PREC_T = float, typename COMPLEX_T>
void ARSSFresnelProp(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &usrc,
                     cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &udst, int ny, int nx, PREC_T dy, PREC_T dx,
                     PREC_T lambda, PREC_T z, PREC_T s, PREC_T oy, PREC_T ox)
{
    olgb::complex64_only<COMPLEX_T>();
    if (!udst) udst = cuda::make_unique<thrust::complex<COMPLEX_T>[]>((size_t)ny * nx);
    olgb::check(olg_arss_prop_c64(usrc.get(), udst.get(), ny, nx, dy, dx, lambda, z, s, oy, ox, 0, nullptr, 0, nullptr),
                "ARSSFresnelProp");
    olgb::sync("ARSSFresnelProp");
}

// golprop.h:990-995
template <typename PREC_T = float, typename COMPLEX_T>
void ARSSFresnelProp(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &usrc,
                     cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &udst, int ny, int nx, PREC_T dy, PREC_T dx,
                     PREC_T lambda, PREC_T z, PREC_T s)
{
    ARSSFresnelProp(usrc, udst, ny, nx, dy, dx, lambda, z, s, (PREC_T)0, (PREC_T)0);
}

// gshiftedAsmProp, golprop.h:537-575 (no band window, 1/Np)
template <typename COMPLEX_T, typename PREC_T>
void gshiftedAsmProp(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &usrc,
                     cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &udst, int ny, int nx, PREC_T dy, PREC_T dx,
                     PREC_T lambda, PREC_T d, PREC_T oy, PREC_T ox)
{
    olgb::complex64_only<COMPLEX_T>();
    if (!udst) udst = cuda::make_unique<thrust::complex<COMPLEX_T>[]>((size_t)ny * nx);
    olgb::check(olg_shifted_asm_prop_c64(usrc.get(), udst.get(), ny, nx, dy, dx, lambda, d, oy, ox, 0, nullptr, 0,
                                         nullptr),
                "gshiftedAsmProp");
    olgb::sync("gshiftedAsmProp");
}

// gshiftedFresnelProp, golprop.h:706-752
template <typename PREC_T = float, typename COMPLEX_T>
void gshiftedFresnelProp(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &usrc,
                         cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &udst, int ny, int nx, PREC_T dy, PREC_T dx,
                         PREC_T lambda, PREC_T z, PREC_T s, PREC_T oy, PREC_T ox)
{
    olgb::complex64_only<COMPLEX_T>();
    if (!udst) udst = cuda::make_unique<thrust::complex<COMPLEX_T>[]>((size_t)ny * nx);
    olgb::check(olg_shifted_fresnel_prop_c64(usrc.get(), udst.get(), ny, nx, dy, dx, lambda, z, s, oy, ox, 0, nullptr,
                                             0, nullptr),
                "gshiftedFresnelProp");
    olgb::sync("gshiftedFresnelProp");
}

// shiftedProp, golprop.h:755-768 (an invalid mode throws where the reference exits)
template <typename COMPLEX_T, typename PREC_T>
void shiftedProp(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &usrc, cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &udst,
                 int ny, int nx, PREC_T dy, PREC_T dx, PREC_T lambda, PREC_T d, PREC_T oy, PREC_T ox,
                 PROPMODE propmode)
{
    olgb::complex64_only<COMPLEX_T>();
    if (!udst) udst = cuda::make_unique<thrust::complex<COMPLEX_T>[]>((size_t)ny * nx);
    const int mode = propmode == PROPMODE::ASM ? OLG_ASM : propmode == PROPMODE::FRESNEL ? OLG_FRESNEL : -1;
    olgb::check(olg_shifted_prop_c64(usrc.get(), udst.get(), ny, nx, dy, dx, lambda, d, oy, ox, mode, 0, nullptr, 0,
                                     nullptr),
                "shiftedProp");
    olgb::sync("shiftedProp");
}

// gsplitProp, golprop.h:772-813: a host field; every block pair runs on the GPU
template <typename PREC_T = float, typename COMPLEX_T>
void gsplitProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int64_t height, int64_t width, PREC_T dy, PREC_T dx,
                PREC_T lambda, PREC_T z, PROPMODE propmode, int blocknum_y = 2, int blocknum_x = 2)
{
    olgb::complex64_only<COMPLEX_T>();
    const int mode = propmode == PROPMODE::ASM ? OLG_ASM : propmode == PROPMODE::FRESNEL ? OLG_FRESNEL : -1;
    const size_t bytes = sizeof(std::complex<float>) * (size_t)height * width;
    void *a = nullptr, *b = nullptr;
    CHECK_CUDA_ERROR(cudaMalloc(&a, bytes));
    CHECK_CUDA_ERROR(cudaMalloc(&b, bytes));
    CHECK_CUDA_ERROR(cudaMemcpy(a, u.get(), bytes, cudaMemcpyHostToDevice));
    const int rc = olg_split_prop_c64(a, b, (int)height, (int)width, dy, dx, lambda, z, mode, blocknum_y, blocknum_x, 0,
                                      nullptr, 0, nullptr);
    if (rc == OLG_OK) CHECK_CUDA_ERROR(cudaMemcpy(u.get(), b, bytes, cudaMemcpyDeviceToHost));
    CHECK_CUDA_ERROR(cudaFree(a));
    CHECK_CUDA_ERROR(cudaFree(b));
    olgb::check(rc, "gsplitProp");
}

// TiltedSourceProp / TiltedReferenceProp on device fields (the host-field
// overloads of olprop.h:414-600 are in olprop.h), in place
template <typename PREC_T = float, typename COMPLEX_T>
void TiltedSourceProp(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T dy, PREC_T dx,
                      PREC_T lambda, PREC_T z, PREC_T angle_src2dst, INTERPOLATION inp = BILINEAR,
                      PROPMODE propmode = ASM)
{
    olgb::complex64_only<COMPLEX_T>();
    olgb::check(olg_tilted_prop_c64(u.get(), u.get(), ny, nx, dy, dx, lambda, z, angle_src2dst, (int)inp,
                                    olgb::tilt_mode(propmode), 0, nullptr, 0, nullptr),
                "TiltedSourceProp");
    olgb::sync("TiltedSourceProp");
}

template <typename PREC_T = float, typename COMPLEX_T>
void TiltedReferenceProp(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &u, int64_t ny, int64_t nx, PREC_T dy,
                         PREC_T dx, PREC_T lambda, PREC_T z, PREC_T rotate, INTERPOLATION inp = BILINEAR,
                         PROPMODE propmode = ASM)
{
    olgb::complex64_only<COMPLEX_T>();
    olgb::check(olg_tilted_prop_c64(u.get(), u.get(), (int)ny, (int)nx, dy, dx, lambda, z, rotate, (int)inp,
                                    olgb::tilt_mode(propmode), 1, nullptr, 0, nullptr),
                "TiltedReferenceProp");
    olgb::sync("TiltedReferenceProp");
}

// golprop.h:578-604 (prints the chosen method, as the reference does)
template <typename COMPLEX_T, typename PREC_T>
void Prop(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T dy, PREC_T dx, PREC_T lambda,
          PREC_T d, PROPMODE propmode = PROPMODE::AUTO)
{
    olgb::complex64_only<COMPLEX_T>();
    const int mode = propmode == PROPMODE::ASM ? OLG_ASM : propmode == PROPMODE::FRESNEL ? OLG_FRESNEL : OLG_AUTO;
    const int flags = OLG_VERBOSE | (std::is_same<PREC_T, float>::value ? OLG_CHECK_F32 : 0);
    olgb::check(olg_prop_c64(u.get(), ny, nx, dy, dx, lambda, d, mode, flags, nullptr, nullptr, 0, nullptr), "Prop");
    olgb::sync("Prop");
}
} // namespace ol
#endif
