/*
 * golcgh.h (drop-in) -- the reference's GPU CGH / WRP templates
 * (include/golcgh.h) with the same names and signatures, forwarding to
 * libolgb300.so.  gCgh runs the Fresnel-form sum on the tensor cores
 * (split-FP16 GEMM) from 1024 points up, on the FP32 direct kernel below.
 * Calls return synchronised; errors throw std::runtime_error.
 */
#ifndef OLGB300_GOLCGH_H
#define OLGB300_GOLCGH_H
#include <thrust/complex.h>

#include <type_traits>

#include "golprop.h"

namespace ol {
namespace olgb {
constexpr int kTensorMinPoints = 1024;
template <typename PREC_T>
constexpr void float_points()
{
    static_assert(std::is_same<PREC_T, float>::value, "libolgb300 takes ol::gObject<float> point clouds");
}
inline void cgh(const void *pts, int n, void *U, float *phase, int ny, int nx, double py, double px, double lambda,
                int flags)
{
    if (!phase && n >= kTensorMinPoints && ny <= 4096 && nx <= 4096)
        check(olg_cgh_fresnel_gemm_c64((const float *)pts, nullptr, nullptr, n, U, ny, nx, py, px, lambda, flags, nullptr,
                                       0, nullptr),
              "gCgh");
    else
        check(olg_cgh_fresnel_c64((const float *)pts, nullptr, nullptr, n, U, phase, ny, nx, py, px, lambda, flags,
                                  nullptr),
              "gCgh");
    sync("gCgh");
}
} // namespace olgb

// complex output, gCghShared (golcgh.h:137-145)
template <typename PREC_T, typename _Tp>
void gCgh(gObject<PREC_T> &gobj, cuda::unique_ptr<_Tp[]> &U, int ny, int nx, PREC_T p, PREC_T lambda)
{
    olgb::float_points<PREC_T>();
    static_assert(std::is_same<_Tp, thrust::complex<float>>::value, "complex64 hologram");
    olgb::cgh(gobj.points.get(), gobj.size, U.get(), nullptr, ny, nx, p, p, lambda, 0);
}

// complex or phase output with separate pitches (golcgh.h:26-45, 108-135)
template <typename PREC_T, typename _Tp>
void gCgh(gObject<PREC_T> &gobj, cuda::unique_ptr<_Tp[]> &U, int ny, int nx, PREC_T py, PREC_T px, PREC_T lambda)
{
    olgb::float_points<PREC_T>();
    if constexpr (std::is_same<_Tp, float>::value)
        olgb::cgh(gobj.points.get(), gobj.size, nullptr, U.get(), ny, nx, py, px, lambda, 0);
    else
        olgb::cgh(gobj.points.get(), gobj.size, U.get(), nullptr, ny, nx, py, px, lambda, 0);
}

// U += hologram, golcgh.h:177-195
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void gCghReduction(gObject<_Tp> &obj, cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &U, int ny, int nx, PREC_T p,
                   PREC_T lambda)
{
    olgb::float_points<_Tp>();
    olgb::cgh(obj.points.get(), obj.size, U.get(), nullptr, ny, nx, p, p, lambda, OLG_ACCUMULATE);
}

// golcgh.h:369-389
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void WRPStep1(gObject<_Tp> &obj, cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &U, int ny, int nx, PREC_T p,
              PREC_T lambda, PREC_T d, PREC_T plimit = 0)
{
    olgb::float_points<_Tp>();
    olgb::check(olg_wrp_step1_c64((const float *)obj.points.get(), obj.size, U.get(), ny, nx, p, lambda, d, plimit,
                                  OLG_WINDOW_CIRCLE, nullptr),
                "WRPStep1");
    olgb::sync("WRPStep1");
}

// golcgh.h:470-491
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void WRPStep1_D(gObject<_Tp> &obj, cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &U, int ny, int nx, PREC_T p,
                PREC_T lambda, PREC_T d, PREC_T plimit = 0)
{
    olgb::float_points<_Tp>();
    olgb::check(olg_wrp_step1_c64((const float *)obj.points.get(), obj.size, U.get(), ny, nx, p, lambda, d, plimit,
                                  OLG_WINDOW_SQUARE, nullptr),
                "WRPStep1_D");
    olgb::sync("WRPStep1_D");
}

// golcgh.h:494-517: propagate the WRP by d.  AUTO takes gAsmProp when
// AsmPropCheck passes; otherwise gFresnelProp when FresnelPropCheck passes,
// else gAsmProp after a warning (not the band-limited Fresnel of Prop).
// Prints the choice like the reference.
template <typename COMPLEX_T, typename PREC_T>
void WRPStep2(cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &U, int ny, int nx, PREC_T p, PREC_T lambda, PREC_T d,
              PROPMODE propmode = PROPMODE::AUTO)
{
    if (propmode == PROPMODE::FRESNEL) {
        gFresnelProp(U, ny, nx, p, p, lambda, d);
    } else if (propmode == PROPMODE::ASM) {
        gAsmProp(U, ny, nx, p, p, lambda, d);
    } else if (propmode == PROPMODE::AUTO) {
        if (AsmPropCheck(ny, nx, p, p, lambda, d)) {
            std::printf("WRP Step2 is AsmProp\n");
            gAsmProp(U, ny, nx, p, p, lambda, d);
        } else if (!FresnelPropCheck(ny, nx, p, p, lambda, d)) {
            std::printf("warning!!\neither AsmProp or FresnelProp does not meet the condition.\n");
            gAsmProp(U, ny, nx, p, p, lambda, d);
        } else {
            std::printf("WRP Step2 is FresnelProp\n");
            gFresnelProp(U, ny, nx, p, p, lambda, d);
        }
    }
}

namespace olgb {
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void wrp_method(gObject<_Tp> &obj, cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &U, int ny, int nx, PREC_T p,
                PREC_T lambda, PREC_T zmin, PREC_T plimit, float s, PROPMODE pm, int window)
{
    float_points<_Tp>();
    const int mode = pm == PROPMODE::ASM ? OLG_ASM : pm == PROPMODE::FRESNEL ? OLG_FRESNEL : OLG_AUTO;
    check(olg_wrp_method_c64((const float *)obj.points.get(), obj.size, U.get(), ny, nx, p, lambda, zmin, s, plimit,
                             window, mode, OLG_VERBOSE, nullptr, nullptr),
          "WRPMethod");
    sync("WRPMethod");
}
} // namespace olgb

// golcgh.h:561-581
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void WRPMethod(gObject<_Tp> &obj, cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &U, int ny, int nx, PREC_T p,
               PREC_T lambda, PREC_T zmin, float s = 0.9, PROPMODE propmode = PROPMODE::AUTO)
{
    olgb::wrp_method(obj, U, ny, nx, p, lambda, zmin, (PREC_T)0, s, propmode, OLG_WINDOW_CIRCLE);
}

// golcgh.h:519-538
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void WRPMethod_D(gObject<_Tp> &obj, cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &U, int ny, int nx, PREC_T p,
                 PREC_T lambda, PREC_T zmin, float s = 0.9, PROPMODE propmode = PROPMODE::AUTO)
{
    olgb::wrp_method(obj, U, ny, nx, p, lambda, zmin, (PREC_T)0, s, propmode, OLG_WINDOW_SQUARE);
}

// golcgh.h:540-559 (p_limit overload)
template <typename _Tp, typename COMPLEX_T, typename PREC_T>
void WRPMethod_D(gObject<_Tp> &obj, cuda::unique_ptr<thrust::complex<COMPLEX_T>[]> &U, int ny, int nx, PREC_T p,
                 PREC_T lambda, PREC_T zmin, PREC_T p_limit, float s = 0.9, PROPMODE propmode = PROPMODE::AUTO)
{
    olgb::wrp_method(obj, U, ny, nx, p, lambda, zmin, p_limit, s, propmode, OLG_WINDOW_SQUARE);
}
} // namespace ol
#endif
