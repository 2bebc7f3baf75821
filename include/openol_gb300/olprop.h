/*
 * olprop.h (drop-in) -- the reference's CPU propagation templates
 * (include/olprop.h) for host fields, with the same names and signatures,
 * computed on the GPU by libolgb300.so (include/olgb300.h).
 *
 * Precision: the reference instantiates these with any PREC_T / COMPLEX_T
 * (double for its accuracy checks).  Here the field always propagates in
 * FP32 (complex64) on the GPU: a std::complex<double> field is rounded to
 * complex64, propagated, and widened back, so results carry FP32 accuracy
 * (relative L2 about 1e-6 against the FP64 path) whatever COMPLEX_T is.  The
 * AUTO checks and the band windows are decided in the caller's PREC_T, as the
 * reference decides them, because they choose what runs.
 *
 * Each call copies the field to the device, runs, copies it back and returns
 * with the device synchronised; errors throw std::runtime_error.
 */
#ifndef OLGB300_OLPROP_H
#define OLGB300_OLPROP_H
#include <complex>
#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../olgb300.h"
#include "golclass.h"
#include "oldefine.h"

namespace ol {
namespace olgb {
inline void check(int rc, const char *where)
{
    if (rc != OLG_OK) throw std::runtime_error(std::string(where) + ": " + olg_last_error());
}
inline void sync(const char *where)
{
    (void)where;
    CHECK_CUDA_ERROR(cudaDeviceSynchronize());
}
template <typename C>
constexpr void complex64_only()
{
    static_assert(std::is_same<C, float>::value, "libolgb300 propagates complex64 (thrust::complex<float>) fields");
}
template <typename PREC_T>
constexpr int check_f32()
{
    return std::is_same<PREC_T, float>::value ? OLG_CHECK_F32 : 0;
}

// A complex64 device copy of a host field of any std::complex<COMPLEX_T>.
template <typename COMPLEX_T>
cuda::unique_ptr<std::complex<float>[]> to_device(const std::complex<COMPLEX_T> *h, size_t n)
{
    auto d = cuda::make_unique<std::complex<float>[]>(n);
    if constexpr (std::is_same<COMPLEX_T, float>::value) {
        CHECK_CUDA_ERROR(cudaMemcpy(d.get(), h, n * sizeof(std::complex<float>), cudaMemcpyHostToDevice));
    } else {
        std::vector<std::complex<float>> t(n);
        for (size_t i = 0; i < n; ++i) t[i] = std::complex<float>((float)h[i].real(), (float)h[i].imag());
        CHECK_CUDA_ERROR(cudaMemcpy(d.get(), t.data(), n * sizeof(std::complex<float>), cudaMemcpyHostToDevice));
    }
    return d;
}

// Device complex64 -> host std::complex<COMPLEX_T>, times `scale`.
template <typename COMPLEX_T>
void to_host(std::complex<COMPLEX_T> *h, const std::complex<float> *d, size_t n, double scale = 1.0)
{
    std::vector<std::complex<float>> t(n);
    CHECK_CUDA_ERROR(cudaMemcpy(t.data(), d, n * sizeof(std::complex<float>), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i)
        h[i] = std::complex<COMPLEX_T>((COMPLEX_T)(t[i].real() * scale), (COMPLEX_T)(t[i].imag() * scale));
}

// fn(device pointer) on a device copy of u (ny x nx), result written back.
template <typename COMPLEX_T, typename F>
void host_field(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int64_t ny, int64_t nx, F &&fn, double scale = 1.0)
{
    const size_t n = (size_t)ny * (size_t)nx;
    auto d = to_device(u.get(), n);
    fn((void *)d.get());
    to_host(u.get(), d.get(), n, scale);
}

inline int tilt_mode(PROPMODE propmode)
{
    return propmode == PROPMODE::ASM ? OLG_ASM : propmode == PROPMODE::FRESNEL ? OLG_FRESNEL : -1;
}
} // namespace olgb

// ol::FresnelPropCheck, olprop.h:109-123 (evaluated in PREC_T)
template <typename PREC_T = double>
bool FresnelPropCheck(size_t ny, size_t nx, PREC_T dy, PREC_T dx, PREC_T lambda, PREC_T z)
{
    return olg_fresnel_prop_check((int)ny, (int)nx, dy, dx, lambda, z, std::is_same<PREC_T, float>::value) == 1;
}

// ol::AsmPropCheck, olprop.h:209-225 (evaluated in PREC_T)
template <typename PREC_T = float>
bool AsmPropCheck(int64_t ny, int64_t nx, PREC_T dy, PREC_T dx, PREC_T lambda, PREC_T z)
{
    return olg_asm_prop_check((int)ny, (int)nx, dy, dx, lambda, z, std::is_same<PREC_T, float>::value) == 1;
}

// ol::AsmProp, olprop.h:227-248: crop(IFFT(H FFT(pad u)) / Np), in place
template <typename PREC_T = double, typename COMPLEX_T>
void AsmProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int64_t height, int64_t width, PREC_T dy, PREC_T dx,
             PREC_T lambda, PREC_T z)
{
    olgb::host_field(u, height, width, [&](void *d) {
        olgb::check(olg_asm_prop_c64(d, d, (int)height, (int)width, dy, dx, lambda, z, 0, nullptr, 0, nullptr),
                    "AsmProp");
    });
}

// ol::FresnelProp, olprop.h:125-148: convolution with the sampled impulse
// response, both spectra scaled by 1/Np, in place
template <typename PREC_T = double, typename COMPLEX_T>
void FresnelProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, size_t height, size_t width, PREC_T dy, PREC_T dx,
                 PREC_T lambda, PREC_T z)
{
    olgb::host_field(u, (int64_t)height, (int64_t)width, [&](void *d) {
        olgb::check(olg_fresnel_prop_c64(d, d, (int)height, (int)width, dy, dx, lambda, z, 0, 0, nullptr, 0, nullptr),
                    "FresnelProp");
    });
}

// ol::FresnelPropBandLimit, olprop.h:150-170: the response zeroed outside the
// x and y limits of FresnelResponseBandLimit (olprop.h:26-50)
template <typename PREC_T = double, typename COMPLEX_T>
void FresnelPropBandLimit(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, size_t height, size_t width, PREC_T dy,
                          PREC_T dx, PREC_T lambda, PREC_T z)
{
    olgb::host_field(u, (int64_t)height, (int64_t)width, [&](void *d) {
        olgb::check(olg_fresnel_prop_c64(d, d, (int)height, (int)width, dy, dx, lambda, z, 2, 0, nullptr, 0, nullptr),
                    "FresnelPropBandLimit");
    });
}

// ol::shiftedAsmProp, olprop.h:307-327: the band window of shiftedAsmTransferF
// (olprop.h:251-305, decided in PREC_T) and 1/Np twice; udst is (re)allocated
// like the reference's del_zero target when empty
template <typename PREC_T = double, typename COMPLEX_T>
void shiftedAsmProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &usrc, std::unique_ptr<std::complex<COMPLEX_T>[]> &udst,
                    int64_t height, int64_t width, PREC_T dy, PREC_T dx, PREC_T lambda, PREC_T z, PREC_T oy, PREC_T ox)
{
    const size_t n = (size_t)height * (size_t)width;
    auto s = olgb::to_device(usrc.get(), n);
    auto o = cuda::make_unique<std::complex<float>[]>(n);
    olgb::check(olg_shifted_asm_prop_c64(s.get(), o.get(), (int)height, (int)width, dy, dx, lambda, z, oy, ox,
                                         OLG_BANDLIMIT | olgb::check_f32<PREC_T>(), nullptr, 0, nullptr),
                "shiftedAsmProp");
    if (!udst) udst = std::make_unique<std::complex<COMPLEX_T>[]>(n);
    olgb::to_host(udst.get(), o.get(), n, 1.0 / (4.0 * (double)n));
}

// ol::shiftedFresnelProp, olprop.h:338-406: the scaled Fresnel chirps without
// windows; one more 1/Np than the device gshiftedFresnelProp; in place
template <typename PREC_T = float, typename COMPLEX_T>
void shiftedFresnelProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int64_t height, int64_t width, PREC_T dy,
                        PREC_T dx, PREC_T lambda, PREC_T z, PREC_T s, PREC_T oy, PREC_T ox)
{
    olgb::host_field(
        u, height, width,
        [&](void *d) {
            olgb::check(olg_shifted_fresnel_prop_c64(d, d, (int)height, (int)width, dy, dx, lambda, z, s, oy, ox, 0,
                                                     nullptr, 0, nullptr),
                        "shiftedFresnelProp");
        },
        1.0 / (4.0 * (double)height * (double)width));
}

// ol::splitAsmProp, olprop.h:618-654: every (source, destination) block pair
// through shiftedAsmProp (band window in PREC_T, 1/Np_block twice); in place
template <typename PREC_T = float, typename COMPLEX_T>
void splitAsmProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int64_t height, int64_t width, PREC_T dy, PREC_T dx,
                  PREC_T lambda, PREC_T z, int blocknum_y = 2, int blocknum_x = 2)
{
    const size_t n = (size_t)height * (size_t)width;
    auto a = olgb::to_device(u.get(), n);
    auto b = cuda::make_unique<std::complex<float>[]>(n);
    olgb::check(olg_split_prop_c64(a.get(), b.get(), (int)height, (int)width, dy, dx, lambda, z, OLG_ASM, blocknum_y,
                                   blocknum_x, OLG_BANDLIMIT | olgb::check_f32<PREC_T>(), nullptr, 0, nullptr),
                "splitAsmProp");
    const double nb = 4.0 * (double)(height / blocknum_y) * (double)(width / blocknum_x);
    olgb::to_host(u.get(), b.get(), n, 1.0 / nb);
}

// ol::TiltedSourceProp, olprop.h:414-521 (the destination plane rotated by
// angle_src2dst about y, as seen from the source); in place
template <typename PREC_T = float, typename COMPLEX_T>
void TiltedSourceProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T dy, PREC_T dx,
                      PREC_T lambda, PREC_T z, PREC_T angle_src2dst, INTERPOLATION inp = BILINEAR,
                      PROPMODE propmode = ASM)
{
    olgb::host_field(u, ny, nx, [&](void *d) {
        olgb::check(olg_tilted_prop_c64(d, d, ny, nx, dy, dx, lambda, z, angle_src2dst, (int)inp,
                                        olgb::tilt_mode(propmode), 0, nullptr, 0, nullptr),
                    "TiltedSourceProp");
    });
}

// ol::TiltedReferenceProp, olprop.h:523-600 (propagate, then resample for a
// plane rotated by `rotate`); in place
template <typename PREC_T = float, typename COMPLEX_T>
void TiltedReferenceProp(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int64_t ny, int64_t nx, PREC_T dy, PREC_T dx,
                         PREC_T lambda, PREC_T z, PREC_T rotate, INTERPOLATION inp = BILINEAR,
                         PROPMODE propmode = ASM)
{
    olgb::host_field(u, ny, nx, [&](void *d) {
        olgb::check(olg_tilted_prop_c64(d, d, (int)ny, (int)nx, dy, dx, lambda, z, rotate, (int)inp,
                                        olgb::tilt_mode(propmode), 1, nullptr, 0, nullptr),
                    "TiltedReferenceProp");
    });
}

// ol::Prop (host fields), olprop.h:656-682: ASM / FRESNEL / AUTO.  AUTO takes
// AsmProp when AsmPropCheck passes, else FresnelProp when FresnelPropCheck
// passes, else FresnelPropBandLimit (the CPU band limit, with its x and y
// limits).  Prints the chosen method like the reference.
template <typename COMPLEX_T, typename PREC_T>
void Prop(std::unique_ptr<std::complex<COMPLEX_T>[]> &u, int ny, int nx, PREC_T dy, PREC_T dx, PREC_T lambda, PREC_T d,
          PROPMODE propmode = ol::PROPMODE::AUTO)
{
    if (propmode == PROPMODE::FRESNEL) {
        std::printf("FresnelProp\n");
        FresnelProp(u, ny, nx, dy, dx, lambda, d);
    } else if (propmode == PROPMODE::ASM) {
        std::printf("AsmProp\n");
        AsmProp(u, ny, nx, dy, dx, lambda, d);
    } else if (propmode == PROPMODE::AUTO) {
        if (AsmPropCheck(ny, nx, dy, dx, lambda, d)) {
            std::printf("AsmProp\n");
            AsmProp(u, ny, nx, dy, dx, lambda, d);
        } else if (!FresnelPropCheck(ny, nx, dy, dx, lambda, d)) {
            std::printf("warning!!\neither AsmProp or FresnelProp does not meet the condition.\n");
            FresnelPropBandLimit(u, ny, nx, dy, dx, lambda, d);
        } else {
            std::printf("FresnelProp\n");
            FresnelProp(u, ny, nx, dy, dx, lambda, d);
        }
    } else {
        throw std::runtime_error("Prop: invalid PROPMODE");
    }
}
} // namespace ol
#endif
