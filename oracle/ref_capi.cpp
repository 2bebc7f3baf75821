/*
 * ref_capi.cpp -- extern "C" entry points over the reference's OWN CPU
 * templates, compiled from the unmodified reference headers (include/olprop.h,
 * include/olcgh.h, include/olutils.h, include/olimg.h) with the shims in
 * refshim/.  TEST INFRASTRUCTURE ONLY: used here to pin the oracle restatement
 * (olcpu.c) and to generate the golden fixtures under tests/golden/.  Output
 * goes to oracle/_ref/ (git-ignored).
 */
#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <memory>

#include "olprop.h"
#include "olcgh.h"
#include "olimg.h"
#include "olobject.h"

using cd = std::complex<double>;

static std::unique_ptr<cd[]> load(const double *p, long n)
{
    auto u = std::make_unique<cd[]>(n);
    std::memcpy((void *)u.get(), p, sizeof(cd) * n);
    return u;
}
static void store(const std::unique_ptr<cd[]> &u, double *p, long n) { std::memcpy(p, (const void *)u.get(), sizeof(cd) * n); }

static ol::Object<double> mkobj(const double *pts, int n)
{
    ol::Object<double> obj(n);
    for (int j = 0; j < n; ++j) obj[j] = ol::Vect3<double>(pts[3 * j], pts[3 * j + 1], pts[3 * j + 2]);
    return obj;
}

extern "C" {

/* ol::AsmProp<double>, olprop.h:227-248 */
void ref_asm_prop(double *u, int ny, int nx, double dy, double dx, double lam, double z)
{
    auto U = load(u, (long)ny * nx);
    ol::AsmProp(U, (int64_t)ny, (int64_t)nx, dy, dx, lam, z);
    store(U, u, (long)ny * nx);
}

/* ol::FresnelProp<double>, olprop.h:125-148 */
void ref_fresnel_prop(double *u, int ny, int nx, double dy, double dx, double lam, double z)
{
    auto U = load(u, (long)ny * nx);
    ol::FresnelProp(U, (size_t)ny, (size_t)nx, dy, dx, lam, z);
    store(U, u, (long)ny * nx);
}

/* ol::FresnelPropBandLimit<double>, olprop.h:150-170 */
void ref_fresnel_prop_bandlimit(double *u, int ny, int nx, double dy, double dx, double lam, double z)
{
    auto U = load(u, (long)ny * nx);
    ol::FresnelPropBandLimit(U, (size_t)ny, (size_t)nx, dy, dx, lam, z);
    store(U, u, (long)ny * nx);
}

/* ol::Prop (CPU dispatcher), olprop.h:656-682; mode = ol::PROPMODE */
void ref_prop(double *u, int ny, int nx, double dy, double dx, double lam, double z, int mode)
{
    auto U = load(u, (long)ny * nx);
    ol::Prop(U, ny, nx, dy, dx, lam, z, (ol::PROPMODE)mode);
    store(U, u, (long)ny * nx);
}

int ref_asm_prop_check(int ny, int nx, double dy, double dx, double lam, double z)
{
    return ol::AsmPropCheck((int64_t)ny, (int64_t)nx, dy, dx, lam, z) ? 1 : 0;
}
int ref_asm_prop_check_f(int ny, int nx, float dy, float dx, float lam, float z)
{
    return ol::AsmPropCheck((int64_t)ny, (int64_t)nx, dy, dx, lam, z) ? 1 : 0;
}
int ref_fresnel_prop_check(int ny, int nx, double dy, double dx, double lam, double z)
{
    return ol::FresnelPropCheck((size_t)ny, (size_t)nx, dy, dx, lam, z) ? 1 : 0;
}
int ref_fresnel_prop_check_f(int ny, int nx, float dy, float dx, float lam, float z)
{
    return ol::FresnelPropCheck((size_t)ny, (size_t)nx, dy, dx, lam, z) ? 1 : 0;
}

/* ol::Cgh complex output, olcgh.h:368-379 -> _CghFresnel olcgh.h:297-313 */
void ref_cgh(const double *pts, int n, double *u, int ny, int nx, double py, double px, double lam)
{
    auto obj = mkobj(pts, n);
    auto U = std::make_unique<cd[]>((long)ny * nx);
    ol::Cgh(obj, U, ny, nx, py, px, lam);
    store(U, u, (long)ny * nx);
}

/* ol::Cgh phase output, olcgh.h:351-365 -> _CghFresnel olcgh.h:276-295 */
void ref_cgh_phase(const double *pts, int n, double *phase, int ny, int nx, double p, double lam)
{
    auto obj = mkobj(pts, n);
    auto ph = std::make_unique<double[]>((long)ny * nx);
    ol::Cgh(obj, ph, ny, nx, p, lam);
    std::memcpy(phase, ph.get(), sizeof(double) * (long)ny * nx);
}

/* ol::complex2img(MODE), olimg.h:348-391 */
void ref_complex2img(const double *u, uint8_t *img, int ny, int nx, int mode)
{
    auto U = load(u, (long)ny * nx);
    auto I = std::make_unique<uint8_t[]>((long)ny * nx);
    ol::complex2img(U, I, ny, nx, (ol::MODE)mode);
    std::memcpy(img, I.get(), (long)ny * nx);
}

/* ol::shiftedAsmProp<double>, olprop.h:307-327 (band window, 1/Np twice) */
void ref_shifted_asm_prop(const double *src, double *dst, int ny, int nx, double dy, double dx, double lam, double z,
                          double oy, double ox)
{
    auto S = load(src, (long)ny * nx);
    auto D = std::make_unique<cd[]>((long)ny * nx);
    ol::shiftedAsmProp(S, D, (int64_t)ny, (int64_t)nx, dy, dx, lam, z, oy, ox);
    store(D, dst, (long)ny * nx);
}

/* ol::shiftedFresnelProp<double>, olprop.h:338-406 (in place; no windows) */
void ref_shifted_fresnel_prop(double *u, int ny, int nx, double dy, double dx, double lam, double z, double s,
                              double oy, double ox)
{
    auto U = load(u, (long)ny * nx);
    ol::shiftedFresnelProp(U, (int64_t)ny, (int64_t)nx, dy, dx, lam, z, s, oy, ox);
    store(U, u, (long)ny * nx);
}

/* ol::splitAsmProp, olprop.h:618-654 (in place).  It only instantiates with
 * PREC_T = float (it passes float block offsets to shiftedAsmProp), so the
 * physical parameters and every phase are single precision there. */
void ref_split_asm_prop(double *u, int ny, int nx, double dy, double dx, double lam, double z, int by, int bx)
{
    auto U = load(u, (long)ny * nx);
    ol::splitAsmProp<float>(U, (int64_t)ny, (int64_t)nx, (float)dy, (float)dx, (float)lam, (float)z, by, bx);
    store(U, u, (long)ny * nx);
}

/* ol::TiltedSourceProp<double> olprop.h:414-521 (reference == 0) and
 * ol::TiltedReferenceProp<double> olprop.h:523-600 (reference != 0), in place;
 * interp 0 BILINEAR / 1 BICUBIC, mode 0 ASM / 1 FRESNEL */
void ref_tilted_prop(double *u, int ny, int nx, double dy, double dx, double lam, double z, double angle, int interp,
                     int mode, int reference)
{
    auto U = load(u, (long)ny * nx);
    const ol::INTERPOLATION ip = interp == 1 ? ol::BICUBIC : ol::BILINEAR;
    const ol::PROPMODE pm = mode == 1 ? ol::FRESNEL : ol::ASM;
    if (reference) ol::TiltedReferenceProp<double>(U, (int64_t)ny, (int64_t)nx, dy, dx, lam, z, angle, ip, pm);
    else ol::TiltedSourceProp<double>(U, ny, nx, dy, dx, lam, z, angle, ip, pm);
    store(U, u, (long)ny * nx);
}

/* ol::objread<float>, olobject.h:79-91 (.3d / .3df); returns n, fills up to cap records */
int ref_objread(const char *path, float *out, int cap)
{
    auto obj = ol::objread<float>(path);
    for (int j = 0; j < obj.size && j < cap; ++j) {
        out[3 * j] = obj[j].x;
        out[3 * j + 1] = obj[j].y;
        out[3 * j + 2] = obj[j].z;
    }
    return obj.size;
}

/* ol::objread<float>(path, Vect3<float> offset, float scale), olobject.h:128-161 */
int ref_objread_scaled(const char *path, float ox, float oy, float oz, float scale, float *out, int cap)
{
    auto obj = ol::objread<float>(path, ol::Vect3<float>(ox, oy, oz), scale);
    for (int j = 0; j < obj.size && j < cap; ++j) {
        out[3 * j] = obj[j].x;
        out[3 * j + 1] = obj[j].y;
        out[3 * j + 2] = obj[j].z;
    }
    return obj.size;
}

static ol::Object<float> mkobjf(const float *p, int n)
{
    ol::Object<float> obj(n);
    for (int j = 0; j < n; ++j) obj[j] = ol::Vect3<float>(p[3 * j], p[3 * j + 1], p[3 * j + 2]);
    return obj;
}
static void storef(ol::Object<float> &obj, float *p)
{
    for (int j = 0; j < obj.size; ++j) {
        p[3 * j] = obj[j].x;
        p[3 * j + 1] = obj[j].y;
        p[3 * j + 2] = obj[j].z;
    }
}

/* ol::objset<float>: y_range < 0 -> one-range form olobject.h:196-230, else
 * the two-range form olobject.h:232-264; mode = ol::OBJSET_MODE; in place */
void ref_objset(float *p, int n, float x_range, float y_range, float ox, float oy, float oz, int mode)
{
    auto obj = mkobjf(p, n);
    if (y_range < 0) ol::objset(obj, x_range, ol::Vect3<float>(ox, oy, oz), (ol::OBJSET_MODE)mode);
    else ol::objset(obj, x_range, y_range, ol::Vect3<float>(ox, oy, oz), (ol::OBJSET_MODE)mode);
    storef(obj, p);
}

/* ol::objsort<float>, olobject.h:176-181, in place */
void ref_objsort(float *p, int n)
{
    auto obj = mkobjf(p, n);
    ol::objsort(obj);
    storef(obj, p);
}

/* ol::bmpwrite, olimg.h:136-160 */
void ref_bmpwrite(const char *fname, uint8_t *img, int ny, int nx) { ol::bmpwrite(fname, img, ny, nx); }

/* ol::quant8bit, olimg.h:178-198 */
void ref_quant8bit(double *real, uint8_t *img, int ny, int nx) { ol::quant8bit(real, img, ny, nx); }

} /* extern "C" */
