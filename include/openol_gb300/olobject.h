/*
 * olobject.h (drop-in) -- the reference's point-cloud helpers
 * (include/olobject.h: objread, objinfo, objset, objsort) and its 8-bit BMP
 * reader / writer (include/olimg.h: bmpread, bmpwrite), with the same names,
 * forwarding to libolgb300.so.  objinfo / objset / objsort run on the GPU:
 * directly on an ol::gObject<float>, or on an ol::Object<float> through a
 * device copy and back.  Errors throw std::runtime_error where the reference
 * called exit(1).
 */
#ifndef OLGB300_OLOBJECT_H
#define OLGB300_OLOBJECT_H
#include <cstdint>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../olgb300.h"
#include "golclass.h"
#include "olclass.h"

namespace ol {

enum OBJSET_MODE { ZMIN, ZMIDDLE };

namespace olgb_obj {
inline void check(int rc, const char *where)
{
    if (rc != OLG_OK) throw std::runtime_error(std::string(where) + ": " + olg_last_error());
}
template <typename T>
constexpr void float_only()
{
    static_assert(std::is_same<T, float>::value, "libolgb300 point clouds are float (x, y, z) records");
}
} // namespace olgb_obj

// objread, olobject.h:79-91 (.3d int32 / .3df float records)
template <typename _Tp>
Object<_Tp> objread(const char *path)
{
    olgb_obj::float_only<_Tp>();
    int n = 0;
    olgb_obj::check(olg_objread(path, nullptr, 0, &n), "objread");
    Object<_Tp> obj(n);
    olgb_obj::check(olg_objread(path, reinterpret_cast<float *>(obj.points.get()), n, &n), "objread");
    return obj;
}

// objread(path, offset, scale), olobject.h:128-161
template <typename _Tp, typename OFFSET_T, typename SCALE_T>
Object<_Tp> objread(const char *path, Vect3<OFFSET_T> offset, SCALE_T scale)
{
    olgb_obj::float_only<_Tp>();
    const float off[3] = {(float)offset.x, (float)offset.y, (float)offset.z};
    int n = 0;
    olgb_obj::check(olg_objread_scaled(path, off, (float)scale, nullptr, 0, &n), "objread");
    Object<_Tp> obj(n);
    olgb_obj::check(olg_objread_scaled(path, off, (float)scale, reinterpret_cast<float *>(obj.points.get()), n, &n),
                    "objread");
    return obj;
}

// objread(path, offset[3], scale), olobject.h:93-126
template <typename _Tp, typename OFFSET_T, typename SCALE_T>
Object<_Tp> objread(const char *path, OFFSET_T *offset, SCALE_T scale)
{
    return objread<_Tp>(path, Vect3<OFFSET_T>(offset[0], offset[1], offset[2]), scale);
}

// device forms
template <typename _Tp>
void objinfo(gObject<_Tp> &obj)
{
    olgb_obj::float_only<_Tp>();
    float m[6];
    olgb_obj::check(olg_obj_minmax_f32(reinterpret_cast<const float *>(obj.points.get()), obj.size, m, nullptr),
                    "objinfo");
    std::printf("xmax: %g  xmin: %g\nymax: %g  ymin: %g\nzmax: %g  zmin: %g\n", m[3], m[0], m[4], m[1], m[5], m[2]);
}
template <typename _Tp>
void objsort(gObject<_Tp> &obj)
{
    olgb_obj::float_only<_Tp>();
    olgb_obj::check(olg_objsort_f32(reinterpret_cast<float *>(obj.points.get()), obj.size, nullptr, 0, nullptr),
                    "objsort");
    CHECK_CUDA_ERROR(cudaDeviceSynchronize());
}
template <typename _Tp>
void objset(gObject<_Tp> &obj, float xy_range, Vect3<_Tp> offset, OBJSET_MODE mode = ZMIN)
{
    olgb_obj::float_only<_Tp>();
    const float off[3] = {offset.x, offset.y, offset.z};
    olgb_obj::check(olg_objset_f32(reinterpret_cast<float *>(obj.points.get()), obj.size, xy_range, -1.0f, off,
                                   mode == ZMIN ? OLG_OBJSET_ZMIN : OLG_OBJSET_ZMIDDLE, OLG_VERBOSE, nullptr),
                    "objset");
    CHECK_CUDA_ERROR(cudaDeviceSynchronize());
}
template <typename _Tp>
void objset(gObject<_Tp> &obj, float x_range, float y_range, Vect3<_Tp> offset, OBJSET_MODE mode = ZMIN)
{
    olgb_obj::float_only<_Tp>();
    const float off[3] = {offset.x, offset.y, offset.z};
    olgb_obj::check(olg_objset_f32(reinterpret_cast<float *>(obj.points.get()), obj.size, x_range, y_range, off,
                                   mode == ZMIN ? OLG_OBJSET_ZMIN : OLG_OBJSET_ZMIDDLE, 0, nullptr),
                    "objset");
    CHECK_CUDA_ERROR(cudaDeviceSynchronize());
}

// host forms (olobject.h:163-264): through a device copy
namespace olgb_obj {
template <typename _Tp, typename F>
void on_device(Object<_Tp> &obj, F &&fn)
{
    gObject<_Tp> g = Object2cuda(obj);
    fn(g);
    CHECK_CUDA_ERROR(cudaMemcpy(obj.points.get(), g.points.get(), sizeof(Vect3<_Tp>) * obj.size, cudaMemcpyDeviceToHost));
}
} // namespace olgb_obj
template <typename _Tp>
void objinfo(Object<_Tp> &obj)
{
    gObject<_Tp> g = Object2cuda(obj);
    objinfo(g);
}
template <typename _Tp>
void objsort(Object<_Tp> &obj)
{
    olgb_obj::on_device(obj, [](gObject<_Tp> &g) { objsort(g); });
}
template <typename _Tp>
void objset(Object<_Tp> &obj, float xy_range, Vect3<_Tp> offset, OBJSET_MODE mode = ZMIN)
{
    olgb_obj::on_device(obj, [&](gObject<_Tp> &g) { objset(g, xy_range, offset, mode); });
}
template <typename _Tp>
void objset(Object<_Tp> &obj, float x_range, float y_range, Vect3<_Tp> offset, OBJSET_MODE mode = ZMIN)
{
    olgb_obj::on_device(obj, [&](gObject<_Tp> &g) { objset(g, x_range, y_range, offset, mode); });
}

// bmpwrite / bmpread, olimg.h:136-165 and 55-99
inline void bmpwrite(const char *fname, uint8_t *img, int ny, int nx)
{
    olgb_obj::check(olg_bmpwrite_u8(fname, img, ny, nx), "bmpwrite");
}
inline void bmpwrite(const char *fname, std::unique_ptr<uint8_t[]> &img, int ny, int nx)
{
    bmpwrite(fname, img.get(), ny, nx);
}
inline void bmpread(const char *fname, uint8_t *img, int ny, int nx)
{
    olgb_obj::check(olg_bmpread_u8(fname, img, ny, nx), "bmpread");
}
} // namespace ol
#endif
