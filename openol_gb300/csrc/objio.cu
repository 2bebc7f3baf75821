// objio.cu -- point clouds and images on either side of the hologram path.
//
// Device side (GB300): the point-cloud set-up of the reference's olobject.h
// on the 12-byte (x, y, z) float records the CGH kernels read --
//   objinfo   (olobject.h:163-174): min / max of x, y, z (one reduction pass),
//   objset    (olobject.h:196-264): scale the larger x/y extent (or the
//             smaller of two scales) and shift, as one elementwise pass whose
//             float roundings are those of the reference's float code,
//   objsort   (olobject.h:176-181): order by z, largest first (a stable radix
//             sort of z with the indices, then a gather).
// Host side: the .3d / .3df point files (olobject.h:9-161) and the 8-bit
// BMP files (olimg.h:55-99, 136-165), byte for byte as the reference reads and
// writes them.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace olg {
namespace {

// order-preserving float <-> int mapping for atomic min / max
__device__ __forceinline__ int of2o(float f)
{
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
inline float o2f_host(int i)
{
    i = i >= 0 ? i : i ^ 0x7fffffff;
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}

__global__ void k_obj_init(int *mm)
{
    if (threadIdx.x < 3) mm[threadIdx.x] = 0x7fffffff;
    else if (threadIdx.x < 6) mm[threadIdx.x] = (int)0x80000000;
}

// mm = {xmin, ymin, zmin, xmax, ymax, zmax} (ordered ints)
__global__ void k_obj_minmax(const float *p, int n, int *mm)
{
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float v = p[3 * (size_t)j + c];
            mn[c] = fminf(mn[c], v);
            mx[c] = fmaxf(mx[c], v);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[c] = fminf(mn[c], __shfl_xor_sync(0xffffffffu, mn[c], o));
            mx[c] = fmaxf(mx[c], __shfl_xor_sync(0xffffffffu, mx[c], o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(mm + c, of2o(mn[c]));
            atomicMax(mm + 3 + c, of2o(mx[c]));
        }
    }
}

// p = p * scale + offset, each product and sum rounded on its own
__global__ void k_obj_affine(float *p, int n, float scale, float ox, float oy, float oz)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    float *q = p + 3 * (size_t)j;
    q[0] = __fadd_rn(__fmul_rn(q[0], scale), ox);
    q[1] = __fadd_rn(__fmul_rn(q[1], scale), oy);
    q[2] = __fadd_rn(__fmul_rn(q[2], scale), oz);
}

__global__ void k_obj_keys(const float *p, int n, float *z, int *idx)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    z[j] = p[3 * (size_t)j + 2];
    idx[j] = j;
}

__global__ void k_obj_gather(const float *src, const int *idx, int n, float *dst)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const size_t s = 3 * (size_t)idx[j];
    dst[3 * (size_t)j] = src[s];
    dst[3 * (size_t)j + 1] = src[s + 1];
    dst[3 * (size_t)j + 2] = src[s + 2];
}

int grid_for(int n, int nt) { return (n + nt - 1) / nt; }

// minimum / maximum of x, y, z on the device, read back (synchronises `st`)
int minmax(const float *p, int n, float out[6], cudaStream_t st)
{
    Scratch sc;
    if (int rc = sc.acquire(nullptr, 0, 6 * sizeof(int), st)) return rc;
    int *mm = (int *)sc.ptr;
    k_obj_init<<<1, 32, 0, st>>>(mm);
    const int g = std::min(grid_for(n, 256), 8 * sm_count());
    k_obj_minmax<<<g, 256, 0, st>>>(p, n, mm);
    count_launch(2);
    if (int rc = check_launch("k_obj_minmax")) return rc;
    int h[6];
    cudaError_t e = cudaMemcpyAsync(h, mm, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "min / max read-back");
    for (int c = 0; c < 6; ++c) out[c] = o2f_host(h[c]);
    return OLG_OK;
}

size_t sort_bytes(int n, size_t *cub_bytes)
{
    size_t tb = 0;
    cub::DeviceRadixSort::SortPairsDescending(nullptr, tb, (const float *)nullptr, (float *)nullptr,
                                              (const int *)nullptr, (int *)nullptr, n);
    if (cub_bytes) *cub_bytes = tb;
    const size_t a = align_up((size_t)n * 4, 256);
    return 4 * a + align_up((size_t)n * 12, 256) + align_up(tb, 256);
}

// file helpers: the reference reads native-endian int32 / float records
struct File {
    FILE *f = nullptr;
    ~File()
    {
        if (f) fclose(f);
    }
};

} // namespace
} // namespace olg

using namespace olg;

extern "C" int olg_obj_minmax_f32(const float *points, int n, float *minmax_out, olg_stream_t stream)
{
    if (!points || n <= 0 || !minmax_out) return fail(OLG_ERR_INVALID_ARG, "need points and a 6-float output");
    return minmax(points, n, minmax_out, (cudaStream_t)stream);
}

extern "C" int olg_objset_f32(float *points, int n, float x_range, float y_range, const float *offset, int mode,
                              int flags, olg_stream_t stream)
{
    if (!points || n <= 0 || !offset) return fail(OLG_ERR_INVALID_ARG, "need points and an offset");
    if (mode != OLG_OBJSET_ZMIN && mode != OLG_OBJSET_ZMIDDLE) return fail(OLG_ERR_INVALID_ARG, "bad objset mode");
    cudaStream_t st = (cudaStream_t)stream;
    float m[6];
    if (int rc = minmax(points, n, m, st)) return rc;
    // the reference's float expressions, operation by operation (olobject.h:208-231, 245-263);
    // this file is compiled with -ffp-contract=off
    volatile float xmin = m[0], ymin = m[1], zmin = m[2], xmax = m[3], ymax = m[4], zmax = m[5];
    volatile float range_x = xmax - xmin, range_y = ymax - ymin, range_z = zmax - zmin;
    volatile float scale;
    if (y_range < 0) { // objset(obj, xy_range, offset, mode)
        scale = (range_x > range_y) ? range_x : range_y;
        scale = x_range / scale;
        if (flags & OLG_VERBOSE) {
            std::printf("xmax: %g  xmin: %g  range%g\n", (double)xmax, (double)xmin, (double)range_x);
            std::printf("ymax: %g  ymin: %g  range%g\n", (double)ymax, (double)ymin, (double)range_y);
            std::printf("zmax: %g  zmin: %g  range%g\n", (double)zmax, (double)zmin, (double)range_z);
        }
    } else { // objset(obj, x_range, y_range, offset, mode): the smaller scale
        volatile float sx = x_range / range_x, sy = y_range / range_y;
        scale = (sx < sy) ? sx : sy;
    }
    volatile float ox = offset[0], oy = offset[1], oz = offset[2];
    volatile float t;
    t = (xmax + xmin) / 2;
    t = t * scale;
    ox = ox - t;
    t = (ymax + ymin) / 2;
    t = t * scale;
    oy = oy - t;
    if (mode == OLG_OBJSET_ZMIN) {
        t = zmin * scale;
    } else {
        t = (zmax + zmin) / 2;
        t = t * scale;
    }
    oz = oz - t;
    k_obj_affine<<<grid_for(n, 256), 256, 0, st>>>(points, n, scale, ox, oy, oz);
    count_launch();
    return check_launch("k_obj_affine");
}

extern "C" size_t olg_objsort_workspace_bytes(int n) { return n > 0 ? sort_bytes(n, nullptr) : 0; }

extern "C" int olg_objsort_f32(float *points, int n, void *work, size_t work_bytes, olg_stream_t stream)
{
    if (!points || n < 0) return fail(OLG_ERR_INVALID_ARG, "need points");
    if (n < 2) return OLG_OK;
    cudaStream_t st = (cudaStream_t)stream;
    size_t tb = 0;
    const size_t need = sort_bytes(n, &tb);
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, need, st)) return rc;
    char *b = (char *)sc.ptr;
    const size_t a = align_up((size_t)n * 4, 256);
    float *zin = (float *)b, *zout = (float *)(b + a);
    int *iin = (int *)(b + 2 * a), *iout = (int *)(b + 3 * a);
    float *tmp = (float *)(b + 4 * a);
    void *cubtmp = b + 4 * a + align_up((size_t)n * 12, 256);
    k_obj_keys<<<grid_for(n, 256), 256, 0, st>>>(points, n, zin, iin);
    cudaError_t e = cub::DeviceRadixSort::SortPairsDescending(cubtmp, tb, zin, zout, iin, iout, n, 0, 32, st);
    if (e != cudaSuccess) return cuda_fail(e, "radix sort of z");
    k_obj_gather<<<grid_for(n, 256), 256, 0, st>>>(points, iout, n, tmp);
    e = cudaMemcpyAsync(points, tmp, (size_t)n * 12, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpyAsync");
    count_launch(2);
    return check_launch("objsort");
}

// ------------------------------------------------------------------ files
extern "C" int olg_objread(const char *path, float *points, int capacity, int *n_out)
{
    if (!path || !n_out) return fail(OLG_ERR_INVALID_ARG, "need a path and n_out");
    const char *ext = std::strrchr(path, '.');
    int fmt = -1; // 0: int32 records (.3d), 1: float records (.3df)
    if (ext && std::strcmp(ext, ".3d") == 0) fmt = 0;
    else if (ext && std::strcmp(ext, ".3df") == 0) fmt = 1;
    if (fmt < 0) return fail(OLG_ERR_INVALID_ARG, "point files are .3d or .3df");
    File F;
    F.f = std::fopen(path, "rb");
    if (!F.f) return fail(OLG_ERR_INVALID_ARG, std::string("cannot open ") + path);
    int32_t N = 0;
    if (std::fread(&N, 4, 1, F.f) != 1 || N < 0) return fail(OLG_ERR_INVALID_ARG, "cannot read the point count");
    *n_out = N;
    if (!points) return OLG_OK;
    if (capacity < N) return fail(OLG_ERR_INVALID_ARG, "points buffer too small");
    std::vector<int32_t> raw((size_t)N * 3);
    if (N && std::fread(raw.data(), 4, raw.size(), F.f) != raw.size())
        return fail(OLG_ERR_INVALID_ARG, "point file shorter than its count");
    for (size_t i = 0; i < raw.size(); ++i) {
        if (fmt == 0) {
            points[i] = (float)raw[i];
        } else {
            float v;
            std::memcpy(&v, &raw[i], 4);
            points[i] = v;
        }
    }
    return OLG_OK;
}

extern "C" int olg_objread_scaled(const char *path, const float *offset, float scale, float *points, int capacity,
                                  int *n_out)
{
    if (!path || !offset || !n_out) return fail(OLG_ERR_INVALID_ARG, "need a path, an offset and n_out");
    File F;
    F.f = std::fopen(path, "rb");
    if (!F.f) return fail(OLG_ERR_INVALID_ARG, std::string("cannot open ") + path);
    int32_t N = 0;
    if (std::fread(&N, 4, 1, F.f) != 1 || N < 0) return fail(OLG_ERR_INVALID_ARG, "cannot read the point count");
    *n_out = N;
    if (!points) return OLG_OK;
    if (capacity < N) return fail(OLG_ERR_INVALID_ARG, "points buffer too small");
    std::vector<int32_t> raw((size_t)N * 3);
    if (N && std::fread(raw.data(), 4, raw.size(), F.f) != raw.size())
        return fail(OLG_ERR_INVALID_ARG, "point file shorter than its count");
    for (size_t i = 0; i < raw.size(); ++i) {
        volatile float p = (float)raw[i] * scale; // xint * scale + offset, float, two roundings
        points[i] = p + offset[i % 3];
    }
    return OLG_OK;
}

namespace {
#pragma pack(push, 1)
struct BmpFile {
    uint16_t type;
    uint32_t size;
    uint16_t r1, r2;
    uint32_t off;
};
struct BmpInfo {
    uint32_t size;
    int32_t width, height;
    uint16_t planes, bits;
    uint32_t compression, image_size;
    int32_t xppm, yppm;
    uint32_t used, important;
};
#pragma pack(pop)
static_assert(sizeof(BmpFile) == 14 && sizeof(BmpInfo) == 40, "BMP headers are packed");
} // namespace

extern "C" int olg_bmpwrite_u8(const char *fname, const uint8_t *img, int ny, int nx)
{
    if (!fname || !img || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad BMP arguments");
    File F;
    F.f = std::fopen(fname, "wb");
    if (!F.f) return fail(OLG_ERR_INVALID_ARG, std::string("cannot create ") + fname);
    // the header fields of olimg.h:137-138: the file size counts no row padding
    const BmpFile bf{19778, 14u + 40u + 1024u + (unsigned)nx * (unsigned)ny, 0, 0, 14 + 40 + 1024};
    const BmpInfo bi{40, nx, ny, 1, 8, 0, 0, 0, 0, 0, 0};
    uint8_t pal[1024];
    for (int i = 0; i < 256; ++i) {
        pal[4 * i] = pal[4 * i + 1] = pal[4 * i + 2] = (uint8_t)i;
        pal[4 * i + 3] = 0;
    }
    bool ok = std::fwrite(&bf, sizeof bf, 1, F.f) == 1 && std::fwrite(&bi, sizeof bi, 1, F.f) == 1 &&
              std::fwrite(pal, sizeof pal, 1, F.f) == 1;
    // rows in memory order, each followed by nx % 4 zero bytes (olimg.h:155-162)
    const uint8_t zeros[4] = {0, 0, 0, 0};
    const int pad = nx % 4;
    for (int n = 0; ok && n < ny; ++n) {
        ok = std::fwrite(img + (size_t)n * nx, 1, nx, F.f) == (size_t)nx;
        if (ok && pad) ok = std::fwrite(zeros, 1, pad, F.f) == (size_t)pad;
    }
    return ok ? OLG_OK : fail(OLG_ERR_INVALID_ARG, "BMP write failed");
}

extern "C" int olg_bmpread_u8(const char *fname, uint8_t *img, int ny, int nx)
{
    if (!fname || !img || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad BMP arguments");
    File F;
    F.f = std::fopen(fname, "rb");
    if (!F.f) return fail(OLG_ERR_INVALID_ARG, std::string("cannot open ") + fname);
    BmpFile bf;
    BmpInfo bi;
    uint8_t pal[1024];
    if (std::fread(&bf, sizeof bf, 1, F.f) != 1 || std::fread(&bi, sizeof bi, 1, F.f) != 1 ||
        std::fread(pal, sizeof pal, 1, F.f) != 1)
        return fail(OLG_ERR_INVALID_ARG, "not an 8-bit BMP written with a 256-entry palette");
    // rows of nx bytes, each followed by nx % 4 bytes skipped (olimg.h:84-98)
    const int pad = nx % 4;
    for (int n = 0; n < ny; ++n) {
        if (std::fread(img + (size_t)n * nx, 1, nx, F.f) != (size_t)nx)
            return fail(OLG_ERR_INVALID_ARG, "BMP shorter than ny rows");
        if (pad && std::fseek(F.f, pad, SEEK_CUR) != 0) return fail(OLG_ERR_INVALID_ARG, "BMP seek failed");
    }
    return OLG_OK;
}
