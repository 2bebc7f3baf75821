// wrp.cu -- wavefront-recording-plane method on GB300 (sm_103a).
//
// Step 1 of the reference (WRPStep1 golcgh.h:303-378, WRPStep1_D
// golcgh.h:403-491) loops every WRP pixel over every point and keeps the few
// inside the point's window: O(pixels x points) tests for ~sum_j pi W_j^2
// useful terms.  Here the points are binned onto 16 x 16 pixel tiles by the
// bounding box of their window, and one CTA per tile sums only the points
// listed for it:
//   k_wrp_prep     per point: window radius (float, as the reference computes
//                  it), tile bounding box and its tile count
//   (CUB scan)     each point's first slot in the (tile, point) pair list
//   k_wrp_pairs    per point: its (tile, point) pairs, in point order
//   (CUB sort)     stable radix sort of the pairs by tile: every tile's list
//                  comes out in increasing point order (deterministic sums)
//   k_wrp_offsets  per tile: start of its list (binary search of the keys)
//   k_wrp_tile     per tile: for each listed point a warp-uniform cull of the
//                  warp's 16 x 8 strip, and for each pixel x kept point: window
//                  test in float32 exactly as the reference evaluates it (each
//                  operation rounded), and the term exp(i pi rho^2 / (lambda dz))
//                  / |dz| with the phase anchored at the tile centre in
//                  double-float arithmetic.
// Step 2 is the fused propagation in prop.cu.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <cmath>
#include <cstdio>

#include "common.cuh"

namespace olg {

constexpr int WT = 16;          // tile edge (pixels)

struct WrpParams {
    const float *pts;
    int n, ny, nx, tiles_x, tiles_y, window;
    float p, lambda, plane_z, plimit;
    float l_hi, l_lo;
    float *R;        // per point: W (circle) or D (square)
    int4 *bbox;      // per point: tile range [tx0, tx1] x [ty0, ty1], tx0 > tx1 if none
    int *pcount;     // per point: tiles in its box (n + 1 entries, last 0)
    int *ppos;       // per point: first pair slot (exclusive scan of pcount; ppos[n] = pairs)
    int *keys, *vals;     // pairs (tile, point), point-major
    const int *skeys;     // pairs sorted by tile
    const int *list;      // their points: every tile's list in increasing point order
    int *offset;     // per tile: start of its list (tiles + 1 entries)
    int pairs;
    float2 *U;
};

// W_j (golcgh.h:291-299) / D_j = W_j sqrt(2) (golcgh.h:392-401): double
// arithmetic on the float inputs, rounded to float once; D rounded again.
__device__ __forceinline__ float wrp_radius(float z, const WrpParams &P)
{
    const double q = (double)P.plimit / (double)P.lambda;
    const double c = 1.0 / sqrt(4.0 * q * q - 1.0);
    const float W = (float)(c * fabs((double)z - (double)P.plane_z));
    if (P.window == 0) return W;
    return __fmul_rn(W, sqrtf(2.0f));
}

__global__ void k_wrp_prep(WrpParams P)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j == P.n) P.pcount[j] = 0;
    if (j >= P.n) return;
    const float x = P.pts[3 * j], y = P.pts[3 * j + 1], z = P.pts[3 * j + 2];
    const float R = wrp_radius(z, P);
    P.R[j] = R;
    // conservative pixel reach of the window (+2 px margin for float rounding)
    const double reach = (P.window == 0 ? (double)R : 0.5 * (double)R) / (double)P.p + 2.0;
    const double cx = (double)x / (double)P.p, cy = (double)y / (double)P.p;
    long w0 = (long)floor(cx - reach), w1 = (long)ceil(cx + reach);
    long h0 = (long)floor(cy - reach), h1 = (long)ceil(cy + reach);
    w0 = max(w0, 0L); h0 = max(h0, 0L);
    w1 = min(w1, (long)P.nx - 1); h1 = min(h1, (long)P.ny - 1);
    int4 bb;
    int cnt = 0;
    if (w0 > w1 || h0 > h1 || !(R > 0.f)) {
        bb = make_int4(1, 0, 1, 0);
    } else {
        bb = make_int4((int)(w0 / WT), (int)(w1 / WT), (int)(h0 / WT), (int)(h1 / WT));
        cnt = (bb.y - bb.x + 1) * (bb.w - bb.z + 1);
    }
    P.bbox[j] = bb;
    P.pcount[j] = cnt;
}

// per point (one warp each, coalesced stores): its (tile, point) pairs from
// slot ppos[j], tiles in raster order
__global__ void k_wrp_pairs(WrpParams P)
{
    const int j = (int)(((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (j >= P.n) return;
    const int4 bb = P.bbox[j];
    const int cnt = P.pcount[j], wdt = bb.y - bb.x + 1, o = P.ppos[j];
    for (int k = lane; k < cnt; k += 32) {
        P.keys[o + k] = (bb.z + k / wdt) * P.tiles_x + bb.x + k % wdt;
        P.vals[o + k] = j;
    }
}

// offset[t] = first slot of tile t in the sorted keys (t = 0 .. tiles)
__global__ void k_wrp_offsets(WrpParams P, int T)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > T) return;
    int lo = 0, hi = P.pairs;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (P.skeys[mid] < t) lo = mid + 1;
        else hi = mid;
    }
    P.offset[t] = lo;
}

// One CTA of two warps per 16 x 16 tile.  Warp w covers the 8-row strip
// [8 w, 8 w + 8); lane l owns column l % 16 and rows r0, r0 + 2, r0 + 4, r0 + 6
// (r0 = 8 w + l / 16), taken as two row pairs on the paired FP32 pipe, so each
// point's constants are read once per 4 pixels.  Before the per-pixel tests a
// warp skips, uniformly, every point whose window cannot reach its strip (a
// conservative test with a 1e-4 relative margin; the exact float test decides
// every pixel it keeps), and every row pair with no pixel inside.  Pixels
// outside the window get weight 0 instead of a branch.
constexpr int WNT = 64; // threads per tile
constexpr int WNB = 64; // points per batch

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

template <int WIN>
__global__ void __launch_bounds__(WNT) k_wrp_tile(WrpParams P)
{
    __shared__ float4 cst[WNB][2]; // {c0, ax, ay, b} {x, y, Rtest, A}
    __shared__ int cls[WNB];       // per point, 2 bits per warp strip: reaches it, holds it whole
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int t = blockIdx.x;
    const int tx_t = t % P.tiles_x, ty_t = t / P.tiles_x;
    const int col = lane & 15, r0 = warp * 8 + (lane >> 4);
    const int w = tx_t * WT + col;
    const float dw = (float)col - 7.5f;
    const float wc = (float)(tx_t * WT) + 7.5f, hc = (float)(ty_t * WT) + 7.5f;
    // per-pixel window-test operands, rounded as the reference's float code;
    // pair k holds rows r0 + 4 k and r0 + 4 k + 2
    const float pw = __fmul_rn(P.p, (float)w);
    float2 php[2], dhp[2], q2p[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int ra = r0 + 4 * k, rb = ra + 2;
        php[k] = make_float2(__fmul_rn(P.p, (float)(ty_t * WT + ra)), __fmul_rn(P.p, (float)(ty_t * WT + rb)));
        dhp[k] = make_float2((float)ra - 7.5f, (float)rb - 7.5f);
        q2p[k] = make_float2(dw * dw + dhp[k].x * dhp[k].x, dw * dw + dhp[k].y * dhp[k].y);
    }
    // the tile's columns in metres (the strips' x range)
    const float xl = __fmul_rn(P.p, (float)(tx_t * WT)), xr = __fmul_rn(P.p, (float)(tx_t * WT + WT - 1));
    const int beg = P.offset[t], cnt = P.offset[t + 1] - beg;
    float2 acc[4]; // (re, im) of rows r0, r0 + 2, r0 + 4, r0 + 6
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = make_float2(0.f, 0.f);
    for (int b0 = 0; b0 < cnt; b0 += WNB) {
        const int k = b0 + tid;
        float4 c0 = make_float4(0.f, 0.f, 0.f, 0.f), c1 = make_float4(0.f, 0.f, -1.f, 0.f);
        if (k < cnt) {
            const int j = P.list[beg + k];
            const float x = P.pts[3 * j], y = P.pts[3 * j + 1], z = P.pts[3 * j + 2];
            const df2 dz = df_two_sum(z, -P.plane_z);
            const df2 Dx = df_add_f(df_two_prod(P.p, wc), -x);
            const df2 Dy = df_add_f(df_two_prod(P.p, hc), -y);
            const df2 rho2 = df_add(df_mul(Dx, Dx), df_mul(Dy, Dy));
            const df2 k2 = df_recip(df_mul(df2{P.l_hi, P.l_lo}, df2{2.0f * dz.hi, 2.0f * dz.lo}));
            const float kk = k2.hi;
            c0 = make_float4(df_frac(df_mul(rho2, k2)), 2.0f * Dx.hi * P.p * kk, 2.0f * Dy.hi * P.p * kk,
                             P.p * P.p * kk);
            const float R = P.R[j];
            const float Rt = WIN == 0 ? __fmul_rn(R, R) : R;
            c1 = make_float4(x, y, Rt, 1.0f / fabsf(dz.hi + dz.lo));
        }
        // Classify this point against both warps' 16 x 8 strips once, here,
        // instead of in every warp's inner loop.  Bit 2s: the window can reach
        // strip s (a conservative cull with a 1e-4 relative margin; the float
        // test decides every pixel it keeps).  Bit 2s + 1: the window holds the
        // whole strip with a 1e-4 margin below its float rounding, so every
        // pixel's test would be true and none is evaluated (float subtraction
        // and squaring are monotone, so no pixel's rounded distance exceeds
        // the strip corner's).
        int cl = 0;
        if (k < cnt) {
#pragma unroll
            for (int s = 0; s < 2; ++s) {
                const float yl = __fmul_rn(P.p, (float)(ty_t * WT + 8 * s));
                const float yr = __fmul_rn(P.p, (float)(ty_t * WT + 8 * s + 7));
                const float ex = fmaxf(fmaxf(xl - c1.x, c1.x - xr), 0.f), ey = fmaxf(fmaxf(yl - c1.y, c1.y - yr), 0.f);
                const float lim = c1.z * 1.0001f;
                const bool reach = WIN == 0 ? ex * ex + ey * ey <= lim : (2.f * ex <= lim && 2.f * ey <= lim);
                const float fx = fmaxf(fabsf(xl - c1.x), fabsf(xr - c1.x));
                const float fy = fmaxf(fabsf(yl - c1.y), fabsf(yr - c1.y));
                const float inner = c1.z * 0.9999f;
                const bool full = WIN == 0 ? fx * fx + fy * fy <= inner : (2.f * fx <= inner && 2.f * fy <= inner);
                cl |= (reach ? 1 : 0) << (2 * s);
                cl |= (reach && full ? 2 : 0) << (2 * s);
            }
        }
        cst[tid][0] = c0;
        cst[tid][1] = c1;
        cls[tid] = cl;
        __syncthreads();
        const int m = min(WNB, cnt - b0);
        float2 part[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) part[q] = make_float2(0.f, 0.f);
        for (int i = 0; i < m; ++i) {
            // warp-uniform class of this point for this warp's strip
            const int cl = (cls[i] >> (2 * warp)) & 3;
            if (!cl) continue;
            const bool full = cl & 2;
            const float4 b = cst[i][1];
            const float4 a = cst[i][0];
            const float base = fmaf(a.y, dw, a.x);
            if (full) {
#pragma unroll
                for (int pr = 0; pr < 2; ++pr) {
                    const float2 cyc = __ffma2_rn(f2(a.z), dhp[pr], __ffma2_rn(f2(a.w), q2p[pr], f2(base)));
                    const float2 r = __fadd2_rn(__fadd2_rn(cyc, f2(12582912.0f)), f2(-12582912.0f));
                    const float2 ang = __fmul2_rn(__ffma2_rn(r, f2(-1.0f), cyc), f2(6.283185307179586f));
                    float sa, ca, sb, cb;
                    __sincosf(ang.x, &sa, &ca);
                    __sincosf(ang.y, &sb, &cb);
                    part[2 * pr] = __ffma2_rn(f2(b.w), make_float2(ca, sa), part[2 * pr]);
                    part[2 * pr + 1] = __ffma2_rn(f2(b.w), make_float2(cb, sb), part[2 * pr + 1]);
                }
                continue;
            }
            const float ddx = __fsub_rn(pw, b.x);
            const float ddx2 = __fmul_rn(ddx, ddx);
            const bool xin = __fmul_rn(fabsf(ddx), 2.0f) <= b.z;
#pragma unroll
            for (int pr = 0; pr < 2; ++pr) {
                // the window test in scalar rounded operations (never contracted);
                // a paired f32x2 form of it (even __fadd2_rn / __fmul2_rn)
                // misclassified edge pixels (9.5e-5 relative L2 on the
                // 20,000-point workload subset)
                const float dya = __fsub_rn(php[pr].x, b.y), dyb = __fsub_rn(php[pr].y, b.y);
                bool in0, in1;
                if (WIN == 0) {
                    in0 = __fadd_rn(ddx2, __fmul_rn(dya, dya)) < b.z;
                    in1 = __fadd_rn(ddx2, __fmul_rn(dyb, dyb)) < b.z;
                } else {
                    in0 = xin && __fmul_rn(fabsf(dya), 2.0f) <= b.z;
                    in1 = xin && __fmul_rn(fabsf(dyb), 2.0f) <= b.z;
                }
                if (!__any_sync(0xffffffffu, in0 || in1)) continue;
                const float wa = in0 ? b.w : 0.f, wb = in1 ? b.w : 0.f;
                const float2 cyc = __ffma2_rn(f2(a.z), dhp[pr], __ffma2_rn(f2(a.w), q2p[pr], f2(base)));
                const float2 r = __fadd2_rn(__fadd2_rn(cyc, f2(12582912.0f)), f2(-12582912.0f));
                const float2 ang = __fmul2_rn(__ffma2_rn(r, f2(-1.0f), cyc), f2(6.283185307179586f));
                float sa, ca, sb, cb;
                __sincosf(ang.x, &sa, &ca);
                __sincosf(ang.y, &sb, &cb);
                part[2 * pr] = __ffma2_rn(f2(wa), make_float2(ca, sa), part[2 * pr]);
                part[2 * pr + 1] = __ffma2_rn(f2(wb), make_float2(cb, sb), part[2 * pr + 1]);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] = __fadd2_rn(acc[q], part[q]);
        __syncthreads();
    }
    if (w < P.nx) {
        // acc[2 pr + e] is row r0 + 4 pr + 2 e
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int h = ty_t * WT + r0 + 4 * (q >> 1) + 2 * (q & 1);
            if (h < P.ny) P.U[(size_t)h * P.nx + w] = acc[q];
        }
    }
}

} // namespace olg

using namespace olg;

extern "C" float olg_wrp_plane_z(int window, int ny, int nx, float p, float plimit, float lambda, float zmin, float s)
{
    if (plimit <= 0.f) plimit = p;
    if (s >= 0.f) return zmin * s;
    if (window == OLG_WINDOW_CIRCLE) {
        // golcgh.h:566-570
        const float Wpow2 = (float)((double)(float)((float)(nx * ny) * p * p) / M_PI * 1 / 1024.f);
        const float q = p / lambda;
        const float d = (float)std::sqrt((4 * std::pow((double)q, 2) - 1) * (double)Wpow2);
        return zmin - d;
    }
    // golcgh.h:524-528 (p_limit overload :543-547)
    const float D = (float)((double)((float)nx * p) * 0.05);
    const float q = plimit / lambda;
    const float d = (float)(std::sqrt(4 * std::pow((double)q, 2) - 1) / std::sqrt(2.0) * (double)D);
    return zmin - d;
}

extern "C" int olg_wrp_step1_c64(const float *points, int n_points, void *U, int ny, int nx, float p, float lambda,
                                 float plane_z, float plimit, int window, olg_stream_t stream)
{
    if ((!points && n_points > 0) || !U) return fail(OLG_ERR_INVALID_ARG, "null pointer");
    if (n_points < 0 || ny <= 0 || nx <= 0) return fail(OLG_ERR_INVALID_ARG, "bad sizes");
    if (!(p > 0.f) || !(lambda > 0.f)) return fail(OLG_ERR_INVALID_ARG, "bad physical parameters");
    if (window != OLG_WINDOW_CIRCLE && window != OLG_WINDOW_SQUARE) return fail(OLG_ERR_INVALID_ARG, "bad window");
    cudaStream_t st = (cudaStream_t)stream;
    WrpParams P{};
    P.pts = points; P.n = n_points; P.ny = ny; P.nx = nx; P.window = window;
    P.p = p; P.lambda = lambda; P.plane_z = plane_z; P.plimit = plimit > 0.f ? plimit : p;
    DF d = split_df((double)lambda); P.l_hi = d.hi; P.l_lo = d.lo;
    P.tiles_x = (nx + WT - 1) / WT;
    P.tiles_y = (ny + WT - 1) / WT;
    const int T = P.tiles_x * P.tiles_y;
    P.U = (float2 *)U;
    const size_t nb = (size_t)(n_points > 0 ? n_points : 1);
    size_t scan_tmp = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, scan_tmp, (const int *)nullptr, (int *)nullptr, n_points + 1);
    const size_t head = align_up(nb * 4, 256) + align_up(nb * 16, 256) + 2 * align_up((nb + 1) * 4, 256) +
                        align_up((size_t)(T + 1) * 4, 256) + align_up(scan_tmp, 256);
    Scratch s1;
    if (int rc = s1.acquire(nullptr, 0, head, st)) return rc;
    char *b = (char *)s1.ptr;
    P.R = (float *)b; b += align_up(nb * 4, 256);
    P.bbox = (int4 *)b; b += align_up(nb * 16, 256);
    P.pcount = (int *)b; b += align_up((nb + 1) * 4, 256);
    P.ppos = (int *)b; b += align_up((nb + 1) * 4, 256);
    P.offset = (int *)b; b += align_up((size_t)(T + 1) * 4, 256);
    void *scan_buf = b;
    int pairs = 0;
    if (n_points > 0) {
        k_wrp_prep<<<(n_points + 1 + 255) / 256, 256, 0, st>>>(P);
        count_launch();
        if (int rc = check_launch("k_wrp_prep")) return rc;
        cudaError_t e = cub::DeviceScan::ExclusiveSum(scan_buf, scan_tmp, P.pcount, P.ppos, n_points + 1, st);
        if (e != cudaSuccess) return cuda_fail(e, "cub::DeviceScan::ExclusiveSum");
        e = cudaMemcpyAsync(&pairs, P.ppos + n_points, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(e, "reading the WRP pair count");
        if (pairs < 0) return fail(OLG_ERR_UNSUPPORTED_SIZE, "too many (tile, point) pairs");
    }
    P.pairs = pairs;
    int end_bit = 1;
    while ((1 << end_bit) < T) ++end_bit;
    size_t sort_tmp = 0;
    if (pairs > 0)
        cub::DeviceRadixSort::SortPairs(nullptr, sort_tmp, (const int *)nullptr, (int *)nullptr, (const int *)nullptr,
                                        (int *)nullptr, pairs, 0, end_bit);
    const size_t pb = align_up((size_t)(pairs > 0 ? pairs : 1) * 4, 256);
    Scratch s2;
    if (int rc = s2.acquire(nullptr, 0, 4 * pb + align_up(sort_tmp, 256), st)) return rc;
    char *c = (char *)s2.ptr;
    P.keys = (int *)c;
    P.vals = (int *)(c + pb);
    int *skeys = (int *)(c + 2 * pb), *svals = (int *)(c + 3 * pb);
    P.skeys = skeys;
    P.list = svals;
    if (pairs > 0) {
        k_wrp_pairs<<<(int)(((long)n_points * 32 + 255) / 256), 256, 0, st>>>(P);
        count_launch();
        if (int rc = check_launch("k_wrp_pairs")) return rc;
        const cudaError_t e = cub::DeviceRadixSort::SortPairs(c + 4 * pb, sort_tmp, P.keys, skeys, P.vals, svals,
                                                              pairs, 0, end_bit, st);
        if (e != cudaSuccess) return cuda_fail(e, "cub::DeviceRadixSort::SortPairs");
    }
    k_wrp_offsets<<<(T + 1 + 255) / 256, 256, 0, st>>>(P, T);
    count_launch();
    if (int rc = check_launch("k_wrp_offsets")) return rc;
    if (window == OLG_WINDOW_CIRCLE) k_wrp_tile<0><<<T, WNT, 0, st>>>(P);
    else k_wrp_tile<1><<<T, WNT, 0, st>>>(P);
    count_launch();
    return check_launch("k_wrp_tile");
}

extern "C" int olg_wrp_method_c64(const float *points, int n_points, void *U, int ny, int nx, float p, float lambda,
                                  float zmin, float s, float plimit, int window, int propmode, int flags,
                                  float *plane_z_out, olg_stream_t stream)
{
    const float pz = olg_wrp_plane_z(window, ny, nx, p, plimit, lambda, zmin, s);
    if (plane_z_out) *plane_z_out = pz;
    if (flags & OLG_VERBOSE) printf("plane z is %f, ratio is %f\n", pz, pz / zmin);
    if (int rc = olg_wrp_step1_c64(points, n_points, U, ny, nx, p, lambda, pz, plimit, window, stream)) return rc;
    // WRPStep2 golcgh.h:494-517: AUTO -> ASM if its check passes, else Fresnel if
    // its check passes, else ASM (not band-limited Fresnel); checks in float.
    int pick;
    if (propmode == OLG_FRESNEL) pick = 1;
    else if (propmode == OLG_ASM) pick = 0;
    else if (propmode == OLG_AUTO) {
        if (olg_asm_prop_check(ny, nx, p, p, lambda, pz, 1)) {
            pick = 0;
            if (flags & OLG_VERBOSE) printf("WRP Step2 is AsmProp\n");
        } else if (!olg_fresnel_prop_check(ny, nx, p, p, lambda, pz, 1)) {
            pick = 0;
            if (flags & OLG_VERBOSE) printf("warning!!\neither AsmProp or FresnelProp does not meet the condition.\n");
        } else {
            pick = 1;
            if (flags & OLG_VERBOSE) printf("WRP Step2 is FresnelProp\n");
        }
    } else {
        return fail(OLG_ERR_INVALID_ARG, "invalid PROPMODE");
    }
    if (pick == 0) return olg_asm_prop_c64(U, U, ny, nx, p, p, lambda, pz, 0, nullptr, 0, stream);
    return olg_fresnel_prop_c64(U, U, ny, nx, p, p, lambda, pz, 0, 0, nullptr, 0, stream);
}
