// wrp.cu -- wavefront-recording-plane method on GB300 (sm_103a).
//
// Step 1 of the reference (WRPStep1 golcgh.h:303-378, WRPStep1_D
// golcgh.h:403-491) loops every WRP pixel over every point and keeps the few
// inside the point's window: O(pixels x points) tests for ~sum_j pi W_j^2
// useful terms.  Here the points are binned onto 16 x 16 pixel tiles by the
// bounding box of their window, and one CTA per tile sums only the points
// listed for it:
//   k_wrp_prep   per point: window radius (float, as the reference computes
//                it), tile bounding box, per-tile counts (atomics)
//   k_wrp_scan   exclusive scan of the counts (one CTA)
//   k_wrp_fill   per point: append its index to each covered tile's list
//   k_wrp_tile   per tile: sort the list (deterministic order), then for each
//                pixel x listed point: window test in float32 exactly as the
//                reference evaluates it (each operation rounded), and the
//                term exp(i pi rho^2 / (lambda dz)) / |dz| with the phase anchored
//                at the tile centre in double-float arithmetic.
// Step 2 is the fused propagation in prop.cu.
#include <cmath>
#include <cstdio>

#include "common.cuh"

namespace olg {

constexpr int WT = 16;          // tile edge (pixels)
constexpr int WLIST_MAX = 4096; // list entries sorted in shared memory

struct WrpParams {
    const float *pts;
    int n, ny, nx, tiles_x, tiles_y, window;
    float p, lambda, plane_z, plimit;
    float l_hi, l_lo;
    float *R;    // per point: W (circle) or D (square)
    int4 *bbox;  // per point: tile range [tx0, tx1] x [ty0, ty1], tx0 > tx1 if none
    int *count;  // tiles + 1
    int *offset; // tiles + 1
    int *cursor; // tiles
    int *list;
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
    if (w0 > w1 || h0 > h1 || !(R > 0.f)) {
        bb = make_int4(1, 0, 1, 0);
    } else {
        bb = make_int4((int)(w0 / WT), (int)(w1 / WT), (int)(h0 / WT), (int)(h1 / WT));
        for (int ty = bb.z; ty <= bb.w; ++ty)
            for (int tx = bb.x; tx <= bb.y; ++tx) atomicAdd(P.count + ty * P.tiles_x + tx, 1);
    }
    P.bbox[j] = bb;
}

// exclusive scan of count[0..T) into offset[0..T], one CTA of 1024 threads
__global__ void __launch_bounds__(1024) k_wrp_scan(const int *count, int *offset, int *cursor, int T)
{
    __shared__ int part[1024];
    const int tid = threadIdx.x;
    const int per = (T + 1023) / 1024;
    const int b = tid * per, e = min(b + per, T);
    int s = 0;
    for (int i = b; i < e; ++i) s += count[i];
    part[tid] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int v = tid >= off ? part[tid - off] : 0;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    int run = part[tid] - s;
    for (int i = b; i < e; ++i) {
        offset[i] = run;
        cursor[i] = run;
        run += count[i];
    }
    if (tid == 1023) offset[T] = part[1023];
}

__global__ void k_wrp_fill(WrpParams P)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= P.n) return;
    const int4 bb = P.bbox[j];
    for (int ty = bb.z; ty <= bb.w; ++ty)
        for (int tx = bb.x; tx <= bb.y; ++tx) {
            const int pos = atomicAdd(P.cursor + ty * P.tiles_x + tx, 1);
            P.list[pos] = j;
        }
}

__device__ __forceinline__ void bitonic_sort(int *a, int n, int tid, int nt)
{
    for (int k = 2; k <= n; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < n; i += nt) {
                const int l = i ^ j;
                if (l > i) {
                    const int ai = a[i], al = a[l];
                    const bool up = (i & k) == 0;
                    if ((ai > al) == up) { a[i] = al; a[l] = ai; }
                }
            }
            __syncthreads();
        }
}

__global__ void __launch_bounds__(256) k_wrp_tile(WrpParams P)
{
    __shared__ int ids[WLIST_MAX];
    __shared__ float4 cst[256][2]; // {c0, ax, ay, b} {x, y, Rtest, A}
    const int tid = threadIdx.x;
    const int t = blockIdx.x;
    const int tx_t = t % P.tiles_x, ty_t = t / P.tiles_x;
    const int w = tx_t * WT + (tid & 15), h = ty_t * WT + (tid >> 4);
    const float dw = (float)(tid & 15) - 7.5f, dh = (float)(tid >> 4) - 7.5f;
    const float q2 = dw * dw + dh * dh;
    const float wc = (float)(tx_t * WT) + 7.5f, hc = (float)(ty_t * WT) + 7.5f;
    // per-pixel window-test operands, rounded as the reference's float code
    const float pw = __fmul_rn(P.p, (float)w), ph = __fmul_rn(P.p, (float)h);
    const int beg = P.offset[t], cnt = P.offset[t + 1] - beg;
    float2 acc = make_float2(0.f, 0.f);
    const bool sorted = cnt <= WLIST_MAX;
    if (sorted) {
        int np2 = 1;
        while (np2 < cnt) np2 <<= 1;
        for (int i = tid; i < np2; i += 256) ids[i] = i < cnt ? P.list[beg + i] : 0x7fffffff;
        __syncthreads();
        bitonic_sort(ids, np2, tid, 256);
    }
    for (int b0 = 0; b0 < cnt; b0 += 256) {
        const int k = b0 + tid;
        float4 c0 = make_float4(0.f, 0.f, 0.f, 0.f), c1 = make_float4(0.f, 0.f, -1.f, 0.f);
        if (k < cnt) {
            const int j = sorted ? ids[k] : P.list[beg + k];
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
            const float Rt = P.window == 0 ? __fmul_rn(R, R) : R;
            c1 = make_float4(x, y, Rt, 1.0f / fabsf(dz.hi + dz.lo));
        }
        cst[tid][0] = c0;
        cst[tid][1] = c1;
        __syncthreads();
        const int m = min(256, cnt - b0);
        float2 part = make_float2(0.f, 0.f);
        for (int i = 0; i < m; ++i) {
            const float4 a = cst[i][0], b = cst[i][1];
            const float ddx = __fsub_rn(pw, b.x), ddy = __fsub_rn(ph, b.y);
            bool inside;
            if (P.window == 0) {
                inside = __fadd_rn(__fmul_rn(ddx, ddx), __fmul_rn(ddy, ddy)) < b.z;
            } else {
                inside = (__fmul_rn(fabsf(ddx), 2.0f) <= b.z) && (__fmul_rn(fabsf(ddy), 2.0f) <= b.z);
            }
            if (inside) {
                const float c = fmaf(a.y, dw, fmaf(a.z, dh, fmaf(a.w, q2, a.x)));
                const float2 e = cis_cycles(wrap_cycles(c));
                part.x = fmaf(b.w, e.x, part.x);
                part.y = fmaf(b.w, e.y, part.y);
            }
        }
        acc.x += part.x;
        acc.y += part.y;
        __syncthreads();
    }
    if (w < P.nx && h < P.ny) P.U[(size_t)h * P.nx + w] = acc;
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
    const size_t head = align_up(nb * 4, 256) + align_up(nb * 16, 256) + 3 * align_up((size_t)(T + 1) * 4, 256);
    Scratch s1;
    if (int rc = s1.acquire(nullptr, 0, head, st)) return rc;
    char *b = (char *)s1.ptr;
    P.R = (float *)b; b += align_up(nb * 4, 256);
    P.bbox = (int4 *)b; b += align_up(nb * 16, 256);
    P.count = (int *)b; b += align_up((size_t)(T + 1) * 4, 256);
    P.offset = (int *)b; b += align_up((size_t)(T + 1) * 4, 256);
    P.cursor = (int *)b;
    cudaError_t e = cudaMemsetAsync(P.count, 0, (size_t)(T + 1) * 4, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
    if (n_points > 0) {
        k_wrp_prep<<<(n_points + 255) / 256, 256, 0, st>>>(P);
        count_launch();
        if (int rc = check_launch("k_wrp_prep")) return rc;
    }
    k_wrp_scan<<<1, 1024, 0, st>>>(P.count, P.offset, P.cursor, T);
    count_launch();
    if (int rc = check_launch("k_wrp_scan")) return rc;
    int total = 0;
    e = cudaMemcpyAsync(&total, P.offset + T, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "reading the WRP pair count");
    Scratch s2;
    if (int rc = s2.acquire(nullptr, 0, (size_t)(total > 0 ? total : 1) * 4, st)) return rc;
    P.list = (int *)s2.ptr;
    if (n_points > 0) {
        k_wrp_fill<<<(n_points + 255) / 256, 256, 0, st>>>(P);
        count_launch();
        if (int rc = check_launch("k_wrp_fill")) return rc;
    }
    k_wrp_tile<<<T, 256, 0, st>>>(P);
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
