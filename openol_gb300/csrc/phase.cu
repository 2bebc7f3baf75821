// phase.cu -- multi-plane phase-only hologram optimisation: loss, gradient by
// the hand-written adjoint, Adam step (olg_phase_*).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <map>
#include <mutex>
#include <set>
#include <vector>

#include "common.cuh"
#include "fft.cuh"
#include "prophost.cuh"

using namespace olg;

// ------------------------------------------- multi-plane phase optimisation
// Phase-only hologram phi (ny x nx) propagated by ASM to P depth planes;
// loss L = sum_p mean((|A_p e^{i phi}|^2 - t_p)^2).  Per plane: the forward
// propagation, whose pass 3 writes the seed dL/dv* = (2/n)(|v|^2 - t) v (and
// sums the loss), then the adjoint propagation (conjugate transfer function)
// of the seed, accumulated into g = dL/du*.  No plane's field is stored.
// dL/dphi = -2 Im(u conj(g)).  For padded heights 256..8192 the planes share
// the forward spectrum of e^{i phi} and sum their adjoint spectra (spec.cu);
// otherwise each plane runs two full three-pass propagations.
namespace olg {

__global__ void k_phase_grad(const float *phi, const float2 *g, float *grad, long n)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float s, c;
        sincosf(phi[i], &s, &c);
        const float2 G = g[i];
        grad[i] = 2.0f * (c * G.y - s * G.x);
    }
}

__global__ void k_adam(float *phi, float *m, float *v, const float2 *g, long n, float lr, float b1, float b2, float eps,
                       float bc1, float bc2)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float ph = phi[i];
        float s, c;
        sincosf(ph, &s, &c);
        const float2 G = g[i];
        const float gr = 2.0f * (c * G.y - s * G.x);
        const float mm = b1 * m[i] + (1.0f - b1) * gr;
        const float vv = b2 * v[i] + (1.0f - b2) * gr * gr;
        m[i] = mm;
        v[i] = vv;
        phi[i] = ph - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
    }
}

__global__ void k_loss_scale(double *loss, double s) { *loss *= s; }

int elem_grid(long n)
{
    long g = (n + 255) / 256;
    const long cap = 8L * sm_count(); // grid-stride beyond eight CTAs per SM
    return (int)(g > cap ? cap : (g < 1 ? 1 : g));
}

PropParams asm_params(const void *in, void *out, int ny, int nx, double dy, double dx, double lambda, double z, bool conj,
                      const Layout &L)
{
    PropParams P = base_params(in, out, ny, nx, L);
    const double NX = 2.0 * nx, NY = 2.0 * ny;
    const double du = 1.0 / (dx * NX), dv = 1.0 / (dy * NY);
    const double zl = z / lambda;
    P.method = M_ASM;
    P.conj = conj ? 1 : 0;
    P.scale = (float)(1.0 / (NX * NY));
    P.c0 = frac_host(zl);
    set_quad(P.ax_hi, P.ax_lo, z * lambda * du * du / 2.0);
    set_quad(P.ay_hi, P.ay_lo, z * lambda * dv * dv / 2.0);
    P.tx = (float)(lambda * lambda * du * du);
    P.ty = (float)(lambda * lambda * dv * dv);
    P.zl = (float)zl;
    P.tf_series = asm_series_ok(NY, NX, dv, du, lambda);
    return P;
}

// [propagation layout][seed][g][loss][F0: NY x NX][G: NY x NX]
size_t phase_ws(int ny, int nx, size_t *off_seed, size_t *off_g, size_t *off_loss, size_t *off_spec = nullptr)
{
    const size_t lb = layout_bytes(ny, nx, nullptr, nullptr);
    const size_t f = align_up((size_t)ny * nx * sizeof(float2), 256);
    if (off_seed) *off_seed = lb;
    if (off_g) *off_g = lb + f;
    if (off_loss) *off_loss = lb + 2 * f;
    if (off_spec) *off_spec = lb + 2 * f + 256;
    return lb + 2 * f + 256 + 2 * 4 * f;
}

int phase_loss_grad(const float *phi, const float *targets, const double *z, int np, int ny, int nx, double dy,
                    double dx, double lambda, char *ws, float2 *g, double *loss, cudaStream_t st)
{
    size_t os, og, ol;
    phase_ws(ny, nx, &os, &og, &ol);
    Layout L;
    layout_bytes(ny, nx, &L, ws);
    float2 *seed = (float2 *)(ws + os);
    const long n = (long)ny * nx;
    cudaError_t e = cudaMemsetAsync(loss, 0, sizeof(double), st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(loss)");
    if (spec_cols_ok(2 * ny)) {
        // Every plane's forward propagation starts from the same e^{i phi}: its
        // padded spectrum F0 is formed once.  The adjoints are linear in their
        // seeds, so their conjugate-transfer-function spectra add into G and
        // one inverse transform gives g.  Per plane this leaves one inverse
        // and one forward column transform and two row passes.
        size_t ospec;
        phase_ws(ny, nx, nullptr, nullptr, nullptr, &ospec);
        float2 *F0 = (float2 *)(ws + ospec);
        float2 *G = F0 + (size_t)4 * n;
        SpecArgs A{};
        A.ny = ny; A.NY = 2 * ny; A.NX = 2 * nx;
        PropParams R = asm_params(nullptr, nullptr, ny, nx, dy, dx, lambda, z[0], false, L);
        R.in_phase = phi;
        if (int rc = rows_pass(R, false, st)) return rc;
        A.in = L.S; A.out = F0; A.tf = 0; A.accumulate = 0;
        if (int rc = spec_cols(A, false, st)) return rc;
        for (int p = 0; p < np; ++p) {
            PropParams F = asm_params(nullptr, seed, ny, nx, dy, dx, lambda, z[p], false, L);
            F.post_mode = OP_SEED;
            F.target = targets + (size_t)p * n;
            F.seed_scale = (float)(2.0 / (double)n);
            F.loss = loss;
            A.in = F0; A.out = L.S; A.tf = 1; A.accumulate = 0; A.P = F;
            if (int rc = spec_cols(A, true, st)) return rc;
            PropParams B = asm_params(seed, nullptr, ny, nx, dy, dx, lambda, z[p], true, L);
            if (2 * nx >= 256) {
                // the seed goes from the forward's inverse row FFT to the
                // adjoint's forward row FFT in registers
                if (int rc = rows_seed_pass(F, st)) return rc;
            } else {
                if (int rc = rows_pass(F, true, st)) return rc;
                if (int rc = rows_pass(B, false, st)) return rc;
            }
            A.in = L.S; A.out = G; A.tf = 1; A.accumulate = p > 0 ? 1 : 0; A.P = B;
            if (int rc = spec_cols(A, false, st)) return rc;
        }
        A.in = G; A.out = L.S; A.tf = 0; A.accumulate = 0;
        if (int rc = spec_cols(A, true, st)) return rc;
        PropParams Gp = asm_params(nullptr, g, ny, nx, dy, dx, lambda, z[0], false, L);
        if (int rc = rows_pass(Gp, true, st)) return rc;
        k_loss_scale<<<1, 1, 0, st>>>(loss, 1.0 / (double)n);
        count_launch();
        return check_launch("k_loss_scale");
    }
    for (int p = 0; p < np; ++p) {
        PropParams F = asm_params(nullptr, seed, ny, nx, dy, dx, lambda, z[p], false, L);
        F.in_phase = phi;
        F.post_mode = OP_SEED;
        F.target = targets + (size_t)p * n;
        F.seed_scale = (float)(2.0 / (double)n);
        F.loss = loss;
        if (int rc = run_passes(F, st)) return rc;
        PropParams B = asm_params(seed, g, ny, nx, dy, dx, lambda, z[p], true, L);
        B.accumulate = p > 0 ? 1 : 0;
        if (int rc = run_passes(B, st)) return rc;
    }
    k_loss_scale<<<1, 1, 0, st>>>(loss, 1.0 / (double)n);
    count_launch();
    return check_launch("k_loss_scale");
}

int phase_checks(const void *phi, const void *targets, const double *z, int np, int ny, int nx)
{
    if (!phi || !targets || !z || np <= 0) return fail(OLG_ERR_INVALID_ARG, "null pointer or no planes");
    if (((uintptr_t)phi & 7) || ((uintptr_t)targets & 7)) return fail(OLG_ERR_INVALID_ARG, "phi / targets must be 8-byte aligned");
    if (!is_pow2(nx) || !is_pow2(ny) || nx < 16 || ny < 16 || 2 * nx > FFT_MAX || 2 * ny > FFT_MAX)
        return fail(OLG_ERR_UNSUPPORTED_SIZE, "ny, nx must be powers of two in [16, 4096]");
    return OLG_OK;
}

} // namespace olg

extern "C" size_t olg_phase_opt_workspace_bytes(int ny, int nx)
{
    if (ny <= 0 || nx <= 0) return 0;
    return phase_ws(ny, nx, nullptr, nullptr, nullptr);
}

extern "C" int olg_phase_loss_grad(const float *phi, const float *targets, const double *z, int n_planes, int ny,
                                   int nx, double dy, double dx, double lambda, float *grad, double *loss,
                                   void *work, size_t work_bytes, olg_stream_t stream)
{
    if (int rc = phase_checks(phi, targets, z, n_planes, ny, nx)) return rc;
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, phase_ws(ny, nx, nullptr, nullptr, nullptr), st)) return rc;
    size_t os, og, ol;
    phase_ws(ny, nx, &os, &og, &ol);
    char *ws = (char *)sc.ptr;
    float2 *g = (float2 *)(ws + og);
    double *dl = loss ? loss : (double *)(ws + ol);
    if (int rc = phase_loss_grad(phi, targets, z, n_planes, ny, nx, dy, dx, lambda, ws, g, dl, st)) return rc;
    if (grad) {
        const long n = (long)ny * nx;
        k_phase_grad<<<elem_grid(n), 256, 0, st>>>(phi, g, grad, n);
        count_launch();
        return check_launch("k_phase_grad");
    }
    return OLG_OK;
}

extern "C" int olg_phase_adam_step(float *phi, float *m, float *v, const float *targets, const double *z, int n_planes,
                                   int ny, int nx, double dy, double dx, double lambda, double lr, double beta1,
                                   double beta2, double eps, int step, double *loss, void *work, size_t work_bytes,
                                   olg_stream_t stream)
{
    if (int rc = phase_checks(phi, targets, z, n_planes, ny, nx)) return rc;
    if (!m || !v || step < 1) return fail(OLG_ERR_INVALID_ARG, "Adam state missing or step < 1");
    if (int rc = ensure_twiddles()) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    Scratch sc;
    if (int rc = sc.acquire(work, work_bytes, phase_ws(ny, nx, nullptr, nullptr, nullptr), st)) return rc;
    size_t os, og, ol;
    phase_ws(ny, nx, &os, &og, &ol);
    char *ws = (char *)sc.ptr;
    float2 *g = (float2 *)(ws + og);
    double *dl = loss ? loss : (double *)(ws + ol);
    if (int rc = phase_loss_grad(phi, targets, z, n_planes, ny, nx, dy, dx, lambda, ws, g, dl, st)) return rc;
    const long n = (long)ny * nx;
    const float bc1 = (float)(1.0 - std::pow(beta1, step)), bc2 = (float)(1.0 - std::pow(beta2, step));
    k_adam<<<elem_grid(n), 256, 0, st>>>(phi, m, v, g, n, (float)lr, (float)beta1, (float)beta2, (float)eps, bc1, bc2);
    count_launch();
    return check_launch("k_adam");
}

