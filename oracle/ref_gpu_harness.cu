// ref_gpu_harness.cu -- runs the reference's OWN GPU templates on given inputs.
//
// TEST INFRASTRUCTURE ONLY: this program generates golden vectors.  It is
// built by `make -C oracle ref-gpu` against an unmodified copy of the
// reference's headers (oracle/_ref/include, never committed) and is run only
// by tests/golden/make_gpu_golden.py.  Nothing in the product links or calls it.
//
// The reference has no CPU code for ARSS (golprop.h:816-995) or the windowed
// WRP step 1 (golcgh.h:291-491); their only implementation is these CUDA
// kernels, so fixtures made here pin those rows to the reference itself.
//
// Binary files are raw little-endian arrays: complex fields as (re, im)
// float32 pairs, row-major; point clouds as n x (x, y, z) float32.
//
//   ref_gpu_harness arss IN OUTDIR ny nx dy dx lambda z s oy ox
//       OUTDIR/arss_u.bin   gARSSFresnelProp_u(IN)        golprop.h:841-859
//       OUTDIR/arss_cz.bin  gARSSFresnelProp_Cz on ones   golprop.h:924-939
//       OUTDIR/arss_h.bin   gARSSFresnelProp_h, 2ny x 2nx golprop.h:886-897
//       OUTDIR/arss_out.bin ARSSFresnelProp(IN)           golprop.h:941-990
//   ref_gpu_harness wrp PTS OUT n ny nx p lambda plane_z window plimit
//       window 0: WRPStep1 (golcgh.h:369-389), 1: WRPStep1_D (golcgh.h:470-491);
//       plimit > 0 selects the p_limit overloads.
//   ref_gpu_harness time-asm|time-fresnel|time-arss ny nx p lambda z reps
//   ref_gpu_harness time-cgh ny nx n p lambda reps
//   ref_gpu_harness time-wrp N n p lambda reps
//       the reference's own gAsmProp / gFresnelProp / ARSSFresnelProp (s = 0.5),
//       gCgh (gCghShared) and WRPMethod timed on the GPU (mean ms per call).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

// golclass.h names std:: inside its own namespace `cuda`; it must come before
// any header that declares cuda::std (thrust, libcu++), or those names bind
// to cuda::std.  golprop.h pulls in thrust and uses the CPU transfer
// functions of olprop.h; golcgh.h's WRPStep2 calls golprop.h's templates.
#include "golclass.h"
#include "olprop.h"
#include "golprop.h"
#include "golcgh.h"

namespace {

using cf = thrust::complex<float>;

bool read_file(const char *path, void *dst, size_t bytes)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    const size_t got = std::fread(dst, 1, bytes, f);
    std::fclose(f);
    return got == bytes;
}

bool write_file(const std::string &path, const void *src, size_t bytes)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const size_t put = std::fwrite(src, 1, bytes, f);
    std::fclose(f);
    return put == bytes;
}

bool dump(cuda::unique_ptr<cf[]> &d, size_t n, const std::string &path)
{
    std::vector<cf> h(n);
    if (cudaMemcpy(h.data(), d.get(), n * sizeof(cf), cudaMemcpyDeviceToHost) != cudaSuccess) return false;
    return write_file(path, h.data(), n * sizeof(cf));
}

bool upload(cuda::unique_ptr<cf[]> &d, const std::vector<cf> &h)
{
    return cudaMemcpy(d.get(), h.data(), h.size() * sizeof(cf), cudaMemcpyHostToDevice) == cudaSuccess;
}

int run_arss(int argc, char **argv)
{
    if (argc != 13) return 2;
    const char *in = argv[2];
    const std::string dir = argv[3];
    const int ny = std::atoi(argv[4]), nx = std::atoi(argv[5]);
    const float dy = std::strtof(argv[6], nullptr), dx = std::strtof(argv[7], nullptr);
    const float lambda = std::strtof(argv[8], nullptr), z = std::strtof(argv[9], nullptr);
    const float s = std::strtof(argv[10], nullptr), oy = std::strtof(argv[11], nullptr);
    const float ox = std::strtof(argv[12], nullptr);
    if (ny < 16 || nx < 16 || ny > 4096 || nx > 4096) return 2;
    const size_t n = (size_t)ny * nx;
    std::vector<cf> h(n);
    if (!read_file(in, h.data(), n * sizeof(cf))) return 3;

    auto src = cuda::make_unique<cf[]>(n);
    auto dst = cuda::make_unique<cf[]>(n);
    if (!upload(src, h)) return 4;

    // stage 1 alone: the windowed pre-chirp
    ol::gARSSFresnelProp_u(src, dst, ny, nx, dy, dx, lambda, z, s, oy, ox);
    if (!dump(dst, n, dir + "/arss_u.bin")) return 5;

    // stage 3 alone on a field of ones: the post-chirp, 1 outside its window
    std::vector<cf> ones(n, cf(1.0f, 0.0f));
    auto c = cuda::make_unique<cf[]>(n);
    if (!upload(c, ones)) return 4;
    ol::gARSSFresnelProp_Cz(c, ny, nx, dy, dx, lambda, z, s, oy, ox);
    if (!dump(c, n, dir + "/arss_cz.bin")) return 5;

    // the impulse-response chirp with its window, on the padded grid
    auto hb = cuda::make_unique<cf[]>(4 * n);
    ol::gARSSFresnelProp_h(hb, 2 * ny, 2 * nx, dy, dx, lambda, z, s);
    if (!dump(hb, 4 * n, dir + "/arss_h.bin")) return 5;

    // the whole propagation
    if (!upload(src, h)) return 4;
    ol::ARSSFresnelProp(src, dst, ny, nx, dy, dx, lambda, z, s, oy, ox);
    if (!dump(dst, n, dir + "/arss_out.bin")) return 5;
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 6;
}

int run_wrp(int argc, char **argv)
{
    if (argc != 12) return 2;
    const char *pts = argv[2];
    const std::string out = argv[3];
    const int n = std::atoi(argv[4]), ny = std::atoi(argv[5]), nx = std::atoi(argv[6]);
    const float p = std::strtof(argv[7], nullptr), lambda = std::strtof(argv[8], nullptr);
    const float plane_z = std::strtof(argv[9], nullptr);
    const int window = std::atoi(argv[10]);
    const float plimit = std::strtof(argv[11], nullptr);
    if (n < 1 || n > 1000000 || ny < 1 || nx < 1 || ny > 4096 || nx > 4096) return 2;
    ol::Object<float> obj(n);
    if (!read_file(pts, obj.points.get(), (size_t)n * sizeof(ol::Vect3<float>))) return 3;
    auto gobj = ol::Object2cuda<float>(obj);
    auto U = cuda::make_unique<cf[]>((size_t)ny * nx);
    if (window == 0) {
        if (plimit > 0) ol::WRPStep1(gobj, U, ny, nx, p, lambda, plane_z, plimit);
        else ol::WRPStep1(gobj, U, ny, nx, p, lambda, plane_z);
    } else {
        if (plimit > 0) ol::WRPStep1_D(gobj, U, ny, nx, p, lambda, plane_z, plimit);
        else ol::WRPStep1_D(gobj, U, ny, nx, p, lambda, plane_z);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return 6;
    return dump(U, (size_t)ny * nx, out) ? 0 : 5;
}

// ---------------------------------------------------------------- timing
// The reference's own GPU calls on the GPU they run on, for comparison with
// this project's kernels on the same GB300.  Each mode prints one line
// "<mode> <mean ms per call> <calls>"; every call is the reference's full
// wrapper (its allocations, plans and synchronisations included), timed with
// CUDA events after two untimed calls.
struct Lcg {
    unsigned long long s;
    float next() { s = s * 6364136223846793005ULL + 1442695040888963407ULL; return (float)((s >> 40) * (1.0 / 16777216.0)); }
};

template <typename F>
double time_calls(int reps, F &&fn)
{
    fn();
    fn();
    cudaDeviceSynchronize();
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a);
    for (int r = 0; r < reps; ++r) fn();
    cudaEventRecord(b);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / reps;
}

cuda::unique_ptr<cf[]> random_field(int ny, int nx, unsigned long long seed)
{
    Lcg g{seed};
    std::vector<cf> h((size_t)ny * nx);
    for (auto &v : h) {
        const float a = g.next() < 0.5f ? 1.f : 0.f, ph = 6.2831853f * g.next();
        v = cf(a * std::cos(ph), a * std::sin(ph));
    }
    auto d = cuda::make_unique<cf[]>(h.size());
    upload(d, h);
    return d;
}

// point cloud: n points uniform in a box of edge `box` centred at
// (cx, cy, cz), or, with depth > 0, uniform over [cx +- box/2] x [cy +- box/2]
// x [cz, cz + depth]
ol::gObject<float> cloud(int n, float cx, float cy, float cz, float box, float depth, unsigned long long seed)
{
    Lcg g{seed};
    ol::Object<float> o(n);
    for (int j = 0; j < n; ++j) {
        const float x = cx + (g.next() - 0.5f) * box, y = cy + (g.next() - 0.5f) * box;
        const float z = depth > 0 ? cz + g.next() * depth : cz + (g.next() - 0.5f) * box;
        o[j] = ol::Vect3<float>(x, y, z);
    }
    return ol::Object2cuda<float>(o);
}

int run_time(int argc, char **argv)
{
    const std::string mode = argv[1];
    if (mode == "time-asm" || mode == "time-fresnel" || mode == "time-arss") {
        // ny nx p lambda z reps
        if (argc != 8) return 2;
        const int ny = std::atoi(argv[2]), nx = std::atoi(argv[3]), reps = std::atoi(argv[7]);
        const float p = std::strtof(argv[4], nullptr), lam = std::strtof(argv[5], nullptr);
        const float z = std::strtof(argv[6], nullptr);
        if (ny < 16 || nx < 16 || ny > 4096 || nx > 4096 || reps < 1) return 2;
        auto u = random_field(ny, nx, 7);
        auto v = cuda::make_unique<cf[]>((size_t)ny * nx);
        double ms;
        if (mode == "time-asm") ms = time_calls(reps, [&] { ol::gAsmProp(u, ny, nx, p, p, lam, z); });
        else if (mode == "time-fresnel") ms = time_calls(reps, [&] { ol::gFresnelProp(u, ny, nx, p, p, lam, z); });
        else ms = time_calls(reps, [&] { ol::ARSSFresnelProp(u, v, ny, nx, p, p, lam, z, 0.5f); });
        std::printf("%s %.6f %d\n", mode.c_str(), ms, reps);
        return cudaDeviceSynchronize() == cudaSuccess ? 0 : 6;
    }
    if (mode == "time-cgh") {
        // ny nx n p lambda reps: the points in a 5 mm box at z = 100 mm over the hologram centre
        if (argc != 8) return 2;
        const int ny = std::atoi(argv[2]), nx = std::atoi(argv[3]), n = std::atoi(argv[4]), reps = std::atoi(argv[7]);
        const float p = std::strtof(argv[5], nullptr), lam = std::strtof(argv[6], nullptr);
        if (ny < 1 || nx < 1 || ny > 8192 || nx > 8192 || n < 1 || n > 10000000 || reps < 1) return 2;
        auto obj = cloud(n, nx / 2 * p, ny / 2 * p, 0.1f, 5e-3f, 0.f, 11);
        auto U = cuda::make_unique<cf[]>((size_t)ny * nx);
        const double ms = time_calls(reps, [&] { ol::gCgh(obj, U, ny, nx, p, lam); });
        std::printf("%s %.6f %d\n", mode.c_str(), ms, reps);
        return cudaDeviceSynchronize() == cudaSuccess ? 0 : 6;
    }
    if (mode == "time-wrp") {
        // N n p lambda reps: n points over 10 x 10 mm, 1..5 mm behind zmin, WRPMethod (plane 0.9 zmin)
        if (argc != 7) return 2;
        const int N = std::atoi(argv[2]), n = std::atoi(argv[3]), reps = std::atoi(argv[6]);
        const float p = std::strtof(argv[4], nullptr), lam = std::strtof(argv[5], nullptr);
        if (N < 16 || N > 4096 || n < 1 || n > 10000000 || reps < 1) return 2;
        const float zmin = 0.15f;
        auto obj = cloud(n, N / 2 * p, N / 2 * p, zmin + 1e-3f, 10e-3f, 4e-3f, 13);
        auto U = cuda::make_unique<cf[]>((size_t)N * N);
        const double ms = time_calls(reps, [&] { ol::WRPMethod(obj, U, N, N, p, lam, zmin); });
        std::printf("%s %.6f %d\n", mode.c_str(), ms, reps);
        return cudaDeviceSynchronize() == cudaSuccess ? 0 : 6;
    }
    return 2;
}

} // namespace

int main(int argc, char **argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: ref_gpu_harness arss|wrp ...\n");
        return 2;
    }
    int rc = 2;
    if (!std::strcmp(argv[1], "arss")) rc = run_arss(argc, argv);
    else if (!std::strcmp(argv[1], "wrp")) rc = run_wrp(argc, argv);
    else if (!std::strncmp(argv[1], "time-", 5)) rc = run_time(argc, argv);
    if (rc) std::fprintf(stderr, "ref_gpu_harness %s: status %d\n", argv[1], rc);
    return rc;
}
