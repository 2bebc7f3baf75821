// A caller written against the reference's GPU API (the shape of the
// reference's tests/gProp_test.cu and tests/CghProp_test.cu), compiled
// against the drop-in headers and linked with libolgb300.so.  Writes each
// result as raw complex64 (or float) to <outdir>/<name>.bin for the parity test.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>

#include "openol_gb300/openol.h"

typedef float PREC_T;

template <typename T>
static void dump(const std::string &path, cuda::unique_ptr<T[]> &d, size_t n)
{
    std::unique_ptr<T[]> h;
    ol::cuda2cpu(d, h, (int)n);
    FILE *f = fopen(path.c_str(), "wb");
    fwrite(h.get(), sizeof(T), n, f);
    fclose(f);
}

int main(int argc, char **argv)
{
    const std::string out = argc > 1 ? argv[1] : ".";
    const int H = 128, W = 256;
    const PREC_T p = 8e-6f, lambda = 532e-9f, d = 0.05f;
    std::mt19937 rng(7);
    std::uniform_real_distribution<float> U01(0.f, 1.f);
    auto u = std::make_unique<std::complex<PREC_T>[]>(H * W);
    for (int i = 0; i < H * W; ++i) {
        const float a = U01(rng) < 0.5f ? 1.f : 0.f, ph = 6.2831853f * U01(rng);
        u[i] = std::complex<PREC_T>(a * std::cos(ph), a * std::sin(ph));
    }
    {
        FILE *f = fopen((out + "/input.bin").c_str(), "wb");
        fwrite(u.get(), sizeof(std::complex<PREC_T>), H * W, f);
        fclose(f);
    }
    auto d_u = cuda::make_unique<thrust::complex<PREC_T>[]>(H * W);
    ol::cpu2cuda(u, d_u, H * W);
    ol::gAsmProp(d_u, H, W, p, p, lambda, d);
    dump(out + "/asm.bin", d_u, H * W);
    ol::cpu2cuda(u, d_u, H * W);
    ol::gFresnelProp(d_u, H, W, p, p, lambda, d);
    dump(out + "/fresnel.bin", d_u, H * W);
    ol::cpu2cuda(u, d_u, H * W);
    auto d_v = cuda::make_unique<thrust::complex<PREC_T>[]>(H * W);
    ol::ARSSFresnelProp(d_u, d_v, H, W, p / 0.5f, p / 0.5f, lambda, d, 0.5f);
    dump(out + "/arss.bin", d_v, H * W);
    ol::cpu2cuda(u, d_u, H * W);
    ol::gshiftedAsmProp(d_u, d_v, H, W, p, p, lambda, d, 2e-4f, -1e-4f);
    dump(out + "/shifted_asm.bin", d_v, H * W);
    {
        auto hs = std::make_unique<std::complex<PREC_T>[]>(H * W);
        for (int i = 0; i < H * W; ++i) hs[i] = u[i];
        ol::gsplitProp(hs, H, W, p, p, lambda, d, ol::PROPMODE::ASM, 2, 2);
        FILE *f = fopen((out + "/split_asm.bin").c_str(), "wb");
        fwrite(hs.get(), sizeof(std::complex<PREC_T>), H * W, f);
        fclose(f);
    }
    {
        // tilted planes: the CPU templates of olprop.h, here on the GPU
        auto ht = std::make_unique<std::complex<PREC_T>[]>(H * W);
        for (int i = 0; i < H * W; ++i) ht[i] = u[i];
        ol::TiltedSourceProp<PREC_T>(ht, H, W, p, p, lambda, d, 0.1f, ol::BICUBIC, ol::PROPMODE::ASM);
        FILE *f = fopen((out + "/tilted_source.bin").c_str(), "wb");
        fwrite(ht.get(), sizeof(std::complex<PREC_T>), H * W, f);
        fclose(f);
    }
    ol::cpu2cuda(u, d_u, H * W);
    ol::TiltedReferenceProp<PREC_T>(d_u, H, W, p, p, lambda, d, 2e-3f, ol::BILINEAR, ol::PROPMODE::FRESNEL);
    dump(out + "/tilted_reference.bin", d_u, H * W);
    ol::cpu2cuda(u, d_u, H * W);
    ol::Prop(d_u, H, W, p, p, lambda, d, ol::PROPMODE::AUTO);
    dump(out + "/prop_auto.bin", d_u, H * W);
    // host-pointer overload (no 1/Np)
    auto hu = std::make_unique<std::complex<PREC_T>[]>(H * W);
    for (int i = 0; i < H * W; ++i) hu[i] = u[i];
    ol::gAsmProp(hu, H, W, p, p, lambda, d);
    {
        FILE *f = fopen((out + "/asm_host.bin").c_str(), "wb");
        fwrite(hu.get(), sizeof(std::complex<PREC_T>), H * W, f);
        fclose(f);
    }
    // point cloud CGH (1500 points -> tensor-core path) and its phase (direct kernel)
    const int N = 1500;
    ol::Object<PREC_T> obj(N);
    for (int j = 0; j < N; ++j)
        obj[j] = ol::Vect3<PREC_T>(U01(rng) * W * p, U01(rng) * H * p, 0.02f + 0.01f * U01(rng));
    {
        FILE *f = fopen((out + "/points.bin").c_str(), "wb");
        fwrite(obj.points.get(), sizeof(ol::Vect3<PREC_T>), N, f);
        fclose(f);
    }
    auto gobj = ol::Object2cuda(obj);
    auto d_c = cuda::make_unique<thrust::complex<PREC_T>[]>(H * W);
    ol::gCgh(gobj, d_c, H, W, p, lambda);
    dump(out + "/cgh.bin", d_c, H * W);
    auto d_ph = cuda::make_unique<float[]>(H * W);
    ol::gCgh(gobj, d_ph, H, W, p, p, lambda);
    dump(out + "/cgh_phase.bin", d_ph, H * W);
    // point file -> objset -> objsort (host Object, through the GPU), and a BMP
    {
        const int M = 300;
        FILE *f = fopen((out + "/cloud.3d").c_str(), "wb");
        const int32_t m = M;
        fwrite(&m, 4, 1, f);
        std::uniform_int_distribution<int> I(-100, 100);
        for (int j = 0; j < 3 * M; ++j) {
            const int32_t v = I(rng);
            fwrite(&v, 4, 1, f);
        }
        fclose(f);
        auto cloud = ol::objread<PREC_T>((out + "/cloud.3d").c_str());
        ol::objset(cloud, 2e-3f, ol::Vect3<PREC_T>(W / 2 * p, H / 2 * p, 0.03f), ol::ZMIN);
        ol::objsort(cloud);
        FILE *g = fopen((out + "/cloud_set_sorted.bin").c_str(), "wb");
        fwrite(cloud.points.get(), sizeof(ol::Vect3<PREC_T>), cloud.size, g);
        fclose(g);
        auto img = std::make_unique<uint8_t[]>(H * W);
        for (int i = 0; i < H * W; ++i) img[i] = (uint8_t)(i * 7);
        ol::bmpwrite((out + "/img.bmp").c_str(), img, H, W);
    }
    printf("compat_demo ok\n");
    return 0;
}
