// A caller written against the reference's GPU API (the shape of the
// reference's tests/gProp_test.cu and tests/CghProp_test.cu), compiled
// against the drop-in headers and linked with libolgb300.so.  Writes each
// result as raw complex64 (or float) to <outdir>/<name>.bin for the parity test.
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <memory>
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
    // host-field templates of olprop.h / olcgh.h (the reference's CPU API)
    {
        auto w32 = [&](const std::string &name, std::unique_ptr<std::complex<float>[]> &a) {
            FILE *f = fopen((out + "/" + name + ".bin").c_str(), "wb");
            fwrite(a.get(), sizeof(std::complex<float>), H * W, f);
            fclose(f);
        };
        auto w64 = [&](const std::string &name, std::unique_ptr<std::complex<double>[]> &a) {
            FILE *f = fopen((out + "/" + name + ".bin").c_str(), "wb");
            fwrite(a.get(), sizeof(std::complex<double>), H * W, f);
            fclose(f);
        };
        auto copy32 = [&]() {
            auto a = std::make_unique<std::complex<float>[]>(H * W);
            for (int i = 0; i < H * W; ++i) a[i] = u[i];
            return a;
        };
        auto copy64 = [&]() {
            auto a = std::make_unique<std::complex<double>[]>(H * W);
            for (int i = 0; i < H * W; ++i) a[i] = std::complex<double>(u[i].real(), u[i].imag());
            return a;
        };
        auto a = copy64();
        ol::AsmProp(a, H, W, (double)p, (double)p, (double)lambda, 0.02);
        w64("host_asm_f64", a);
        auto b = copy32();
        ol::AsmProp<float>(b, H, W, p, p, lambda, 0.02f);
        w32("host_asm_f32", b);
        auto c = copy64();
        ol::FresnelProp(c, H, W, (double)p, (double)p, (double)lambda, 0.1);
        w64("host_fresnel", c);
        auto e = copy64();
        ol::FresnelPropBandLimit(e, H, W, (double)p, (double)p, (double)lambda, 0.05);
        w64("host_fresnel_bl", e);
        const double zs[3] = {0.02, 0.05, 0.1};
        for (int k = 0; k < 3; ++k) {
            auto f = copy64();
            ol::Prop(f, H, W, (double)p, (double)p, (double)lambda, zs[k], ol::PROPMODE::AUTO);
            w64("host_prop_auto" + std::to_string(k), f);
        }
        auto g = copy64();
        std::unique_ptr<std::complex<double>[]> gd;
        ol::shiftedAsmProp(g, gd, H, W, (double)p, (double)p, (double)lambda, 0.02, 2e-4, -1e-4);
        w64("host_shifted_asm", gd);
        auto sf = copy32();
        ol::shiftedFresnelProp(sf, H, W, p, p, lambda, 0.05f, 0.7f, 1e-4f, 0.f);
        w32("host_shifted_fresnel", sf);
        auto sp = copy32();
        ol::splitAsmProp(sp, H, W, p, p, lambda, 0.02f, 2, 2);
        w32("host_split_asm", sp);
        // Cgh: the four overloads, float and double clouds
        ol::Object<double> objd(N);
        for (int j = 0; j < N; ++j) objd[j] = ol::Vect3<double>(obj[j].x, obj[j].y, obj[j].z);
        std::unique_ptr<std::complex<double>[]> hc;
        ol::Cgh(objd, hc, H, W, (double)p, (double)lambda);
        w64("host_cgh", hc);
        std::unique_ptr<std::complex<float>[]> hc2;
        ol::Cgh(obj, hc2, H, W, p, p, lambda);
        w32("host_cgh_pypx", hc2);
        std::unique_ptr<float[]> hp;
        ol::Cgh(obj, hp, H, W, p, lambda);
        std::unique_ptr<double[]> hp2;
        ol::Cgh(objd, hp2, H, W, (double)p, (double)p, (double)lambda);
        {
            FILE *f = fopen((out + "/host_cgh_phase.bin").c_str(), "wb");
            fwrite(hp.get(), sizeof(float), H * W, f);
            fclose(f);
            f = fopen((out + "/host_cgh_phase_f64.bin").c_str(), "wb");
            fwrite(hp2.get(), sizeof(double), H * W, f);
            fclose(f);
        }
        std::unique_ptr<std::complex<float>[]> hw;
        ol::WRPStep1(obj, hw, H, W, p, lambda, 0.f);
        w32("host_wrp_step1", hw);
        // WRPStep2 on a device field: AUTO at 0.02 (ASM) and 0.1 (Fresnel)
        for (int k = 0; k < 2; ++k) {
            ol::cpu2cuda(u, d_u, H * W);
            ol::WRPStep2(d_u, H, W, p, lambda, k == 0 ? 0.02f : 0.1f);
            dump(out + "/wrp_step2_" + std::to_string(k) + ".bin", d_u, H * W);
        }
    }
    printf("compat_demo ok\n");
    return 0;
}
