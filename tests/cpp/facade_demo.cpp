// Drives the six reference class shapes of include/tw_dic.hpp on one image
// pair and writes their outputs for tests/test_cpp_facade.py.
//   facade_demo W H r grid margin ref.raw tar.raw out.raw
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tw_dic.hpp"

using namespace TW::paDIC;

static std::vector<unsigned char> read_raw(const char* path, size_t n) {
    std::vector<unsigned char> b(n);
    FILE* f = std::fopen(path, "rb");
    if (!f || std::fread(b.data(), 1, n, f) != n) {
        std::fprintf(stderr, "cannot read %s\n", path);
        std::exit(2);
    }
    std::fclose(f);
    return b;
}

template <typename T>
static void put(FILE* f, const T* p, size_t n) {
    std::fwrite(p, sizeof(T), n, f);
}

int main(int argc, char** argv) {
    if (argc != 9) {
        std::fprintf(stderr, "usage: facade_demo W H r grid margin ref.raw tar.raw out.raw\n");
        return 2;
    }
    const int W = std::atoi(argv[1]), H = std::atoi(argv[2]), r = std::atoi(argv[3]);
    const int grid = std::atoi(argv[4]), m = std::atoi(argv[5]);
    const std::vector<unsigned char> ref = read_raw(argv[6], (size_t)W * H), tar = read_raw(argv[7], (size_t)W * H);
    FILE* out = std::fopen(argv[8], "wb");
    try {
        // host classes
        Fftcc2D_CPU f(W, H, 1, 1, W - 2, H - 2, r, r, grid, grid, m, m, paDICThreadFlag::Multicore);
        int*** poi = nullptr;
        float **U = nullptr, **V = nullptr, **Z = nullptr;
        f.InitializeFFTCC(ImageView(ref.data(), W, H), poi, U, V, Z);
        f.Algorithm_FFTCC(ImageView(tar.data(), W, H), poi, U, V, Z);
        const int n = f.GetNumPOIs();
        ICGN2D_CPU ic(ImageView(ref.data(), W, H), W, H, 1, 1, W - 2, H - 2, r, r, f.GetNumPOIsX(), f.GetNumPOIsY(),
                      20, 0.001f, ICGN2DInterpolationFLag::Bicubic, paDICThreadFlag::Multicore);
        std::vector<float> u(U[0], U[0] + n), v(V[0], V[0] + n);
        std::vector<int> it(n, 0);
        ic.ICGN2D_Algorithm(u.data(), v.data(), it.data(), poi[0][0], ImageView(tar.data(), W, H));
        const int32_t hdr[2] = {n, 0};
        put(out, hdr, 2);
        put(out, poi[0][0], 2 * (size_t)n);
        put(out, U[0], n);
        put(out, V[0], n);
        put(out, Z[0], n);
        put(out, u.data(), n);
        put(out, v.data(), n);
        put(out, it.data(), n);
        put(out, ic.Flags().data(), n);
        put(out, ic.Deformation().data(), 6 * (size_t)n);
        // device classes
        unsigned char *d_ref = nullptr, *d_tar = nullptr;
        int* d_poi = nullptr;
        cudaMalloc(&d_ref, (size_t)W * H);
        cudaMalloc(&d_tar, (size_t)W * H);
        cudaMalloc(&d_poi, sizeof(int) * 2 * (size_t)n);
        cudaMemcpy(d_ref, ref.data(), (size_t)W * H, cudaMemcpyHostToDevice);
        cudaMemcpy(d_tar, tar.data(), (size_t)W * H, cudaMemcpyHostToDevice);
        cudaMemcpy(d_poi, poi[0][0], sizeof(int) * 2 * (size_t)n, cudaMemcpyHostToDevice);
        cuFFTCC2D cf(W, H, W - 2, H - 2, 1, 1, r, r, grid, grid, m, m);
        float *dU = nullptr, *dV = nullptr, *dZ = nullptr;
        cf.cuInitializeFFTCC(dU, dV, dZ, ImageView(d_ref, W, H, W, true));
        cf.cuComputeFFTCC(dU, dV, dZ, ImageView(d_tar, W, H, W, true));
        cuICGN2D cic(W, H, 1, 1, W - 2, H - 2, r, r, cf.GetNumPOIsX(), cf.GetNumPOIsY(), 20, 0.001f,
                     ICGN2DInterpolationFLag::Bicubic);
        cic.cuInitialize(reinterpret_cast<uchar1*>(d_ref));
        cic.cuCompute(reinterpret_cast<uchar1*>(d_tar), d_poi, dU, dV);
        std::vector<float> gu(n), gv(n);
        cudaMemcpy(gu.data(), dU, sizeof(float) * n, cudaMemcpyDeviceToHost);
        cudaMemcpy(gv.data(), dV, sizeof(float) * n, cudaMemcpyDeviceToHost);
        put(out, gu.data(), n);
        put(out, gv.data(), n);
        // the B-spline interpolation flag (ICGN2DInterpolationFLag::BicubicSpline)
        ICGN2D_CPU bic(ImageView(ref.data(), W, H), W, H, 1, 1, W - 2, H - 2, r, r, f.GetNumPOIsX(),
                       f.GetNumPOIsY(), 20, 0.001f, ICGN2DInterpolationFLag::BicubicSpline, paDICThreadFlag::Multicore);
        std::vector<float> bu(U[0], U[0] + n), bv(V[0], V[0] + n);
        std::vector<int> bit(n, 0);
        bic.ICGN2D_Algorithm(bu.data(), bv.data(), bit.data(), poi[0][0], ImageView(tar.data(), W, H));
        put(out, bu.data(), n);
        put(out, bv.data(), n);
        put(out, bit.data(), n);
        put(out, bic.Flags().data(), n);
        cic.cuFinalize();
        cf.cuDestroyFFTCC(dU, dV, dZ);
        f.FinalizeFFTCC(poi, U, V, Z);
        cudaFree(d_ref);
        cudaFree(d_tar);
        cudaFree(d_poi);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    std::fclose(out);
    // constructor errors surface as std::logic_error
    try {
        Fftcc2D_CPU bad(100, 100, 0, 0, 100, 100, 60, 60, 5, 5, 0, 0, paDICThreadFlag::Single);
        std::fprintf(stderr, "expected a logic_error\n");
        return 1;
    } catch (const std::logic_error&) {
    }
    std::printf("ok\n");
    return 0;
}
