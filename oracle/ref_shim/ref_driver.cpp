// TEST INFRASTRUCTURE ONLY -- C entry points over the reference's own CPU
// classes, compiled with the reference's sources into oracle/_ref/libtwref.so
// by oracle/build_ref.py.  They let tests run the reference's FFT-CC and
// IC-GN on the same inputs as the oracle restatement (tw_oracle.cpp) and
// compare the two.
//
//   twref_fftcc : Fftcc2D_CPU(...) + InitializeFFTCC + Algorithm_FFTCC
//                 (TW_paDIC_FFTCC2D_CPU.cpp:8-80, 127-216, 222-326)
//   twref_icgn  : ICGN2D_CPU(refImg, ...) + ICGN2D_Algorithm, then
//                 ICGN2D_Compute once more per POI for its return flag, which
//                 ICGN2D_Algorithm discards (TW_paDIC_ICGN2D_CPU.cpp:36-132,
//                 481-925)
#include <cstdint>
#include <cstring>
#include <iostream>
#include <sstream>
#include <vector>

#include "TW_paDIC_FFTCC2D_CPU.h"
#include "TW_paDIC_ICGN2D_CPU.h"
#include "TW_MemManager.h"

using namespace TW;
using namespace TW::paDIC;

namespace {
// the reference prints timings to std::cout; keep them out of the test output
struct QuietCout {
    std::ostringstream sink;
    std::streambuf* old;
    QuietCout() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~QuietCout() { std::cout.rdbuf(old); }
};
}  // namespace

extern "C" {

// Returns the POI count, or -1 when the reference's constructor rejects the
// geometry.  poi_yx receives (y, x) pairs in the reference's order; u, v, zncc
// hold the reference's outputs (dark subsets keep the zero the reference's
// calloc gave them).  multicore: the reference's paDICThreadFlag.
int twref_fftcc(const uint8_t* ref, const uint8_t* tar, int img_w, int img_h, int sx, int sy, int roi_w, int roi_h,
                int rx, int ry, int gx, int gy, int mx, int my, int multicore, int capacity, int* poi_yx, float* u,
                float* v, float* zncc) {
    QuietCout quiet;
    try {
        Fftcc2D_CPU f(img_w, img_h, sx, sy, roi_w, roi_h, rx, ry, gx, gy, mx, my,
                      multicore ? paDICThreadFlag::Multicore : paDICThreadFlag::Single);
        const int n = f.GetNumPOIs();
        if (n > capacity) return -2;
        cv::Mat rm(img_h, img_w, CV_8UC1, const_cast<uint8_t*>(ref));
        cv::Mat tm(img_h, img_w, CV_8UC1, const_cast<uint8_t*>(tar));
        int*** POI = nullptr;
        real_t** U = nullptr;
        real_t** V = nullptr;
        real_t** Z = nullptr;
        f.InitializeFFTCC(rm, POI, U, V, Z);
        f.Algorithm_FFTCC(tm, POI, U, V, Z);
        const int nx = f.GetNumPOIsX();
        for (int i = 0; i < n; ++i) {
            const int y = i / nx, x = i % nx;
            poi_yx[2 * i] = POI[y][x][0];
            poi_yx[2 * i + 1] = POI[y][x][1];
            u[i] = U[y][x];
            v[i] = V[y][x];
            zncc[i] = Z[y][x];
        }
        f.FinalizeFFTCC(POI, U, V, Z);
        return n;
    } catch (const std::exception&) {
        return -1;
    }
}

// IC-GN of n POIs ((y, x) pairs) from the guesses in u, v (updated in place);
// iters is updated as the reference updates it (callers pass it zeroed);
// flags receives ICGN2D_Compute's return value per POI.  interp: 0 bicubic,
// 1 bicubic B-spline.  Returns 0, or 1 when the second pass did not
// reproduce ICGN2D_Algorithm's outputs.
int twref_icgn(const uint8_t* ref, const uint8_t* tar, int img_w, int img_h, int sx, int sy, int roi_w, int roi_h,
               int rx, int ry, int n, int max_iter, float delta_p, int interp, int multicore, const int* poi_yx,
               float* u, float* v, int* iters, uint8_t* flags) {
    QuietCout quiet;
    cv::Mat rm(img_h, img_w, CV_8UC1, const_cast<uint8_t*>(ref));
    cv::Mat tm(img_h, img_w, CV_8UC1, const_cast<uint8_t*>(tar));
    ICGN2D_CPU ic(rm, img_w, img_h, sx, sy, roi_w, roi_h, rx, ry, n, 1, max_iter, delta_p,
                  interp ? ICGN2DInterpolationFLag::BicubicSpline : ICGN2DInterpolationFLag::Bicubic,
                  multicore ? paDICThreadFlag::Multicore : paDICThreadFlag::Single);
    std::vector<float> u0(u, u + n), v0(v, v + n);
    std::vector<int> it0(iters, iters + n);
    ic.ICGN2D_Algorithm(u, v, iters, const_cast<int*>(poi_yx), tm);
    int mismatch = 0;
    for (int i = 0; i < n; ++i) {
        float uu = u0[i], vv = v0[i];
        int it = it0[i];
        const ICGN2DFlag fl = ic.ICGN2D_Compute(uu, vv, it, poi_yx[2 * i + 1], poi_yx[2 * i], i);
        flags[i] = (uint8_t)fl;
        if (uu != u[i] || vv != v[i] || it != iters[i]) mismatch = 1;
    }
    return mismatch;
}

}  // extern "C"
