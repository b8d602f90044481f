// TEST INFRASTRUCTURE ONLY -- the oracle.
//
// CPU restatement of TW_Engine's reference CPU path for 2D DIC (integer-pixel
// FFT-CC followed by first-order IC-GN with a bicubic LUT).  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this
// library, and only as the parity reference / the timed CPU baseline.  The product
// (tw_gb300/) never calls it.
//
// Parity status: PINNED to the reference's own code.  The reference's
// Fftcc2D_CPU and ICGN2D_CPU are compiled from their sources
// (oracle/build_ref.py, with stand-ins for FFTW, LAPACKE, OpenCV and Qt) and
// their outputs on seeded inputs are stored in tests/golden/ref_*.npz;
// tests/test_ref_pin.py requires this restatement to reproduce them (integer
// FFT-CC equal, IC-GN flags and iteration counts equal, u and v within 1e-4
// px).  The third-party arithmetic is pinned separately: the DFT against
// numpy.fft and the Cholesky routines against the LAPACK that scipy links
// (tests/test_oracle.py).
//
// Every function follows a reference file:line (paths relative to the
// TWANG006/TW project root):
//   POI count          TW/TW_Engine/TW_paDIC_FFTCC2D.cpp:88-94
//   POI positions      TW/TW_Engine/TW_utils.cpp:29-49
//   FFT-CC per POI     TW/TW_Engine/TW_paDIC_FFTCC2D_CPU.cpp:222-326
//   gradients          TW/TW_Engine/TW_utils.cpp:232-305
//   bicubic LUT        TW/TW_Engine/TW_utils.cpp:604-700
//   IC-GN per POI      TW/TW_Engine/TW_paDIC_ICGN2D_CPU.cpp:481-925
//   IC-GN precompute   TW/TW_Engine/TW_paDIC_ICGN2D_CPU.cpp:287-319
//
// Floating-point contract: the reference was built with MSVC x64 /fp:precise
// (SSE scalar float, no contraction into FMA).  This file is compiled with
// -ffp-contract=off so every a*b+c rounds twice, as there.  Where the
// reference promotes to double (std::pow(float,int), sqrt of a double sum)
// the restatement promotes at the same place.
//
// Third-party arithmetic restated here (none of it is vendored by the
// reference, and no version is pinned there):
//   * FFTW3 single precision r2c/c2r 2D, FFTW_ESTIMATE: restated as an exact
//     unnormalised DFT (mixed-radix Cooley-Tukey, complex, row-column) in the
//     same precision.  FFTW's own rounding pattern is not reproducible.
//   * LAPACK spotrf('L') / spotrs('L'): restated as reference LAPACK's
//     unblocked spotf2 and the two strsm triangular solves.

#include <cstdint>
#include <cstring>
#include <cmath>
#include <cfloat>
#include <complex>
#include <vector>
#include <limits>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum Flag : uint8_t { kSuccess = 0, kDarkSubset = 1, kSingularHessian = 2, kSingularWarp = 3, kOutofROI = 4 };

// ---------------------------------------------------------------- FFT ----
// Mixed-radix decimation-in-time DFT of arbitrary length n (any prime factor
// handled by a direct DFT of that size).  Twiddles are computed in long double
// and rounded once to T, as FFTW's precomputed trig tables are.
template <typename T>
struct Dft1D {
    int n = 0;
    std::vector<int> fac;
    std::vector<std::complex<T>> tw;  // exp(-2 pi i k / n), k < n

    explicit Dft1D(int n_) : n(n_) {
        int m = n;
        for (int p : {4, 2, 3, 5}) {
            while (m % p == 0) { fac.push_back(p); m /= p; }
        }
        for (int p = 7; m > 1; p += 2) {
            while (m % p == 0) { fac.push_back(p); m /= p; }
        }
        tw.resize(n);
        const long double two_pi = 6.283185307179586476925286766559L;
        for (int k = 0; k < n; ++k) {
            long double a = -two_pi * (long double)k / (long double)n;
            tw[k] = std::complex<T>((T)cosl(a), (T)sinl(a));
        }
    }

    // out[k] = sum_j in[j*is] * w^(+-jk)
    void run(const std::complex<T>* in, int is, std::complex<T>* out, bool inverse) const {
        rec(in, is, out, n, 0, inverse);
    }

  private:
    std::complex<T> w(long idx, bool inverse) const {
        std::complex<T> t = tw[idx % n];
        return inverse ? std::conj(t) : t;
    }
    void rec(const std::complex<T>* in, int is, std::complex<T>* out, int len, int fi, bool inv) const {
        if (len == 1) { out[0] = in[0]; return; }
        const int p = fac[fi];
        const int m = len / p;
        for (int r = 0; r < p; ++r) rec(in + r * is, is * p, out + r * m, m, fi + 1, inv);
        const long step = n / len;  // w_len^e = w_n^(e*step)
        std::vector<std::complex<T>> tmp(len);
        for (int k = 0; k < m; ++k) {
            for (int q = 0; q < p; ++q) {
                const int kk = k + q * m;
                std::complex<T> acc = out[k];
                for (int r = 1; r < p; ++r) {
                    acc += out[r * m + k] * w((long)r * kk * step, inv);
                }
                tmp[kk] = acc;
            }
        }
        for (int k = 0; k < len; ++k) out[k] = tmp[k];
    }
};

// 2D unnormalised DFT of an [h][w] row-major complex array, in place.
template <typename T>
void dft2d(std::vector<std::complex<T>>& a, int h, int w, const Dft1D<T>& dw, const Dft1D<T>& dh, bool inverse) {
    std::vector<std::complex<T>> line(std::max(h, w)), res(std::max(h, w));
    for (int y = 0; y < h; ++y) {
        dw.run(&a[(size_t)y * w], 1, res.data(), inverse);
        for (int x = 0; x < w; ++x) a[(size_t)y * w + x] = res[x];
    }
    for (int x = 0; x < w; ++x) {
        dh.run(&a[x], w, res.data(), inverse);
        for (int y = 0; y < h; ++y) a[(size_t)y * w + x] = res[y];
    }
}

// ------------------------------------------------------------- FFT-CC ----
// Restates Fftcc2D_CPU::ComputeFFTCC (TW_paDIC_FFTCC2D_CPU.cpp:222-326).
// Returns false for a dark subset (the reference returns early and leaves the
// outputs untouched, :272-275).
template <typename T>
bool fftcc_poi(const uint8_t* ref, const uint8_t* tar, int img_w, int py, int px, int rx, int ry,
               const Dft1D<T>& dw, const Dft1D<T>& dh, std::vector<std::complex<T>>& f,
               std::vector<std::complex<T>>& g, T& out_u, T& out_v, T& out_zncc) {
    const int W = 2 * rx, H = 2 * ry;  // FFT window, no padding (:24-25)
    const int n = W * H;
    std::vector<T> s1(n), s2(n);
    T ave_r = 0, ave_t = 0;
    // fill + sums (:239-252)
    for (int i = 0; i < H; ++i) {
        for (int j = 0; j < W; ++j) {
            const size_t off = (size_t)(py - ry + i) * img_w + (px - rx + j);
            T t = s1[i * W + j] = (T)ref[off];
            ave_r += t;
            t = s2[i * W + j] = (T)tar[off];
            ave_t += t;
        }
    }
    ave_r = ave_r / T(n);
    ave_t = ave_t / T(n);
    // centre + squared norms (:256-270)
    T nor_r = 0, nor_t = 0;
    for (int i = 0; i < H; ++i) {
        for (int j = 0; j < W; ++j) {
            T t = s1[i * W + j] -= ave_r;
            nor_r += t * t;
            t = s2[i * W + j] -= ave_t;
            nor_t += t * t;
        }
    }
    // dark subset: early return, outputs untouched (:272-275)
    if (nor_r < 0.0000001 || nor_t < 0.0000001) return false;
    for (int k = 0; k < n; ++k) { f[k] = std::complex<T>(s1[k], 0); g[k] = std::complex<T>(s2[k], 0); }
    dft2d(f, H, W, dw, dh, false);
    dft2d(g, H, W, dw, dh, false);
    // conj(F) * G (:285-293)
    for (int k = 0; k < n; ++k) {
        const T ar = f[k].real(), ai = f[k].imag(), br = g[k].real(), bi = g[k].imag();
        f[k] = std::complex<T>(ar * br + ai * bi, ar * bi - ai * br);
    }
    dft2d(f, H, W, dw, dh, true);  // unnormalised c2r (:294-298)
    // first strict maximum in row-major order, initialised to -2 (:300-311)
    T zncc = -2;
    int peak = 0;
    for (int k = 0; k < n; ++k) {
        const T c = f[k].real();
        if (zncc < c) { zncc = c; peak = k; }
    }
    zncc /= std::sqrt(nor_r * nor_t) * T(n);  // (:313)
    int iu = peak % W, iv = peak / W;        // wrap to +-r (:316-325)
    if (iu > rx) iu -= W;
    if (iv > ry) iv -= H;
    out_u = (T)iu;
    out_v = (T)iv;
    out_zncc = zncc;
    return true;
}

// ---------------------------------------------------- LAPACK restated ----
// spotrf('L'), reference LAPACK spotf2 ordering: for each column j,
// ajj = a(j,j) - dot(row j), info = j if ajj <= 0 or NaN, then the column
// below the diagonal is updated with a gemv and scaled by 1/ajj.
// `a` is row-major 6x6 holding the lower triangle (LAPACKE row-major 'L').
template <typename T>
int potrf6(T* a) {
    const int n = 6;
    for (int j = 0; j < n; ++j) {
        T dot = 0;
        for (int k = 0; k < j; ++k) dot += a[j * n + k] * a[j * n + k];
        T ajj = a[j * n + j] - dot;
        if (ajj <= 0 || std::isnan(ajj)) { a[j * n + j] = ajj; return j + 1; }
        ajj = std::sqrt(ajj);
        a[j * n + j] = ajj;
        for (int i = j + 1; i < n; ++i) {
            T s = 0;
            for (int k = 0; k < j; ++k) s += a[i * n + k] * a[j * n + k];
            a[i * n + j] = a[i * n + j] - s;
        }
        const T rec = T(1) / ajj;
        for (int i = j + 1; i < n; ++i) a[i * n + j] *= rec;
    }
    return 0;
}

// spotrs('L'): L y = b (column-oriented strsm, division by the diagonal),
// then L^T x = y (dot-product strsm).
template <typename T>
void potrs6(const T* a, T* b) {
    const int n = 6;
    for (int k = 0; k < n; ++k) {
        if (b[k] != 0) {
            b[k] = b[k] / a[k * n + k];
            for (int i = k + 1; i < n; ++i) b[i] -= b[k] * a[i * n + k];
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        T t = b[i];
        for (int k = i + 1; k < n; ++k) t -= a[k * n + i] * b[k];
        b[i] = t / a[i * n + i];
    }
}

// ------------------------------------------------------- IC-GN context ----
template <typename T>
struct IcgnImages {
    const uint8_t* ref;
    const uint8_t* tar;
    int img_w, img_h, sx, sy, roi_w, roi_h;
    std::vector<T> Rx, Ry, Tx, Ty, Txy;  // [roi_h][roi_w]
    std::vector<T> lut;                  // [roi_h][roi_w][4][4], zero-initialised
};

// GradientXY_2Images_s (TW_utils.cpp:232-305), Quadratic order.
template <typename T>
void gradients(IcgnImages<T>& c) {
    const int rw = c.roi_w, rh = c.roi_h, W = c.img_w;
    c.Rx.assign((size_t)rw * rh, 0); c.Ry.assign((size_t)rw * rh, 0);
    c.Tx.assign((size_t)rw * rh, 0); c.Ty.assign((size_t)rw * rh, 0); c.Txy.assign((size_t)rw * rh, 0);
    for (int i = c.sy; i < c.sy + rh; ++i) {
        for (int j = c.sx; j < c.sx + rw; ++j) {
            auto R = [&](int y, int x) { return (int)c.ref[(size_t)y * W + x]; };
            auto G = [&](int y, int x) { return (int)c.tar[(size_t)y * W + x]; };
            const size_t o = (size_t)(i - c.sy) * rw + (j - c.sx);
            c.Rx[o] = (T)(0.5 * T(R(i, j + 1) - R(i, j - 1)));
            c.Ry[o] = (T)(0.5 * T(R(i + 1, j) - R(i - 1, j)));
            c.Tx[o] = (T)(0.5 * T(G(i, j + 1) - G(i, j - 1)));
            c.Ty[o] = (T)(0.5 * T(G(i + 1, j) - G(i - 1, j)));
            c.Txy[o] = (T)(0.25 * T(G(i + 1, j + 1) - G(i - 1, j + 1) - G(i + 1, j - 1) + G(i - 1, j - 1)));
        }
    }
}

// The 16x16 Hermite bicubic coefficient matrix (TW_utils.cpp:622-638):
// alpha = M * tau, tau = [f00 f01 f10 f11 | fx.. | fy.. | fxy..] with corner
// order (i,j),(i,j+1),(i+1,j),(i+1,j+1); alpha[4k+n] multiplies fy^k fx^n.
const int kBicubicM[16][16] = {
    { 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    { 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {-3, 3, 0, 0,-2,-1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    { 2,-2, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    { 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0},
    { 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0},
    { 0, 0, 0, 0, 0, 0, 0, 0,-3, 3, 0, 0,-2,-1, 0, 0},
    { 0, 0, 0, 0, 0, 0, 0, 0, 2,-2, 0, 0, 1, 1, 0, 0},
    {-3, 0, 3, 0, 0, 0, 0, 0,-2, 0,-1, 0, 0, 0, 0, 0},
    { 0, 0, 0, 0,-3, 0, 3, 0, 0, 0, 0, 0,-2, 0,-1, 0},
    { 9,-9,-9, 9, 6, 3,-6,-3, 6,-6, 3,-3, 4, 2, 2, 1},
    {-6, 6, 6,-6,-3,-3, 3, 3,-4, 4,-2, 2,-2,-2,-1,-1},
    { 2, 0,-2, 0, 0, 0, 0, 0, 1, 0, 1, 0, 0, 0, 0, 0},
    { 0, 0, 0, 0, 2, 0,-2, 0, 0, 0, 0, 0, 1, 0, 1, 0},
    {-6, 6, 6,-6,-4,-2, 4, 2,-3, 3,-3, 3,-2,-1,-2,-1},
    { 4,-4,-4, 4, 2, 2,-2,-2, 2,-2, 2,-2, 1, 1, 1, 1}};

// BicubicCoefficients_s (TW_utils.cpp:604-700).  The last ROI row and column
// are never written (calloc zeros) and the corner is zeroed explicitly.
template <typename T>
void bicubic_lut(IcgnImages<T>& c) {
    const int rw = c.roi_w, rh = c.roi_h, W = c.img_w;
    c.lut.assign((size_t)rw * rh * 16, 0);
    for (int i = 0; i < rh - 1; ++i) {
        for (int j = 0; j < rw - 1; ++j) {
            T tau[16];
            auto G = [&](int y, int x) { return (T)c.tar[(size_t)y * W + x]; };
            const size_t o = (size_t)i * rw + j;
            tau[0] = G(i + c.sy, j + c.sx);
            tau[1] = G(i + c.sy, j + c.sx + 1);
            tau[2] = G(i + c.sy + 1, j + c.sx);
            tau[3] = G(i + c.sy + 1, j + c.sx + 1);
            tau[4] = c.Tx[o]; tau[5] = c.Tx[o + 1]; tau[6] = c.Tx[o + rw]; tau[7] = c.Tx[o + rw + 1];
            tau[8] = c.Ty[o]; tau[9] = c.Ty[o + 1]; tau[10] = c.Ty[o + rw]; tau[11] = c.Ty[o + rw + 1];
            tau[12] = c.Txy[o]; tau[13] = c.Txy[o + 1]; tau[14] = c.Txy[o + rw]; tau[15] = c.Txy[o + rw + 1];
            for (int k = 0; k < 16; ++k) {
                T a = 0;
                for (int l = 0; l < 16; ++l) a += T(kBicubicM[k][l]) * tau[l];
                c.lut[o * 16 + k] = a;
            }
        }
    }
    for (int k = 0; k < 16; ++k) c.lut[((size_t)(rh - 1) * rw + (rw - 1)) * 16 + k] = 0;
}

// BicubicSplineCoefficients_s (TW_utils.cpp:521-602): per ROI pixel, the 4x4
// neighbourhood Omega (rows y-1..y+2, columns x-1..x+2) is prefiltered by
// the local B-spline interpolation matrix CP on both sides (Beta), mapped to
// polynomial coefficients by the cubic B-spline basis matrix (Base), and the
// 4x4 result is reversed in both indices so that entry [k][l] multiplies
// fy^k fx^l.  All ROI pixels are written.  Pixels outside the image read as 0
// (the reference reads one row and column past a one-pixel border).  The
// matrices are rounded to T once, then every product and sum is rounded in
// the reference's order.
template <typename T>
void bspline_lut(IcgnImages<T>& c) {
    const T CP[4][4] = {{T(71 / 56.0), T(-19 / 56.0), T(5 / 56.0), T(-1 / 56.0)},
                        {T(-19 / 56.0), T(95 / 56.0), T(-25 / 56.0), T(5 / 56.0)},
                        {T(5 / 56.0), T(-25 / 56.0), T(95 / 56.0), T(-19 / 56.0)},
                        {T(-1 / 56.0), T(5 / 56.0), T(-19 / 56.0), T(71 / 56.0)}};
    const T Base[4][4] = {{T(-1 / 6.0), T(3 / 6.0), T(-3 / 6.0), T(1 / 6.0)},
                          {T(3 / 6.0), T(-6 / 6.0), T(3 / 6.0), T(0)},
                          {T(-3 / 6.0), T(0), T(3 / 6.0), T(0)},
                          {T(1 / 6.0), T(4 / 6.0), T(1 / 6.0), T(0)}};
    const int rw = c.roi_w, rh = c.roi_h, W = c.img_w, H = c.img_h;
    c.lut.assign((size_t)rw * rh * 16, 0);
    for (int i = 0; i < rh; ++i) {
        for (int j = 0; j < rw; ++j) {
            T om[4][4], be[4][4], bs[4][4];
            for (int k = 0; k < 4; ++k)
                for (int l = 0; l < 4; ++l) {
                    const int y = i + c.sy - 1 + k, x = j + c.sx - 1 + l;
                    om[k][l] = (y >= 0 && y < H && x >= 0 && x < W) ? (T)c.tar[(size_t)y * W + x] : T(0);
                }
            for (int k = 0; k < 4; ++k)
                for (int l = 0; l < 4; ++l) {
                    T a = 0;
                    for (int m = 0; m < 4; ++m)
                        for (int n = 0; n < 4; ++n) a += CP[k][m] * CP[l][n] * om[n][m];
                    be[k][l] = a;
                }
            for (int k = 0; k < 4; ++k)
                for (int l = 0; l < 4; ++l) {
                    T a = 0;
                    for (int m = 0; m < 4; ++m)
                        for (int n = 0; n < 4; ++n) a += Base[k][m] * Base[l][n] * be[n][m];
                    bs[k][l] = a;
                }
            const size_t o = (size_t)i * rw + j;
            for (int k = 0; k < 4; ++k)
                for (int l = 0; l < 4; ++l) c.lut[o * 16 + k * 4 + l] = bs[3 - k][3 - l];
        }
    }
}

template <typename T>
inline T warp_coord(int base, T a, int d0, T b, int d1, T c) {
    // iPOIx + W[0][0]*(m - r) + W[0][1]*(l - r) + W[0][2], left to right
    T t = T(base) + a * T(d0);
    t = t + b * T(d1);
    return t + c;
}

// Closed-form W(P) <- W(P) o W(dP)^-1 (TW_paDIC_ICGN2D_CPU.cpp:713-745).
// Returns false for a singular warp.
template <typename T>
bool update_warp(T P[6], const T d[6], T Wm[6]) {
    const T eps = std::numeric_limits<T>::epsilon();
    const T det = (1 + d[1]) * (1 + d[5]) - d[2] * d[4];
    if (std::abs(det) <= eps) return false;
    Wm[0] = ((1 + P[1]) * (1 + d[5]) - P[2] * d[4]) / det;
    Wm[1] = (P[2] * (1 + d[1]) - (1 + P[1]) * d[2]) / det;
    Wm[2] = P[0] + (P[2] * (d[0] * d[4] - d[3] - d[3] * d[1]) - (1 + P[1]) * (d[0] * d[5] + d[0] - d[2] * d[3])) / det;
    Wm[3] = (P[4] * (1 + d[5]) - (1 + P[5]) * d[4]) / det;
    Wm[4] = ((1 + P[5]) * (1 + d[1]) - P[4] * d[2]) / det;
    Wm[5] = P[3] + ((1 + P[5]) * (d[0] * d[4] - d[3] - d[3] * d[1]) - P[4] * (d[0] * d[5] + d[0] - d[2] * d[3])) / det;
    P[0] = Wm[2];
    P[1] = Wm[0] - 1;
    P[2] = Wm[1];
    P[3] = Wm[5];
    P[4] = Wm[3];
    P[5] = Wm[4] - 1;
    return true;
}

template <typename T>
double dp_norm(const T d[6], int rx, int ry) {
    // sqrt(pow(dP0,2) + pow(dP1*rx,2) + ...) with std::pow promoting to double
    const T a1 = d[1] * T(rx), a2 = d[2] * T(ry), a4 = d[4] * T(rx), a5 = d[5] * T(ry);
    return std::sqrt(std::pow((double)d[0], 2) + std::pow((double)a1, 2) + std::pow((double)a2, 2) +
                     std::pow((double)d[3], 2) + std::pow((double)a4, 2) + std::pow((double)a5, 2));
}

// ICGN2D_CPU::ICGN2D_Compute (TW_paDIC_ICGN2D_CPU.cpp:481-925) for one POI.
// On return P holds the last accepted deformation, iters the reference's
// iteration counter (left at its input value if the POI aborts before the
// first solve), and the function value is the ICGN2DFlag.
template <typename T>
Flag icgn_poi(const IcgnImages<T>& c, int px, int py, int rx, int ry, int max_iter, float delta_p, T P[6],
              int& iters, std::vector<T>& subR, std::vector<T>& subT, std::vector<T>& desc) {
    const int SW = 2 * rx + 1, SH = 2 * ry + 1, S = SW * SH;
    const int rw = c.roi_w, W = c.img_w;
    const T eps = std::numeric_limits<T>::epsilon();
    T Hs[36];
    for (int k = 0; k < 36; ++k) Hs[k] = 0;
    P[1] = 0; P[2] = 0; P[4] = 0; P[5] = 0;  // v_P = (u,0,0,v,0,0) (:499, :601-602)
    T mean_r = 0, norm_r = 0, mean_t = 0, norm_t = 0;
    // reference subset, steepest descent, Hessian lower triangle (:516-564)
    for (int l = 0; l < SH; ++l) {
        for (int m = 0; m < SW; ++m) {
            const int idY = py - ry + l, idX = px - rx + m;
            T r = subR[l * SW + m] = (T)c.ref[(size_t)idY * W + idX];
            mean_r += r;
            const T J0[6] = {1, T(m - rx), T(l - ry), 0, 0, 0};
            const T J1[6] = {0, 0, 0, 1, T(m - rx), T(l - ry)};
            const size_t g = (size_t)(idY - c.sy) * rw + (idX - c.sx);
            T* sd = &desc[(size_t)(l * SW + m) * 6];
            for (int k = 0; k < 6; ++k) sd[k] = c.Rx[g] * J0[k] + c.Ry[g] * J1[k];
            for (int k = 0; k < 6; ++k)
                for (int n = 0; n <= k; ++n) Hs[k * 6 + n] += sd[k] * sd[n];
        }
    }
    mean_r /= T(S);  // (:580-582)
    if (std::abs(mean_r) <= eps) return kDarkSubset;
    for (int k = 0; k < S; ++k) {
        subR[k] = subR[k] - mean_r;
        norm_r += subR[k] * subR[k];
    }
    norm_r = std::sqrt(norm_r);
    if (std::abs(norm_r) <= eps) return kDarkSubset;

    T Wm[6] = {1 + P[1], P[2], P[0], P[4], 1 + P[5], P[3]};

    // iteration 1: integer-pixel target subset, no interpolation (:609-637)
    for (int l = 0; l < SH; ++l) {
        for (int m = 0; m < SW; ++m) {
            const T wx = warp_coord(px, Wm[0], m - rx, Wm[1], l - ry, Wm[2]);
            const T wy = warp_coord(py, Wm[3], m - rx, Wm[4], l - ry, Wm[5]);
            const int ix = int(wx), iy = int(wy);
            if (ix >= c.sx && iy >= c.sy && ix < c.sx + c.roi_w && iy < c.sy + c.roi_h) {
                T t = subT[l * SW + m] = (T)c.tar[(size_t)iy * W + ix];
                mean_t += t;
            } else {
                return kOutofROI;
            }
        }
    }
    mean_t /= T(S);
    if (std::abs(mean_t) <= eps) return kDarkSubset;
    for (int k = 0; k < S; ++k) {
        subT[k] = subT[k] - mean_t;
        norm_t += subT[k] * subT[k];
    }
    norm_t = std::sqrt(norm_t);
    if (std::abs(norm_t) <= eps) return kDarkSubset;
    T rhs[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < S; ++k) {
        const T e = (norm_r / norm_t) * subT[k] - subR[k];
        const T* sd = &desc[(size_t)k * 6];
        for (int j = 0; j < 6; ++j) rhs[j] += sd[j] * e;
    }
    if (potrf6(Hs) > 0) return kSingularHessian;  // (:676-693)
    potrs6(Hs, rhs);
    if (!update_warp(P, rhs, Wm)) return kSingularWarp;
    iters = 1;

    // Gauss-Newton loop (:749-908)
    while (iters < max_iter && dp_norm(rhs, rx, ry) >= (double)delta_p) {
        ++iters;
        mean_t = 0;
        norm_t = 0;
        for (int l = 0; l < SH; ++l) {
            for (int m = 0; m < SW; ++m) {
                const T wx = warp_coord(px, Wm[0], m - rx, Wm[1], l - ry, Wm[2]);
                const T wy = warp_coord(py, Wm[3], m - rx, Wm[4], l - ry, Wm[5]);
                const int ix = int(wx), iy = int(wy);
                if (ix >= c.sx && iy >= c.sy && ix < c.sx + c.roi_w && iy < c.sy + c.roi_h) {
                    const T fx = wx - T(ix), fy = wy - T(iy);
                    // sum_k sum_n LUT[k][n] * pow(fy,k) * pow(fx,n): std::pow(float,int)
                    // is evaluated in double; the float accumulator rounds per term.
                    const double dy = (double)fy, dx = (double)fx;
                    const double py4[4] = {1.0, dy, dy * dy, dy * dy * dy};
                    const double px4[4] = {1.0, dx, dx * dx, dx * dx * dx};
                    const T* a = &c.lut[((size_t)(iy - c.sy) * rw + (ix - c.sx)) * 16];
                    T t = 0;
                    for (int k = 0; k < 4; ++k)
                        for (int n = 0; n < 4; ++n) t = (T)((double)t + (double)a[k * 4 + n] * py4[k] * px4[n]);
                    subT[l * SW + m] = t;
                    mean_t += t;
                } else {
                    return kOutofROI;
                }
            }
        }
        mean_t /= T(S);
        if (std::abs(mean_t) <= eps) return kDarkSubset;
        for (int k = 0; k < S; ++k) {
            subT[k] = subT[k] - mean_t;
            norm_t += subT[k] * subT[k];
        }
        norm_t = std::sqrt(norm_t);
        if (std::abs(norm_t) <= eps) return kDarkSubset;
        for (int j = 0; j < 6; ++j) rhs[j] = 0;
        for (int k = 0; k < S; ++k) {
            T e = (norm_r / norm_t) * subT[k];
            e -= subR[k];
            const T* sd = &desc[(size_t)k * 6];
            for (int j = 0; j < 6; ++j) rhs[j] += sd[j] * e;
        }
        potrs6(Hs, rhs);
        if (!update_warp(P, rhs, Wm)) return kSingularWarp;
    }
    return kSuccess;
}

inline int set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    return omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

template <typename T>
int icgn_run(const uint8_t* ref, const uint8_t* tar, int W, int H, int sx, int sy, int rw, int rh, int rx, int ry,
             const int32_t* poi_yx, int n_poi, int max_iter, float delta_p, int nthreads, T* p6, int32_t* iters,
             uint8_t* flags, int interp = 0) {
    // ROI must leave a one-pixel border for the gradients and the LUT
    // (TW_utils.cpp:254-257, :615-619).
    if (sx < 1 || sy < 1 || sx + rw + 1 > W || sy + rh + 1 > H) return -1;
    IcgnImages<T> c;
    c.ref = ref; c.tar = tar; c.img_w = W; c.img_h = H; c.sx = sx; c.sy = sy; c.roi_w = rw; c.roi_h = rh;
    gradients(c);
    if (interp == 1)
        bspline_lut(c);  // ICGN2DInterpolationFLag::BicubicSpline (TW_paDIC_ICGN2D_CPU.cpp:322-345)
    else
        bicubic_lut(c);
    set_threads(nthreads);
    const int S = (2 * rx + 1) * (2 * ry + 1);
#pragma omp parallel
    {
        std::vector<T> subR(S), subT(S), desc((size_t)S * 6);
#pragma omp for schedule(dynamic, 16)
        for (int i = 0; i < n_poi; ++i) {
            const int py = poi_yx[2 * i + 0], px = poi_yx[2 * i + 1];
            T* P = &p6[(size_t)i * 6];
            // a subset outside the ROI cannot be formed (the reference reads
            // out of bounds there); report it as OutofROI.
            if (py - ry < sy || px - rx < sx || py + ry >= sy + rh || px + rx >= sx + rw) {
                flags[i] = kOutofROI;
                continue;
            }
            int it = iters[i];
            flags[i] = icgn_poi(c, px, py, rx, ry, max_iter, delta_p, P, it, subR, subT, desc);
            iters[i] = it;
        }
    }
    return 0;
}

template <typename T>
int fftcc_run(const uint8_t* ref, const uint8_t* tar, int W, int H, const int32_t* poi_yx, int n_poi, int rx, int ry,
              int nthreads, T* u, T* v, T* zncc, uint8_t* dark) {
    const Dft1D<T> dw(2 * rx), dh(2 * ry);
    set_threads(nthreads);
#pragma omp parallel
    {
        std::vector<std::complex<T>> f(4 * rx * ry), g(4 * rx * ry);
#pragma omp for schedule(dynamic, 16)
        for (int i = 0; i < n_poi; ++i) {
            const int py = poi_yx[2 * i + 0], px = poi_yx[2 * i + 1];
            if (py - ry < 0 || px - rx < 0 || py + ry > H || px + rx > W) { dark[i] = 2; continue; }
            const bool ok = fftcc_poi(ref, tar, W, py, px, rx, ry, dw, dh, f, g, u[i], v[i], zncc[i]);
            dark[i] = ok ? 0 : 1;
        }
    }
    return 0;
}

}  // namespace

extern "C" {

// Fftcc2D::recomputeNumPOI (TW_paDIC_FFTCC2D.cpp:88-94).
int or_num_pois(int roi_w, int roi_h, int rx, int ry, int gx, int gy, int mx, int my, int* nx, int* ny) {
    *nx = int(std::floor((roi_w - rx * 2 - mx * 2) / float(gx))) + 1;
    *ny = int(std::floor((roi_h - ry * 2 - my * 2) / float(gy))) + 1;
    return (*nx > 0 && *ny > 0) ? 0 : -1;
}

// ComputePOIPositions_s (TW_utils.cpp:29-49): (y, x) pairs, x fastest.
void or_poi_positions(int sx, int sy, int nx, int ny, int mx, int my, int rx, int ry, int gx, int gy, int32_t* yx) {
    for (int i = 0; i < ny; ++i)
        for (int j = 0; j < nx; ++j) {
            yx[2 * ((size_t)i * nx + j) + 0] = sy + my + ry + i * gy;
            yx[2 * ((size_t)i * nx + j) + 1] = sx + mx + rx + j * gx;
        }
}

// Gradients of both images and the target LUT, float32, for KATs.
int or_precompute_f32(const uint8_t* ref, const uint8_t* tar, int W, int H, int sx, int sy, int rw, int rh, float* Rx,
                      float* Ry, float* Tx, float* Ty, float* Txy, float* lut) {
    if (sx < 1 || sy < 1 || sx + rw + 1 > W || sy + rh + 1 > H) return -1;
    IcgnImages<float> c;
    c.ref = ref; c.tar = tar; c.img_w = W; c.img_h = H; c.sx = sx; c.sy = sy; c.roi_w = rw; c.roi_h = rh;
    gradients(c);
    bicubic_lut(c);
    const size_t n = (size_t)rw * rh;
    std::memcpy(Rx, c.Rx.data(), n * 4); std::memcpy(Ry, c.Ry.data(), n * 4);
    std::memcpy(Tx, c.Tx.data(), n * 4); std::memcpy(Ty, c.Ty.data(), n * 4);
    std::memcpy(Txy, c.Txy.data(), n * 4); std::memcpy(lut, c.lut.data(), n * 64);
    return 0;
}

// Integer-pixel FFT-CC over a POI list.  dark[i] = 1 for a dark subset (the
// outputs of that POI are left untouched), 2 for a window outside the image.
int or_fftcc_f32(const uint8_t* ref, const uint8_t* tar, int W, int H, const int32_t* poi_yx, int n_poi, int rx, int ry,
                 int nthreads, float* u, float* v, float* zncc, uint8_t* dark) {
    return fftcc_run<float>(ref, tar, W, H, poi_yx, n_poi, rx, ry, nthreads, u, v, zncc, dark);
}
int or_fftcc_f64(const uint8_t* ref, const uint8_t* tar, int W, int H, const int32_t* poi_yx, int n_poi, int rx, int ry,
                 int nthreads, double* u, double* v, double* zncc, uint8_t* dark) {
    return fftcc_run<double>(ref, tar, W, H, poi_yx, n_poi, rx, ry, nthreads, u, v, zncc, dark);
}

// Exact integer circular cross-correlation sum_x f(x) g(x+k) of one POI's raw
// windows, [2ry][2rx] row-major.  Its ordering equals the ordering of the
// mean-subtracted correlation (they differ by a constant), so it decides exact
// ties of the FFT-CC peak.
void or_fftcc_exact_surface(const uint8_t* ref, const uint8_t* tar, int W, int py, int px, int rx, int ry,
                            int64_t* c) {
    const int w = 2 * rx, h = 2 * ry;
    for (int ky = 0; ky < h; ++ky)
        for (int kx = 0; kx < w; ++kx) {
            int64_t s = 0;
            for (int y = 0; y < h; ++y)
                for (int x = 0; x < w; ++x) {
                    const int yy = (y + ky) % h, xx = (x + kx) % w;
                    s += (int64_t)ref[(size_t)(py - ry + y) * W + (px - rx + x)] *
                         (int64_t)tar[(size_t)(py - ry + yy) * W + (px - rx + xx)];
                }
            c[ky * w + kx] = s;
        }
}

// IC-GN over a POI list.  p6[i*6..] holds (u, ux, uy, v, vx, vy): on input
// p6[i*6+0] and p6[i*6+3] are the initial guesses (u, v from FFT-CC), on
// output the last accepted deformation.  iters[i] is updated as the
// reference updates it; flags[i] receives the ICGN2DFlag value.
int or_icgn_f32(const uint8_t* ref, const uint8_t* tar, int W, int H, int sx, int sy, int rw, int rh, int rx, int ry,
                const int32_t* poi_yx, int n_poi, int max_iter, float delta_p, int nthreads, float* p6, int32_t* iters,
                uint8_t* flags, int interp) {
    return icgn_run<float>(ref, tar, W, H, sx, sy, rw, rh, rx, ry, poi_yx, n_poi, max_iter, delta_p, nthreads, p6,
                           iters, flags, interp);
}

// The target's B-spline coefficient LUT, float32 ([rh][rw][16], entry 4k+l
// multiplies fy^k fx^l), for KATs and the GPU table's equality test.
void or_bspline_lut_f32(const uint8_t* tar, int W, int H, int sx, int sy, int rw, int rh, float* lut) {
    IcgnImages<float> c;
    c.ref = tar; c.tar = tar; c.img_w = W; c.img_h = H; c.sx = sx; c.sy = sy; c.roi_w = rw; c.roi_h = rh;
    bspline_lut(c);
    std::memcpy(lut, c.lut.data(), (size_t)rw * rh * 64);
}
int or_icgn_f64(const uint8_t* ref, const uint8_t* tar, int W, int H, int sx, int sy, int rw, int rh, int rx, int ry,
                const int32_t* poi_yx, int n_poi, int max_iter, float delta_p, int nthreads, double* p6,
                int32_t* iters, uint8_t* flags, int interp) {
    return icgn_run<double>(ref, tar, W, H, sx, sy, rw, rh, rx, ry, poi_yx, n_poi, max_iter, delta_p, nthreads, p6,
                            iters, flags, interp);
}

// Restated LAPACK kernels, exported so tests can pin them against LAPACK.
int or_potrf6_f32(float* a) { return potrf6<float>(a); }
void or_potrs6_f32(const float* a, float* b) { potrs6<float>(a, b); }

// The restated DFT, exported so tests can pin it against numpy.fft.
void or_dft2d_f64(const double* re_in, const double* im_in, int h, int w, int inverse, double* re_out, double* im_out) {
    const Dft1D<double> dw(w), dh(h);
    std::vector<std::complex<double>> a((size_t)h * w);
    for (size_t k = 0; k < a.size(); ++k) a[k] = std::complex<double>(re_in[k], im_in[k]);
    dft2d(a, h, w, dw, dh, inverse != 0);
    for (size_t k = 0; k < a.size(); ++k) { re_out[k] = a[k].real(); im_out[k] = a[k].imag(); }
}

int or_max_threads() { return set_threads(0); }

}  // extern "C"
