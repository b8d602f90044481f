// TEST INFRASTRUCTURE ONLY -- implementations behind the stand-in headers of
// this folder, linked only into oracle/_ref/libtwref.so (the reference's own
// CPU sources compiled by oracle/build_ref.py).
//
// * FFTW3 single-precision 2D r2c / c2r (the calls of
//   TW_paDIC_FFTCC2D_CPU.cpp:62-73, 279-298): FFTW's definition of the
//   unnormalised transforms, evaluated as separable direct DFTs in double with
//   exactly reduced angles ((k j) mod n) and rounded once to float.  This is an
//   independent evaluation from the oracle's FP32 mixed-radix FFT, so the two
//   agree on the integer peak except where the correlation values tie within
//   FP32 rounding.
// * LAPACKE_spotrf / LAPACKE_spotrs in row-major layout (the calls of
//   TW_paDIC_ICGN2D_CPU.cpp:682-683, 853): LAPACKE's row-major convention
//   (transpose in, Fortran routine, transpose out) over the Fortran spotrf_ /
//   spotrs_ whose addresses the test process hands over (the LAPACK scipy
//   links), so the Cholesky arithmetic is a real LAPACK's, not a restatement.
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fftw3.h"
#include "mkl.h"

namespace {

enum PlanKind { kR2C, kC2R };

struct PlanF {
    PlanKind kind;
    int n0, n1;
    float* real;          // r2c input / c2r output
    fftwf_complex* cplx;  // r2c output / c2r input
};

// e^{sign 2 pi i m / n} with the angle reduced exactly
std::complex<double> cis(long long m, int n, int sign) {
    const long long r = ((m % n) + n) % n;
    const double a = 6.283185307179586476925286766559 * (double)r / (double)n;
    return std::complex<double>(std::cos(a), sign * std::sin(a));
}

void exec_r2c(const PlanF& p) {
    const int n0 = p.n0, n1 = p.n1, h = n1 / 2 + 1;
    std::vector<std::complex<double>> rows((size_t)n0 * h);
    for (int j0 = 0; j0 < n0; ++j0)
        for (int k1 = 0; k1 < h; ++k1) {
            std::complex<double> s = 0;
            for (int j1 = 0; j1 < n1; ++j1) s += (double)p.real[(size_t)j0 * n1 + j1] * cis((long long)k1 * j1, n1, -1);
            rows[(size_t)j0 * h + k1] = s;
        }
    for (int k0 = 0; k0 < n0; ++k0)
        for (int k1 = 0; k1 < h; ++k1) {
            std::complex<double> s = 0;
            for (int j0 = 0; j0 < n0; ++j0) s += rows[(size_t)j0 * h + k1] * cis((long long)k0 * j0, n0, -1);
            p.cplx[(size_t)k0 * h + k1][0] = (float)s.real();
            p.cplx[(size_t)k0 * h + k1][1] = (float)s.imag();
        }
}

void exec_c2r(const PlanF& p) {
    const int n0 = p.n0, n1 = p.n1, h = n1 / 2 + 1;
    // inverse along n0 for every stored column k1
    std::vector<std::complex<double>> cols((size_t)n0 * h);
    for (int j0 = 0; j0 < n0; ++j0)
        for (int k1 = 0; k1 < h; ++k1) {
            std::complex<double> s = 0;
            for (int k0 = 0; k0 < n0; ++k0) {
                const std::complex<double> x(p.cplx[(size_t)k0 * h + k1][0], p.cplx[(size_t)k0 * h + k1][1]);
                s += x * cis((long long)k0 * j0, n0, +1);
            }
            cols[(size_t)j0 * h + k1] = s;
        }
    // Hermitian inverse along n1: the columns k1 > n1/2 are the conjugates of
    // n1 - k1, so every column strictly between DC and Nyquist counts twice
    for (int j0 = 0; j0 < n0; ++j0)
        for (int j1 = 0; j1 < n1; ++j1) {
            double s = cols[(size_t)j0 * h].real();
            for (int k1 = 1; k1 < h; ++k1) {
                const double w = (2 * k1 == n1) ? 1.0 : 2.0;
                s += w * (cols[(size_t)j0 * h + k1] * cis((long long)k1 * j1, n1, +1)).real();
            }
            p.real[(size_t)j0 * n1 + j1] = (float)s;
        }
}

typedef void (*spotrf_t)(char*, int*, float*, int*, int*);
typedef void (*spotrs_t)(char*, int*, int*, float*, int*, float*, int*, int*);
spotrf_t g_spotrf = nullptr;
spotrs_t g_spotrs = nullptr;

}  // namespace

extern "C" {

void* fftw_malloc(size_t n) { return std::malloc(n); }
void fftw_free(void* p) { std::free(p); }
void* fftwf_malloc(size_t n) { return std::malloc(n); }
void fftwf_free(void* p) { std::free(p); }

fftwf_plan fftwf_plan_dft_r2c_2d(int n0, int n1, float* in, fftwf_complex* out, unsigned) {
    return reinterpret_cast<fftwf_plan>(new PlanF{kR2C, n0, n1, in, out});
}
fftwf_plan fftwf_plan_dft_c2r_2d(int n0, int n1, fftwf_complex* in, float* out, unsigned) {
    return reinterpret_cast<fftwf_plan>(new PlanF{kC2R, n0, n1, out, in});
}
void fftwf_execute(const fftwf_plan p) {
    const PlanF& q = *reinterpret_cast<const PlanF*>(p);
    if (q.kind == kR2C)
        exec_r2c(q);
    else
        exec_c2r(q);
}
void fftwf_destroy_plan(fftwf_plan p) { delete reinterpret_cast<PlanF*>(p); }

// Fortran LAPACK entry points (spotrf_, spotrs_ signatures)
void twref_set_lapack(void* spotrf, void* spotrs) {
    g_spotrf = reinterpret_cast<spotrf_t>(spotrf);
    g_spotrs = reinterpret_cast<spotrs_t>(spotrs);
}

int LAPACKE_spotrf(int layout, char uplo, int n, float* a, int lda) {
    if (!g_spotrf) std::abort();
    int info = 0;
    if (layout == LAPACK_COL_MAJOR) {
        g_spotrf(&uplo, &n, a, &lda, &info);
        return info;
    }
    std::vector<float> t((size_t)n * n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) t[(size_t)i + (size_t)j * n] = a[(size_t)i * lda + j];
    int ldt = n;
    g_spotrf(&uplo, &n, t.data(), &ldt, &info);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) a[(size_t)i * lda + j] = t[(size_t)i + (size_t)j * n];
    return info;
}

int LAPACKE_spotrs(int layout, char uplo, int n, int nrhs, const float* a, int lda, float* b, int ldb) {
    if (!g_spotrs) std::abort();
    int info = 0;
    std::vector<float> at((size_t)n * n), bt((size_t)n * nrhs);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            at[(size_t)i + (size_t)j * n] = layout == LAPACK_COL_MAJOR ? a[(size_t)i + (size_t)j * lda]
                                                                      : a[(size_t)i * lda + j];
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < nrhs; ++k)
            bt[(size_t)i + (size_t)k * n] = layout == LAPACK_COL_MAJOR ? b[(size_t)i + (size_t)k * ldb]
                                                                      : b[(size_t)i * ldb + k];
    int ldt = n, ldbt = n;
    g_spotrs(&uplo, &n, &nrhs, at.data(), &ldt, bt.data(), &ldbt, &info);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < nrhs; ++k) {
            if (layout == LAPACK_COL_MAJOR)
                b[(size_t)i + (size_t)k * ldb] = bt[(size_t)i + (size_t)k * n];
            else
                b[(size_t)i * ldb + k] = bt[(size_t)i + (size_t)k * n];
        }
    return info;
}

// double precision is compiled only with the reference's TW_USE_DOUBLE
int LAPACKE_dpotrf(int, char, int, double*, int) { std::abort(); }
int LAPACKE_dpotrs(int, char, int, int, const double*, int, double*, int) { std::abort(); }

}  // extern "C"
