// Shared device-side definitions of the GB300 DIC hot path.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cfloat>

namespace twdic {

// Hermite bicubic matrix M (TW_utils.cpp:622-638): alpha = M tau, with tau
// the four corner values, then d/dx, d/dy and d2/dxdy at the corners
// (0,0), (0,1), (1,0), (1,1); alpha[4k+n] multiplies fy^k fx^n.
static __constant__ signed char c_bicubic_m[16][16] = {
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


// Geometry of one image pair / POI grid as the kernels see it.  Field names
// follow the reference constructors (TW/TW_Engine/TW_paDIC_ICGN2D.h:38-60).
struct Geom {
    int img_w, img_h, pitch;  // pitch = bytes per image row
    int sx, sy, rw, rh;       // ROI
    int rx, ry;               // subset half sizes
    int max_iter;
    float delta_p;
    int grid_x = 0;           // POI grid step along x (0: unknown), sizes FFT-CC window boxes
};

enum : uint8_t { kSuccess = 0, kDarkSubset = 1, kSingularHessian = 2, kSingularWarp = 3, kOutofROI = 4 };

// ------------------------------------------------------------ reductions --
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum of K values over the whole CTA; every thread receives the totals.
// `scratch` holds at least K * (THREADS/32) elements.  Contains two
// __syncthreads and must be reached by every thread of the CTA.
template <int THREADS, int K, typename T>
__device__ __forceinline__ void block_sum(T (&v)[K], T* scratch) {
    constexpr int NW = THREADS / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) scratch[k * NW + wid] = v[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        T s = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w) s += scratch[k * NW + w];
        v[k] = s;
    }
    __syncthreads();
}

// Arg-max with the reference's tie rule: the first (lowest row-major index)
// of equal maxima wins (TW_paDIC_FFTCC2D_CPU.cpp:300-311).
__device__ __forceinline__ void argmax_merge(float& v, int& i, float v2, int i2) {
    if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}
__device__ __forceinline__ void warp_argmax(float& v, int& i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        argmax_merge(v, i, v2, i2);
    }
}

// ---------------------------------------------- restated LAPACK, 6x6 'L' --
// spotrf/dpotrf('L') in reference LAPACK's unblocked spotf2 order on a
// row-major 6x6 lower triangle; returns info (0 = ok, j = leading minor j is
// not positive).  Used by LAPACKE_spotrf in TW_paDIC_ICGN2D_CPU.cpp:682.
template <typename T>
__host__ __device__ __forceinline__ int potrf6(T* a) {
    for (int j = 0; j < 6; ++j) {
        T dot = 0;
        for (int k = 0; k < j; ++k) dot += a[j * 6 + k] * a[j * 6 + k];
        T ajj = a[j * 6 + j] - dot;
        if (!(ajj > T(0))) { a[j * 6 + j] = ajj; return j + 1; }
        ajj = sqrt(ajj);
        a[j * 6 + j] = ajj;
        for (int i = j + 1; i < 6; ++i) {
            T s = 0;
            for (int k = 0; k < j; ++k) s += a[i * 6 + k] * a[j * 6 + k];
            a[i * 6 + j] = a[i * 6 + j] - s;
        }
        const T rec = T(1) / ajj;
        for (int i = j + 1; i < 6; ++i) a[i * 6 + j] *= rec;
    }
    return 0;
}

// spotrs('L') (TW_paDIC_ICGN2D_CPU.cpp:683, :853): L y = b then L^T x = y.
template <typename T>
__host__ __device__ __forceinline__ void potrs6(const T* a, T* b) {
    for (int k = 0; k < 6; ++k) {
        if (b[k] != T(0)) {
            b[k] = b[k] / a[k * 6 + k];
            for (int i = k + 1; i < 6; ++i) b[i] -= b[k] * a[i * 6 + k];
        }
    }
    for (int i = 5; i >= 0; --i) {
        T t = b[i];
        for (int k = i + 1; k < 6; ++k) t -= a[k * 6 + i] * b[k];
        b[i] = t / a[i * 6 + i];
    }
}

// ------------------------------------------------------ warp arithmetic --
// Warp coordinate iPOI + W0*(m-r) + W1*(l-r) + W2 evaluated left to right with
// one rounding per operation, as the reference's /fp:precise build does
// (TW_paDIC_ICGN2D_CPU.cpp:618-619, :761-762).  Explicit _rn intrinsics keep
// nvcc from contracting into FMA.
__device__ __forceinline__ float warp_coord(int base, float a, int d0, float b, int d1, float c) {
    float t = __fadd_rn((float)base, __fmul_rn(a, (float)d0));
    t = __fadd_rn(t, __fmul_rn(b, (float)d1));
    return __fadd_rn(t, c);
}

// W(P) <- W(P) o W(dP)^-1 in closed form (TW_paDIC_ICGN2D_CPU.cpp:713-745).
// W = {W00, W01, W02, W10, W11, W12}.  Returns false for a singular warp.
__device__ __forceinline__ bool update_warp(float P[6], const float d[6], float Wm[6]) {
    const float det = __fsub_rn(__fmul_rn(1.f + d[1], 1.f + d[5]), __fmul_rn(d[2], d[4]));
    if (fabsf(det) <= FLT_EPSILON) return false;
    const float a = __fsub_rn(__fsub_rn(__fmul_rn(d[0], d[4]), d[3]), __fmul_rn(d[3], d[1]));
    const float b = __fsub_rn(__fadd_rn(__fmul_rn(d[0], d[5]), d[0]), __fmul_rn(d[2], d[3]));
    const float w00 = __fdiv_rn(__fsub_rn(__fmul_rn(1.f + P[1], 1.f + d[5]), __fmul_rn(P[2], d[4])), det);
    const float w01 = __fdiv_rn(__fsub_rn(__fmul_rn(P[2], 1.f + d[1]), __fmul_rn(1.f + P[1], d[2])), det);
    const float w02 = __fadd_rn(P[0], __fdiv_rn(__fsub_rn(__fmul_rn(P[2], a), __fmul_rn(1.f + P[1], b)), det));
    const float w10 = __fdiv_rn(__fsub_rn(__fmul_rn(P[4], 1.f + d[5]), __fmul_rn(1.f + P[5], d[4])), det);
    const float w11 = __fdiv_rn(__fsub_rn(__fmul_rn(1.f + P[5], 1.f + d[1]), __fmul_rn(P[4], d[2])), det);
    const float w12 = __fadd_rn(P[3], __fdiv_rn(__fsub_rn(__fmul_rn(1.f + P[5], a), __fmul_rn(P[4], b)), det));
    Wm[0] = w00; Wm[1] = w01; Wm[2] = w02; Wm[3] = w10; Wm[4] = w11; Wm[5] = w12;
    P[0] = w02;
    P[1] = w00 - 1.f;
    P[2] = w01;
    P[3] = w12;
    P[4] = w10;
    P[5] = w11 - 1.f;
    return true;
}

// Scaled ||dP|| of the convergence test, evaluated in double as the
// reference's std::pow / sqrt do (TW_paDIC_ICGN2D_CPU.cpp:750-751).
__device__ __forceinline__ double dp_norm(const float d[6], int rx, int ry) {
    const double a0 = d[0], a1 = __fmul_rn(d[1], (float)rx), a2 = __fmul_rn(d[2], (float)ry);
    const double a3 = d[3], a4 = __fmul_rn(d[4], (float)rx), a5 = __fmul_rn(d[5], (float)ry);
    double s = __dmul_rn(a0, a0);
    s = __dadd_rn(s, __dmul_rn(a1, a1));
    s = __dadd_rn(s, __dmul_rn(a2, a2));
    s = __dadd_rn(s, __dmul_rn(a3, a3));
    s = __dadd_rn(s, __dmul_rn(a4, a4));
    s = __dadd_rn(s, __dmul_rn(a5, a5));
    return sqrt(s);
}

// Device error word: bit 0 = a bounded wait gave up.
constexpr unsigned kErrTimeout = 1u;

}  // namespace twdic
