// Fast IC-GN path.
//
// Per reference image (cached): per POI mean(R), ||R - mean(R)|| and the FP64
// Cholesky factor of the 6x6 Hessian -- 184 bytes per POI instead of the
// seven subset-sized planes of the plain path.  The steepest-descent images
// are rebuilt on chip from the reference image (R_x, R_y are exact half
// integers) when a POI is picked up.
//
// Per frame: one persistent kernel.  Each CTA takes the next POI from an
// atomic work counter (row-major order, so CTAs in flight share image rows in
// L2), stages the target window around the FFT-CC guess in shared memory and
// runs the whole Gauss-Newton loop there.  The target is interpolated on the
// fly: the reference's Hermite bicubic LUT with central-difference
// derivatives (TW_utils.cpp:604-700) is algebraically the separable
// Catmull-Rom kernel on the 4x4 neighbourhood, so no per-frame LUT is built.
// The LUT's zero last ROI row and column are reproduced explicitly.
#include "dic_common.cuh"
#include "dic_kernels.h"

namespace twdic {

namespace {

constexpr int kPreThreads = 128;

__device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }

// Per-reference precompute (TW_paDIC_ICGN2D_CPU.cpp:516-595, :676-693).
// Sums: FP32 per thread (exact for the integer intensity sum), FP64 across
// threads; Cholesky in FP64.
__global__ void __launch_bounds__(kPreThreads) k_ref_precompute_fast(Geom g, const uint8_t* __restrict__ ref,
                                                                      const int2* __restrict__ poi, int n,
                                                                      float2* refstat, double* chol,
                                                                      uint8_t* rflag) {
    const int p = blockIdx.x;
    if (p >= n) return;
    const int SW = 2 * g.rx + 1, SH = 2 * g.ry + 1, S = SW * SH;
    const int2 pyx = poi[p];
    const int tid = threadIdx.x;
    constexpr int NW = kPreThreads / 32;
    __shared__ double dred[22 * NW];
    __shared__ int ired[NW];
    if (pyx.x - g.ry < g.sy || pyx.y - g.rx < g.sx || pyx.x + g.ry >= g.sy + g.rh || pyx.y + g.rx >= g.sx + g.rw) {
        if (tid == 0) rflag[p] = kOutofROI;
        return;
    }
    float h[21];
#pragma unroll
    for (int k = 0; k < 21; ++k) h[k] = 0.f;
    int isum[1] = {0};
    for (int k = tid; k < S; k += kPreThreads) {
        const int l = k / SW, m = k - l * SW;
        const uint8_t* r = ref + (size_t)(pyx.x - g.ry + l) * g.pitch + (pyx.y - g.rx + m);
        isum[0] += r[0];
        const float rx = 0.5f * (float)((int)r[1] - (int)r[-1]);
        const float ry = 0.5f * (float)((int)r[g.pitch] - (int)r[-g.pitch]);
        const float dx = (float)(m - g.rx), dy = (float)(l - g.ry);
        const float d[6] = {rx, rx * dx, rx * dy, ry, ry * dx, ry * dy};
        int q = 0;
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int b = 0; b <= a; ++b) h[q++] += d[a] * d[b];
    }
    block_sum<kPreThreads, 1>(isum, ired);
    const float mean = (float)isum[0] / (float)S;  // bit-equal to the reference's mean
    float nrm = 0.f;
    for (int k = tid; k < S; k += kPreThreads) {
        const int l = k / SW, m = k - l * SW;
        const float t = (float)ref[(size_t)(pyx.x - g.ry + l) * g.pitch + (pyx.y - g.rx + m)] - mean;
        nrm += t * t;
    }
    // FP64 combination of the per-thread FP32 partial sums
    double dv[22];
#pragma unroll
    for (int k = 0; k < 21; ++k) dv[k] = (double)h[k];
    dv[21] = (double)nrm;
    block_sum<kPreThreads, 22>(dv, dred);
    if (tid == 0) {
        const float rs = (float)sqrt(dv[21]);
        uint8_t f = kSuccess;
        if (fabsf(mean) <= FLT_EPSILON || fabsf(rs) <= FLT_EPSILON) f = kDarkSubset;
        double a[36];
        int q = 0;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) a[i * 6 + j] = (j <= i) ? dv[q++] : 0.0;
        if (f == kSuccess && potrf6(a) > 0) f = kSingularHessian;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j <= i; ++j) chol[(size_t)p * 21 + tri(i, j)] = a[i * 6 + j];
        refstat[p] = make_float2(mean, rs);
        rflag[p] = f;
    }
}

// Catmull-Rom weights (the Hermite bicubic with central differences).
__device__ __forceinline__ void cr_weights(float t, float& w0, float& w1, float& w2, float& w3) {
    const float t2 = t * t;
    w0 = t * (t * (-0.5f * t + 1.0f) - 0.5f);
    w1 = t2 * (1.5f * t - 2.5f) + 1.0f;
    w2 = t * (t * (-1.5f * t + 2.0f) + 0.5f);
    w3 = t2 * (0.5f * t - 0.5f);
}

// Sum of K floats over the CTA: FP32 within warps, FP64 across warps.
template <int THREADS, int K>
__device__ __forceinline__ void cta_sum(float (&v)[K], double* scratch) {
    constexpr int NW = THREADS / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) scratch[k * NW + wid] = (double)v[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < NW; ++w) s += scratch[k * NW + w];
        v[k] = (float)s;
    }
    __syncthreads();
}

template <int THREADS, int MAXPT, bool USE_LUT>
__global__ void __launch_bounds__(THREADS) k_icgn_fast(Geom g, const uint8_t* __restrict__ ref,
                                                       const uint8_t* __restrict__ tar,
                                                       const int2* __restrict__ poi, int n,
                                                       const float2* __restrict__ refstat,
                                                       const double* __restrict__ chol,
                                                       const uint8_t* __restrict__ rflag,
                                                       const float4* __restrict__ lut, int* work, float* u,
                                                       float* v, float* p6, int* iters, uint8_t* flags, int ws) {
    constexpr int NW = THREADS / 32;
    extern __shared__ __align__(16) float win[];  // [ws][ws] target window
    __shared__ double red[6 * NW];
    __shared__ float sW[6];
    __shared__ int sctl[3];
    const int tid = threadIdx.x;
    const int SW = 2 * g.rx + 1, SH = 2 * g.ry + 1, S = SW * SH;
    const size_t plane = (size_t)g.rw * g.rh;

    for (;;) {
        if (tid == 0) sctl[2] = atomicAdd(work, 1);
        __syncthreads();
        const int p = sctl[2];
        if (p >= n) break;
        const int2 pyx = poi[p];
        const int py = pyx.x, px = pyx.y;
        float P[6] = {u[p], 0.f, 0.f, v[p], 0.f, 0.f};
        const uint8_t rf = rflag[p];
        bool done = false;
        auto finish = [&](uint8_t flag, int it, bool set_it) {
            if (tid == 0) {
                flags[p] = flag;
                for (int k = 0; k < 6; ++k) p6[(size_t)p * 6 + k] = P[k];
                u[p] = P[0];
                v[p] = P[3];
                if (set_it) iters[p] = it;
            }
            done = true;
        };
        if (rf == kDarkSubset || rf == kOutofROI) finish(rf, 0, false);

        // ---- stage the target window and the reference-side data
        const int wx0 = px + (int)floorf(P[0]) - g.rx - 4;
        const int wy0 = py + (int)floorf(P[3]) - g.ry - 4;
        if (!USE_LUT && !done) {
            for (int k = tid; k < ws * ws; k += THREADS) {
                const int yy = wy0 + k / ws, xx = wx0 + k % ws;
                float t = 0.f;
                if (yy >= 0 && yy < g.img_h && xx >= 0 && xx < g.img_w) t = (float)tar[(size_t)yy * g.pitch + xx];
                win[k] = t;
            }
        }
        const float2 rst = refstat[p];
        float Rt[MAXPT], Gx[MAXPT], Gy[MAXPT], T[MAXPT];
#pragma unroll
        for (int j = 0; j < MAXPT; ++j) {
            const int k = tid + j * THREADS;
            Rt[j] = 0.f; Gx[j] = 0.f; Gy[j] = 0.f;
            if (!done && k < S) {
                const int l = k / SW, m = k - l * SW;
                const uint8_t* r = ref + (size_t)(py - g.ry + l) * g.pitch + (px - g.rx + m);
                Rt[j] = (float)r[0] - rst.x;
                Gx[j] = 0.5f * (float)((int)r[1] - (int)r[-1]);
                Gy[j] = 0.5f * (float)((int)r[g.pitch] - (int)r[-g.pitch]);
            }
        }
        __syncthreads();
        float Wm[6] = {1.f, 0.f, P[0], 0.f, 1.f, P[3]};
        int it = 0;  // solves completed; see the plain kernel for the counter rule
        while (!done) {
            int oor = 0;
            float s1[1] = {0.f};
#pragma unroll
            for (int j = 0; j < MAXPT; ++j) {
                const int k = tid + j * THREADS;
                T[j] = 0.f;
                if (k < S) {
                    const int l = k / SW, m = k - l * SW;
                    const float wx = warp_coord(px, Wm[0], m - g.rx, Wm[1], l - g.ry, Wm[2]);
                    const float wy = warp_coord(py, Wm[3], m - g.rx, Wm[4], l - g.ry, Wm[5]);
                    const int ix = (int)wx, iy = (int)wy;
                    if (ix >= g.sx && iy >= g.sy && ix < g.sx + g.rw && iy < g.sy + g.rh) {
                        float t;
                        const int lx = ix - wx0, ly = iy - wy0;
                        if (it == 0) {
                            t = (!USE_LUT && lx >= 0 && ly >= 0 && lx < ws && ly < ws)
                                    ? win[ly * ws + lx]
                                    : (float)tar[(size_t)iy * g.pitch + ix];
                        } else if (iy - g.sy == g.rh - 1 || ix - g.sx == g.rw - 1) {
                            t = 0.f;  // the reference LUT's never-written last row / column
                        } else {
                            const float fx = wx - (float)ix, fy = wy - (float)iy;
                            if (USE_LUT) {
                                const size_t o = (size_t)(iy - g.sy) * g.rw + (ix - g.sx);
                                const float4 a0 = lut[o], a1 = lut[plane + o], a2 = lut[2 * plane + o],
                                             a3 = lut[3 * plane + o];
                                const float r0 = ((a0.w * fx + a0.z) * fx + a0.y) * fx + a0.x;
                                const float r1 = ((a1.w * fx + a1.z) * fx + a1.y) * fx + a1.x;
                                const float r2 = ((a2.w * fx + a2.z) * fx + a2.y) * fx + a2.x;
                                const float r3 = ((a3.w * fx + a3.z) * fx + a3.y) * fx + a3.x;
                                t = ((r3 * fy + r2) * fy + r1) * fy + r0;
                            } else {
                                float cx0, cx1, cx2, cx3, cy0, cy1, cy2, cy3;
                                cr_weights(fx, cx0, cx1, cx2, cx3);
                                cr_weights(fy, cy0, cy1, cy2, cy3);
                                float rr[4];
                                if (lx >= 1 && ly >= 1 && lx + 2 < ws && ly + 2 < ws) {
                                    const float* w0 = win + (ly - 1) * ws + (lx - 1);
#pragma unroll
                                    for (int a = 0; a < 4; ++a) {
                                        const float* w = w0 + a * ws;
                                        rr[a] = cx0 * w[0] + cx1 * w[1] + cx2 * w[2] + cx3 * w[3];
                                    }
                                } else {  // outside the staged window: read the image
                                    const uint8_t* w0 = tar + (size_t)(iy - 1) * g.pitch + (ix - 1);
#pragma unroll
                                    for (int a = 0; a < 4; ++a) {
                                        const uint8_t* w = w0 + a * g.pitch;
                                        rr[a] = cx0 * (float)w[0] + cx1 * (float)w[1] + cx2 * (float)w[2] +
                                                cx3 * (float)w[3];
                                    }
                                }
                                t = cy0 * rr[0] + cy1 * rr[1] + cy2 * rr[2] + cy3 * rr[3];
                            }
                        }
                        T[j] = t;
                        s1[0] += t;
                    } else {
                        oor = 1;
                    }
                }
            }
            if (__syncthreads_or(oor)) { finish(kOutofROI, it + 1, it > 0); break; }
            cta_sum<THREADS, 1>(s1, red);
            const float mean = s1[0] / (float)S;
            if (fabsf(mean) <= FLT_EPSILON) { finish(kDarkSubset, it + 1, it > 0); break; }
            float s2[1] = {0.f};
#pragma unroll
            for (int j = 0; j < MAXPT; ++j) {
                const int k = tid + j * THREADS;
                if (k < S) {
                    T[j] -= mean;
                    s2[0] += T[j] * T[j];
                }
            }
            cta_sum<THREADS, 1>(s2, red);
            const float ts = sqrtf(s2[0]);
            if (fabsf(ts) <= FLT_EPSILON) { finish(kDarkSubset, it + 1, it > 0); break; }
            const float q = rst.y / ts;
            float rhs[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int j = 0; j < MAXPT; ++j) {
                const int k = tid + j * THREADS;
                if (k < S) {
                    const int l = k / SW, m = k - l * SW;
                    const float dx = (float)(m - g.rx), dy = (float)(l - g.ry);
                    const float e = q * T[j] - Rt[j];
                    const float a = Gx[j] * e, b = Gy[j] * e;
                    rhs[0] += a; rhs[1] += a * dx; rhs[2] += a * dy;
                    rhs[3] += b; rhs[4] += b * dx; rhs[5] += b * dy;
                }
            }
            cta_sum<THREADS, 6>(rhs, red);
            if (it == 0 && rf == kSingularHessian) { finish(kSingularHessian, 0, false); break; }
            if (tid == 0) {
                // FP64 solve with the cached FP64 factor
                const double* L = chol + (size_t)p * 21;
                double b[6];
                for (int k = 0; k < 6; ++k) b[k] = (double)rhs[k];
                for (int k = 0; k < 6; ++k) {
                    double s = b[k];
                    for (int i = 0; i < k; ++i) s -= L[tri(k, i)] * b[i];
                    b[k] = s / L[tri(k, k)];
                }
                for (int k = 5; k >= 0; --k) {
                    double s = b[k];
                    for (int i = k + 1; i < 6; ++i) s -= L[tri(i, k)] * b[i];
                    b[k] = s / L[tri(k, k)];
                }
                float d[6];
                for (int k = 0; k < 6; ++k) d[k] = (float)b[k];
                int flag = kSuccess, cont = 0;
                if (!update_warp(P, d, Wm)) {
                    flag = kSingularWarp;
                } else {
                    ++it;
                    cont = (it < g.max_iter && dp_norm(d, g.rx, g.ry) >= (double)g.delta_p) ? 1 : 0;
                }
                for (int k = 0; k < 6; ++k) sW[k] = Wm[k];
                sctl[0] = flag;
                sctl[1] = cont;
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < 6; ++k) Wm[k] = sW[k];
            const int flag = sctl[0], cont = sctl[1];
            if (tid != 0 && flag == kSuccess) ++it;
            if (flag != kSuccess) { finish((uint8_t)flag, it + 1, it > 0); break; }
            if (!cont) { finish(kSuccess, it, true); break; }
            __syncthreads();
        }
        __syncthreads();  // window and sctl are reused by the next POI
    }
}

}  // namespace

cudaError_t launch_ref_precompute_fast(const Geom& g, const uint8_t* ref, const int2* poi, int n, float2* refstat,
                                       double* chol, uint8_t* rflag, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_ref_precompute_fast<<<n, kPreThreads, 0, st>>>(g, ref, poi, n, refstat, chol, rflag);
    return cudaGetLastError();
}

int icgn_fast_window(const Geom& g) { return 2 * (g.rx > g.ry ? g.rx : g.ry) + 1 + 10; }

template <int THREADS, int MAXPT, bool LUT>
static cudaError_t launch_icgn_fast_t(const Geom& g, const uint8_t* ref, const uint8_t* tar, const int2* poi,
                                      int n, const float2* refstat, const double* chol, const uint8_t* rflag,
                                      const float4* lut, int* work, float* u, float* v, float* p6, int* iters,
                                      uint8_t* flags, int ctas_per_sm, cudaStream_t st) {
    const int ws = icgn_fast_window(g);
    const size_t smem = LUT ? 16 : sizeof(float) * (size_t)ws * ws;
    auto kern = k_icgn_fast<THREADS, MAXPT, LUT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, THREADS, smem);
    if (e != cudaSuccess) return e;
    if (ctas_per_sm > 0 && ctas_per_sm < occ) occ = ctas_per_sm;
    if (occ < 1) occ = 1;
    int grid = sms * occ;
    if (grid > n) grid = n;
    e = cudaMemsetAsync(work, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    kern<<<grid, THREADS, smem, st>>>(g, ref, tar, poi, n, refstat, chol, rflag, lut, work, u, v, p6, iters, flags,
                                      ws);
    return cudaGetLastError();
}

cudaError_t launch_icgn_fast(const Geom& g, const uint8_t* ref, const uint8_t* tar, const int2* poi, int n,
                             const float2* refstat, const double* chol, const uint8_t* rflag, const float4* lut,
                             int* work, float* u, float* v, float* p6, int* iters, uint8_t* flags,
                             const IcgnTune& tune, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int S = (2 * g.rx + 1) * (2 * g.ry + 1);
    const bool use_lut = tune.use_lut != 0;
#define TWDIC_ICGN_FAST(TH, PT)                                                                                  \
    return use_lut ? launch_icgn_fast_t<TH, PT, true>(g, ref, tar, poi, n, refstat, chol, rflag, lut, work, u, v, \
                                                      p6, iters, flags, tune.ctas_per_sm, st)                      \
                   : launch_icgn_fast_t<TH, PT, false>(g, ref, tar, poi, n, refstat, chol, rflag, lut, work, u, v, \
                                                       p6, iters, flags, tune.ctas_per_sm, st)
    if (tune.threads == 256) {
        if (S <= 256 * 8) { TWDIC_ICGN_FAST(256, 8); }
        TWDIC_ICGN_FAST(256, 16);
    }
    if (S <= 128 * 8) { TWDIC_ICGN_FAST(128, 8); }
    if (S <= 128 * 16) { TWDIC_ICGN_FAST(128, 16); }
    TWDIC_ICGN_FAST(128, 32);
#undef TWDIC_ICGN_FAST
}

}  // namespace twdic
