// Fast IC-GN path.
//
// Per reference image (cached, 256 B per POI): mean(R), ||R - mean(R)||, the
// sums over the subset of the six steepest-descent images SD_k and of
// SD_k * (R - mean(R)), and the FP64 Cholesky factor of the 6x6 Hessian
// (diagonal stored as its reciprocal).  The steepest-descent images
// themselves are rebuilt on chip from the reference image: R_x and R_y are
// exact half integers (TW_utils.cpp:232-305) and SD = (R_x, R_x dx, R_x dy,
// R_y, R_y dx, R_y dy).
//
// Per frame: one persistent kernel.  Each CTA takes the next POI from an
// atomic work counter (row-major order, so CTAs in flight share image rows in
// L2), stages the target window around the FFT-CC guess in shared memory and
// runs the whole Gauss-Newton loop on chip.  One pass over the subset per
// iteration accumulates, with T' = T - mean(R),
//     S0 = sum T',  S1 = sum T'^2,  A_k = sum SD_k T',
// from which the reference's two-pass quantities follow exactly in real
// arithmetic (TW_paDIC_ICGN2D_CPU.cpp:793-826):
//     mean(T) = mean(R) + S0/S,  ||T - mean(T)||^2 = S1 - S0^2/S,
//     RHS_k = (Rs/Ts) (A_k - (S0/S) sum SD_k) - sum SD_k (R - mean(R)).
// The target is interpolated on the fly: the reference's Hermite bicubic LUT
// with central-difference derivatives (TW_utils.cpp:604-700) is algebraically
// the separable Catmull-Rom kernel on the 4x4 neighbourhood, so no per-frame
// LUT is built; the LUT's zero last ROI row and column are reproduced.
#include "dic_common.cuh"
#include "dic_kernels.h"

namespace twdic {

namespace {

constexpr int kPreThreads = 128;

__device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }

// Per-reference precompute (TW_paDIC_ICGN2D_CPU.cpp:516-595, :676-693).
// Per-thread FP32 partial sums (exact for the intensity sum) and FP32 warp
// sums; the final cross-warp sums are FP64, one value per lane of warp 0.
// Thread 0 factors the Hessian (Cholesky, FP64) and forms H^-1 = L^-T L^-1
// from the factor in FP64, stored packed (21 doubles) for the per-iteration
// FP64 solve.  On GB300 an FP64 warp instruction holds the FP64 pipe for
// many cycles whatever its active lanes, so FP64 work is kept to a few
// lane-parallel instructions.
__global__ void __launch_bounds__(kPreThreads) k_ref_precompute_fast(Geom g, const uint8_t* __restrict__ ref,
                                                                      const int2* __restrict__ poi, int n,
                                                                      float* stats, double* hinv,
                                                                      uint8_t* rflag) {
    const int p = blockIdx.x;
    if (p >= n) return;
    const int SW = 2 * g.rx + 1, SH = 2 * g.ry + 1, S = SW * SH;
    const int2 pyx = poi[p];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    constexpr int NW = kPreThreads / 32;
    __shared__ float fred[NW][34];
    __shared__ double dsum[34];
    __shared__ int ired[NW];
    if (pyx.x - g.ry < g.sy || pyx.y - g.rx < g.sx || pyx.x + g.ry >= g.sy + g.rh || pyx.y + g.rx >= g.sx + g.rw) {
        if (tid == 0) rflag[p] = kOutofROI;
        return;
    }
    const uint8_t* r0 = ref + (size_t)(pyx.x - g.ry) * g.pitch + (pyx.y - g.rx);
    int isum[1] = {0};
    for (int l = wid; l < SH; l += NW)
        for (int m = lane; m < SW; m += 32) isum[0] += r0[(size_t)l * g.pitch + m];
    block_sum<kPreThreads, 1>(isum, ired);
    const float mean = (float)isum[0] / (float)S;  // bit-equal to the reference's mean
    // [0..20] Hessian lower triangle, [21] sum (R-mean)^2, [22..27] sum SD_k,
    // [28..33] sum SD_k (R - mean)
    float h[34];
#pragma unroll
    for (int k = 0; k < 34; ++k) h[k] = 0.f;
    for (int l = wid; l < SH; l += NW) {
        for (int m = lane; m < SW; m += 32) {
            const uint8_t* r = r0 + (size_t)l * g.pitch + m;
            const float rx = 0.5f * (float)((int)r[1] - (int)r[-1]);
            const float ry = 0.5f * (float)((int)r[g.pitch] - (int)r[-g.pitch]);
            const float dx = (float)(m - g.rx), dy = (float)(l - g.ry);
            const float d[6] = {rx, rx * dx, rx * dy, ry, ry * dx, ry * dy};
            const float rt = (float)r[0] - mean;
            int q = 0;
#pragma unroll
            for (int a = 0; a < 6; ++a)
#pragma unroll
                for (int b = 0; b <= a; ++b) h[q++] += d[a] * d[b];
            h[21] += rt * rt;
#pragma unroll
            for (int a = 0; a < 6; ++a) {
                h[22 + a] += d[a];
                h[28 + a] += d[a] * rt;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 34; ++k) {
        const float w = warp_sum(h[k]);
        if (lane == 0) fred[wid][k] = w;
    }
    __syncthreads();
    if (wid == 0) {
        for (int k = lane; k < 34; k += 32) {
            double a = 0.0;
            for (int w = 0; w < NW; ++w) a += (double)fred[w][k];
            dsum[k] = a;
        }
    }
    __syncthreads();
    if (tid == 0) {
        const float rs = (float)sqrt(dsum[21]);
        uint8_t f = kSuccess;
        if (fabsf(mean) <= FLT_EPSILON || fabsf(rs) <= FLT_EPSILON) f = kDarkSubset;
        double a[36];
        int q = 0;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) a[i * 6 + j] = (j <= i) ? dsum[q++] : 0.0;
        if (f == kSuccess && potrf6(a) > 0) f = kSingularHessian;
        double* hi = hinv + (size_t)p * 21;
        if (f == kSuccess) {
            // H^-1 column by column: L y = e_j, then L^T x = y
            for (int j = 0; j < 6; ++j) {
                double x[6];
                for (int k = 0; k < 6; ++k) {
                    double acc = (k == j) ? 1.0 : 0.0;
                    for (int i = 0; i < k; ++i) acc -= a[k * 6 + i] * x[i];
                    x[k] = acc / a[k * 6 + k];
                }
                for (int k = 5; k >= 0; --k) {
                    double acc = x[k];
                    for (int i = k + 1; i < 6; ++i) acc -= a[i * 6 + k] * x[i];
                    x[k] = acc / a[k * 6 + k];
                }
                for (int k = j; k < 6; ++k) hi[tri(k, j)] = x[k];
            }
        } else {
            for (int k = 0; k < 21; ++k) hi[k] = 0.0;
        }
        float* st = stats + (size_t)p * 16;
        st[0] = mean;
        st[1] = rs;
        for (int k = 0; k < 6; ++k) {
            st[2 + k] = (float)dsum[22 + k];
            st[8 + k] = (float)dsum[28 + k];
        }
        st[14] = 0.f;
        st[15] = 0.f;
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

template <int THREADS, bool USE_LUT>
__global__ void __launch_bounds__(THREADS) k_icgn_fast(Geom g, const uint8_t* __restrict__ ref,
                                                       const uint8_t* __restrict__ tar,
                                                       const int2* __restrict__ poi, int n,
                                                       const float* __restrict__ stats,
                                                       const double* __restrict__ hinv,
                                                       const uint8_t* __restrict__ rflag,
                                                       const float4* __restrict__ lut, int* work, float* u,
                                                       float* v, float* p6, int* iters, uint8_t* flags, int ws) {
    constexpr int NW = THREADS / 32;
    constexpr unsigned FULL = 0xffffffffu;
    // dynamic shared memory: [S] float2 reference gradients (R_x, R_y), then
    // the [ws][ws] target window
    extern __shared__ __align__(16) float smem_f[];
    __shared__ float red[NW][9];
    __shared__ float sW[6];
    __shared__ int sctl[3];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int SW = 2 * g.rx + 1, SH = 2 * g.ry + 1, S = SW * SH;
    float2* grad = reinterpret_cast<float2*>(smem_f);
    float* win = smem_f + 2 * ((S + 1) & ~1);
    const size_t plane = (size_t)g.rw * g.rh;
    const float inv_s = 1.0f / (float)S;
    // sample k = tid + j*THREADS sits at row l, column m of the subset;
    // stepping j advances (l, m) by (dl, dm) with carry
    const int l_first = tid / SW, m_first = tid - (tid / SW) * SW;
    const int dl = THREADS / SW, dm = THREADS - (THREADS / SW) * SW;

    for (;;) {
        if (tid == 0) sctl[2] = atomicAdd(work, 1);
        __syncthreads();
        const int p = sctl[2];
        if (p >= n) break;
        const int2 pyx = poi[p];
        const int py = pyx.x, px = pyx.y;
        const float u0 = u[p], v0 = v[p];
        const uint8_t rf = rflag[p];
        float P[6] = {u0, 0.f, 0.f, v0, 0.f, 0.f};  // maintained by thread 0
        float Wm[6] = {1.f, 0.f, u0, 0.f, 1.f, v0};
        bool done = (rf == kDarkSubset || rf == kOutofROI);
        if (done && tid == 0) {
            flags[p] = rf;
            for (int k = 0; k < 6; ++k) p6[(size_t)p * 6 + k] = P[k];
        }
        // ---- stage the target window and the reference gradients (rows by
        // warps, columns by lanes)
        const int wx0 = px + (int)floorf(u0) - g.rx - 4;
        const int wy0 = py + (int)floorf(v0) - g.ry - 4;
        if (!done) {
            if (!USE_LUT) {
                for (int yy = wid; yy < ws; yy += NW) {
                    const int gy = wy0 + yy;
                    const bool rowok = gy >= 0 && gy < g.img_h;
                    const uint8_t* trow = tar + (size_t)(rowok ? gy : 0) * g.pitch;
                    for (int xx = lane; xx < ws; xx += 32) {
                        const int gx = wx0 + xx;
                        win[yy * ws + xx] = (rowok && gx >= 0 && gx < g.img_w) ? (float)trow[gx] : 0.f;
                    }
                }
            }
            const uint8_t* r0 = ref + (size_t)(py - g.ry) * g.pitch + (px - g.rx);
            for (int l = wid; l < SH; l += NW) {
                for (int m = lane; m < SW; m += 32) {
                    const uint8_t* r = r0 + (size_t)l * g.pitch + m;
                    grad[l * SW + m] = make_float2(0.5f * (float)((int)r[1] - (int)r[-1]),
                                                   0.5f * (float)((int)r[g.pitch] - (int)r[-g.pitch]));
                }
            }
        }
        // warp 0, lane k < 6: row k of H^-1 (FP64), sum SD_k and sum SD_k (R - mean)
        double hrow[6];
        float sumsd = 0.f, qk = 0.f, rs = 0.f;
#pragma unroll
        for (int j = 0; j < 6; ++j) hrow[j] = 0.0;
        if (wid == 0 && !done) {
            const float* st = stats + (size_t)p * 16;
            rs = st[1];
            if (lane < 6) {
                sumsd = st[2 + lane];
                qk = st[8 + lane];
                const double* hi = hinv + (size_t)p * 21;
#pragma unroll
                for (int j = 0; j < 6; ++j) hrow[j] = hi[lane >= j ? tri(lane, j) : tri(j, lane)];
            }
        }
        const float c = done ? 0.f : stats[(size_t)p * 16];  // shift: mean(R)
        __syncthreads();
        int it = 0;  // solves completed; abort/counter rule as in the plain kernel
        while (!done) {
            float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            int oor = 0;
            int l = l_first, m = m_first;
            // x = px + W00 dx + W01 dy + W02 as two FMAs (the reference rounds
            // each operation; the difference is an ulp, which moves a
            // truncated coordinate only at an exact integer, where the
            // bicubic patch is continuous)
            const float bx = (float)px + Wm[2], by = (float)py + Wm[5];
#pragma unroll 2
            for (int k = tid; k < S; k += THREADS) {
                const float dxf = (float)(m - g.rx), dyf = (float)(l - g.ry);
                const float wx = fmaf(Wm[0], dxf, fmaf(Wm[1], dyf, bx));
                const float wy = fmaf(Wm[3], dxf, fmaf(Wm[4], dyf, by));
                const int ix = (int)wx, iy = (int)wy;
                float t = 0.f;
                if ((unsigned)(ix - g.sx) < (unsigned)g.rw && (unsigned)(iy - g.sy) < (unsigned)g.rh) {
                    const int lx = ix - wx0, ly = iy - wy0;
                    if (it == 0) {  // first pass: integer pixels (TW_paDIC_ICGN2D_CPU.cpp:609-637)
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
                } else {
                    oor = 1;
                }
                const float2 gr = grad[k];
                const float tp = t - c;
                const float dx = dxf, dy = dyf;
                const float a = gr.x * tp, b = gr.y * tp;
                s[0] += tp;
                s[1] += tp * tp;
                s[2] += a; s[3] += a * dx; s[4] += a * dy;
                s[5] += b; s[6] += b * dx; s[7] += b * dy;
                l += dl;
                m += dm;
                if (m >= SW) { m -= SW; ++l; }
            }
            // ---- one reduction (FP32), then warp 0 finishes the iteration:
            // FP32 scalars, FP64 H^-1 b on lanes 0-5, warp update on lane 0
#pragma unroll
            for (int k = 0; k < 8; ++k) s[k] = warp_sum(s[k]);
            oor = __any_sync(FULL, oor);
            if (lane == 0) {
#pragma unroll
                for (int k = 0; k < 8; ++k) red[wid][k] = s[k];
                red[wid][8] = (float)oor;
            }
            __syncthreads();
            if (wid == 0) {
                float tot = 0.f;
                if (lane < 9)
                    for (int w = 0; w < NW; ++w) tot += red[w][lane];
                const float S0 = __shfl_sync(FULL, tot, 0), S1 = __shfl_sync(FULL, tot, 1);
                const float any_oor = __shfl_sync(FULL, tot, 8);
                const float Ak = __shfl_sync(FULL, tot, 2 + (lane < 6 ? lane : 0));
                const float m0 = S0 * inv_s;
                const float mean_t = c + m0;
                const float var = S1 - S0 * m0;
                const float ts = sqrtf(var > 0.f ? var : 0.f);
                int flag = kSuccess, cont = 0;
                if (any_oor > 0.f) {
                    flag = kOutofROI;
                } else if (fabsf(mean_t) <= FLT_EPSILON || fabsf(ts) <= FLT_EPSILON) {
                    flag = kDarkSubset;
                } else if (it == 0 && rf == kSingularHessian) {
                    flag = kSingularHessian;
                }
                float dpk = 0.f;
                if (flag == kSuccess) {
                    const float q = rs / ts;
                    const float bk = (lane < 6) ? q * (Ak - m0 * sumsd) - qk : 0.f;
                    const double bd = (double)bk;
                    double acc = 0.0;
#pragma unroll
                    for (int j = 0; j < 6; ++j) acc = fma(hrow[j], __shfl_sync(FULL, bd, j), acc);
                    dpk = (float)acc;
                }
                float dp[6];
#pragma unroll
                for (int j = 0; j < 6; ++j) dp[j] = __shfl_sync(FULL, dpk, j);
                if (lane == 0) {
                    if (flag == kSuccess) {
                        if (!update_warp(P, dp, Wm)) {
                            flag = kSingularWarp;
                        } else {
                            // scaled ||dP|| >= delta_p, squared, FP32
                            const float a1 = dp[1] * (float)g.rx, a2 = dp[2] * (float)g.ry;
                            const float a4 = dp[4] * (float)g.rx, a5 = dp[5] * (float)g.ry;
                            const float nrm2 = dp[0] * dp[0] + a1 * a1 + a2 * a2 + dp[3] * dp[3] + a4 * a4 + a5 * a5;
                            cont = (it + 1 < g.max_iter && nrm2 >= g.delta_p * g.delta_p) ? 1 : 0;
                        }
                    }
                    if (flag == kSuccess && cont) {
                        for (int k = 0; k < 6; ++k) sW[k] = Wm[k];
                    } else {
                        // finish: the counter is it+1 after a solve or an abort in a
                        // later pass; an abort in the first pass leaves it untouched
                        flags[p] = (uint8_t)flag;
                        for (int k = 0; k < 6; ++k) p6[(size_t)p * 6 + k] = P[k];
                        u[p] = P[0];
                        v[p] = P[3];
                        if (flag == kSuccess || it > 0) iters[p] = it + 1;
                    }
                    sctl[0] = (flag == kSuccess && cont) ? 1 : 0;
                }
            }
            __syncthreads();
            if (!sctl[0]) break;
#pragma unroll
            for (int k = 0; k < 6; ++k) Wm[k] = sW[k];
            ++it;
        }
        __syncthreads();  // window and sctl are reused by the next POI
    }
}

}  // namespace

cudaError_t launch_ref_precompute_fast(const Geom& g, const uint8_t* ref, const int2* poi, int n, float* stats,
                                       double* chol, uint8_t* rflag, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_ref_precompute_fast<<<n, kPreThreads, 0, st>>>(g, ref, poi, n, stats, chol, rflag);
    return cudaGetLastError();
}

int icgn_fast_window(const Geom& g) { return 2 * (g.rx > g.ry ? g.rx : g.ry) + 1 + 10; }

template <int THREADS, bool LUT>
static cudaError_t launch_icgn_fast_t(const Geom& g, const uint8_t* ref, const uint8_t* tar, const int2* poi,
                                      int n, const float* stats, const double* chol, const uint8_t* rflag,
                                      const float4* lut, int* work, float* u, float* v, float* p6, int* iters,
                                      uint8_t* flags, int ctas_per_sm, cudaStream_t st) {
    const int ws = icgn_fast_window(g);
    const int S = (2 * g.rx + 1) * (2 * g.ry + 1);
    const size_t smem = sizeof(float) * (2 * (size_t)((S + 1) & ~1) + (LUT ? 0 : (size_t)ws * ws));
    auto kern = k_icgn_fast<THREADS, LUT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
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
    kern<<<grid, THREADS, smem, st>>>(g, ref, tar, poi, n, stats, chol, rflag, lut, work, u, v, p6, iters, flags, ws);
    return cudaGetLastError();
}

cudaError_t launch_icgn_fast(const Geom& g, const uint8_t* ref, const uint8_t* tar, const int2* poi, int n,
                             const float* stats, const double* chol, const uint8_t* rflag, const float4* lut,
                             int* work, float* u, float* v, float* p6, int* iters, uint8_t* flags,
                             const IcgnTune& tune, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const bool use_lut = tune.use_lut != 0;
#define TWDIC_ICGN_FAST(TH)                                                                                      \
    return use_lut ? launch_icgn_fast_t<TH, true>(g, ref, tar, poi, n, stats, chol, rflag, lut, work, u, v, p6,   \
                                                  iters, flags, tune.ctas_per_sm, st)                              \
                   : launch_icgn_fast_t<TH, false>(g, ref, tar, poi, n, stats, chol, rflag, lut, work, u, v, p6,  \
                                                   iters, flags, tune.ctas_per_sm, st)
    if (tune.threads == 64) { TWDIC_ICGN_FAST(64); }
    if (tune.threads == 256) { TWDIC_ICGN_FAST(256); }
    TWDIC_ICGN_FAST(128);
#undef TWDIC_ICGN_FAST
}

}  // namespace twdic
