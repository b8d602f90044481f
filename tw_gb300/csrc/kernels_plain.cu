// Plain FP32 SIMT path: one CTA per POI, the reference-side steepest-descent
// images and the per-frame target bicubic LUT kept in HBM.  This is the
// project's own straightforward sm_103a implementation of the reference CPU
// semantics, used as the comparator of the fast path.
#include "dic_common.cuh"
#include "dic_kernels.h"

namespace twdic {

namespace {

constexpr int kFftThreads = 128;
constexpr int kIcgnThreads = 128;

// ------------------------------------------------------------- FFT-CC ----
// Fftcc2D_CPU::ComputeFFTCC (TW_paDIC_FFTCC2D_CPU.cpp:222-326) as a direct
// FP32 DFT: half-spectrum row DFT, column DFT, conj(F)*G, inverse column DFT,
// c2r row DFT fused with the first-maximum search.
__global__ void __launch_bounds__(kFftThreads) k_fftcc_plain(Geom g, const uint8_t* __restrict__ ref,
                                                               const uint8_t* __restrict__ tar,
                                                               const int2* __restrict__ poi, int n,
                                                               const float2* __restrict__ tw, float* u, float* v,
                                                               float* zncc, uint8_t* status) {
    const int p = blockIdx.x;
    if (p >= n) return;
    const int Nx = 2 * g.rx, Ny = 2 * g.ry, Hx = g.rx + 1, NN = Nx * Ny;
    extern __shared__ __align__(16) unsigned char smem[];
    float2* twx = reinterpret_cast<float2*>(smem);  // [Nx] exp(-2 pi i k / Nx)
    float2* twy = twx + 64;                          // [Ny]
    float2* bufA = twy + 64;                          // windows, then F/G then C
    float2* bufB = bufA + 2 * Ny * Hx;                // X then Z
    __shared__ float red[8 * (kFftThreads / 32)];
    __shared__ int ired[2 * (kFftThreads / 32)];

    const int tid = threadIdx.x;
    for (int k = tid; k < 128; k += kFftThreads) twx[k] = tw[k];
    const int2 pyx = poi[p];
    const int y0 = pyx.x - g.ry, x0 = pyx.y - g.rx;
    float* fw = reinterpret_cast<float*>(bufA);  // [Ny][Nx]
    float* gw = fw + NN;
    int isum[2] = {0, 0};
    for (int k = tid; k < NN; k += kFftThreads) {
        const int i = k / Nx, j = k - i * Nx;
        const size_t off = (size_t)(y0 + i) * g.pitch + (x0 + j);
        const int a = ref[off], b = tar[off];
        fw[k] = (float)a;
        gw[k] = (float)b;
        isum[0] += a;
        isum[1] += b;
    }
    block_sum<kFftThreads, 2>(isum, ired);
    // mean = (sum of integers, exact) / n: the reference's float running sum is
    // exact below 2^24, so this equals its fSubAveR/fSubAveT bit for bit.
    const float mf = (float)isum[0] / (float)NN, mg = (float)isum[1] / (float)NN;
    float nrm[2] = {0.f, 0.f};
    for (int k = tid; k < NN; k += kFftThreads) {
        const float a = fw[k] - mf, b = gw[k] - mg;
        fw[k] = a;
        gw[k] = b;
        nrm[0] += a * a;
        nrm[1] += b * b;
    }
    block_sum<kFftThreads, 2>(nrm, red);
    if (nrm[0] < 0.0000001f || nrm[1] < 0.0000001f) {  // dark subset: outputs untouched
        if (tid == 0) status[p] = 1;
        return;
    }
    // row DFT, half spectrum: X[y][k] = sum_x w[y][x] e^{-2 pi i k x / Nx}
    float2* Xf = bufB;
    float2* Xg = bufB + Ny * Hx;
    for (int o = tid; o < Ny * Hx; o += kFftThreads) {
        const int y = o / Hx, k = o - y * Hx;
        float fr = 0.f, fi = 0.f, gr = 0.f, gi = 0.f;
        int e = 0;
        for (int x = 0; x < Nx; ++x) {
            const float2 w = twx[e];
            const float a = fw[y * Nx + x], b = gw[y * Nx + x];
            fr += a * w.x; fi += a * w.y;
            gr += b * w.x; gi += b * w.y;
            e += k; if (e >= Nx) e -= Nx;
        }
        Xf[o] = make_float2(fr, fi);
        Xg[o] = make_float2(gr, gi);
    }
    __syncthreads();
    // column DFT and cross power C = conj(F) G
    float2* C = bufA;
    for (int o = tid; o < Ny * Hx; o += kFftThreads) {
        const int ky = o / Hx, k = o - ky * Hx;
        float fr = 0.f, fi = 0.f, gr = 0.f, gi = 0.f;
        int e = 0;
        for (int y = 0; y < Ny; ++y) {
            const float2 w = twy[e];
            const float2 a = Xf[y * Hx + k], b = Xg[y * Hx + k];
            fr += a.x * w.x - a.y * w.y; fi += a.x * w.y + a.y * w.x;
            gr += b.x * w.x - b.y * w.y; gi += b.x * w.y + b.y * w.x;
            e += ky; if (e >= Ny) e -= Ny;
        }
        // separate store after all reads of bufA windows is guaranteed by
        // the barrier above: the windows are no longer needed.
        C[o] = make_float2(fr * gr + fi * gi, fr * gi - fi * gr);
    }
    __syncthreads();
    // inverse column DFT: Z[y][k] = sum_ky C[ky][k] e^{+2 pi i ky y / Ny}
    float2* Z = bufB;
    for (int o = tid; o < Ny * Hx; o += kFftThreads) {
        const int y = o / Hx, k = o - y * Hx;
        float zr = 0.f, zi = 0.f;
        int e = 0;
        for (int ky = 0; ky < Ny; ++ky) {
            const float2 w = twy[e];
            const float2 c = C[ky * Hx + k];
            zr += c.x * w.x + c.y * w.y;
            zi += c.y * w.x - c.x * w.y;
            e += y; if (e >= Ny) e -= Ny;
        }
        Z[o] = make_float2(zr, zi);
    }
    __syncthreads();
    // c2r along x fused with the first-maximum search
    float best = -3.4e38f;
    int bidx = 0x7fffffff;
    for (int o = tid; o < NN; o += kFftThreads) {
        const int y = o / Nx, x = o - y * Nx;
        const float2* zr = Z + y * Hx;
        float c = zr[0].x + ((x & 1) ? -zr[g.rx].x : zr[g.rx].x);
        float s = 0.f;
        int e = x;
        for (int k = 1; k < g.rx; ++k) {
            const float2 w = twx[e];
            s += zr[k].x * w.x + zr[k].y * w.y;  // Re(Z e^{+i theta})
            e += x; if (e >= Nx) e -= Nx;
        }
        c += 2.f * s;
        argmax_merge(best, bidx, c, o);
    }
    warp_argmax(best, bidx);
    __shared__ float sbest[kFftThreads / 32];
    __shared__ int sidx[kFftThreads / 32];
    if ((tid & 31) == 0) { sbest[tid >> 5] = best; sidx[tid >> 5] = bidx; }
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < kFftThreads / 32; ++w) argmax_merge(best, bidx, sbest[w], sidx[w]);
        int iu = bidx % Nx, iv = bidx / Nx;
        if (iu > g.rx) iu -= Nx;
        if (iv > g.ry) iv -= Ny;
        u[p] = (float)iu;
        v[p] = (float)iv;
        zncc[p] = best / (sqrtf(nrm[0] * nrm[1]) * (float)NN);
        status[p] = 0;
    }
}

// ----------------------------------------------- reference precompute ----
// Per POI, cached per reference image: R - mean(R), the six steepest-descent
// images (stored as three float2 planes), the FP32 Hessian and its FP32
// Cholesky factor, ||R - mean(R)|| and the reference-side flag
// (TW_paDIC_ICGN2D_CPU.cpp:516-595, :676-693).
__global__ void __launch_bounds__(kIcgnThreads) k_ref_precompute_plain(Geom g, const uint8_t* __restrict__ ref,
                                                                        const int2* __restrict__ poi, int n,
                                                                        float* subR, float2* sd, float* chol,
                                                                        float* refnorm, uint8_t* rflag) {
    const int p = blockIdx.x;
    if (p >= n) return;
    const int SW = 2 * g.rx + 1, SH = 2 * g.ry + 1, S = SW * SH;
    const int2 pyx = poi[p];
    const int tid = threadIdx.x;
    __shared__ float red[21 * (kIcgnThreads / 32)];
    __shared__ int ired[kIcgnThreads / 32];
    if (pyx.x - g.ry < g.sy || pyx.y - g.rx < g.sx || pyx.x + g.ry >= g.sy + g.rh || pyx.y + g.rx >= g.sx + g.rw) {
        if (tid == 0) rflag[p] = kOutofROI;
        return;
    }
    float h[21];
#pragma unroll
    for (int k = 0; k < 21; ++k) h[k] = 0.f;
    int isum[1] = {0};
    float* sR = subR + (size_t)p * S;
    float2* sd0 = sd + (size_t)p * 3 * S;
    for (int k = tid; k < S; k += kIcgnThreads) {
        const int l = k / SW, m = k - l * SW;
        const int y = pyx.x - g.ry + l, x = pyx.y - g.rx + m;
        const uint8_t* r = ref + (size_t)y * g.pitch + x;
        const int rv = r[0];
        isum[0] += rv;
        const float rx = 0.5f * (float)((int)r[1] - (int)r[-1]);
        const float ry = 0.5f * (float)((int)r[g.pitch] - (int)r[-g.pitch]);
        const float dx = (float)(m - g.rx), dy = (float)(l - g.ry);
        const float d[6] = {rx, rx * dx, rx * dy, ry, ry * dx, ry * dy};  // exact products
        sd0[k] = make_float2(d[0], d[1]);
        sd0[S + k] = make_float2(d[2], d[3]);
        sd0[2 * S + k] = make_float2(d[4], d[5]);
        sR[k] = (float)rv;
        int q = 0;
#pragma unroll
        for (int a = 0; a < 6; ++a)
#pragma unroll
            for (int b = 0; b <= a; ++b) h[q++] += d[a] * d[b];
    }
    block_sum<kIcgnThreads, 1>(isum, ired);
    const float mean = (float)isum[0] / (float)S;
    float nrm[1] = {0.f};
    for (int k = tid; k < S; k += kIcgnThreads) {
        const float t = sR[k] - mean;
        sR[k] = t;
        nrm[0] += t * t;
    }
    block_sum<kIcgnThreads, 1>(nrm, red);
    block_sum<kIcgnThreads, 21>(h, red);
    if (tid == 0) {
        const float rs = sqrtf(nrm[0]);
        uint8_t f = kSuccess;
        if (fabsf(mean) <= FLT_EPSILON || fabsf(rs) <= FLT_EPSILON) f = kDarkSubset;
        float a[36];
        int q = 0;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) a[i * 6 + j] = (j <= i) ? h[q++] : 0.f;
        if (f == kSuccess && potrf6(a) > 0) f = kSingularHessian;
        for (int i = 0; i < 36; ++i) chol[(size_t)p * 36 + i] = a[i];
        refnorm[p] = rs;
        rflag[p] = f;
    }
}

// ------------------------------------------------ per-frame target LUT ----
// BicubicCoefficients (TW_utils.cpp:604-700) with the target gradients of
// GradientXY_2Images (TW_utils.cpp:232-305) computed on the fly.  All values
// are quarter integers, so alpha = M tau is exact in FP32 in any order and the
// table equals the reference's bit for bit.  Layout: four float4 planes,
// plane k holding the coefficients of fy^k fx^0..3 for every ROI pixel.
// (M: c_bicubic_m in dic_common.cuh)

__global__ void k_bicubic_lut(Geom g, const uint8_t* __restrict__ tar, float4* __restrict__ lut) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.rh || j >= g.rw) return;
    const size_t plane = (size_t)g.rw * g.rh;
    const size_t o = (size_t)i * g.rw + j;
    if (i == g.rh - 1 || j == g.rw - 1) {  // never written by the reference: calloc zeros
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        lut[o] = z; lut[plane + o] = z; lut[2 * plane + o] = z; lut[3 * plane + o] = z;
        return;
    }
    const uint8_t* t = tar + (size_t)(i + g.sy) * g.pitch + (j + g.sx);
    const int P = g.pitch;
    auto G = [&](int dy, int dx) { return (int)t[dy * P + dx]; };
    float tau[16];
    tau[0] = (float)G(0, 0); tau[1] = (float)G(0, 1); tau[2] = (float)G(1, 0); tau[3] = (float)G(1, 1);
    const int cy[4] = {0, 0, 1, 1}, cx[4] = {0, 1, 0, 1};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int y = cy[c], x = cx[c];
        tau[4 + c] = 0.5f * (float)(G(y, x + 1) - G(y, x - 1));
        tau[8 + c] = 0.5f * (float)(G(y + 1, x) - G(y - 1, x));
        tau[12 + c] = 0.25f * (float)(G(y + 1, x + 1) - G(y - 1, x + 1) - G(y + 1, x - 1) + G(y - 1, x - 1));
    }
    float a[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        float s = 0.f;
#pragma unroll
        for (int l = 0; l < 16; ++l) s += (float)c_bicubic_m[k][l] * tau[l];
        a[k] = s;
    }
    lut[o] = make_float4(a[0], a[1], a[2], a[3]);
    lut[plane + o] = make_float4(a[4], a[5], a[6], a[7]);
    lut[2 * plane + o] = make_float4(a[8], a[9], a[10], a[11]);
    lut[3 * plane + o] = make_float4(a[12], a[13], a[14], a[15]);
}

// ---------------------------------------------------------------- IC-GN ----
// ICGN2D_CPU::ICGN2D_Compute (TW_paDIC_ICGN2D_CPU.cpp:481-925), one CTA per
// POI, FP32 throughout: integer-pixel first iteration, LUT interpolation
// afterwards, block reductions for the means, norms and the six RHS sums,
// FP32 Cholesky solve with the cached factor.
template <int MAXPT>
__global__ void __launch_bounds__(kIcgnThreads) k_icgn_plain(Geom g, const uint8_t* __restrict__ tar,
                                                               const int2* __restrict__ poi, int n,
                                                               const float* __restrict__ subR,
                                                               const float2* __restrict__ sd,
                                                               const float* __restrict__ chol,
                                                               const float* __restrict__ refnorm,
                                                               const uint8_t* __restrict__ rflag,
                                                               const float4* __restrict__ lut, float* u, float* v,
                                                               float* p6, int* iters, uint8_t* flags) {
    const int p = blockIdx.x;
    if (p >= n) return;
    const int tid = threadIdx.x;
    const int SW = 2 * g.rx + 1, SH = 2 * g.ry + 1, S = SW * SH;
    const int2 pyx = poi[p];
    const int py = pyx.x, px = pyx.y;
    __shared__ float red[6 * (kIcgnThreads / 32)];
    __shared__ float sW[6];
    __shared__ int sctl[2];  // [0] = flag, [1] = continue
    float P[6] = {u[p], 0.f, 0.f, v[p], 0.f, 0.f};
    const uint8_t rf = rflag[p];
    auto finish = [&](uint8_t flag, int it, bool set_it) {
        if (tid == 0) {
            flags[p] = flag;
            for (int k = 0; k < 6; ++k) p6[(size_t)p * 6 + k] = P[k];
            u[p] = P[0];
            v[p] = P[3];
            if (set_it) iters[p] = it;
        }
    };
    if (rf == kDarkSubset || rf == kOutofROI) { finish(rf, 0, false); return; }

    float Wm[6] = {1.f, 0.f, P[0], 0.f, 1.f, P[3]};
    const float* sR = subR + (size_t)p * S;
    const float2* sd0 = sd + (size_t)p * 3 * S;
    const float rs = refnorm[p];
    const size_t plane = (size_t)g.rw * g.rh;
    float T[MAXPT];
    // it = Gauss-Newton solves completed.  The reference's counter is 1 after
    // the first solve and is pre-incremented at the top of every later pass,
    // so an abort during pass it > 0 leaves it at it + 1, and an abort during
    // the first pass leaves it untouched (TW_paDIC_ICGN2D_CPU.cpp:749-753).
    int it = 0;
    for (;;) {
        // --- sample the target subset
        int oor = 0;
        float sum[1] = {0.f};
#pragma unroll
        for (int j = 0; j < MAXPT; ++j) {
            const int k = tid + j * kIcgnThreads;
            T[j] = 0.f;
            if (k < S) {
                const int l = k / SW, m = k - l * SW;
                const float wx = warp_coord(px, Wm[0], m - g.rx, Wm[1], l - g.ry, Wm[2]);
                const float wy = warp_coord(py, Wm[3], m - g.rx, Wm[4], l - g.ry, Wm[5]);
                const int ix = (int)wx, iy = (int)wy;
                if (ix >= g.sx && iy >= g.sy && ix < g.sx + g.rw && iy < g.sy + g.rh) {
                    float t;
                    if (it == 0) {
                        t = (float)tar[(size_t)iy * g.pitch + ix];
                    } else {
                        const float fx = wx - (float)ix, fy = wy - (float)iy;
                        const size_t o = (size_t)(iy - g.sy) * g.rw + (ix - g.sx);
                        const float4 a0 = lut[o], a1 = lut[plane + o], a2 = lut[2 * plane + o],
                                     a3 = lut[3 * plane + o];
                        const float r0 = ((a0.w * fx + a0.z) * fx + a0.y) * fx + a0.x;
                        const float r1 = ((a1.w * fx + a1.z) * fx + a1.y) * fx + a1.x;
                        const float r2 = ((a2.w * fx + a2.z) * fx + a2.y) * fx + a2.x;
                        const float r3 = ((a3.w * fx + a3.z) * fx + a3.y) * fx + a3.x;
                        t = ((r3 * fy + r2) * fy + r1) * fy + r0;
                    }
                    T[j] = t;
                    sum[0] += t;
                } else {
                    oor = 1;
                }
            }
        }
        if (__syncthreads_or(oor)) { finish(kOutofROI, it + 1, it > 0); return; }
        block_sum<kIcgnThreads, 1>(sum, red);
        const float mean = sum[0] / (float)S;
        if (fabsf(mean) <= FLT_EPSILON) { finish(kDarkSubset, it + 1, it > 0); return; }
        float nrm[1] = {0.f};
#pragma unroll
        for (int j = 0; j < MAXPT; ++j) {
            const int k = tid + j * kIcgnThreads;
            if (k < S) {
                T[j] -= mean;
                nrm[0] += T[j] * T[j];
            }
        }
        block_sum<kIcgnThreads, 1>(nrm, red);
        const float ts = sqrtf(nrm[0]);
        if (fabsf(ts) <= FLT_EPSILON) { finish(kDarkSubset, it + 1, it > 0); return; }
        const float q = rs / ts;
        float rhs[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int j = 0; j < MAXPT; ++j) {
            const int k = tid + j * kIcgnThreads;
            if (k < S) {
                const float e = q * T[j] - sR[k];
                const float2 d0 = sd0[k], d1 = sd0[S + k], d2 = sd0[2 * S + k];
                rhs[0] += d0.x * e; rhs[1] += d0.y * e;
                rhs[2] += d1.x * e; rhs[3] += d1.y * e;
                rhs[4] += d2.x * e; rhs[5] += d2.y * e;
            }
        }
        block_sum<kIcgnThreads, 6>(rhs, red);
        if (it == 0 && rf == kSingularHessian) { finish(kSingularHessian, it, false); return; }
        if (tid == 0) {
            potrs6(chol + (size_t)p * 36, rhs);
            int flag = kSuccess, cont = 0;
            if (!update_warp(P, rhs, Wm)) {
                flag = kSingularWarp;
            } else {
                ++it;
                cont = (it < g.max_iter && dp_norm(rhs, g.rx, g.ry) >= (double)g.delta_p) ? 1 : 0;
            }
            for (int k = 0; k < 6; ++k) sW[k] = Wm[k];
            sctl[0] = flag;
            sctl[1] = cont;
        }
        __syncthreads();
        // only thread 0 holds P; the others need the warp matrix
#pragma unroll
        for (int k = 0; k < 6; ++k) Wm[k] = sW[k];
        const int flag = sctl[0], cont = sctl[1];
        if (tid != 0 && flag == kSuccess) ++it;  // thread 0 advanced its counter in the solve
        if (flag != kSuccess) { finish((uint8_t)flag, it + 1, it > 0); return; }
        if (!cont) { finish(kSuccess, it, true); return; }
        __syncthreads();  // sctl/sW reused next iteration
    }
}

}  // namespace

// ------------------------------------------------------------ launchers ----
cudaError_t launch_fftcc_plain(const Geom& g, const uint8_t* ref, const uint8_t* tar, const int2* poi, int n,
                               const float2* tw, float* u, float* v, float* zncc, uint8_t* status, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int Ny = 2 * g.ry, Hx = g.rx + 1;
    const size_t smem = sizeof(float2) * (128 + 4 * (size_t)Ny * Hx);
    cudaError_t e = cudaFuncSetAttribute(k_fftcc_plain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_fftcc_plain<<<n, kFftThreads, smem, st>>>(g, ref, tar, poi, n, tw, u, v, zncc, status);
    return cudaGetLastError();
}

cudaError_t launch_ref_precompute_plain(const Geom& g, const uint8_t* ref, const int2* poi, int n, float* subR,
                                        float2* sd, float* chol, float* refnorm, uint8_t* rflag, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_ref_precompute_plain<<<n, kIcgnThreads, 0, st>>>(g, ref, poi, n, subR, sd, chol, refnorm, rflag);
    return cudaGetLastError();
}

// BicubicSplineCoefficients_s (TW_utils.cpp:521-602): the B-spline
// coefficient LUT of the target, same layout as k_bicubic_lut (plane k holds
// the coefficients of fy^k fx^0..3).  Per ROI pixel the 4x4 neighbourhood is
// prefiltered on both sides by the local B-spline interpolation matrix and
// mapped to polynomial coefficients by the cubic B-spline basis, then both
// indices are reversed.  Every product and sum is rounded separately, in the
// reference's order, so the table equals the reference's FP32 table.  Pixels
// outside the image read as 0 (the reference reads one row and column past a
// one-pixel border); all ROI pixels are written.
namespace {
__device__ const float kBsCP[4][4] = {{(float)(71 / 56.0), (float)(-19 / 56.0), (float)(5 / 56.0), (float)(-1 / 56.0)},
                                      {(float)(-19 / 56.0), (float)(95 / 56.0), (float)(-25 / 56.0), (float)(5 / 56.0)},
                                      {(float)(5 / 56.0), (float)(-25 / 56.0), (float)(95 / 56.0), (float)(-19 / 56.0)},
                                      {(float)(-1 / 56.0), (float)(5 / 56.0), (float)(-19 / 56.0), (float)(71 / 56.0)}};
__device__ const float kBsBase[4][4] = {{(float)(-1 / 6.0), (float)(3 / 6.0), (float)(-3 / 6.0), (float)(1 / 6.0)},
                                        {(float)(3 / 6.0), (float)(-6 / 6.0), (float)(3 / 6.0), 0.f},
                                        {(float)(-3 / 6.0), 0.f, (float)(3 / 6.0), 0.f},
                                        {(float)(1 / 6.0), (float)(4 / 6.0), (float)(1 / 6.0), 0.f}};
}  // namespace

__global__ void k_bspline_lut(Geom g, const uint8_t* __restrict__ tar, float4* __restrict__ lut) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.rh || j >= g.rw) return;
    float om[4][4], be[4][4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const int y = i + g.sy - 1 + k, x = j + g.sx - 1 + l;
            om[k][l] = (y >= 0 && y < g.img_h && x >= 0 && x < g.img_w) ? (float)tar[(size_t)y * g.pitch + x] : 0.f;
        }
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            float a = 0.f;
#pragma unroll
            for (int m = 0; m < 4; ++m)
#pragma unroll
                for (int n = 0; n < 4; ++n) a = __fadd_rn(a, __fmul_rn(__fmul_rn(kBsCP[k][m], kBsCP[l][n]), om[n][m]));
            be[k][l] = a;
        }
    const size_t plane = (size_t)g.rw * g.rh;
    const size_t o = (size_t)i * g.rw + j;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        float c[4];
#pragma unroll
        for (int ll = 0; ll < 4; ++ll) {
            const int k = 3 - kk, l = 3 - ll;  // reversed indices
            float a = 0.f;
#pragma unroll
            for (int m = 0; m < 4; ++m)
#pragma unroll
                for (int n = 0; n < 4; ++n)
                    a = __fadd_rn(a, __fmul_rn(__fmul_rn(kBsBase[k][m], kBsBase[l][n]), be[n][m]));
            c[ll] = a;
        }
        lut[kk * plane + o] = make_float4(c[0], c[1], c[2], c[3]);
    }
}

cudaError_t launch_bspline_lut(const Geom& g, const uint8_t* tar, float4* lut, cudaStream_t st) {
    dim3 blk(32, 8), grd((g.rw + 31) / 32, (g.rh + 7) / 8);
    k_bspline_lut<<<grd, blk, 0, st>>>(g, tar, lut);
    return cudaGetLastError();
}

cudaError_t launch_bicubic_lut(const Geom& g, const uint8_t* tar, float4* lut, cudaStream_t st) {
    dim3 blk(32, 8), grd((g.rw + 31) / 32, (g.rh + 7) / 8);
    k_bicubic_lut<<<grd, blk, 0, st>>>(g, tar, lut);
    return cudaGetLastError();
}

cudaError_t launch_icgn_plain(const Geom& g, const uint8_t* tar, const int2* poi, int n, const float* subR,
                              const float2* sd, const float* chol, const float* refnorm, const uint8_t* rflag,
                              const float4* lut, float* u, float* v, float* p6, int* iters, uint8_t* flags,
                              cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int S = (2 * g.rx + 1) * (2 * g.ry + 1);
    const int pt = (S + kIcgnThreads - 1) / kIcgnThreads;
    if (pt <= 8)
        k_icgn_plain<8><<<n, kIcgnThreads, 0, st>>>(g, tar, poi, n, subR, sd, chol, refnorm, rflag, lut, u, v, p6,
                                                     iters, flags);
    else if (pt <= 16)
        k_icgn_plain<16><<<n, kIcgnThreads, 0, st>>>(g, tar, poi, n, subR, sd, chol, refnorm, rflag, lut, u, v, p6,
                                                      iters, flags);
    else
        k_icgn_plain<32><<<n, kIcgnThreads, 0, st>>>(g, tar, poi, n, subR, sd, chol, refnorm, rflag, lut, u, v, p6,
                                                      iters, flags);
    return cudaGetLastError();
}

}  // namespace twdic
