// Fast IC-GN path.
//
// Per reference image (cached): per POI 16 floats (mean(R), ||R - mean(R)||,
// the subset sums of the six steepest-descent images SD_k and of
// SD_k * (R - mean(R))) and the packed FP64 inverse Hessian (21 doubles, from
// an FP64 Cholesky factor), and per ROI pixel the reference gradients
// (R_x, R_y) as float2 -- half integers, exact (TW_utils.cpp:232-305).  The
// steepest-descent images are never stored: SD = (R_x, R_x dx, R_x dy, R_y,
// R_y dx, R_y dy) is formed per sample.
//
// Per target frame: the 4x4 byte neighbourhood of every ROI pixel (16 B,
// k_nbhd_table), then one persistent kernel that runs the whole Gauss-Newton
// loop of each POI on chip.  Default layout (k_icgn_warp): one POI per warp,
// the 32 warps of a CTA walking runs of consecutive POIs so that their
// overlapping subsets are served from L1.  One-POI-per-CTA layout
// (k_icgn_fast): 32 to 256 threads per POI, gradients staged in shared
// memory, optionally sampling a target window staged in shared memory
// instead of a table (the no-allocation entry point).  One pass over the
// subset per iteration accumulates, with T' = T - mean(R),
//     S0 = sum T',  S1 = sum T'^2,  A_k = sum SD_k T',
// from which the reference's two-pass quantities follow exactly in real
// arithmetic (TW_paDIC_ICGN2D_CPU.cpp:793-826):
//     mean(T) = mean(R) + S0/S,  ||T - mean(T)||^2 = S1 - S0^2/S,
//     RHS_k = (Rs/Ts) (A_k - (S0/S) sum SD_k) - sum SD_k (R - mean(R)).
// The reference's Hermite bicubic LUT with central-difference derivatives
// (TW_utils.cpp:604-700) is algebraically the separable Catmull-Rom kernel on
// the 4x4 neighbourhood, evaluated from the table's bytes; the LUT's zero
// last ROI row and column are reproduced by zero table entries.
#include <cuda_fp16.h>

#include <algorithm>

#include "dic_common.cuh"
#include "dic_kernels.h"

namespace twdic {

namespace {


__device__ __forceinline__ constexpr int tri(int i, int j) { return i * (i + 1) / 2 + j; }

// Per-reference precompute (TW_paDIC_ICGN2D_CPU.cpp:516-595, :676-693), in
// two kernels.
// k_ref_sums: one warp per POI.  The subset is walked in row-major sample
// order k = lane + 32 j (every lane busy whatever the subset width): first
// the integer sum of its pixels (the mean, bit-equal to the reference's),
// then the 34 FP32 sums (Hessian lower triangle, sum (R - mean)^2, sum SD_k,
// sum SD_k (R - mean)) on the packed FP32 pipe, lane partials reduced over
// the warp.  The Hessian sums are staged, as floats, in the POI's own slot of
// the inverse-Hessian array.
// k_ref_factor: one POI per thread, in FP64: Cholesky (spotrf's steps, as
// potrf6), then H^-1 = L^-T L^-1 packed (21 doubles) for the per-iteration
// solve, dividing by the diagonal through its six reciprocals.  On GB300 an
// FP64 warp instruction holds the FP64 pipe for many cycles whatever its
// active lanes, so each serves 32 POIs.
constexpr int kSumWarps = 4;  // measured at 2048², 41x41: 4 to 16 warps per CTA within 6 %
constexpr int kFactorThreads = 128;

__global__ void __launch_bounds__(kSumWarps * 32) k_ref_sums(Geom g, const uint8_t* __restrict__ ref,
                                                               const int2* __restrict__ poi, int n,
                                                               float* __restrict__ stats, double* hinv,
                                                               uint8_t* __restrict__ rflag) {
    const int lane = threadIdx.x & 31;
    const int p = blockIdx.x * kSumWarps + (threadIdx.x >> 5);
    if (p >= n) return;
    const int2 pyx = poi[p];
    if (pyx.x - g.ry < g.sy || pyx.y - g.rx < g.sx || pyx.x + g.ry >= g.sy + g.rh || pyx.y + g.rx >= g.sx + g.rw) {
        if (lane == 0) rflag[p] = kOutofROI;
        return;
    }
    const int SW = 2 * g.rx + 1, SH = 2 * g.ry + 1, S = SW * SH;
    const int pitch = g.pitch;
    const uint8_t* r0 = ref + (size_t)(pyx.x - g.ry) * pitch + (pyx.y - g.rx);
    // sample k = lane + 32 j at row l, column m of the subset (offset o);
    // a step adds 32 samples: dm columns and 32 / SW rows, then a carry
    const int m_first = lane % SW, l_first = lane / SW;
    const int dm = 32 % SW, dofs = (32 / SW) * pitch + dm, wrap = pitch - SW;
    const int o_first = l_first * pitch + m_first;
    int isum = 0;
    {
        int m = m_first, o = o_first;
        for (int k = lane; k < S; k += 32) {
            isum += r0[o];
            o += dofs;
            m += dm;
            if (m >= SW) {
                m -= SW;
                o += wrap;
            }
        }
    }
    isum = warp_sum(isum);
    const float mean = (float)isum / (float)S;  // bit-equal to the reference's mean
    // SD = (d0 .. d5) = (g_x, g_x dx, g_x dy, g_y, g_y dx, g_y dy) as
    // D0 = (d0, d1), D1 = (d2, d3), D2 = (d4, d5); Hessian entry (a, b) of the
    // lower triangle is element tri(a, b) of h below
    const float2 zero = make_float2(0.f, 0.f);
    float2 A0 = zero, A1 = zero, A2 = zero, A3 = zero, A4 = zero, A5 = zero, A6 = zero, A7 = zero, A8 = zero,
           A9 = zero, A10 = zero, B0 = zero, B1 = zero, B2 = zero, C0 = zero, C1 = zero, C2 = zero;
    {
        int m = m_first, o = o_first;
        float2 dd = make_float2((float)(m_first - g.rx), (float)(l_first - g.ry));
        const float2 dstep = make_float2((float)dm, (float)(32 / SW)), dwrap = make_float2(-(float)SW, 1.f);
        for (int k = lane; k < S; k += 32) {
            const uint8_t* r = r0 + o;
            const float gx = 0.5f * (float)((int)r[1] - (int)r[-1]);
            const float gy = 0.5f * (float)((int)r[pitch] - (int)r[-pitch]);
            const float rt = (float)r[0] - mean;
            const float2 gxd = __fmul2_rn(make_float2(gx, gx), dd), gyd = __fmul2_rn(make_float2(gy, gy), dd);
            const float2 D0 = make_float2(gx, gxd.x), D1 = make_float2(gxd.y, gy), D2 = gyd;
            const float2 rr = make_float2(rt, rt);
            A0 = __ffma2_rn(make_float2(D0.x, D1.x), make_float2(D0.x, D1.x), A0);  // (0,0), (2,2)
            A1 = __ffma2_rn(make_float2(D0.y, D0.y), D0, A1);                      // (1,0), (1,1)
            A2 = __ffma2_rn(make_float2(D1.x, D1.x), D0, A2);                      // (2,0), (2,1)
            A3 = __ffma2_rn(make_float2(D1.y, D1.y), D0, A3);                      // (3,0), (3,1)
            A4 = __ffma2_rn(make_float2(D1.y, D1.y), D1, A4);                      // (3,2), (3,3)
            A5 = __ffma2_rn(make_float2(D2.x, D2.x), D0, A5);                      // (4,0), (4,1)
            A6 = __ffma2_rn(make_float2(D2.x, D2.x), D1, A6);                      // (4,2), (4,3)
            A7 = __ffma2_rn(make_float2(D2.x, rt), make_float2(D2.x, rt), A7);     // (4,4), (R - mean)^2
            A8 = __ffma2_rn(make_float2(D2.y, D2.y), D0, A8);                      // (5,0), (5,1)
            A9 = __ffma2_rn(make_float2(D2.y, D2.y), D1, A9);                      // (5,2), (5,3)
            A10 = __ffma2_rn(make_float2(D2.y, D2.y), D2, A10);                    // (5,4), (5,5)
            B0 = __fadd2_rn(B0, D0);
            B1 = __fadd2_rn(B1, D1);
            B2 = __fadd2_rn(B2, D2);
            C0 = __ffma2_rn(D0, rr, C0);
            C1 = __ffma2_rn(D1, rr, C1);
            C2 = __ffma2_rn(D2, rr, C2);
            o += dofs;
            m += dm;
            dd = __fadd2_rn(dd, dstep);
            if (m >= SW) {
                m -= SW;
                o += wrap;
                dd = __fadd2_rn(dd, dwrap);
            }
        }
    }
    // [0..20] H lower (tri order), [21] sum (R-mean)^2, [22..27] sum SD, [28..33] sum SD (R-mean)
    float h[34] = {A0.x, A1.x, A1.y, A2.x, A2.y, A0.y, A3.x, A3.y, A4.x, A4.y, A5.x, A5.y,
                   A6.x, A6.y, A7.x, A8.x, A8.y, A9.x, A9.y, A10.x, A10.y, A7.y, B0.x, B0.y,
                   B1.x, B1.y, B2.x, B2.y, C0.x, C0.y, C1.x, C1.y, C2.x, C2.y};
#pragma unroll
    for (int k = 0; k < 34; ++k) h[k] = warp_sum(h[k]);  // every lane holds the totals
    if (lane == 0) {
        const float rs = (float)sqrt((double)h[21]);
        uint8_t f = kSuccess;  // pending the factorization
        if (fabsf(mean) <= FLT_EPSILON || fabsf(rs) <= FLT_EPSILON) f = kDarkSubset;
        float* st = stats + (size_t)p * 16;
        st[0] = mean;
        st[1] = rs;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            st[2 + k] = h[22 + k];
            st[8 + k] = h[28 + k];
        }
        st[14] = 0.f;
        st[15] = 0.f;
        float* hs = reinterpret_cast<float*>(hinv + (size_t)p * 21);
#pragma unroll
        for (int k = 0; k < 21; ++k) hs[k] = h[k];
        rflag[p] = f;
    }
}

__global__ void __launch_bounds__(kFactorThreads) k_ref_factor(int n, double* hinv, uint8_t* __restrict__ rflag) {
    const int p = blockIdx.x * kFactorThreads + threadIdx.x;
    if (p >= n) return;
    const uint8_t f = rflag[p];
    if (f == kOutofROI) return;
    double* hi = hinv + (size_t)p * 21;
    if (f != kSuccess) {
#pragma unroll
        for (int k = 0; k < 21; ++k) hi[k] = 0.0;
        return;
    }
    // the staged FP32 sums, all read before the slot is rewritten (every
    // output below depends on all of them through the factorization)
    const float* hs = reinterpret_cast<const float*>(hi);
    double L[21];
#pragma unroll
    for (int k = 0; k < 21; ++k) L[k] = (double)hs[k];
    // (loops of constant trip count with the bounds as predicates, so that
    // they unroll before L is assigned to registers)
    double rinv[6];
    bool ok = true;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double dot = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (k < j) dot += L[tri(j, k)] * L[tri(j, k)];
        double ajj = L[tri(j, j)] - dot;
        if (!(ajj > 0.0)) {
            ok = false;
            ajj = 1.0;
        }
        ajj = __dsqrt_rn(ajj);
        L[tri(j, j)] = ajj;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            if (i <= j) continue;
            double s2 = 0.0;
#pragma unroll
            for (int k = 0; k < 6; ++k)
                if (k < j) s2 += L[tri(i, k)] * L[tri(j, k)];
            L[tri(i, j)] = L[tri(i, j)] - s2;
        }
        rinv[j] = __drcp_rn(ajj);
#pragma unroll
        for (int i = 0; i < 6; ++i)
            if (i > j) L[tri(i, j)] *= rinv[j];
    }
    if (!ok) {
#pragma unroll
        for (int k = 0; k < 21; ++k) hi[k] = 0.0;
        rflag[p] = kSingularHessian;
        return;
    }
    // H^-1 column by column: L y = e_j (y_k = 0 for k < j), then L^T x = y
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double x[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            if (k < j) {
                x[k] = 0.0;
                continue;
            }
            double acc = (k == j) ? 1.0 : 0.0;
#pragma unroll
            for (int i = j; i < k; ++i) acc -= L[tri(k, i)] * x[i];
            x[k] = acc * rinv[k];
        }
#pragma unroll
        for (int k = 5; k >= j; --k) {
            double acc = x[k];
#pragma unroll
            for (int i = k + 1; i < 6; ++i) acc -= L[tri(i, k)] * x[i];
            x[k] = acc * rinv[k];
        }
#pragma unroll
        for (int k = j; k < 6; ++k) hi[tri(k, j)] = x[k];
    }
}

// 4x4 byte neighbourhood of every ROI pixel (i, j) of the target: rows
// i-1 .. i+2, columns j-1 .. j+2 of the ROI-relative pixel, one 32-bit word
// per row, lowest byte leftmost.  Bicubic (full = 0): zero on the ROI's last
// row and column, the entries the reference's LUT never writes
// (TW_MemManager.cpp calloc).  The ROI has one pixel of border on every side
// (validated on the host), and the neighbourhood of the other last-but-one
// pixels stays inside the image.  B-spline (full = 1): every ROI pixel, with
// the bytes outside the image zero, as the reference's B-spline LUT reads
// them (TW_utils.cpp:521-602).
__device__ __forceinline__ uint4 nbhd_entry(const Geom& g, const uint8_t* __restrict__ tar, int i, int j, int full) {
    uint4 q = make_uint4(0u, 0u, 0u, 0u);
    const int y0 = i + g.sy - 1, x0 = j + g.sx - 1;
    if (!full && (i == g.rh - 1 || j == g.rw - 1)) {
        // bicubic: the LUT's unwritten last row and column
    } else if (y0 >= 0 && x0 >= 0 && y0 + 3 < g.img_h && x0 + 3 < g.img_w) {
        const uint8_t* t = tar + (size_t)y0 * g.pitch + x0;
        uint32_t w[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const uint8_t* r = t + (size_t)a * g.pitch;
            w[a] = (uint32_t)r[0] | ((uint32_t)r[1] << 8) | ((uint32_t)r[2] << 16) | ((uint32_t)r[3] << 24);
        }
        q = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
        // B-spline near the image edge: bytes outside the image are zero
        uint32_t w[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            w[a] = 0u;
            const int y = y0 + a;
            if (y < 0 || y >= g.img_h) continue;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int x = x0 + b;
                if (x >= 0 && x < g.img_w) w[a] |= (uint32_t)tar[(size_t)y * g.pitch + x] << (8 * b);
            }
        }
        q = make_uint4(w[0], w[1], w[2], w[3]);
    }
    return q;
}

__global__ void k_nbhd_table(Geom g, const uint8_t* __restrict__ tar, uint4* __restrict__ table, int full) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.rh || j >= g.rw) return;
    table[(size_t)i * g.rw + j] = nbhd_entry(g, tar, i, j, full);
}

// The per-frame preparation of a batch in one launch: the neighbourhood
// tables of every frame that has one, then the zeroing of every frame's
// output arrays that start at zero.  Items are numbered over all frames
// (table pixels first, row-major per frame, then one item per POI); each
// thread finds its frame by binary search over the frames' first items.
__global__ void k_batch_prepare(const __grid_constant__ PrepJobs J) {
    const long long total = J.px_total + J.z_total;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const bool px = k < J.px_total;
        const long long item = px ? k : k - J.px_total;
        int lo = 0, hi = J.njobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if ((px ? J.job[mid].px_begin : J.job[mid].z_begin) <= item) lo = mid; else hi = mid - 1;
        }
        const PrepJob& jb = J.job[lo];
        if (px) {
            const long long o = item - jb.px_begin;
            const int i = (int)(o / jb.g.rw), j = (int)(o - (long long)i * jb.g.rw);
            jb.table[o] = nbhd_entry(jb.g, jb.tar, i, j, jb.full);
        } else {
            const long long p = item - jb.z_begin;
            for (int a = 0; a < 3; ++a)
                if (jb.zero_f[a]) jb.zero_f[a][p] = 0.f;
            if (jb.zero_i) jb.zero_i[p] = 0;
        }
    }
}

// Catmull-Rom interpolation along one row of four pixels v0..v3 (bytes of
// w, v0 lowest) at fraction t:
//   h(t) = v1 + (t/2) (e1 + t (e2 + t e3)),
//   e1 = v2 - v0, e2 = 2 v0 - 5 v1 + 4 v2 - v3, e3 = -v0 + 3 v1 - 3 v2 + v3,
// the integer coefficients by one DP4A each (unsigned pixel bytes times signed
// weight bytes), exact; then Horner in FP32, two rows at a time on the
// packed FP32 pipe (f32x2).  The conversions are split between pipes: the
// coefficients by I2F; v1 by a byte permute into the low mantissa bits of
// 1.5 * 2^23 and one exact packed subtraction of 1.5 * 2^23 for both rows.
__device__ __forceinline__ int dp4a_us(uint32_t a, uint32_t b) {
    int d;
    asm("dp4a.u32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(0));
    return d;
}
__device__ __forceinline__ float v1_biased(uint32_t w) {
    return __int_as_float((int)__byte_perm(w, 0x4B400000u, 0x7651));  // bytes (v1, 0x00, 0x40, 0x4B)
}
__device__ __forceinline__ float2 cr_row_pair(uint32_t wa, uint32_t wb, float t) {
    const float2 v1 = __fadd2_rn(make_float2(v1_biased(wa), v1_biased(wb)), make_float2(-12582912.0f, -12582912.0f));
    const float2 e1 = make_float2((float)dp4a_us(wa, 0x000100FFu), (float)dp4a_us(wb, 0x000100FFu));  // (-1, 0, 1, 0)
    const float2 e2 = make_float2((float)dp4a_us(wa, 0xFF04FB02u), (float)dp4a_us(wb, 0xFF04FB02u));  // (2, -5, 4, -1)
    const float2 e3 = make_float2((float)dp4a_us(wa, 0x01FD03FFu), (float)dp4a_us(wb, 0x01FD03FFu));  // (-1, 3, -3, 1)
    const float2 tt = make_float2(t, t), th = make_float2(0.5f * t, 0.5f * t);
    return __ffma2_rn(__ffma2_rn(__ffma2_rn(e3, tt, e2), tt, e1), th, v1);
}
// Catmull-Rom combination in fraction t of four row values
// (H01 = (h_0, h_1), H23 = (h_2, h_3)): twice the interpolated value.
__device__ __forceinline__ float cr_combine4x4(float2 H01, float2 H23, float t) {
    const float f1 = H23.x - H01.x;
    const float f2 = fmaf(2.f, H01.x, fmaf(-5.f, H01.y, fmaf(4.f, H23.x, -H23.y)));
    const float f3 = fmaf(3.f, H01.y - H23.x, H23.y - H01.x);
    const float f0 = 2.f * H01.y;
    return fmaf(fmaf(fmaf(f3, t, f2), t, f1), t, f0);
}

// The reference's B-spline interpolant (BicubicSplineCoefficients_s,
// TW_utils.cpp:521-602: the 4x4 neighbourhood prefiltered on both sides by
// the local interpolation matrix CP, then mapped by the cubic B-spline basis
// matrix Base) is a tensor product of one 4-tap filter whose weights are
// cubics in the fraction: the rows of Base CP, powers of t increasing, are
// (0, 1, 0, 0), (3/56) (-11, -1, 15, -3), (3/56) (19, -39, 25, -5) and
// (1/7) (-3, 8, -8, 3).  Along one row of four pixels v0..v3 at fraction t
//   h(t) = v1 + (3/56) t (e1 + t (e2 + (8/3) t e3)),
//   e1 = -11 v0 - v1 + 15 v2 - 3 v3, e2 = 19 v0 - 39 v1 + 25 v2 - 5 v3,
//   e3 = -3 v0 + 8 v1 - 8 v2 + 3 v3,
// the integer coefficients by DP4A and v1 by the byte permute, as for
// Catmull-Rom; the four row values are combined by the same weights in the
// other fraction.
__device__ __forceinline__ float2 bs_row_pair(uint32_t wa, uint32_t wb, float t) {
    const float2 v1 = __fadd2_rn(make_float2(v1_biased(wa), v1_biased(wb)), make_float2(-12582912.0f, -12582912.0f));
    const float2 e1 = make_float2((float)dp4a_us(wa, 0xFD0FFFF5u), (float)dp4a_us(wb, 0xFD0FFFF5u));  // (-11, -1, 15, -3)
    const float2 e2 = make_float2((float)dp4a_us(wa, 0xFB19D913u), (float)dp4a_us(wb, 0xFB19D913u));  // (19, -39, 25, -5)
    const float2 e3 = make_float2((float)dp4a_us(wa, 0x03F808FDu), (float)dp4a_us(wb, 0x03F808FDu));  // (-3, 8, -8, 3)
    const float ta = (3.0f / 56.0f) * t, tb = (8.0f / 3.0f) * t;
    return __ffma2_rn(__ffma2_rn(__ffma2_rn(e3, make_float2(tb, tb), e2), make_float2(t, t), e1), make_float2(ta, ta),
                      v1);
}
// B-spline combination in fraction t of four row values (H01 = (h_0, h_1),
// H23 = (h_2, h_3)): the interpolated value, with the scalings in the
// weights ((3/56) e1 and (3/56) e2 together on the packed pipe).
__device__ __forceinline__ float bs_combine4x4(float2 H01, float2 H23, float t) {
    constexpr float k = 3.0f / 56.0f;
    const float2 f12 = __ffma2_rn(
        make_float2(H23.y, H23.y), make_float2(-3.f * k, -5.f * k),
        __ffma2_rn(make_float2(H23.x, H23.x), make_float2(15.f * k, 25.f * k),
                   __ffma2_rn(make_float2(H01.y, H01.y), make_float2(-k, -39.f * k),
                              __fmul2_rn(make_float2(H01.x, H01.x), make_float2(-11.f * k, 19.f * k)))));
    const float f3 = fmaf(3.0f / 7.0f, H23.y - H01.x, (8.0f / 7.0f) * (H01.y - H23.x));
    return fmaf(fmaf(fmaf(f3, t, f12.y), t, f12.x), t, H01.y);
}

// Per-sample sums of one IC-GN pass on packed FP32: (sum t', sum t'^2),
// (sum R_x t', sum R_y t'), (sum R_x t' dx, sum R_y t' dx),
// (sum R_x t' dy, sum R_y t' dy), t' = T - mean(R).
struct PassSums {
    float2 s01 = make_float2(0.f, 0.f), s25 = make_float2(0.f, 0.f);
    float2 s36 = make_float2(0.f, 0.f), s47 = make_float2(0.f, 0.f);
    __device__ __forceinline__ void add(float tp, float2 gr, float2 d) {
        const float2 tt = make_float2(tp, tp);
        s01 = __ffma2_rn(tt, make_float2(1.f, tp), s01);
        const float2 ab = __fmul2_rn(gr, tt);
        s25 = __fadd2_rn(s25, ab);
        s36 = __ffma2_rn(ab, make_float2(d.x, d.x), s36);
        s47 = __ffma2_rn(ab, make_float2(d.y, d.y), s47);
    }
    // the eight sums in the order sum t', sum t'^2, R_x t', R_x t' dx,
    // R_x t' dy, R_y t', R_y t' dx, R_y t' dy
    __device__ __forceinline__ void unpack(float* s) const {
        s[0] = s01.x; s[1] = s01.y;
        s[2] = s25.x; s[3] = s36.x; s[4] = s47.x;
        s[5] = s25.y; s[6] = s36.y; s[7] = s47.y;
    }
};

// The eight sums of a warp by recursive halving: each exchange sends half of
// the values still held and adds the received half, so after the exchanges
// at lane distances 16, 8 and 4 a lane holds partial sums of one value, and
// two butterfly steps finish it.  Lane l returns sum number (l >> 2) & 7
// (12 shuffles instead of 40).
__device__ __forceinline__ float warp_reduce8(const float* s) {
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    float t4[4], t2[2];
    const bool b16 = lane & 16, b8 = lane & 8, b4 = lane & 4;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float keep = b16 ? s[i + 4] : s[i], send = b16 ? s[i] : s[i + 4];
        t4[i] = keep + __shfl_xor_sync(FULL, send, 16);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const float keep = b8 ? t4[i + 2] : t4[i], send = b8 ? t4[i] : t4[i + 2];
        t2[i] = keep + __shfl_xor_sync(FULL, send, 8);
    }
    const float keep = b4 ? t2[1] : t2[0], send = b4 ? t2[0] : t2[1];
    float v = keep + __shfl_xor_sync(FULL, send, 4);
    v += __shfl_xor_sync(FULL, v, 2);
    v += __shfl_xor_sync(FULL, v, 1);
    return v;
}

// Catmull-Rom weights (the Hermite bicubic with central differences).
__device__ __forceinline__ void cr_weights(float t, float& w0, float& w1, float& w2, float& w3) {
    const float t2 = t * t;
    w0 = t * (t * (-0.5f * t + 1.0f) - 0.5f);
    w1 = t2 * (1.5f * t - 2.5f) + 1.0f;
    w2 = t * (t * (-1.5f * t + 2.0f) + 0.5f);
    w3 = t2 * (0.5f * t - 0.5f);
}

// Affine warp of subset offset (dx, dy) as two FMAs per coordinate.  The
// reference rounds each operation; the difference is an ulp, which moves a
// truncated coordinate only at an exact integer, where the bicubic patch is
// continuous.  Each FMA rounds once, so the result is non-decreasing in dx
// and in dy separately: its extremes over the subset lie at the corners.
__device__ __forceinline__ float warp_x(const float* Wm, float bx, float dx, float dy) {
    return fmaf(Wm[0], dx, fmaf(Wm[1], dy, bx));
}
__device__ __forceinline__ float warp_y(const float* Wm, float by, float dx, float dy) {
    return fmaf(Wm[3], dx, fmaf(Wm[4], dy, by));
}

// OutofROI test of one pass (TW_paDIC_ICGN2D_CPU.cpp:625-635, :765-770):
// some sample truncates outside the ROI exactly when one of the four corner
// samples does, since truncation is monotone and the warp's extremes lie at
// the corners.
__device__ __forceinline__ bool pass_out_of_roi(const Geom& g, const float* Wm, float bx, float by) {
    const float rx = (float)g.rx, ry = (float)g.ry;
    bool out = false;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float dx = (c & 1) ? rx : -rx, dy = (c & 2) ? ry : -ry;
        const int ix = (int)warp_x(Wm, bx, dx, dy), iy = (int)warp_y(Wm, by, dx, dy);
        out |= (unsigned)(ix - g.sx) >= (unsigned)g.rw || (unsigned)(iy - g.sy) >= (unsigned)g.rh;
    }
    return out;
}

// The same test with one corner per lane (lanes 0-3) and a warp vote.
__device__ __forceinline__ bool pass_out_of_roi_warp(const Geom& g, const float* Wm, float bx, float by) {
    const int lane = threadIdx.x & 31, c = lane & 3;
    const float rx = (float)g.rx, ry = (float)g.ry;
    const float dx = (c & 1) ? rx : -rx, dy = (c & 2) ? ry : -ry;
    const int ix = (int)warp_x(Wm, bx, dx, dy), iy = (int)warp_y(Wm, by, dx, dy);
    const bool out = lane < 4 && ((unsigned)(ix - g.sx) >= (unsigned)g.rw || (unsigned)(iy - g.sy) >= (unsigned)g.rh);
    return __any_sync(0xffffffffu, out);
}

// Persistent IC-GN kernel, one POI per CTA at a time.  The target sampler:
//   kSampWindow: the target window around the guess is staged in shared
//     memory and interpolated with the separable Catmull-Rom weights;
//   kSampLut: the per-frame bicubic coefficient LUT (four float4 planes,
//     k_bicubic_lut), evaluated by Horner's rule;
//   kSampNbhd: the per-frame 4x4 neighbourhood table (16 bytes per ROI
//     pixel, k_nbhd_table), one 16-byte gather per sample, Catmull-Rom;
//   kSampNbhdBs: the same table over every ROI pixel, the reference's
//     B-spline interpolant (bs_row_pair, bs_combine4x4).
// The Catmull-Rom form with central-difference derivatives is algebraically
// the reference's Hermite bicubic LUT (TW_utils.cpp:604-700).
template <int THREADS, int SAMPLER, bool MULTI>
__global__ void __launch_bounds__(THREADS, (THREADS == 64 ? 16 : 2048 / THREADS / 2))
    k_icgn_fast(const __grid_constant__ IcgnJobs J, int* work) {
    constexpr int NW = THREADS / 32;
    constexpr unsigned FULL = 0xffffffffu;
    // dynamic shared memory: [S] half2 reference gradients (R_x, R_y: half
    // integers of magnitude <= 127.5, exact in FP16), then (window path) the
    // [ws][ws] target window; sized for the largest subset of the launch
    extern __shared__ __align__(16) float smem_f[];
    __shared__ float red[NW][8];
    __shared__ float sW[6];
    __shared__ int sctl[3];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

    for (;;) {
        if (tid == 0) sctl[2] = atomicAdd(work, 1);
        __syncthreads();
        const int pg = sctl[2];
        if (pg >= J.total) break;
        // the job (image pair, POI set) this POI belongs to; POIs of job j
        // are the global indices [begin_j, begin_j + n_j)
        int jj = 0;
        if (MULTI) {
            while (jj + 1 < J.njobs && pg >= J.job[jj + 1].begin) ++jj;
        }
        const IcgnJob& jb = J.job[jj];
        const Geom& g = jb.g;
        const uint8_t* __restrict__ ref = jb.ref;
        const uint8_t* __restrict__ tar = jb.tar;
        const int2* __restrict__ poi = jb.poi;
        const float* __restrict__ stats = jb.stats;
        const double* __restrict__ hinv = jb.hinv;
        const uint8_t* __restrict__ rflag = jb.rflag;
        float* u = jb.u;
        float* v = jb.v;
        float* p6 = jb.p6;
        int* iters = jb.iters;
        uint8_t* flags = jb.flags;
        const int p = pg - jb.begin;
        const int ws = 2 * (g.rx > g.ry ? g.rx : g.ry) + 11;
        const int SW = 2 * g.rx + 1, SH = 2 * g.ry + 1, S = SW * SH;
        __half2* grad = reinterpret_cast<__half2*>(smem_f);
        float* win = smem_f + ((S + 3) & ~3);
        const float inv_s = 1.0f / (float)S;
        // sample k = tid + j*THREADS sits at subset offset (dx, dy); stepping j
        // advances it by (ddx, ddy) with carry (small integers, exact in FP32)
        const float dx_first = (float)(tid % SW - g.rx), dy_first = (float)(tid / SW - g.ry);
        const float ddx = (float)(THREADS % SW), ddy = (float)(THREADS / SW);
        const float rxf = (float)g.rx, swf = (float)SW;
        // plane-0 LUT entry of image pixel (ix, iy) is lut0[iy * rw + ix]
        const size_t plane = (size_t)g.rw * g.rh;
        const float4* lut0 = static_cast<const float4*>(jb.table) - ((size_t)g.sy * g.rw + g.sx);
        const uint4* nb0 = static_cast<const uint4*>(jb.table) - ((size_t)g.sy * g.rw + g.sx);
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
        // ---- stage the reference gradients (and the target window)
        const int wx0 = px + (int)floorf(u0) - g.rx - 4;
        const int wy0 = py + (int)floorf(v0) - g.ry - 4;
        if (!done) {
            if (SAMPLER == kSampWindow) {
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
                    grad[l * SW + m] = __floats2half2_rn(0.5f * (float)((int)r[1] - (int)r[-1]),
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
            float s[8];
            PassSums ps;
            const float bx = (float)px + Wm[2], by = (float)py + Wm[5];
            // uniform over the CTA: every thread evaluates the same corners
            const bool oor = pass_out_of_roi(g, Wm, bx, by);
            if (!oor) {
                // (dx, dy) of the current sample; warp_x / warp_y on packed FP32
                float2 d = make_float2(dx_first, dy_first);
                const float2 dd = make_float2(ddx, ddy), wrap = make_float2(-swf, 1.f);
                const float2 w03 = make_float2(Wm[0], Wm[3]), w14 = make_float2(Wm[1], Wm[4]);
                const float2 bxy = make_float2(bx, by);
                const __half2* gp = grad + tid;
                if (it == 0) {
                    // first pass: integer pixels (TW_paDIC_ICGN2D_CPU.cpp:609-637)
#pragma unroll 4
                    for (int k = tid; k < S; k += THREADS) {
                        const float2 wxy = __ffma2_rn(w03, make_float2(d.x, d.x),
                                                      __ffma2_rn(w14, make_float2(d.y, d.y), bxy));
                        const int ix = (int)wxy.x, iy = (int)wxy.y;
                        const int lx = ix - wx0, ly = iy - wy0;
                        const float t = (SAMPLER == kSampWindow && lx >= 0 && ly >= 0 && lx < ws && ly < ws)
                                            ? win[ly * ws + lx]
                                            : (float)tar[(size_t)iy * g.pitch + ix];
                        ps.add(t - c, __half22float2(*gp), d);
                        gp += THREADS;
                        d = __fadd2_rn(d, dd);
                        if (d.x > rxf) d = __fadd2_rn(d, wrap);
                    }
                } else {
#pragma unroll 4
                    for (int k = tid; k < S; k += THREADS) {
                        const float2 wxy = __ffma2_rn(w03, make_float2(d.x, d.x),
                                                      __ffma2_rn(w14, make_float2(d.y, d.y), bxy));
                        const int ix = (int)wxy.x, iy = (int)wxy.y;
                        const float2 fxy = __fadd2_rn(wxy, make_float2(-(float)ix, -(float)iy));
                        const float fx = fxy.x, fy = fxy.y;
                        float tp;
                        if (SAMPLER == kSampNbhd) {
                            // 4x4 pixels around (ix, iy), row-major bytes; zero on the
                            // ROI's last row and column, as the reference LUT is there
                            const uint4 q = nb0[(size_t)iy * g.rw + ix];
                            const float2 h01 = cr_row_pair(q.x, q.y, fx), h23 = cr_row_pair(q.z, q.w, fx);
                            tp = fmaf(0.5f, cr_combine4x4(h01, h23, fy), -c);
                        } else if (SAMPLER == kSampNbhdBs) {
                            const uint4 q = nb0[(size_t)iy * g.rw + ix];
                            const float2 h01 = bs_row_pair(q.x, q.y, fx), h23 = bs_row_pair(q.z, q.w, fx);
                            tp = bs_combine4x4(h01, h23, fy) - c;
                        } else if (SAMPLER == kSampLut) {
                            const float4* q = lut0 + ((size_t)iy * g.rw + ix);
                            const float4 a0 = q[0], a1 = q[plane], a2 = q[2 * plane], a3 = q[3 * plane];
                            const float2 tx = make_float2(fx, fx);
                            const float2 r01 = __ffma2_rn(
                                __ffma2_rn(__ffma2_rn(make_float2(a0.w, a1.w), tx, make_float2(a0.z, a1.z)), tx,
                                           make_float2(a0.y, a1.y)),
                                tx, make_float2(a0.x, a1.x));
                            const float2 r23 = __ffma2_rn(
                                __ffma2_rn(__ffma2_rn(make_float2(a2.w, a3.w), tx, make_float2(a2.z, a3.z)), tx,
                                           make_float2(a2.y, a3.y)),
                                tx, make_float2(a2.x, a3.x));
                            tp = (((r23.y * fy + r23.x) * fy + r01.y) * fy + r01.x) - c;
                        } else if (iy - g.sy == g.rh - 1 || ix - g.sx == g.rw - 1) {
                            tp = 0.f - c;  // the reference LUT's never-written last row / column
                        } else {
                            const int lx = ix - wx0, ly = iy - wy0;
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
                            tp = (cy0 * rr[0] + cy1 * rr[1] + cy2 * rr[2] + cy3 * rr[3]) - c;
                        }
                        ps.add(tp, __half22float2(*gp), d);
                        gp += THREADS;
                        d = __fadd2_rn(d, dd);
                        if (d.x > rxf) d = __fadd2_rn(d, wrap);
                    }
                }
                ps.unpack(s);
                // ---- one reduction (FP32)
                const float v8 = warp_reduce8(s);
                if ((lane & 3) == 0) red[wid][(lane >> 2) & 7] = v8;
                __syncthreads();
            }
            // ---- warp 0 finishes the iteration: FP32 scalars, FP64 H^-1 b on
            // lanes 0-5, warp update on lane 0
            if (wid == 0) {
                float tot = 0.f;
                if (!oor && lane < 8)
                    for (int w = 0; w < NW; ++w) tot += red[w][lane];
                const float S0 = __shfl_sync(FULL, tot, 0), S1 = __shfl_sync(FULL, tot, 1);
                const float Ak = __shfl_sync(FULL, tot, 2 + (lane < 6 ? lane : 0));
                const float m0 = S0 * inv_s;
                const float mean_t = c + m0;
                const float var = S1 - S0 * m0;
                const float ts = sqrtf(var > 0.f ? var : 0.f);
                int flag = kSuccess, cont = 0;
                if (oor) {
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

// Reference gradients of every ROI pixel as float2 (R_x, R_y): central
// differences (TW_utils.cpp:232-305), half integers of magnitude <= 127.5.
// (FP32 rather than FP16 pairs: the sample loop of k_icgn_warp then loads them
// without conversion, 2 % faster at 2048^2.)  The ROI has one pixel of border on every side, so every
// neighbour read lies in the image.
__global__ void k_ref_grad(Geom g, const uint8_t* __restrict__ ref, float2* __restrict__ grad) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= g.rh || j >= g.rw) return;
    const uint8_t* r = ref + (size_t)(i + g.sy) * g.pitch + (j + g.sx);
    grad[(size_t)i * g.rw + j] = make_float2(0.5f * (float)((int)r[1] - (int)r[-1]),
                                                   0.5f * (float)((int)r[g.pitch] - (int)r[-g.pitch]));
}

// Persistent IC-GN kernel, one POI per warp.  The warps of a CTA walk runs
// of CHUNK consecutive POIs (CTA b takes runs b, b + gridDim.x, ...; its
// warps draw POIs from them in order through a shared counter), so the
// subsets a CTA has in flight overlap and their target-table entries and
// reference gradients (global, per-reference float2 image) are re-read from
// L1 across neighbouring POIs and across iterations.  The arithmetic per
// POI is that of k_icgn_fast<32, ...>: the same sample order per lane, the
// same sums, reduction, solve and update, so the results are identical.
template <int NW, int SAMPLER, bool MULTI, int UNROLL>
__global__ void __launch_bounds__(NW * 32, (NW >= 32 ? 1 : 32 / NW))
    k_icgn_warp(const __grid_constant__ IcgnJobs J, int chunk) {
    constexpr unsigned FULL = 0xffffffffu;
    __shared__ int s_next;
    __shared__ double s_h[NW][36];  // rows of H^-1 of each warp's POI
    __shared__ float s_p[NW][6];     // each warp's warp parameters P (lane 0)
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    double* hw = s_h[wid];
    float* pw = s_p[wid];
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(&s_next, 1);
        t = __shfl_sync(FULL, t, 0);
        const long long pgl = ((long long)blockIdx.x + (long long)(t / chunk) * gridDim.x) * chunk + t % chunk;
        if (pgl >= J.total) break;
        const int pg = (int)pgl;
        int jj = 0;
        if (MULTI) {
            while (jj + 1 < J.njobs && pg >= J.job[jj + 1].begin) ++jj;
        }
        const IcgnJob& jb = J.job[jj];
        const Geom& g = jb.g;
        const int p = pg - jb.begin;
        const int SW = 2 * g.rx + 1, SH = 2 * g.ry + 1, S = SW * SH;
        const float inv_s = 1.0f / (float)S;
        const size_t plane = (size_t)g.rw * g.rh;
        const float4* lut0 = static_cast<const float4*>(jb.table) - ((size_t)g.sy * g.rw + g.sx);
        const uint4* nb0 = static_cast<const uint4*>(jb.table) - ((size_t)g.sy * g.rw + g.sx);
        const int2 pyx = jb.poi[p];
        const int py = pyx.x, px = pyx.y;
        const float u0 = jb.u[p], v0 = jb.v[p];
        const uint8_t rf = jb.rflag[p];
        float Wm[6] = {1.f, 0.f, u0, 0.f, 1.f, v0};
        if (rf == kDarkSubset || rf == kOutofROI) {
            if (lane == 0) {
                jb.flags[p] = rf;
                const float P0[6] = {u0, 0.f, 0.f, v0, 0.f, 0.f};
                for (int k = 0; k < 6; ++k) jb.p6[(size_t)p * 6 + k] = P0[k];
            }
            continue;
        }
        // P in shared memory (lane 0 updates it); lane k < 6: row k of H^-1
        // (FP64); the statistics are re-read at each solve, not held in
        // registers through the sample loop
        if (lane == 0) {
            pw[0] = u0; pw[1] = 0.f; pw[2] = 0.f; pw[3] = v0; pw[4] = 0.f; pw[5] = 0.f;
        }
        const float* st = jb.stats + (size_t)p * 16;
        const float c = st[0];
        if (lane < 6) {
            const double* hi = jb.hinv + (size_t)p * 21;
#pragma unroll
            for (int j = 0; j < 6; ++j) hw[lane * 6 + j] = hi[lane >= j ? tri(lane, j) : tri(j, lane)];
        }
        __syncwarp();
        // sample k = lane + 32 j: its offset (dx, dy) and its column and row
        // in the subset from the sample table (one L1-resident load in place
        // of stepping with a carry), its reference gradient at ROI offset
        // row * rw + column from grad0
        const float2* grad0 = jb.grad + ((size_t)(py - g.ry - g.sy) * g.rw + (px - g.rx - g.sx));
        const float4* smp0 = jb.samples + lane;
        int it = 0;
        for (;;) {
            const float bx = (float)px + Wm[2], by = (float)py + Wm[5];
            const bool oor = pass_out_of_roi_warp(g, Wm, bx, by);
            float s[8];
            float v8 = 0.f;
            if (!oor) {
                PassSums ps;
                const float4* smp = smp0;
                const float2 w03 = make_float2(Wm[0], Wm[3]), w14 = make_float2(Wm[1], Wm[4]);
                const float2 bxy = make_float2(bx, by);
                if (it == 0) {
                    // first pass: integer pixels (TW_paDIC_ICGN2D_CPU.cpp:609-637)
#pragma unroll UNROLL
                    for (int k = lane; k < S; k += 32) {
                        const float4 e4 = __ldg(smp);
                        smp += 32;
                        const float2 d = make_float2(e4.x, e4.y);
                        const int gofs = __float_as_int(e4.w) * g.rw + __float_as_int(e4.z);
                        const float2 wxy = __ffma2_rn(w03, make_float2(d.x, d.x),
                                                      __ffma2_rn(w14, make_float2(d.y, d.y), bxy));
                        const int ix = (int)wxy.x, iy = (int)wxy.y;
                        ps.add((float)jb.tar[(size_t)iy * g.pitch + ix] - c, grad0[gofs], d);
                    }
                } else {
#pragma unroll UNROLL
                    for (int k = lane; k < S; k += 32) {
                        const float4 e4 = __ldg(smp);
                        smp += 32;
                        const float2 d = make_float2(e4.x, e4.y);
                        const int gofs = __float_as_int(e4.w) * g.rw + __float_as_int(e4.z);
                        const float2 wxy = __ffma2_rn(w03, make_float2(d.x, d.x),
                                                      __ffma2_rn(w14, make_float2(d.y, d.y), bxy));
                        const int ix = (int)wxy.x, iy = (int)wxy.y;
                        const float2 fxy = __fadd2_rn(wxy, make_float2(-(float)ix, -(float)iy));
                        const float fx = fxy.x, fy = fxy.y;
                        float tp;
                        if (SAMPLER == kSampNbhd) {
                            const uint4 q = nb0[(unsigned)(iy * g.rw + ix)];  // < 2^31 entries
                            const float2 h01 = cr_row_pair(q.x, q.y, fx), h23 = cr_row_pair(q.z, q.w, fx);
                            tp = fmaf(0.5f, cr_combine4x4(h01, h23, fy), -c);
                        } else if (SAMPLER == kSampNbhdBs) {
                            const uint4 q = nb0[(unsigned)(iy * g.rw + ix)];
                            const float2 h01 = bs_row_pair(q.x, q.y, fx), h23 = bs_row_pair(q.z, q.w, fx);
                            tp = bs_combine4x4(h01, h23, fy) - c;
                        } else {
                            const float4* q = lut0 + (unsigned)(iy * g.rw + ix);
                            const float4 a0 = q[0], a1 = q[plane], a2 = q[2 * plane], a3 = q[3 * plane];
                            const float2 tx = make_float2(fx, fx);
                            const float2 r01 = __ffma2_rn(
                                __ffma2_rn(__ffma2_rn(make_float2(a0.w, a1.w), tx, make_float2(a0.z, a1.z)), tx,
                                           make_float2(a0.y, a1.y)),
                                tx, make_float2(a0.x, a1.x));
                            const float2 r23 = __ffma2_rn(
                                __ffma2_rn(__ffma2_rn(make_float2(a2.w, a3.w), tx, make_float2(a2.z, a3.z)), tx,
                                           make_float2(a2.y, a3.y)),
                                tx, make_float2(a2.x, a3.x));
                            tp = (((r23.y * fy + r23.x) * fy + r01.y) * fy + r01.x) - c;
                        }
                        ps.add(tp, grad0[gofs], d);
                    }
                }
                ps.unpack(s);
                v8 = warp_reduce8(s);
            }
            // FP32 scalars, FP64 H^-1 b on lanes 0-5, warp update on lanes 0-5;
            // sum k is held by lanes 4k .. 4k+3
            const float S0 = __shfl_sync(FULL, v8, 0), S1 = __shfl_sync(FULL, v8, 4);
            const float Ak = __shfl_sync(FULL, v8, 8 + 4 * (lane < 6 ? lane : 0));
            const float m0 = S0 * inv_s;
            const float mean_t = c + m0;
            const float var = S1 - S0 * m0;
            const float ts = sqrtf(var > 0.f ? var : 0.f);
            int flag = kSuccess, cont = 0;
            if (oor) {
                flag = kOutofROI;
            } else if (fabsf(mean_t) <= FLT_EPSILON || fabsf(ts) <= FLT_EPSILON) {
                flag = kDarkSubset;
            } else if (it == 0 && rf == kSingularHessian) {
                flag = kSingularHessian;
            }
            float dpk = 0.f;
            if (flag == kSuccess) {
                const float q = st[1] / ts;  // ||R - mean(R)|| / ||T - mean(T)||
                const float sumsd = lane < 6 ? st[2 + lane] : 0.f, qk = lane < 6 ? st[8 + lane] : 0.f;
                const float bk = (lane < 6) ? q * (Ak - m0 * sumsd) - qk : 0.f;
                const double bd = (double)bk;
                double acc = 0.0;
#pragma unroll
                for (int j = 0; j < 6; ++j) {
                    const double bj = __shfl_sync(FULL, bd, j);
                    if (lane < 6) acc = fma(hw[lane * 6 + j], bj, acc);
                }
                dpk = (float)acc;
            }
            float dp[6];
#pragma unroll
            for (int j = 0; j < 6; ++j) dp[j] = __shfl_sync(FULL, dpk, j);
            // W(P) o W(dP)^-1 (update_warp's operations), coefficient k on lane k:
            // w_k = base_k + (x_k y_k - z_k v_k) / det
            bool singular = false;
            float wk = 0.f;
            if (flag == kSuccess) {
                const float P0 = pw[0], P1 = pw[1], P2 = pw[2], P3 = pw[3], P4 = pw[4], P5 = pw[5];
                const float det = __fsub_rn(__fmul_rn(1.f + dp[1], 1.f + dp[5]), __fmul_rn(dp[2], dp[4]));
                singular = fabsf(det) <= FLT_EPSILON;
                if (!singular && lane < 6) {
                    const float a = __fsub_rn(__fsub_rn(__fmul_rn(dp[0], dp[4]), dp[3]), __fmul_rn(dp[3], dp[1]));
                    const float b = __fsub_rn(__fadd_rn(__fmul_rn(dp[0], dp[5]), dp[0]), __fmul_rn(dp[2], dp[3]));
                    const int r3 = lane % 3;  // 0: (1+d5, d4), 1: (1+d1, d2), 2: (a, b)
                    const float y = r3 == 0 ? 1.f + dp[5] : (r3 == 1 ? 1.f + dp[1] : a);
                    const float v = r3 == 0 ? dp[4] : (r3 == 1 ? dp[2] : b);
                    const float x = lane == 0 ? 1.f + P1 : (lane <= 2 ? P2 : (lane == 3 ? P4 : 1.f + P5));
                    const float z = lane == 0 ? P2 : (lane <= 2 ? 1.f + P1 : (lane == 3 ? 1.f + P5 : P4));
                    const float q = __fdiv_rn(__fsub_rn(__fmul_rn(x, y), __fmul_rn(z, v)), det);
                    wk = lane == 2 ? __fadd_rn(P0, q) : (lane == 5 ? __fadd_rn(P3, q) : q);
                }
            }
            float Wn[6];
#pragma unroll
            for (int j = 0; j < 6; ++j) Wn[j] = __shfl_sync(FULL, wk, j);
            if (lane == 0) {
                float P[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) P[k] = pw[k];
                if (flag == kSuccess) {
                    if (singular) {
                        flag = kSingularWarp;
                    } else {
#pragma unroll
                        for (int k = 0; k < 6; ++k) Wm[k] = Wn[k];
                        P[0] = Wn[2];
                        P[1] = Wn[0] - 1.f;
                        P[2] = Wn[1];
                        P[3] = Wn[5];
                        P[4] = Wn[3];
                        P[5] = Wn[4] - 1.f;
                        // scaled ||dP|| >= delta_p, squared, FP32
                        const float a1 = dp[1] * (float)g.rx, a2 = dp[2] * (float)g.ry;
                        const float a4 = dp[4] * (float)g.rx, a5 = dp[5] * (float)g.ry;
                        const float nrm2 = dp[0] * dp[0] + a1 * a1 + a2 * a2 + dp[3] * dp[3] + a4 * a4 + a5 * a5;
                        cont = (it + 1 < g.max_iter && nrm2 >= g.delta_p * g.delta_p) ? 1 : 0;
                    }
                }
                if (!(flag == kSuccess && cont)) {
                    // finish: the counter is it+1 after a solve or an abort in a
                    // later pass; an abort in the first pass leaves it untouched
                    jb.flags[p] = (uint8_t)flag;
                    for (int k = 0; k < 6; ++k) jb.p6[(size_t)p * 6 + k] = P[k];
                    jb.u[p] = P[0];
                    jb.v[p] = P[3];
                    if (flag == kSuccess || it > 0) jb.iters[p] = it + 1;
                }
#pragma unroll
                for (int k = 0; k < 6; ++k) pw[k] = P[k];
            }
            cont = __shfl_sync(FULL, (flag == kSuccess && cont) ? 1 : 0, 0);
            if (!cont) break;
            // every lane has the new warp; lane 0's P is read by all at the next update
#pragma unroll
            for (int k = 0; k < 6; ++k) Wm[k] = Wn[k];
            __syncwarp();
            ++it;
        }
        __syncwarp();  // hw is rewritten by the warp's next POI
    }
}

}  // namespace

cudaError_t launch_ref_precompute_fast(const Geom& g, const uint8_t* ref, const int2* poi, int n, float* stats,
                                       double* chol, uint8_t* rflag, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_ref_sums<<<(n + kSumWarps - 1) / kSumWarps, kSumWarps * 32, 0, st>>>(g, ref, poi, n, stats, chol, rflag);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_ref_factor<<<(n + kFactorThreads - 1) / kFactorThreads, kFactorThreads, 0, st>>>(n, chol, rflag);
    return cudaGetLastError();
}

cudaError_t launch_nbhd_table(const Geom& g, const uint8_t* tar, uint4* table, cudaStream_t st, bool full) {
    dim3 blk(32, 8), grd((g.rw + 31) / 32, (g.rh + 7) / 8);
    k_nbhd_table<<<grd, blk, 0, st>>>(g, tar, table, full ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_batch_prepare(const PrepJobs& J, cudaStream_t st) {
    const long long total = J.px_total + J.z_total;
    if (total <= 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long blocks = std::min<long long>((total + 255) / 256, (long long)sms * 8);
    k_batch_prepare<<<(int)blocks, 256, 0, st>>>(J);
    return cudaGetLastError();
}

int icgn_fast_window(const Geom& g) { return 2 * (g.rx > g.ry ? g.rx : g.ry) + 1 + 10; }

template <int THREADS, int SAMPLER, bool MULTI>
static cudaError_t launch_icgn_fast_t(const IcgnJobs& J, int* work, int ctas_per_sm, cudaStream_t st) {
    int S_max = 0, ws_max = 0;
    for (int j = 0; j < J.njobs; ++j) {
        const Geom& g = J.job[j].g;
        S_max = std::max(S_max, (2 * g.rx + 1) * (2 * g.ry + 1));
        ws_max = std::max(ws_max, icgn_fast_window(g));
    }
    const size_t smem =
        sizeof(float) * ((size_t)((S_max + 3) & ~3) + (SAMPLER == kSampWindow ? (size_t)ws_max * ws_max : 0));
    auto kern = k_icgn_fast<THREADS, SAMPLER, MULTI>;
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
    if (grid > J.total) grid = J.total;
    e = cudaMemsetAsync(work, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    kern<<<grid, THREADS, smem, st>>>(J, work);
    return cudaGetLastError();
}

int icgn_fast_residency(const Geom& g, const IcgnTune& tune) {
    // one POI per warp: no per-POI shared memory, one residency for all
    if (tune.chunk > 0 && tune.sampler != kSampWindow && tune.threads >= 128) return 32 * 32 / tune.threads;
    const int S = (2 * g.rx + 1) * (2 * g.ry + 1), ws = icgn_fast_window(g);
    const size_t smem = sizeof(float) * ((size_t)((S + 3) & ~3) + (tune.sampler == kSampWindow ? (size_t)ws * ws : 0));
    const int threads = tune.threads == 32 || tune.threads == 64 || tune.threads == 256 ? tune.threads : 128;
    const int by_regs = 65536 / (64 * threads);            // the kernels' 64-register budget
    const int by_smem = (int)((228u * 1024u) / (smem + 1024u));  // 1 KB per CTA reserved by the runtime
    return std::max(1, std::min(std::min(32, by_regs), by_smem));
}

// Entry k of the sample table: the offset (dx, dy) from the POI and the
// column and row within the subset, k = row * (2 rx + 1) + column.
__global__ void k_sample_table(int rx, int ry, float4* out) {
    const int SW = 2 * rx + 1, S = SW * (2 * ry + 1);
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= S) return;
    const int ox = k % SW, oy = k / SW;
    out[k] = make_float4((float)(ox - rx), (float)(oy - ry), __int_as_float(ox), __int_as_float(oy));
}

cudaError_t launch_sample_table(int rx, int ry, float4* out, cudaStream_t st) {
    const int S = (2 * rx + 1) * (2 * ry + 1);
    k_sample_table<<<(S + 255) / 256, 256, 0, st>>>(rx, ry, out);
    return cudaGetLastError();
}

cudaError_t launch_ref_grad(const Geom& g, const uint8_t* ref, float2* grad, cudaStream_t st) {
    dim3 blk(32, 8), grd((g.rw + 31) / 32, (g.rh + 7) / 8);
    k_ref_grad<<<grd, blk, 0, st>>>(g, ref, grad);
    return cudaGetLastError();
}

template <int NW, int SAMPLER, bool MULTI>
static cudaError_t launch_icgn_warp_t(const IcgnJobs& J, int chunk, int ctas_per_sm, int unroll, cudaStream_t st) {
    // sample-loop unrolling: 2, 4 or 8 for the one-CTA-per-SM shape, 4 otherwise
    auto kern = k_icgn_warp<NW, SAMPLER, MULTI, 4>;
    if (NW == 32 && unroll == 2) kern = k_icgn_warp<NW, SAMPLER, MULTI, (NW == 32 ? 2 : 4)>;
    if (NW == 32 && unroll == 8) kern = k_icgn_warp<NW, SAMPLER, MULTI, (NW == 32 ? 8 : 4)>;
    // a few KB of shared memory: leave the rest of the SM's 256 KB to L1
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, NW * 32, 0);
    if (e != cudaSuccess) return e;
    if (ctas_per_sm > 0 && ctas_per_sm < occ) occ = ctas_per_sm;
    if (occ < 1) occ = 1;
    long long grid = (long long)sms * occ;
    const long long runs = ((long long)J.total + chunk - 1) / chunk;
    if (grid > runs) grid = runs;
    kern<<<(int)grid, NW * 32, 0, st>>>(J, chunk);
    return cudaGetLastError();
}

// One POI per warp over a per-reference gradient image: every job needs
// grad, the sample table, a table sampler and table offsets below 2^31
// (otherwise the one-POI-per-CTA kernel runs).
static bool icgn_warp_eligible(const IcgnJobs& J, const IcgnTune& tune) {
    if (tune.chunk <= 0 || tune.sampler == kSampWindow) return false;
    if (tune.threads != 128 && tune.threads != 256 && tune.threads != 512 && tune.threads != 1024) return false;
    for (int j = 0; j < J.njobs; ++j) {
        if (!J.job[j].grad || !J.job[j].samples) return false;
        // the kernel indexes the table with 32-bit image offsets iy * rw + ix
        if ((long long)J.job[j].g.img_h * J.job[j].g.rw >= (1ll << 31)) return false;
    }
    return true;
}

cudaError_t launch_icgn_fast_jobs(const IcgnJobs& J, int* work, const IcgnTune& tune, cudaStream_t st) {
    if (J.njobs < 1 || J.njobs > kMaxJobs) return cudaErrorInvalidValue;
    if (J.total <= 0) return cudaSuccess;
    if (icgn_warp_eligible(J, tune)) {
        for (int j = 0; j < J.njobs; ++j)
            if (!J.job[j].table) return cudaErrorInvalidValue;
        const bool multi = J.njobs > 1;
#define TWDIC_ICGN_WARP(NW, SA)                                                                  \
    return multi ? launch_icgn_warp_t<NW, SA, true>(J, tune.chunk, tune.ctas_per_sm, tune.unroll, st)  \
                 : launch_icgn_warp_t<NW, SA, false>(J, tune.chunk, tune.ctas_per_sm, tune.unroll, st)
#define TWDIC_ICGN_WARP_N(NW)                                                                    \
    if (tune.sampler == kSampLut) { TWDIC_ICGN_WARP(NW, kSampLut); }                              \
    if (tune.sampler == kSampNbhdBs) { TWDIC_ICGN_WARP(NW, kSampNbhdBs); }                        \
    TWDIC_ICGN_WARP(NW, kSampNbhd)
        if (tune.threads == 128) { TWDIC_ICGN_WARP_N(4); }
        if (tune.threads == 256) { TWDIC_ICGN_WARP_N(8); }
        if (tune.threads == 512) { TWDIC_ICGN_WARP_N(16); }
        TWDIC_ICGN_WARP_N(32);
#undef TWDIC_ICGN_WARP_N
#undef TWDIC_ICGN_WARP
    }
    // one POI per CTA: 32 to 256 threads; where the one-POI-per-warp layout was
    // asked for but cannot run (window sampler, oversized image), one-warp CTAs
    IcgnTune t1 = tune;
    if (t1.chunk > 0 && t1.threads > 256) t1.threads = 32;
    if (t1.threads != 32 && t1.threads != 64 && t1.threads != 128 && t1.threads != 256)
        return cudaErrorInvalidValue;
    for (int j = 0; j < J.njobs; ++j)
        if (t1.sampler != kSampWindow && !J.job[j].table) return cudaErrorInvalidValue;
    const bool multi = J.njobs > 1;
#define TWDIC_ICGN_FAST(TH, SA)                                                                  \
    return multi ? launch_icgn_fast_t<TH, SA, true>(J, work, t1.ctas_per_sm, st)               \
                 : launch_icgn_fast_t<TH, SA, false>(J, work, t1.ctas_per_sm, st)
#define TWDIC_ICGN_FAST_T(TH)                                                                    \
    if (t1.sampler == kSampLut) { TWDIC_ICGN_FAST(TH, kSampLut); }                              \
    if (t1.sampler == kSampNbhd) { TWDIC_ICGN_FAST(TH, kSampNbhd); }                            \
    if (t1.sampler == kSampNbhdBs) { TWDIC_ICGN_FAST(TH, kSampNbhdBs); }                        \
    TWDIC_ICGN_FAST(TH, kSampWindow)
    if (t1.threads == 32) { TWDIC_ICGN_FAST_T(32); }
    if (t1.threads == 64) { TWDIC_ICGN_FAST_T(64); }
    if (t1.threads == 256) { TWDIC_ICGN_FAST_T(256); }
    TWDIC_ICGN_FAST_T(128);
#undef TWDIC_ICGN_FAST_T
#undef TWDIC_ICGN_FAST
}

cudaError_t launch_icgn_fast(const Geom& g, const uint8_t* ref, const uint8_t* tar, const int2* poi, int n,
                             const float* stats, const double* chol, const uint8_t* rflag, const void* table,
                             int* work, float* u, float* v, float* p6, int* iters, uint8_t* flags,
                             const IcgnTune& tune, cudaStream_t st, const float2* grad,
                             const float4* samples) {
    if (n <= 0) return cudaSuccess;
    IcgnJobs J;
    J.njobs = 1;
    J.total = n;
    IcgnJob& jb = J.job[0];
    jb.g = g;
    jb.ref = ref;
    jb.tar = tar;
    jb.poi = poi;
    jb.stats = stats;
    jb.hinv = chol;
    jb.rflag = rflag;
    jb.table = table;
    jb.grad = grad;
    jb.samples = samples;
    jb.u = u;
    jb.v = v;
    jb.p6 = p6;
    jb.iters = iters;
    jb.flags = flags;
    jb.n = n;
    jb.begin = 0;
    return launch_icgn_fast_jobs(J, work, tune, st);
}

}  // namespace twdic
