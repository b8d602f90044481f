// Tracking-loop kernels: the reference-refresh POI update and the
// displacement colour map of TW_Core's FFT-CC worker thread
// (TW/TW_Core/fftcctworkerthread.cpp:228-330, :408-438; kernels at
// TW/TW_Core/cuda_utils.cu:109-240).
#include <algorithm>

#include "dic_common.cuh"
#include "dic_kernels.h"

namespace twdic {

namespace {

// At a reference refresh: the accumulated displacement takes the last
// frame's (accumulateUV), and every POI moves by the truncated displacement
// (updatePOIpos: y += int(v), x += int(u)).  A POI is held inside
// [lo, hi] so that its subset stays in the ROI (the reference then reads
// outside the image).
__global__ void k_track_update(int2* __restrict__ poi, const float* __restrict__ u, const float* __restrict__ v,
                               float* __restrict__ acc_u, float* __restrict__ acc_v, int n, int lo_y, int hi_y,
                               int lo_x, int hi_x) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x) {
        acc_u[i] += u[i];
        acc_v[i] += v[i];
        int2 p = poi[i];
        p.x = min(max(p.x + (int)v[i], lo_y), hi_y);
        p.y = min(max(p.y + (int)u[i], lo_x), hi_x);
        poi[i] = p;
    }
}

// Jet colour map of 256 entries as RGBA bytes (R lowest): with
// a(k) = round(255 k / 64), k = 0..64, the blue channel rises from a(33)
// over the first 32 entries, then green rises, red rises while blue falls,
// green falls, and red falls to a(32) at the last entry.
__device__ __forceinline__ uint32_t jet256(int i) {
    auto a = [](int k) { return (uint32_t)((255 * k + 32) / 64); };
    uint32_t r, g, b;
    if (i < 32) {
        r = 0; g = 0; b = a(i + 33);
    } else if (i < 96) {
        r = 0; g = a(i - 31); b = 255;
    } else if (i < 160) {
        r = a(i - 95); g = 255; b = a(159 - i);
    } else if (i < 224) {
        r = 255; g = a(223 - i); b = 0;
    } else {
        r = a(287 - i); g = 0; b = 0;
    }
    return 0xFF000000u | (b << 16) | (g << 8) | r;
}

__device__ __forceinline__ uint32_t jet_of(float t, float lo, float hi) {
    t = t > hi ? hi : t;
    t = t < lo ? lo : t;
    t = t - lo;
    int k = (int)(255.f * t / (hi - lo));
    k = k < 0 ? 0 : (k > 255 ? 255 : k);
    return jet256(k);
}

// constructTextImageFixedMinMax with the display positions of
// accumulatePOI: POI i is drawn at poi + (int(v), int(u)) as a 3x3 block
// of the colour of its total displacement (acc + current, clamped to
// [min, max]) in two ROI-sized RGBA images.  Pixels outside the ROI are
// skipped (the reference writes outside its buffers there).
__global__ void k_colormap(uint32_t* __restrict__ tex_u, uint32_t* __restrict__ tex_v,
                           const int2* __restrict__ poi, const float* __restrict__ u, const float* __restrict__ v,
                           const float* __restrict__ acc_u, const float* __restrict__ acc_v, int n, int sx, int sy,
                           int rw, int rh, float min_u, float max_u, float min_v, float max_v) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x) {
        const uint32_t cu = jet_of(u[i] + acc_u[i], min_u, max_u);
        const uint32_t cv = jet_of(v[i] + acc_v[i], min_v, max_v);
        const int y = poi[i].x + (int)v[i] - sy, x = poi[i].y + (int)u[i] - sx;
        for (int dy = -1; dy <= 1; ++dy) {
            const int yy = y + dy;
            if (yy < 0 || yy >= rh) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                const int xx = x + dx;
                if (xx < 0 || xx >= rw) continue;
                tex_u[(size_t)yy * rw + xx] = cu;
                tex_v[(size_t)yy * rw + xx] = cv;
            }
        }
    }
}

// Device POIs of the IC-GN handle: copied into the handle's array, read as
// 32-bit words (the caller's array need only be 4-byte aligned); *changed is
// set when any pair differs from the array's previous contents, for which
// the per-reference precompute was made.
__global__ void k_poi_refresh(const int32_t* __restrict__ src, int2* __restrict__ dst, int n, int* changed) {
    int diff = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += blockDim.x * gridDim.x) {
        const int2 a = make_int2(src[2 * i], src[2 * i + 1]);
        const int2 b = dst[i];
        if (a.x != b.x || a.y != b.y) {
            dst[i] = a;
            diff = 1;
        }
    }
    if (__syncthreads_or(diff) && threadIdx.x == 0) atomicOr(changed, 1);
}

}  // namespace

cudaError_t launch_track_update(int2* poi, const float* u, const float* v, float* acc_u, float* acc_v, int n,
                                int lo_y, int hi_y, int lo_x, int hi_x, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int grid = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    k_track_update<<<grid, 256, 0, st>>>(poi, u, v, acc_u, acc_v, n, lo_y, hi_y, lo_x, hi_x);
    return cudaGetLastError();
}

cudaError_t launch_colormap(uint32_t* tex_u, uint32_t* tex_v, const int2* poi, const float* u, const float* v,
                            const float* acc_u, const float* acc_v, int n, const Geom& g, float min_u, float max_u,
                            float min_v, float max_v, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int grid = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    k_colormap<<<grid, 256, 0, st>>>(tex_u, tex_v, poi, u, v, acc_u, acc_v, n, g.sx, g.sy, g.rw, g.rh, min_u, max_u,
                                     min_v, max_v);
    return cudaGetLastError();
}

cudaError_t launch_poi_refresh(const int32_t* src, int2* dst, int n, int* changed, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int grid = std::min((n + 255) / 256, 1024);
    k_poi_refresh<<<grid, 256, 0, st>>>(src, dst, n, changed);
    return cudaGetLastError();
}

}  // namespace twdic
