// IC-GN entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the point where they need sub-pixel
// registration: a real-time camera loop (like the reference's capture ->
// FFT-CC -> IC-GN worker threads) whose frame deadline cannot absorb an
// allocation's implicit device-wide synchronisation or an out-of-memory
// failure in the middle of a stream, and applications whose device memory is
// fully budgeted up front by another framework or allocator.  For them this
// file runs the fast IC-GN path (per-reference precompute + persistent IC-GN
// kernel) with its scratch -- the per-POI reference cache and the work
// counter -- in one file-scope __device__ array of fixed size instead of
// handle-owned cudaMalloc buffers.  Every GPU that loads the library holds
// that array until the process exits.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "dic_common.cuh"
#include "dic_kernels.h"
#include "../../include/tw_dic.h"

namespace twdic {

void set_error_message(const char* msg);  // capi.cu

namespace {

constexpr size_t kAlign = 256;
constexpr size_t round_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

// Scratch carving, per POI: 16 floats of reference statistics (64 B), the
// packed FP64 inverse Hessian (21 doubles, 168 B) and a flag byte; then one
// work counter.
constexpr size_t kStatsOff = 0;
constexpr size_t kCholOff = kStatsOff + round_up(size_t(TWDIC_NOALLOC_MAX_POIS) * 64);
constexpr size_t kFlagOff = kCholOff + round_up(size_t(TWDIC_NOALLOC_MAX_POIS) * 168);
constexpr size_t kWorkOff = kFlagOff + round_up(size_t(TWDIC_NOALLOC_MAX_POIS));
constexpr size_t kScratchBytes = kWorkOff + kAlign;

static __device__ __align__(256) unsigned char g_icgn_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_ptr[kMaxDevices] = {};

int fail_msg(int code, const char* msg) {
    set_error_message(msg);
    return code;
}

// Device address of the scratch array on the current device.  The first call
// per device resolves it with cudaGetSymbolAddress (which may load the
// module on that device); later calls reuse the cached address.
int scratch_address(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_msg(TWDIC_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail_msg(TWDIC_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_icgn_scratch);
        if (e != cudaSuccess || !p) {
            char buf[256];
            snprintf(buf, sizeof(buf), "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
            return fail_msg(TWDIC_ERR_CUDA, buf);
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return TWDIC_OK;
}

}  // namespace
}  // namespace twdic

extern "C" TWDIC_API int twdic_icgn_compute_noalloc(const twdic_params* p, const uint8_t* d_ref,
                                                    const uint8_t* d_tar, const int32_t* d_poi_yx,
                                                    int32_t num_pois, float* d_u, float* d_v, float* d_p6,
                                                    int32_t* d_iters, uint8_t* d_flags, void* stream) {
    using namespace twdic;
    if (!p || !d_ref || !d_tar || !d_poi_yx || !d_u || !d_v || !d_p6 || !d_iters || !d_flags)
        return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL argument (every buffer is required)");
    if (num_pois <= 0) return fail_msg(TWDIC_ERR_NO_POI, "Number of POIs is below 0!");
    if (num_pois > TWDIC_NOALLOC_MAX_POIS)
        return fail_msg(TWDIC_ERR_UNSUPPORTED,
                        "twdic_icgn_compute_noalloc: num_pois exceeds TWDIC_NOALLOC_MAX_POIS (196608)");
    if (reinterpret_cast<uintptr_t>(d_poi_yx) % 8 != 0)
        return fail_msg(TWDIC_ERR_INVALID_ARG, "POI array must be 8-byte aligned");
    if (p->img_width <= 0 || p->img_height <= 0 || p->roi_width <= 0 || p->roi_height <= 0)
        return fail_msg(TWDIC_ERR_INVALID_ARG, "image and ROI sizes must be positive");
    if (p->subset_x < 1 || p->subset_y < 1) return fail_msg(TWDIC_ERR_INVALID_ARG, "subset half size must be >= 1");
    if (p->subset_x > 31 || p->subset_y > 31) return fail_msg(TWDIC_ERR_UNSUPPORTED, "subset half size exceeds 31");
    if (p->max_iterations < 1 || !(p->delta_p >= 0.f))
        return fail_msg(TWDIC_ERR_INVALID_ARG, "max_iterations must be >= 1 and delta_p >= 0");
    if (p->start_x < 1 || p->start_y < 1 || p->start_x + p->roi_width + 1 > p->img_width ||
        p->start_y + p->roi_height + 1 > p->img_height)
        return fail_msg(TWDIC_ERR_BORDER, "Not enough boundary pixels for gradients!");

    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc != TWDIC_OK) return rc;
    unsigned char* base = static_cast<unsigned char*>(scratch);
    float* stats = reinterpret_cast<float*>(base + kStatsOff);
    double* chol = reinterpret_cast<double*>(base + kCholOff);
    uint8_t* rflag = base + kFlagOff;
    int* work = reinterpret_cast<int*>(base + kWorkOff);

    Geom g;
    g.img_w = p->img_width; g.img_h = p->img_height; g.pitch = p->img_width;
    g.sx = p->start_x; g.sy = p->start_y; g.rw = p->roi_width; g.rh = p->roi_height;
    g.rx = p->subset_x; g.ry = p->subset_y;
    g.max_iter = p->max_iterations; g.delta_p = p->delta_p;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int2* poi = reinterpret_cast<const int2*>(d_poi_yx);

    // The reference cache is rewritten for every POI by the precompute kernel
    // before the IC-GN kernel reads it; the work counter is zeroed by the
    // launcher (cudaMemsetAsync) on every call.
    cudaError_t e = launch_ref_precompute_fast(g, d_ref, poi, num_pois, stats, chol, rflag, st);
    if (e == cudaSuccess) {
        IcgnTune tune;  // 128 threads, staged window (no per-frame LUT buffer)
        e = launch_icgn_fast(g, d_ref, d_tar, poi, num_pois, stats, chol, rflag, nullptr, work, d_u, d_v, d_p6,
                             d_iters, d_flags, tune, st);
    }
    if (e != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf), "twdic_icgn_compute_noalloc launch failed: %s", cudaGetErrorString(e));
        return fail_msg(TWDIC_ERR_CUDA, buf);
    }
    return TWDIC_OK;
}
