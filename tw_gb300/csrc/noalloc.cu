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

void set_error_message(const char* msg);                                      // capi.cu
int validate_params(const twdic_params* p, bool need_grid, bool need_border);  // capi.cu

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
void* g_scratch_ctx[kMaxDevices] = {};  // the context the address was resolved in

int fail_msg(int code, const char* msg) {
    set_error_message(msg);
    return code;
}

// cuCtxGetCurrent, resolved once through the runtime (no link-time
// dependency on libcuda)
typedef int (*ctx_get_current_t)(void**);
ctx_get_current_t ctx_get_current() {
    static ctx_get_current_t fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<ctx_get_current_t>(f);
    }();
    return fn;
}

// Device address of the scratch array in the current context.  The first
// call on a device (and the first after another context is made current on
// it) resolves it with cudaGetSymbolAddress, which may load the library's
// module there; later calls reuse it.
int scratch_address(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail_msg(TWDIC_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail_msg(TWDIC_ERR_UNSUPPORTED, "device ordinal out of range");
    auto current_ctx = [] {
        void* c = nullptr;
        if (auto fn = ctx_get_current()) fn(&c);
        return c;
    };
    void* ctx = current_ctx();
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev] || g_scratch_ctx[dev] != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_icgn_scratch);
        if (e != cudaSuccess || !p) {
            char buf[256];
            snprintf(buf, sizeof(buf), "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
            return fail_msg(TWDIC_ERR_CUDA, buf);
        }
        g_scratch_ptr[dev] = p;
        g_scratch_ctx[dev] = current_ctx();  // the runtime has made its context current by now
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
    if (!d_ref || !d_tar || !d_poi_yx || !d_u || !d_v || !d_p6 || !d_iters || !d_flags)
        return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL argument (every buffer is required)");
    // the parameter checks of the handle entry points (twdic_icgn_create)
    int rc = validate_params(p, false, true);
    if (rc != TWDIC_OK) return rc;
    if (p->path != TWDIC_PATH_FAST)
        return fail_msg(TWDIC_ERR_UNSUPPORTED, "twdic_icgn_compute_noalloc runs the fast path only (path = 1)");
    if (num_pois <= 0) return fail_msg(TWDIC_ERR_NO_POI, "Number of POIs is below 0!");
    if (num_pois > TWDIC_NOALLOC_MAX_POIS)
        return fail_msg(TWDIC_ERR_UNSUPPORTED,
                        "twdic_icgn_compute_noalloc: num_pois exceeds TWDIC_NOALLOC_MAX_POIS (196608)");
    if (reinterpret_cast<uintptr_t>(d_poi_yx) % 8 != 0)
        return fail_msg(TWDIC_ERR_INVALID_ARG, "POI array must be 8-byte aligned");

    void* scratch = nullptr;
    rc = scratch_address(&scratch);
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
