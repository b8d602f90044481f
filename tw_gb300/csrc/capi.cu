// C ABI of the GB300 DIC hot path (declared in include/tw_dic.h).
//
// Host orchestration in C++: parameter validation with the reference's error
// conditions turned into status codes, device buffers owned by the handles,
// host<->device staging on the handle's stream, and the per-reference cache.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "dic_common.cuh"
#include "dic_kernels.h"
#include "../../include/tw_dic.h"

namespace twdic {
namespace {

thread_local std::string g_last_error = "no error";

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

bool valid_icgn_threads(int t) { return t == 32 || t == 64 || t == 128 || t == 256 || t == 512 || t == 1024; }

#define TW_CUDA(call)                                                                                   \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            return fail(e_ == cudaErrorMemoryAllocation ? TWDIC_ERR_NO_MEMORY : TWDIC_ERR_CUDA,         \
                        "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);    \
    } while (0)

#define TW_TRY(expr)                 \
    do {                             \
        int r_ = (expr);             \
        if (r_ != TWDIC_OK) return r_; \
    } while (0)

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    int ensure(size_t b) {
        if (b <= bytes && p) return TWDIC_OK;
        release();
        if (b == 0) return TWDIC_OK;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && b + (size_t(256) << 20) > free_b)
            return fail(TWDIC_ERR_NO_MEMORY, "device budget: %zu bytes requested, %zu free", b, free_b);
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(TWDIC_ERR_NO_MEMORY, "cudaMalloc(%zu) failed: %s", b, cudaGetErrorString(e));
        }
        bytes = b;
        return TWDIC_OK;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

int num_pois_of(const twdic_params& p, int* nx, int* ny) {
    // Fftcc2D::recomputeNumPOI (TW_paDIC_FFTCC2D.cpp:88-94)
    *nx = int(std::floor((p.roi_width - p.subset_x * 2 - p.margin_x * 2) / float(p.grid_space_x))) + 1;
    *ny = int(std::floor((p.roi_height - p.subset_y * 2 - p.margin_y * 2) / float(p.grid_space_y))) + 1;
    return (*nx > 0 && *ny > 0) ? TWDIC_OK : fail(TWDIC_ERR_NO_POI, "Number of POIs is below 0!");
}

int validate(const twdic_params* p, bool need_grid, bool need_border) {
    if (!p) return fail(TWDIC_ERR_INVALID_ARG, "params is NULL");
    if (p->img_width <= 0 || p->img_height <= 0) return fail(TWDIC_ERR_INVALID_ARG, "image size must be positive");
    if (p->roi_width <= 0 || p->roi_height <= 0) return fail(TWDIC_ERR_INVALID_ARG, "ROI size must be positive");
    if (p->start_x < 0 || p->start_y < 0 || p->start_x + p->roi_width > p->img_width ||
        p->start_y + p->roi_height > p->img_height)
        return fail(TWDIC_ERR_INVALID_ARG, "ROI lies outside the image");
    if (p->subset_x < 1 || p->subset_y < 1) return fail(TWDIC_ERR_INVALID_ARG, "subset half size must be >= 1");
    if (p->subset_x > 31 || p->subset_y > 31)
        return fail(TWDIC_ERR_UNSUPPORTED, "subset half size %d x %d exceeds 31", p->subset_x, p->subset_y);
    if (p->path != TWDIC_PATH_PLAIN && p->path != TWDIC_PATH_FAST)
        return fail(TWDIC_ERR_INVALID_ARG, "unknown path %d", p->path);
    if (need_grid) {
        if (p->grid_space_x < 1 || p->grid_space_y < 1) return fail(TWDIC_ERR_INVALID_ARG, "grid space must be >= 1");
        if (p->margin_x < 0 || p->margin_y < 0) return fail(TWDIC_ERR_INVALID_ARG, "margin must be >= 0");
    }
    if (need_border) {
        if (p->max_iterations < 1) return fail(TWDIC_ERR_INVALID_ARG, "max_iterations must be >= 1");
        if (!(p->delta_p >= 0.f)) return fail(TWDIC_ERR_INVALID_ARG, "delta_p must be >= 0");
        // GradientXY_2Images / BicubicCoefficients (TW_utils.cpp:254-257, :615-619)
        if (p->start_x < 1 || p->start_y < 1 || p->start_x + p->roi_width + 1 > p->img_width ||
            p->start_y + p->roi_height + 1 > p->img_height)
            return fail(TWDIC_ERR_BORDER, "Not enough boundary pixels for gradients!");
    }
    return TWDIC_OK;
}

Geom make_geom(const twdic_params& p) {
    Geom g;
    g.img_w = p.img_width; g.img_h = p.img_height;
    // engine-owned image rows are padded to 16 bytes: the tensor-memory-access
    // (TMA) loads of the tensor-core FFT-CC need 16-byte-multiple row strides
    g.pitch = (p.img_width + 15) & ~15;
    g.sx = p.start_x; g.sy = p.start_y; g.rw = p.roi_width; g.rh = p.roi_height;
    g.rx = p.subset_x; g.ry = p.subset_y;
    g.max_iter = p.max_iterations; g.delta_p = p.delta_p;
    g.grid_x = p.grid_space_x;
    return g;
}

void grid_positions(const twdic_params& p, int nx, int ny, int32_t* yx) {
    // ComputePOIPositions_s (TW_utils.cpp:29-49)
    for (int i = 0; i < ny; ++i)
        for (int j = 0; j < nx; ++j) {
            yx[2 * ((size_t)i * nx + j) + 0] = p.start_y + p.margin_y + p.subset_y + i * p.grid_space_y;
            yx[2 * ((size_t)i * nx + j) + 1] = p.start_x + p.margin_x + p.subset_x + j * p.grid_space_x;
        }
}

// -------------------------------------------------------------- Engine ----
struct Engine {
    twdic_params prm{};
    Geom g{};
    int n = 0;  // POIs of the handle
    int nx = 0, ny = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    bool have_ref = false, have_tar = false;
    IcgnTune icgn_tune;
    FftccTune fftcc_tune;
    int interp = TWDIC_INTERP_BICUBIC;  // target interpolation of IC-GN (ICGN2DInterpolationFLag)
    // batched calls: 1 = no FFT-CC, IC-GN starts from the u, v arrays passed in
    // (the last frame's displacements); 0 = FFT-CC then IC-GN
    int guess = 0;

    DevBuf d_ref, d_tar, d_poi;
    DevBuf d_u, d_v, d_zncc, d_fst, d_p6, d_iters, d_flags, d_err, d_work, d_tw;
    // per-reference cache
    bool cache_valid = false;
    std::vector<int32_t> cache_poi_host;
    DevBuf c_subR, c_sd, c_chol, c_norm, c_flag;  // plain
    DevBuf c_stat, c_chol64, c_flag64, c_grad, c_samp;  // fast
    DevBuf d_lut;
    // TMA descriptors of d_ref / d_tar for the tensor-core FFT-CC: a pinned
    // host copy and the device copy the kernels read, re-encoded when the
    // launch shape changes
    DevBuf d_tcmaps;
    void* h_tcmaps = nullptr;
    TcMapInfo tcmaps{0, 0, 0};
    // per-reference cache of the tensor-core FFT-CC: the reference windows'
    // spectra and integer sums at the POIs (dropped with the IC-GN cache)
    DevBuf c_fspec, c_fsum;
    bool fspec_valid = false;
    cudaEvent_t ev[7] = {};
    cudaEvent_t ev_sync = nullptr;  // orders this handle's stream with a batch stream
    float last_times[6] = {0, 0, 0, 0, 0, 0};
    bool times_pending = false;

    ~Engine() {
        if (h_tcmaps) cudaFreeHost(h_tcmaps);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (ev_sync) cudaEventDestroy(ev_sync);
        if (own_stream) cudaStreamDestroy(own_stream);
    }

    int init(const twdic_params& p, int num_pois) {
        prm = p;
        // fastest measured IC-GN shape on GB300 at 41x41 subsets: one warp
        // per POI, one 32-warp CTA per SM walking runs of 32 consecutive
        // POIs, gathering the per-frame 4x4 neighbourhood table (16 B per ROI
        // pixel) through L1 (the autotuner may change it)
        icgn_tune.threads = 1024;
        icgn_tune.chunk = 32;
        icgn_tune.sampler = kSampNbhd;
        g = make_geom(p);
        n = num_pois;
        TW_CUDA(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking));
        stream = own_stream;
        for (auto& e : ev) TW_CUDA(cudaEventCreate(&e));
        TW_CUDA(cudaEventCreateWithFlags(&ev_sync, cudaEventDisableTiming));
        // 16 spare bytes: the FFT-CC kernel reads whole aligned 32-bit words
        // around a window's last byte
        const size_t img = (size_t)g.pitch * p.img_height + 16;
        TW_TRY(d_ref.ensure(img));
        TW_TRY(d_tar.ensure(img));
        TW_TRY(d_poi.ensure(sizeof(int2) * (size_t)n));
        TW_TRY(d_u.ensure(sizeof(float) * (size_t)n));
        TW_TRY(d_v.ensure(sizeof(float) * (size_t)n));
        TW_TRY(d_zncc.ensure(sizeof(float) * (size_t)n));
        TW_TRY(d_fst.ensure((size_t)n));
        TW_TRY(d_p6.ensure(sizeof(float) * 6 * (size_t)n));
        TW_TRY(d_iters.ensure(sizeof(int) * (size_t)n));
        TW_TRY(d_flags.ensure((size_t)n));
        TW_TRY(d_err.ensure(sizeof(unsigned)));
        TW_TRY(d_work.ensure(sizeof(int) * 4));
        TW_TRY(d_tcmaps.ensure(kTcMapsBytes));
        TW_CUDA(cudaMallocHost(&h_tcmaps, kTcMapsBytes));
        TW_CUDA(cudaMemsetAsync(d_err.p, 0, sizeof(unsigned), stream));
        // DFT twiddles exp(-2 pi i k / N) of the two window sizes, rounded once
        // from double (the FP32 SIMT FFT-CC kernel reads them)
        std::vector<float> tw(4 * 64, 0.f);
        const double two_pi = 6.283185307179586476925286766559;
        for (int t = 0; t < 2; ++t) {
            const int N = 2 * (t == 0 ? p.subset_x : p.subset_y);
            for (int k = 0; k < N; ++k) {
                tw[t * 128 + 2 * k] = (float)std::cos(-two_pi * k / N);
                tw[t * 128 + 2 * k + 1] = (float)std::sin(-two_pi * k / N);
            }
        }
        TW_TRY(d_tw.ensure(tw.size() * sizeof(float)));
        TW_CUDA(cudaMemcpyAsync(d_tw.p, tw.data(), tw.size() * sizeof(float), cudaMemcpyHostToDevice, stream));
        TW_CUDA(cudaStreamSynchronize(stream));
        return TWDIC_OK;
    }

    int upload_image(DevBuf& dst, const uint8_t* img, int32_t stride, int mem) {
        if (!img) return fail(TWDIC_ERR_INVALID_ARG, "image pointer is NULL");
        if (stride == 0) stride = prm.img_width;
        if (stride < prm.img_width) return fail(TWDIC_ERR_INVALID_ARG, "stride %d < width %d", stride, prm.img_width);
        if (mem != TWDIC_MEM_HOST && mem != TWDIC_MEM_DEVICE) return fail(TWDIC_ERR_INVALID_ARG, "bad mem kind");
        TW_CUDA(cudaMemcpy2DAsync(dst.p, g.pitch, img, stride, prm.img_width, prm.img_height,
                                  mem == TWDIC_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, stream));
        return TWDIC_OK;
    }

    int set_ref(const uint8_t* img, int32_t stride, int mem) {
        TW_TRY(upload_image(d_ref, img, stride, mem));
        have_ref = true;
        cache_valid = false;
        fspec_valid = false;
        return TWDIC_OK;
    }

    int set_tar(const uint8_t* img, int32_t stride, int mem) {
        TW_TRY(upload_image(d_tar, img, stride, mem));
        have_tar = true;
        return TWDIC_OK;
    }

    int check_err() {
        unsigned h = 0;
        TW_CUDA(cudaMemcpyAsync(&h, d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
        TW_CUDA(cudaStreamSynchronize(stream));
        if (h & kErrTimeout) {
            cudaMemsetAsync(d_err.p, 0, sizeof(unsigned), stream);
            return fail(TWDIC_ERR_TIMEOUT, "a bounded device-side wait gave up");
        }
        return TWDIC_OK;
    }

    // TMA descriptors of the images for a tensor-core FFT-CC launch of this
    // shape: encoded and copied on this handle's stream when the shape
    // changed (after the previous copy has read the host descriptors).
    int ensure_tc_maps(const FftccTune& tune) {
        const uint64_t key = fftcc_tc_maps_key(g, tune);
        if (key != 0 && key == tcmaps.key) return TWDIC_OK;
        if (tcmaps.key != 0) TW_CUDA(cudaStreamSynchronize(stream));
        tcmaps.key = 0;
        if (!fftcc_tc_encode_maps(g, d_ref.as<uint8_t>(), d_tar.as<uint8_t>(), tune, h_tcmaps, &tcmaps))
            return fail(TWDIC_ERR_UNSUPPORTED, "tensor-core FFT-CC: tensor maps could not be encoded");
        TW_CUDA(cudaMemcpyAsync(d_tcmaps.p, h_tcmaps, kTcMapsBytes, cudaMemcpyHostToDevice, stream));
        return TWDIC_OK;
    }

    // The reference spectra of the tensor-core FFT-CC: once per reference
    // (and POI set), by the per-reference pass, on this handle's stream.
    int ensure_fspec(const FftccTune& tune) {
        if (fspec_valid) return TWDIC_OK;
        if (!have_ref) return fail(TWDIC_ERR_STATE, "FFT-CC needs a reference image");
        TW_TRY(c_fspec.ensure(fftcc_tc_spectrum_bytes(g, n)));
        TW_TRY(c_fsum.ensure(sizeof(int2) * (size_t)n));
        TW_TRY(ensure_tc_maps(tune));
        TW_CUDA(launch_fftcc_tc(g, d_ref.as<uint8_t>(), d_tar.as<uint8_t>(), d_tcmaps.p, tcmaps.key, tcmaps.uw,
                                tcmaps.utoff, c_fspec.as<uint32_t>(), c_fsum.as<int2>(), d_poi.as<int2>(), n, nullptr,
                                nullptr, nullptr, nullptr, d_err.as<unsigned>(), d_work.as<int>() + 1, tune, stream,
                                true));
        fspec_valid = true;
        return TWDIC_OK;
    }

    // FFT-CC of all POIs into device arrays.
    int fftcc(float* u, float* v, float* z, uint8_t* st) {
        if (!have_ref || !have_tar) return fail(TWDIC_ERR_STATE, "FFT-CC needs a reference and a target image");
        const int2* poi = d_poi.as<int2>();
        if (prm.path == TWDIC_PATH_FAST && fftcc_tune.use_tc && fftcc_tc_supported(g)) {
            TW_TRY(ensure_fspec(fftcc_tune));
            TW_TRY(ensure_tc_maps(fftcc_tune));
            TW_CUDA(launch_fftcc_tc(g, d_ref.as<uint8_t>(), d_tar.as<uint8_t>(), d_tcmaps.p, tcmaps.key, tcmaps.uw,
                                    tcmaps.utoff, c_fspec.as<uint32_t>(), c_fsum.as<int2>(), poi, n, u, v, z, st,
                                    d_err.as<unsigned>(), d_work.as<int>() + 1, fftcc_tune, stream));
        } else {
            TW_CUDA(launch_fftcc_plain(g, d_ref.as<uint8_t>(), d_tar.as<uint8_t>(), poi, n, d_tw.as<float2>(), u, v, z,
                                       st, stream));
        }
        return TWDIC_OK;
    }

    int ensure_cache(float* t_pre) {
        if (cache_valid) return TWDIC_OK;
        const int S = (2 * g.rx + 1) * (2 * g.ry + 1);
        if (prm.path == TWDIC_PATH_PLAIN) {
            TW_TRY(c_subR.ensure(sizeof(float) * (size_t)n * S));
            TW_TRY(c_sd.ensure(sizeof(float2) * 3 * (size_t)n * S));
            TW_TRY(c_chol.ensure(sizeof(float) * 36 * (size_t)n));
            TW_TRY(c_norm.ensure(sizeof(float) * (size_t)n));
            TW_TRY(c_flag.ensure((size_t)n));
            TW_CUDA(launch_ref_precompute_plain(g, d_ref.as<uint8_t>(), d_poi.as<int2>(), n, c_subR.as<float>(),
                                                c_sd.as<float2>(), c_chol.as<float>(), c_norm.as<float>(),
                                                c_flag.as<uint8_t>(), stream));
        } else {
            TW_TRY(c_stat.ensure(sizeof(float) * 16 * (size_t)n));
            TW_TRY(c_chol64.ensure(sizeof(double) * 21 * (size_t)n));
            TW_TRY(c_flag64.ensure((size_t)n));
            TW_CUDA(launch_ref_precompute_fast(g, d_ref.as<uint8_t>(), d_poi.as<int2>(), n, c_stat.as<float>(),
                                               c_chol64.as<double>(), c_flag64.as<uint8_t>(), stream));
            TW_TRY(c_grad.ensure(sizeof(float2) * (size_t)g.rw * g.rh));
            TW_CUDA(launch_ref_grad(g, d_ref.as<uint8_t>(), c_grad.as<float2>(), stream));
            TW_TRY(c_samp.ensure(sizeof(float4) * (size_t)S));
            TW_CUDA(launch_sample_table(g.rx, g.ry, c_samp.as<float4>(), stream));
        }
        cache_valid = true;
        if (t_pre) *t_pre = 1.f;
        return TWDIC_OK;
    }

    // IC-GN of all POIs; u, v in/out device arrays.
    int icgn(float* u, float* v, float* p6, int* iters, uint8_t* flags) {
        TW_TRY(prepare_target());
        return icgn_solve(u, v, p6, iters, flags);
    }

    // Per-target preparation: the table the IC-GN variant reads, the bicubic
    // (TW_utils.cpp:604-700) or B-spline (TW_utils.cpp:521-602) coefficient
    // LUT of the target or its 4x4 neighbourhood table.
    int prepare_target() {
        if (!have_ref || !have_tar) return fail(TWDIC_ERR_STATE, "IC-GN needs a reference and a target image");
        if (interp == TWDIC_INTERP_BSPLINE && prm.path == TWDIC_PATH_FAST && solve_tune().sampler == kSampNbhdBs) {
            TW_TRY(d_lut.ensure(sizeof(uint4) * (size_t)g.rw * g.rh));
            TW_CUDA(launch_nbhd_table(g, d_tar.as<uint8_t>(), d_lut.as<uint4>(), stream, true));
        } else if (interp == TWDIC_INTERP_BSPLINE) {
            TW_TRY(d_lut.ensure(sizeof(float4) * 4 * (size_t)g.rw * g.rh));
            TW_CUDA(launch_bspline_lut(g, d_tar.as<uint8_t>(), d_lut.as<float4>(), stream));
        } else if (prm.path == TWDIC_PATH_PLAIN || icgn_tune.sampler == kSampLut) {
            TW_TRY(d_lut.ensure(sizeof(float4) * 4 * (size_t)g.rw * g.rh));
            TW_CUDA(launch_bicubic_lut(g, d_tar.as<uint8_t>(), d_lut.as<float4>(), stream));
        } else if (icgn_tune.sampler == kSampNbhd) {
            TW_TRY(d_lut.ensure(sizeof(uint4) * (size_t)g.rw * g.rh));
            TW_CUDA(launch_nbhd_table(g, d_tar.as<uint8_t>(), d_lut.as<uint4>(), stream));
        }
        return TWDIC_OK;
    }

    // the fast IC-GN launch shape; B-spline from the neighbourhood table
    // (kSampNbhdBs) or from its coefficient LUT (the window sampler is
    // Catmull-Rom only)
    IcgnTune solve_tune() const {
        IcgnTune t = icgn_tune;
        if (interp == TWDIC_INTERP_BSPLINE) t.sampler = t.sampler == kSampNbhd ? kSampNbhdBs : kSampLut;
        return t;
    }

    int icgn_solve(float* u, float* v, float* p6, int* iters, uint8_t* flags) {
        if (!have_ref || !have_tar) return fail(TWDIC_ERR_STATE, "IC-GN needs a reference and a target image");
        TW_TRY(ensure_cache(nullptr));
        const int2* poi = d_poi.as<int2>();
        if (prm.path == TWDIC_PATH_PLAIN) {
            TW_CUDA(launch_icgn_plain(g, d_tar.as<uint8_t>(), poi, n, c_subR.as<float>(), c_sd.as<float2>(),
                                      c_chol.as<float>(), c_norm.as<float>(), c_flag.as<uint8_t>(),
                                      d_lut.as<float4>(), u, v, p6, iters, flags, stream));
        } else {
            TW_CUDA(launch_icgn_fast(g, d_ref.as<uint8_t>(), d_tar.as<uint8_t>(), poi, n, c_stat.as<float>(),
                                     c_chol64.as<double>(), c_flag64.as<uint8_t>(), d_lut.p,
                                     d_work.as<int>(), u, v, p6, iters, flags, solve_tune(), stream,
                                     c_grad.as<float2>(), c_samp.as<float4>()));
        }
        return TWDIC_OK;
    }
};

int copy_in(void* dst, const void* src, size_t bytes, int mem, cudaStream_t st) {
    if (!src || bytes == 0) return TWDIC_OK;
    TW_CUDA(cudaMemcpyAsync(dst, src, bytes, mem == TWDIC_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                            st));
    return TWDIC_OK;
}
int copy_out(void* dst, const void* src, size_t bytes, int mem, cudaStream_t st) {
    if (!dst || bytes == 0) return TWDIC_OK;
    TW_CUDA(cudaMemcpyAsync(dst, src, bytes, mem == TWDIC_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                            st));
    return TWDIC_OK;
}
int check_mem(int mem) {
    return (mem == TWDIC_MEM_HOST || mem == TWDIC_MEM_DEVICE) ? TWDIC_OK
                                                               : fail(TWDIC_ERR_INVALID_ARG, "bad mem kind %d", mem);
}

}  // namespace

// Error message setter for entry points defined in other translation units.
void set_error_message(const char* msg) { g_last_error = msg; }
int validate_params(const twdic_params* p, bool need_grid, bool need_border) {
    return validate(p, need_grid, need_border);
}

}  // namespace twdic

using namespace twdic;

struct twdic_fftcc { Engine e; };
struct twdic_icgn { Engine e; };
struct twdic_frame { Engine e; };

extern "C" {

const char* twdic_last_error(void) { return g_last_error.c_str(); }
int twdic_abi_version(void) { return TWDIC_ABI_VERSION; }

int twdic_num_pois(const twdic_params* p, int32_t* num_x, int32_t* num_y) {
    TW_TRY(validate(p, true, false));
    if (!num_x || !num_y) return fail(TWDIC_ERR_INVALID_ARG, "NULL output");
    int nx, ny;
    TW_TRY(num_pois_of(*p, &nx, &ny));
    *num_x = nx;
    *num_y = ny;
    return TWDIC_OK;
}

int twdic_poi_positions(const twdic_params* p, int32_t* poi_yx) {
    int32_t nx, ny;
    TW_TRY(twdic_num_pois(p, &nx, &ny));
    if (!poi_yx) return fail(TWDIC_ERR_INVALID_ARG, "NULL output");
    grid_positions(*p, nx, ny, poi_yx);
    return TWDIC_OK;
}

static int engine_grid_init(Engine& e, const twdic_params* p, bool border) {
    TW_TRY(validate(p, true, border));
    int nx, ny;
    TW_TRY(num_pois_of(*p, &nx, &ny));
    if ((size_t)nx * ny > (size_t)1 << 30) return fail(TWDIC_ERR_UNSUPPORTED, "too many POIs");
    e.nx = nx;
    e.ny = ny;
    TW_TRY(e.init(*p, nx * ny));
    std::vector<int32_t> yx(2 * (size_t)nx * ny);
    grid_positions(*p, nx, ny, yx.data());
    TW_CUDA(cudaMemcpyAsync(e.d_poi.p, yx.data(), yx.size() * 4, cudaMemcpyHostToDevice, e.stream));
    TW_CUDA(cudaStreamSynchronize(e.stream));
    return TWDIC_OK;
}

// ------------------------------------------------------------ FFT-CC ABI --
int twdic_fftcc_create(const twdic_params* p, twdic_fftcc** out) {
    if (!out) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle output");
    *out = nullptr;
    auto* h = new (std::nothrow) twdic_fftcc;
    if (!h) return fail(TWDIC_ERR_NO_MEMORY, "host allocation failed");
    int r = engine_grid_init(h->e, p, false);
    if (r != TWDIC_OK) { delete h; return r; }
    *out = h;
    return TWDIC_OK;
}
int twdic_fftcc_num_pois(const twdic_fftcc* h, int32_t* num_x, int32_t* num_y) {
    if (!h || !num_x || !num_y) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    *num_x = h->e.nx;
    *num_y = h->e.ny;
    return TWDIC_OK;
}
int twdic_fftcc_poi_positions(const twdic_fftcc* h, int32_t* poi_yx, int mem) {
    if (!h || !poi_yx) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    TW_TRY(check_mem(mem));
    TW_TRY(copy_out(poi_yx, h->e.d_poi.p, sizeof(int2) * (size_t)h->e.n, mem, h->e.stream));
    TW_CUDA(cudaStreamSynchronize(h->e.stream));
    return TWDIC_OK;
}
int twdic_fftcc_reset_ref(twdic_fftcc* h, const uint8_t* img, int32_t stride, int mem) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    return h->e.set_ref(img, stride, mem);
}
int twdic_fftcc_set_tar(twdic_fftcc* h, const uint8_t* img, int32_t stride, int mem) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    return h->e.set_tar(img, stride, mem);
}
int twdic_fftcc_compute(twdic_fftcc* h, float* u, float* v, float* zncc, uint8_t* status, int mem) {
    if (!h || !u || !v || !zncc) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    TW_TRY(check_mem(mem));
    Engine& e = h->e;
    const size_t fb = sizeof(float) * (size_t)e.n;
    float *du = u, *dv = v, *dz = zncc;
    uint8_t* ds = (mem == TWDIC_MEM_DEVICE && status) ? status : e.d_fst.as<uint8_t>();
    if (mem == TWDIC_MEM_HOST) {
        // dark subsets leave their outputs untouched: stage the caller's values
        du = e.d_u.as<float>(); dv = e.d_v.as<float>(); dz = e.d_zncc.as<float>();
        TW_TRY(copy_in(du, u, fb, mem, e.stream));
        TW_TRY(copy_in(dv, v, fb, mem, e.stream));
        TW_TRY(copy_in(dz, zncc, fb, mem, e.stream));
    }
    TW_TRY(e.fftcc(du, dv, dz, ds));
    if (mem == TWDIC_MEM_HOST) {
        TW_TRY(copy_out(u, du, fb, mem, e.stream));
        TW_TRY(copy_out(v, dv, fb, mem, e.stream));
        TW_TRY(copy_out(zncc, dz, fb, mem, e.stream));
        TW_TRY(copy_out(status, ds, (size_t)e.n, mem, e.stream));
    }
    return e.check_err();
}
int twdic_fftcc_destroy(twdic_fftcc* h) {
    delete h;
    return TWDIC_OK;
}

// ------------------------------------------------------------- IC-GN ABI --
int twdic_icgn_create(const twdic_params* p, int32_t num_x, int32_t num_y, twdic_icgn** out) {
    if (!out) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle output");
    *out = nullptr;
    TW_TRY(validate(p, false, true));
    if (num_x <= 0 || num_y <= 0) return fail(TWDIC_ERR_NO_POI, "Number of POIs is below 0!");
    if ((size_t)num_x * num_y > (size_t)1 << 30) return fail(TWDIC_ERR_UNSUPPORTED, "too many POIs");
    auto* h = new (std::nothrow) twdic_icgn;
    if (!h) return fail(TWDIC_ERR_NO_MEMORY, "host allocation failed");
    h->e.nx = num_x;
    h->e.ny = num_y;
    int r = h->e.init(*p, num_x * num_y);
    if (r != TWDIC_OK) { delete h; return r; }
    *out = h;
    return TWDIC_OK;
}
int twdic_icgn_reset_ref(twdic_icgn* h, const uint8_t* img, int32_t stride, int mem) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    return h->e.set_ref(img, stride, mem);
}
int twdic_icgn_compute(twdic_icgn* h, const uint8_t* tar, int32_t stride, const int32_t* poi_yx, int mem_in,
                       float* u, float* v, float* p6, int32_t* iters, uint8_t* flags, int mem_out) {
    if (!h || !tar || !poi_yx || !u || !v) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    TW_TRY(check_mem(mem_in));
    TW_TRY(check_mem(mem_out));
    Engine& e = h->e;
    const size_t n = (size_t)e.n;
    TW_TRY(e.set_tar(tar, stride, mem_in));
    // POIs: the per-reference cache is keyed on their contents.  Host POIs
    // are compared with a host copy; device POIs are copied into the handle's
    // array on every call by a kernel that reports whether any pair changed
    // (the caller may rewrite the same buffer, or an allocator may hand its
    // address to new POIs).
    if (mem_in == TWDIC_MEM_HOST) {
        if (e.cache_poi_host.size() != 2 * n || std::memcmp(e.cache_poi_host.data(), poi_yx, 8 * n) != 0) {
            e.cache_poi_host.assign(poi_yx, poi_yx + 2 * n);
            TW_TRY(copy_in(e.d_poi.p, poi_yx, 8 * n, mem_in, e.stream));
            e.cache_valid = false;
            e.fspec_valid = false;
        }
    } else {
        int* changed_d = e.d_work.as<int>() + 2;
        int changed = 0;
        TW_CUDA(cudaMemsetAsync(changed_d, 0, sizeof(int), e.stream));
        TW_CUDA(launch_poi_refresh(poi_yx, e.d_poi.as<int2>(), (int)n, changed_d, e.stream));
        TW_CUDA(cudaMemcpyAsync(&changed, changed_d, sizeof(int), cudaMemcpyDeviceToHost, e.stream));
        TW_CUDA(cudaStreamSynchronize(e.stream));
        if (changed) {
            e.cache_poi_host.clear();
            e.cache_valid = false;
            e.fspec_valid = false;
        }
    }
    float *du = u, *dv = v, *dp6 = p6 ? p6 : e.d_p6.as<float>();
    int* dit = iters;
    uint8_t* dfl = flags ? flags : e.d_flags.as<uint8_t>();
    if (mem_out == TWDIC_MEM_HOST) {
        du = e.d_u.as<float>(); dv = e.d_v.as<float>(); dp6 = e.d_p6.as<float>();
        dit = e.d_iters.as<int>(); dfl = e.d_flags.as<uint8_t>();
        TW_TRY(copy_in(du, u, 4 * n, mem_out, e.stream));
        TW_TRY(copy_in(dv, v, 4 * n, mem_out, e.stream));
        if (iters) TW_TRY(copy_in(dit, iters, 4 * n, mem_out, e.stream));
        else TW_CUDA(cudaMemsetAsync(dit, 0, 4 * n, e.stream));
    } else if (!iters) {
        dit = e.d_iters.as<int>();
        TW_CUDA(cudaMemsetAsync(dit, 0, 4 * n, e.stream));
    }
    TW_TRY(e.icgn(du, dv, dp6, dit, dfl));
    if (mem_out == TWDIC_MEM_HOST) {
        TW_TRY(copy_out(u, du, 4 * n, mem_out, e.stream));
        TW_TRY(copy_out(v, dv, 4 * n, mem_out, e.stream));
        TW_TRY(copy_out(p6, dp6, 24 * n, mem_out, e.stream));
        TW_TRY(copy_out(iters, dit, 4 * n, mem_out, e.stream));
        TW_TRY(copy_out(flags, dfl, n, mem_out, e.stream));
    }
    return e.check_err();
}
int twdic_icgn_destroy(twdic_icgn* h) {
    delete h;
    return TWDIC_OK;
}

// ------------------------------------------------------------- frame ABI --
int twdic_frame_create(const twdic_params* p, twdic_frame** out) {
    if (!out) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle output");
    *out = nullptr;
    auto* h = new (std::nothrow) twdic_frame;
    if (!h) return fail(TWDIC_ERR_NO_MEMORY, "host allocation failed");
    int r = engine_grid_init(h->e, p, true);
    if (r != TWDIC_OK) { delete h; return r; }
    *out = h;
    return TWDIC_OK;
}
int twdic_frame_num_pois(const twdic_frame* h, int32_t* num_x, int32_t* num_y) {
    if (!h || !num_x || !num_y) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    *num_x = h->e.nx;
    *num_y = h->e.ny;
    return TWDIC_OK;
}
int twdic_frame_poi_positions(const twdic_frame* h, int32_t* poi_yx, int mem) {
    if (!h || !poi_yx) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    TW_TRY(check_mem(mem));
    TW_TRY(copy_out(poi_yx, h->e.d_poi.p, sizeof(int2) * (size_t)h->e.n, mem, h->e.stream));
    TW_CUDA(cudaStreamSynchronize(h->e.stream));
    return TWDIC_OK;
}
int twdic_frame_set_reference(twdic_frame* h, const uint8_t* img, int32_t stride, int mem) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    return h->e.set_ref(img, stride, mem);
}
int twdic_frame_set_stream(twdic_frame* h, void* stream) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    h->e.stream = stream ? static_cast<cudaStream_t>(stream) : h->e.own_stream;
    return TWDIC_OK;
}
int twdic_frame_process(twdic_frame* h, const uint8_t* tar, int32_t stride, int mem_in, float* u, float* v,
                        float* zncc, float* p6, int32_t* iters, uint8_t* flags, int mem_out) {
    if (!h || !tar || !u || !v) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    TW_TRY(check_mem(mem_in));
    TW_TRY(check_mem(mem_out));
    Engine& e = h->e;
    if (!e.have_ref) return fail(TWDIC_ERR_STATE, "no reference image set");
    const size_t n = (size_t)e.n;
    const bool dev = mem_out == TWDIC_MEM_DEVICE;
    float* du = dev ? u : e.d_u.as<float>();
    float* dv = dev ? v : e.d_v.as<float>();
    float* dz = (dev && zncc) ? zncc : e.d_zncc.as<float>();
    float* dp6 = (dev && p6) ? p6 : e.d_p6.as<float>();
    int* dit = (dev && iters) ? iters : e.d_iters.as<int>();
    uint8_t* dfl = (dev && flags) ? flags : e.d_flags.as<uint8_t>();
    TW_CUDA(cudaEventRecord(e.ev[0], e.stream));
    TW_TRY(e.set_tar(tar, stride, mem_in));
    TW_CUDA(cudaEventRecord(e.ev[1], e.stream));
    const bool cached = e.cache_valid;
    TW_TRY(e.ensure_cache(nullptr));
    TW_CUDA(cudaEventRecord(e.ev[2], e.stream));
    // a frame starts from zero displacements for dark FFT-CC subsets and a
    // zero iteration count, as a freshly calloc'd reference buffer would
    TW_CUDA(cudaMemsetAsync(du, 0, 4 * n, e.stream));
    TW_CUDA(cudaMemsetAsync(dv, 0, 4 * n, e.stream));
    TW_CUDA(cudaMemsetAsync(dz, 0, 4 * n, e.stream));
    TW_CUDA(cudaMemsetAsync(dit, 0, 4 * n, e.stream));
    TW_TRY(e.fftcc(du, dv, dz, e.d_fst.as<uint8_t>()));
    TW_CUDA(cudaEventRecord(e.ev[3], e.stream));
    TW_TRY(e.prepare_target());
    TW_CUDA(cudaEventRecord(e.ev[6], e.stream));
    TW_TRY(e.icgn_solve(du, dv, dp6, dit, dfl));
    TW_CUDA(cudaEventRecord(e.ev[4], e.stream));
    if (!dev) {
        TW_TRY(copy_out(u, du, 4 * n, mem_out, e.stream));
        TW_TRY(copy_out(v, dv, 4 * n, mem_out, e.stream));
        TW_TRY(copy_out(zncc, dz, 4 * n, mem_out, e.stream));
        TW_TRY(copy_out(p6, dp6, 24 * n, mem_out, e.stream));
        TW_TRY(copy_out(iters, dit, 4 * n, mem_out, e.stream));
        TW_TRY(copy_out(flags, dfl, n, mem_out, e.stream));
    }
    TW_CUDA(cudaEventRecord(e.ev[5], e.stream));
    e.times_pending = true;
    e.last_times[5] = cached ? -1.f : 0.f;
    if (!dev) return e.check_err();
    return TWDIC_OK;
}
int twdic_frame_table(twdic_frame* h, int which, float* dst) {
    if (!h || !dst) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    Engine& e = h->e;
    const Geom& g = e.g;
    const size_t px = (size_t)g.rw * g.rh;
    if (which == TWDIC_TABLE_BICUBIC_LUT || which == TWDIC_TABLE_BSPLINE_LUT) {
        if (!e.have_tar) return fail(TWDIC_ERR_STATE, "the LUT needs a target image (process a frame first)");
        DevBuf lut;
        TW_TRY(lut.ensure(sizeof(float4) * 4 * px));
        if (which == TWDIC_TABLE_BICUBIC_LUT)
            TW_CUDA(launch_bicubic_lut(g, e.d_tar.as<uint8_t>(), lut.as<float4>(), e.stream));
        else
            TW_CUDA(launch_bspline_lut(g, e.d_tar.as<uint8_t>(), lut.as<float4>(), e.stream));
        std::vector<float4> hb(4 * px);
        TW_CUDA(cudaMemcpyAsync(hb.data(), lut.p, sizeof(float4) * 4 * px, cudaMemcpyDeviceToHost, e.stream));
        TW_CUDA(cudaStreamSynchronize(e.stream));
        // device layout: plane k of float4 (n = 0..3) per ROI pixel
        for (size_t o = 0; o < px; ++o)
            for (int k = 0; k < 4; ++k) {
                const float4 c = hb[k * px + o];
                float* d = dst + o * 16 + k * 4;
                d[0] = c.x; d[1] = c.y; d[2] = c.z; d[3] = c.w;
            }
        return TWDIC_OK;
    }
    if (which == TWDIC_TABLE_REF_GRADIENT) {
        if (!e.have_ref) return fail(TWDIC_ERR_STATE, "the gradients need a reference image");
        DevBuf grad;
        TW_TRY(grad.ensure(sizeof(float2) * px));
        TW_CUDA(launch_ref_grad(g, e.d_ref.as<uint8_t>(), grad.as<float2>(), e.stream));
        std::vector<float2> hb(px);
        TW_CUDA(cudaMemcpyAsync(hb.data(), grad.p, sizeof(float2) * px, cudaMemcpyDeviceToHost, e.stream));
        TW_CUDA(cudaStreamSynchronize(e.stream));
        for (size_t o = 0; o < px; ++o) {
            dst[2 * o] = hb[o].x;
            dst[2 * o + 1] = hb[o].y;
        }
        return TWDIC_OK;
    }
    if (which == TWDIC_TABLE_SUBSET_GRADIENT) {
        if (e.prm.path != TWDIC_PATH_PLAIN) return fail(TWDIC_ERR_STATE, "per-subset gradients: plain path only");
        if (!e.have_ref) return fail(TWDIC_ERR_STATE, "the gradients need a reference image");
        TW_TRY(e.ensure_cache(nullptr));
        const size_t S = (size_t)(2 * g.rx + 1) * (2 * g.ry + 1), n = (size_t)e.n;
        std::vector<float2> hb(3 * S * n);
        TW_CUDA(cudaMemcpyAsync(hb.data(), e.c_sd.p, sizeof(float2) * 3 * S * n, cudaMemcpyDeviceToHost,
                                e.stream));
        TW_CUDA(cudaStreamSynchronize(e.stream));
        // steepest-descent planes per POI: (R_x, R_x dx), (R_x dy, R_y), (R_y dx, R_y dy)
        for (size_t p = 0; p < n; ++p)
            for (size_t k = 0; k < S; ++k) {
                dst[(p * S + k) * 2] = hb[p * 3 * S + k].x;
                dst[(p * S + k) * 2 + 1] = hb[p * 3 * S + S + k].y;
            }
        return TWDIC_OK;
    }
    return fail(TWDIC_ERR_INVALID_ARG, "unknown table %d", which);
}
int twdic_frame_phase_times(const twdic_frame* hc, float* t6) {
    if (!hc || !t6) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    auto* h = const_cast<twdic_frame*>(hc);
    Engine& e = h->e;
    if (e.times_pending) {
        TW_CUDA(cudaEventSynchronize(e.ev[5]));
        float a = 0, b = 0, c = 0, d = 0, f = 0, pr = 0;
        TW_CUDA(cudaEventElapsedTime(&a, e.ev[0], e.ev[1]));
        TW_CUDA(cudaEventElapsedTime(&f, e.ev[1], e.ev[2]));
        TW_CUDA(cudaEventElapsedTime(&b, e.ev[2], e.ev[3]));
        TW_CUDA(cudaEventElapsedTime(&pr, e.ev[3], e.ev[6]));
        TW_CUDA(cudaEventElapsedTime(&c, e.ev[6], e.ev[4]));
        TW_CUDA(cudaEventElapsedTime(&d, e.ev[4], e.ev[5]));
        const bool cached = e.last_times[5] < 0.f;
        e.last_times[0] = a;
        e.last_times[1] = b;
        e.last_times[2] = pr;  // target LUT
        e.last_times[3] = c;
        e.last_times[4] = d;
        e.last_times[5] = cached ? 0.f : f;
        e.times_pending = false;
    }
    for (int i = 0; i < 6; ++i) t6[i] = e.last_times[i];
    return TWDIC_OK;
}
int twdic_frame_destroy(twdic_frame* h) {
    delete h;
    return TWDIC_OK;
}

// Device memory of a frame handle after its first fast-path frame (the
// allocations of Engine::init, the per-reference cache and the default
// neighbourhood table), each rounded up to the 2 MiB the allocator may
// reserve for it.  Host-only: no CUDA call.
int twdic_frame_device_bytes(const twdic_params* p, uint64_t* bytes) {
    if (!bytes) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    TW_TRY(validate(p, true, true));
    int nx = 0, ny = 0;
    TW_TRY(num_pois_of(*p, &nx, &ny));
    const uint64_t n = (uint64_t)nx * ny;
    const uint64_t pitch = (uint64_t)((p->img_width + 15) & ~15);
    const uint64_t img = pitch * (uint64_t)p->img_height + 16;
    auto r = [](uint64_t b) { return (b + (2ull << 20) - 1) / (2ull << 20) * (2ull << 20); };
    uint64_t t = 0;
    t += 2 * r(img);                                        // reference, target
    t += r(8 * n);                                          // POIs
    t += 3 * r(4 * n) + r(n) + r(24 * n) + r(4 * n) + r(n);  // u, v, zncc, status, p6, iters, flags
    t += 4 * r(1024);                                       // error flag, work counter, twiddles, TMA descriptors
    if (p->path == TWDIC_PATH_PLAIN) {
        const uint64_t S = (uint64_t)(2 * p->subset_x + 1) * (2 * p->subset_y + 1);
        t += r(4 * n * S) + r(24 * n * S) + r(144 * n) + r(4 * n) + r(n);
        t += r(64 * (uint64_t)p->roi_width * p->roi_height);  // float LUT
    } else {
        t += r(64 * n) + r(168 * n) + r(n);                 // statistics, inverse Hessian, flags
        t += r(8 * (uint64_t)p->roi_width * p->roi_height);   // reference gradient image (float2)
        t += r(16 * (uint64_t)(2 * p->subset_x + 1) * (2 * p->subset_y + 1));  // sample table
        if (p->subset_x == p->subset_y && p->subset_x >= 4 && p->subset_x <= 32) {
            // the tensor-core FFT-CC's reference spectra (N/2 + 1 rows of N
            // rounded up to 4 FP16 pairs per POI) and window sums
            const uint64_t N = 2 * (uint64_t)p->subset_x;
            t += r(n * (N / 2 + 1) * ((N + 3) / 4 * 4) * 4) + r(8 * n);
        }
        t += r(16 * (uint64_t)p->roi_width * p->roi_height);  // neighbourhood table
    }
    *bytes = t;
    return TWDIC_OK;
}

// ICGN2DInterpolationFLag (TW/TW_Engine/TW_paDIC.h:89-93), the Iflag of the
// ICGN2D_CPU / cuICGN2D constructors.
static int set_interp(Engine& e, int mode) {
    if (mode != TWDIC_INTERP_BICUBIC && mode != TWDIC_INTERP_BSPLINE)
        return fail(TWDIC_ERR_INVALID_ARG, "interpolation must be TWDIC_INTERP_BICUBIC or TWDIC_INTERP_BSPLINE");
    e.interp = mode;
    return TWDIC_OK;
}
int twdic_icgn_set_interpolation(twdic_icgn* h, int mode) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    return set_interp(h->e, mode);
}
int twdic_frame_set_interpolation(twdic_frame* h, int mode) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    return set_interp(h->e, mode);
}

// Tuning (internal to the Python autotuner; not part of the reference interface).
int twdic_frame_set_tuning(twdic_frame* h, int icgn_threads, int icgn_ctas_per_sm, int icgn_sampler,
                           int fftcc_use_tc) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    if (!valid_icgn_threads(icgn_threads))
        return fail(TWDIC_ERR_INVALID_ARG, "threads must be 32, 64, 128, 256, 512 or 1024");
    h->e.icgn_tune.threads = icgn_threads;
    h->e.icgn_tune.ctas_per_sm = icgn_ctas_per_sm;
    if (icgn_sampler < kSampWindow || icgn_sampler > kSampNbhd)
        return fail(TWDIC_ERR_INVALID_ARG, "sampler must be 0 (window), 1 (LUT) or 2 (neighbourhood table)");
    h->e.icgn_tune.sampler = icgn_sampler;
    h->e.fftcc_tune.use_tc = fftcc_use_tc;
    return TWDIC_OK;
}


int twdic_frame_set_icgn_layout(twdic_frame* h, int chunk) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    if (chunk < 0) return fail(TWDIC_ERR_INVALID_ARG, "chunk must be >= 0");
    h->e.icgn_tune.chunk = chunk;
    return TWDIC_OK;
}

int twdic_frame_set_guess_mode(twdic_frame* h, int mode) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    if (mode != 0 && mode != 1) return fail(TWDIC_ERR_INVALID_ARG, "guess mode must be 0 or 1");
    h->e.guess = mode;
    return TWDIC_OK;
}

int twdic_frame_set_icgn_unroll(twdic_frame* h, int unroll) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    if (unroll != 2 && unroll != 4 && unroll != 8) return fail(TWDIC_ERR_INVALID_ARG, "unroll must be 2, 4 or 8");
    h->e.icgn_tune.unroll = unroll;
    return TWDIC_OK;
}

int twdic_frame_set_fftcc_tuning(twdic_frame* h, int use_tc, int groups, int pois_per_group) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    if (groups < 0 || groups > 5 || pois_per_group < 0) return fail(TWDIC_ERR_INVALID_ARG, "bad FFT-CC tuning");
    h->e.fftcc_tune.use_tc = use_tc;
    h->e.fftcc_tune.groups = groups;
    h->e.fftcc_tune.pois_per_group = pois_per_group;
    return TWDIC_OK;
}

int twdic_frame_set_fftcc_twiddles(twdic_frame* h, int hi_lo) {
    if (!h) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    h->e.fftcc_tune.twiddle_lo = hi_lo ? 1 : 0;
    return TWDIC_OK;
}

int twdic_frame_get_tuning(const twdic_frame* h, twdic_tuning* out) {
    if (!h || !out) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    out->icgn_threads = h->e.icgn_tune.threads;
    out->icgn_ctas_per_sm = h->e.icgn_tune.ctas_per_sm;
    out->icgn_sampler = h->e.icgn_tune.sampler;
    out->icgn_chunk = h->e.icgn_tune.chunk;
    out->icgn_unroll = h->e.icgn_tune.unroll;
    out->fftcc_use_tc = h->e.fftcc_tune.use_tc;
    out->fftcc_groups = h->e.fftcc_tune.groups;
    out->fftcc_pois_per_group = h->e.fftcc_tune.pois_per_group;
    return TWDIC_OK;
}

}  // extern "C"

namespace {

// Key of a tuning cache entry: the GPU and every parameter that changes the
// launch shapes' costs.
std::string tuning_key(const Engine& e) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    std::memset(&prop, 0, sizeof(prop));
    cudaGetDeviceProperties(&prop, dev);
    std::string name(prop.name);
    for (char& c : name)
        if (c == ' ' || c == '|') c = '_';
    const twdic_params& p = e.prm;
    char buf[256];
    snprintf(buf, sizeof(buf), "%s|sm%d|%dx%d|roi%dx%d|r%dx%d|g%dx%d|m%dx%d|path%d", name.c_str(),
             prop.multiProcessorCount, p.img_width, p.img_height, p.roi_width, p.roi_height, p.subset_x, p.subset_y,
             p.grid_space_x, p.grid_space_y, p.margin_x, p.margin_y, p.path);
    return buf;
}

// A cache entry is taken only with the values the setters accept
// (twdic_frame_set_tuning, _icgn_layout, _icgn_unroll, _fftcc_tuning); a
// hand-edited or damaged line is skipped, so the shapes are measured again.
bool cached_tuning_valid(const twdic_tuning& c) {
    return valid_icgn_threads(c.icgn_threads) && c.icgn_ctas_per_sm >= 0 && c.icgn_sampler >= kSampWindow &&
           c.icgn_sampler <= kSampNbhd && c.icgn_chunk >= 0 &&
           (c.icgn_unroll == 2 || c.icgn_unroll == 4 || c.icgn_unroll == 8) &&
           (c.fftcc_use_tc == 0 || c.fftcc_use_tc == 1) && c.fftcc_groups >= 0 && c.fftcc_groups <= 5 &&
           c.fftcc_pois_per_group >= 0;
}

bool cache_lookup(const char* path, const std::string& key, twdic_tuning* t) {
    FILE* f = path ? std::fopen(path, "r") : nullptr;
    if (!f) return false;
    char line[512];
    bool found = false;
    while (std::fgets(line, sizeof(line), f)) {
        const size_t k = key.size();
        if (std::strncmp(line, key.c_str(), k) != 0 || line[k] != ' ') continue;
        twdic_tuning c;
        std::memset(&c, 0, sizeof(c));
        if (std::sscanf(line + k, " %d %d %d %d %d %d %d %d %f %f", &c.icgn_threads, &c.icgn_ctas_per_sm,
                        &c.icgn_sampler, &c.icgn_chunk, &c.icgn_unroll, &c.fftcc_use_tc, &c.fftcc_groups,
                        &c.fftcc_pois_per_group, &c.fftcc_ms, &c.icgn_ms) == 10 &&
            cached_tuning_valid(c)) {
            *t = c;  // the last entry for a key wins
            found = true;
        }
    }
    std::fclose(f);
    return found;
}

}  // namespace

extern "C" {

// Measures the launch shapes on this frame's target and keeps the fastest:
// the FFT-CC tile (groups per CTA, POIs per group batch) by the FFT-CC phase
// time, the IC-GN shape (threads per CTA, target sampler) by the time of
// target preparation plus IC-GN; each candidate takes one warm-up and three
// timed frames (median).  With cache_path, an entry for this GPU and these
// parameters is reused without timing, and a new choice is appended.
int twdic_frame_autotune(twdic_frame* h, const uint8_t* tar, int32_t stride, int mem, const char* cache_path,
                         twdic_tuning* out) {
    if (!h || !tar || !out) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    Engine& e = h->e;
    if (!e.have_ref) return fail(TWDIC_ERR_STATE, "autotune needs a reference image");
    const std::string key = tuning_key(e);
    twdic_tuning t;
    std::memset(&t, 0, sizeof(t));
    if (cache_lookup(cache_path, key, &t)) {
        e.icgn_tune.threads = t.icgn_threads;
        e.icgn_tune.ctas_per_sm = t.icgn_ctas_per_sm;
        e.icgn_tune.sampler = t.icgn_sampler;
        e.icgn_tune.chunk = t.icgn_chunk;
        e.icgn_tune.unroll = t.icgn_unroll;
        e.fftcc_tune.use_tc = t.fftcc_use_tc;
        e.fftcc_tune.groups = t.fftcc_groups;
        e.fftcc_tune.pois_per_group = t.fftcc_pois_per_group;
        t.from_cache = 1;
        *out = t;
        return TWDIC_OK;
    }
    const IcgnTune icgn0 = e.icgn_tune;
    const FftccTune fft0 = e.fftcc_tune;
    auto measure = [&](float* fftcc_ms, float* icgn_ms) -> int {
        std::vector<float> fa, ia;
        for (int r = 0; r < 4; ++r) {
            TW_TRY(twdic_frame_process(h, tar, stride, mem, e.d_u.as<float>(), e.d_v.as<float>(),
                                       e.d_zncc.as<float>(), e.d_p6.as<float>(), e.d_iters.as<int>(),
                                       e.d_flags.as<uint8_t>(), TWDIC_MEM_DEVICE));
            float t6[6];
            TW_TRY(twdic_frame_phase_times(h, t6));
            if (r == 0) continue;
            fa.push_back(t6[1]);
            ia.push_back(t6[2] + t6[3]);
        }
        std::sort(fa.begin(), fa.end());
        std::sort(ia.begin(), ia.end());
        *fftcc_ms = fa[fa.size() / 2];
        *icgn_ms = ia[ia.size() / 2];
        return TWDIC_OK;
    };
    // FFT-CC tile shapes (the IC-GN shape stays as it was)
    FftccTune best_f = fft0;
    float best_fms = 1e30f;
    if (e.prm.path == TWDIC_PATH_FAST && fftcc_tc_supported(e.g)) {
        for (int groups : {0, 4, 2, 1}) {
            for (int ppg : {0, 2, 1}) {
                FftccTune c;
                c.use_tc = 1;
                c.groups = groups;
                c.pois_per_group = ppg;
                c.twiddle_lo = fft0.twiddle_lo;  // the precision stays the caller's choice
                e.fftcc_tune = c;
                float f = 0, ic = 0;
                const int rc = measure(&f, &ic);
                if (rc != TWDIC_OK) {
                    e.fftcc_tune = fft0;
                    e.icgn_tune = icgn0;
                    return rc;
                }
                if (f < best_fms) {
                    best_fms = f;
                    best_f = c;
                }
            }
        }
    }
    e.fftcc_tune = best_f;
    // IC-GN shapes
    IcgnTune best_i = icgn0;
    float best_ims = 1e30f, fms = best_fms;
    if (e.prm.path == TWDIC_PATH_FAST) {
        // (threads, chunk): one POI per warp over runs of consecutive POIs,
        // then one POI per CTA
        const int shapes[][2] = {{1024, 32}, {1024, 64}, {512, 32}, {32, 0}, {64, 0}, {128, 0}, {256, 0}};
        for (const auto& sh : shapes) {
            for (int sampler : {kSampNbhd, kSampLut, kSampWindow}) {
                if (sh[1] > 0 && sampler == kSampWindow) continue;
                IcgnTune c;
                c.threads = sh[0];
                c.chunk = sh[1];
                c.ctas_per_sm = 0;
                c.sampler = sampler;
                e.icgn_tune = c;
                float f = 0, ic = 0;
                const int rc = measure(&f, &ic);
                if (rc != TWDIC_OK) {
                    e.fftcc_tune = fft0;
                    e.icgn_tune = icgn0;
                    return rc;
                }
                if (ic < best_ims) {
                    best_ims = ic;
                    best_i = c;
                    if (best_fms >= 1e30f) fms = f;
                }
            }
        }
        // sample-loop unrolling of the chosen one-POI-per-warp shape
        if (best_i.chunk > 0 && best_i.threads == 1024) {
            for (int unroll : {2, 4}) {
                IcgnTune c = best_i;
                c.unroll = unroll;
                e.icgn_tune = c;
                float f = 0, ic = 0;
                const int rc = measure(&f, &ic);
                if (rc != TWDIC_OK) {
                    e.fftcc_tune = fft0;
                    e.icgn_tune = icgn0;
                    return rc;
                }
                if (ic < best_ims) {
                    best_ims = ic;
                    best_i = c;
                }
            }
        }
    } else {
        float f = 0, ic = 0;
        TW_TRY(measure(&f, &ic));
        best_ims = ic;
        fms = f;
    }
    e.icgn_tune = best_i;
    t.icgn_threads = best_i.threads;
    t.icgn_ctas_per_sm = best_i.ctas_per_sm;
    t.icgn_sampler = best_i.sampler;
    t.icgn_chunk = best_i.chunk;
    t.icgn_unroll = best_i.unroll;
    t.fftcc_use_tc = e.fftcc_tune.use_tc;
    t.fftcc_groups = e.fftcc_tune.groups;
    t.fftcc_pois_per_group = e.fftcc_tune.pois_per_group;
    t.fftcc_ms = fms < 1e30f ? fms : 0.f;
    t.icgn_ms = best_ims;
    t.from_cache = 0;
    if (cache_path) {
        FILE* f = std::fopen(cache_path, "a");
        if (f) {
            std::fprintf(f, "%s %d %d %d %d %d %d %d %d %.4f %.4f\n", key.c_str(), t.icgn_threads,
                         t.icgn_ctas_per_sm, t.icgn_sampler, t.icgn_chunk, t.icgn_unroll, t.fftcc_use_tc,
                         t.fftcc_groups, t.fftcc_pois_per_group, t.fftcc_ms, t.icgn_ms);
            std::fclose(f);
        }
    }
    *out = t;
    return TWDIC_OK;
}
}  // extern "C"

// ------------------------------------------------------------- batches ----
// Several frame handles' targets in one set of launches: the fast-path frames
// share one tensor-core FFT-CC launch (all window sizes) and one persistent
// IC-GN launch per sampler (kMaxJobs frames per launch).  No reference
// counterpart (the reference runs one frame per call).
struct twdic_batch {
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    DevBuf d_work, d_err;
    IcgnTune tune;
    FftccTune fftcc_tune;
    bool use_graph = false;
    cudaGraphExec_t exec = nullptr;
    std::vector<uintptr_t> key;  // the call the instantiated graph replays
    cudaEvent_t done = nullptr;
    // phase boundaries of the last call run without a graph: start,
    // preparation done, FFT-CC done, float LUTs done, IC-GN done
    cudaEvent_t ph[5] = {};
    bool ph_recorded = false;
    ~twdic_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (done) cudaEventDestroy(done);
        for (auto& e : ph)
            if (e) cudaEventDestroy(e);
        if (own_stream) cudaStreamDestroy(own_stream);
    }
};

namespace {

struct BatchArgs {
    int count;
    twdic_frame* const* frames;
    const uint8_t* const* tars;
    const int32_t* strides;
    int mem_in;
    float* const* u;
    float* const* v;
    float* const* zncc;
    float* const* p6;
    int32_t* const* iters;
    uint8_t* const* flags;
    int mem_out;
};

// Per-frame device outputs of a batch call: the caller's arrays (device
// outputs) or the handle's own buffers (host outputs, copied out after).
struct FrameOut {
    float *u, *v, *z, *p6;
    int* it;
    uint8_t* fl;
};

FrameOut frame_out(Engine& e, const BatchArgs& a, int i) {
    const bool dev = a.mem_out == TWDIC_MEM_DEVICE;
    FrameOut o;
    o.u = dev ? a.u[i] : e.d_u.as<float>();
    o.v = dev ? a.v[i] : e.d_v.as<float>();
    o.z = (dev && a.zncc && a.zncc[i]) ? a.zncc[i] : e.d_zncc.as<float>();
    o.p6 = (dev && a.p6 && a.p6[i]) ? a.p6[i] : e.d_p6.as<float>();
    o.it = (dev && a.iters && a.iters[i]) ? a.iters[i] : e.d_iters.as<int>();
    o.fl = (dev && a.flags && a.flags[i]) ? a.flags[i] : e.d_flags.as<uint8_t>();
    return o;
}

// The sampler a fast-path frame runs with under the batch's launch shape:
// B-spline frames read the neighbourhood table with the B-spline weights, or
// the B-spline LUT (the window sampler is Catmull-Rom only).
int batch_sampler(const IcgnTune& tune, const Engine& e) {
    if (e.interp != TWDIC_INTERP_BSPLINE) return tune.sampler;
    return tune.sampler == kSampNbhd ? kSampNbhdBs : kSampLut;
}

// The frame's per-frame target table for its sampler.
int prepare_target_for(Engine& e, int sampler) {
    const Geom& g = e.g;
    if (sampler == kSampLut) {
        TW_TRY(e.d_lut.ensure(sizeof(float4) * 4 * (size_t)g.rw * g.rh));
        if (e.interp == TWDIC_INTERP_BSPLINE)
            TW_CUDA(launch_bspline_lut(g, e.d_tar.as<uint8_t>(), e.d_lut.as<float4>(), e.stream));
        else
            TW_CUDA(launch_bicubic_lut(g, e.d_tar.as<uint8_t>(), e.d_lut.as<float4>(), e.stream));
    } else if (sampler == kSampNbhd || sampler == kSampNbhdBs) {
        TW_TRY(e.d_lut.ensure(sizeof(uint4) * (size_t)g.rw * g.rh));
        TW_CUDA(launch_nbhd_table(g, e.d_tar.as<uint8_t>(), e.d_lut.as<uint4>(), e.stream, sampler == kSampNbhdBs));
    }
    return TWDIC_OK;
}

// All work of one batch call on b->stream (the frames' streams are switched
// to it for the duration).  Nothing here allocates once the frames' buffers
// exist, so a second identical call can be captured into a graph.
int batch_enqueue(twdic_batch* b, const BatchArgs& a) {
    const int count = a.count;
    // phase events on calls that run now (a capture records none)
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    TW_CUDA(cudaStreamIsCapturing(b->stream, &cap));
    const bool timed = cap == cudaStreamCaptureStatusNone;
    auto mark = [&](int k) -> int {
        if (timed) TW_CUDA(cudaEventRecord(b->ph[k], b->stream));
        return TWDIC_OK;
    };
    TW_TRY(mark(0));
    std::vector<int> fast_tc, fast_ic;
    // per frame: its target into the handle, guesses in (host outputs), and
    // its part of the preparation launch (neighbourhood table; outputs that
    // start at zero: the counters always, u, v, zncc unless IC-GN starts from
    // the given displacements)
    std::vector<PrepJob> prep;
    for (int i = 0; i < count; ++i) {
        Engine& e = a.frames[i]->e;
        e.stream = b->stream;
        TW_TRY(e.ensure_cache(nullptr));
        TW_TRY(e.set_tar(a.tars[i], a.strides ? a.strides[i] : 0, a.mem_in));
        const FrameOut o = frame_out(e, a, i);
        const size_t n = (size_t)e.n;
        const bool fast = e.prm.path == TWDIC_PATH_FAST;
        PrepJob pj{};
        pj.g = e.g;
        pj.tar = e.d_tar.as<uint8_t>();
        pj.n = e.n;
        pj.zero_i = o.it;
        if (fast) {
            const int sampler = batch_sampler(b->tune, e);
            if (sampler == kSampNbhd || sampler == kSampNbhdBs) {
                TW_TRY(e.d_lut.ensure(sizeof(uint4) * (size_t)e.g.rw * e.g.rh));
                pj.table = e.d_lut.as<uint4>();
                pj.full = sampler == kSampNbhdBs ? 1 : 0;
            }
        }
        if (e.guess) {
            // IC-GN from the displacements in u, v (ZNCC is not recomputed)
            if (a.mem_out == TWDIC_MEM_HOST) {
                TW_CUDA(cudaMemcpyAsync(o.u, a.u[i], 4 * n, cudaMemcpyHostToDevice, b->stream));
                TW_CUDA(cudaMemcpyAsync(o.v, a.v[i], 4 * n, cudaMemcpyHostToDevice, b->stream));
            }
        } else {
            pj.zero_f[0] = o.u;
            pj.zero_f[1] = o.v;
            pj.zero_f[2] = o.z;
            if (fast && e.fftcc_tune.use_tc && fftcc_tc_supported(e.g)) fast_tc.push_back(i);
        }
        if (fast) fast_ic.push_back(i);
        prep.push_back(pj);
    }
    for (size_t k0 = 0; k0 < prep.size(); k0 += kMaxPrepJobs) {
        PrepJobs P;
        for (size_t k = k0; k < prep.size() && k < k0 + kMaxPrepJobs; ++k) {
            PrepJob& pj = P.job[P.njobs++];
            pj = prep[k];
            pj.px_begin = P.px_total;
            pj.z_begin = P.z_total;
            if (pj.table) P.px_total += (long long)pj.g.rw * pj.g.rh;
            P.z_total += pj.n;
        }
        TW_CUDA(launch_batch_prepare(P, b->stream));
    }
    TW_TRY(mark(1));
    // FFT-CC of the frames off the tensor-core path, one call each
    for (int i = 0; i < count; ++i) {
        Engine& e = a.frames[i]->e;
        if (e.guess || std::find(fast_tc.begin(), fast_tc.end(), i) != fast_tc.end()) continue;
        const FrameOut o = frame_out(e, a, i);
        TW_TRY(e.fftcc(o.u, o.v, o.z, e.d_fst.as<uint8_t>()));
    }
    // tensor-core FFT-CC: one launch over every window size (the launch takes
    // the frames in segments of one window size), per kMaxTcJobsPerLaunch frames
    {
        std::vector<FftccJob> jobs;
        for (size_t m = 0; m < fast_tc.size(); ++m) {
            const int i = fast_tc[m];
            Engine& e = a.frames[i]->e;
            TW_TRY(e.ensure_fspec(b->fftcc_tune));
            TW_TRY(e.ensure_tc_maps(b->fftcc_tune));
            const FrameOut o = frame_out(e, a, i);
            jobs.push_back(FftccJob{e.g, e.d_tcmaps.p, e.tcmaps.key, e.tcmaps.uw, e.tcmaps.utoff,
                                    e.d_ref.as<uint8_t>(), e.d_tar.as<uint8_t>(), e.c_fspec.as<uint32_t>(), e.c_fsum.as<int2>(), e.d_poi.as<int2>(), e.n, o.u,
                                    o.v, o.z, e.d_fst.as<uint8_t>()});
            if ((int)jobs.size() == kMaxTcJobsPerLaunch || m + 1 == fast_tc.size()) {
                TW_CUDA(launch_fftcc_tc_jobs(jobs.data(), (int)jobs.size(), b->fftcc_tune, b->d_err.as<unsigned>(),
                                             b->d_work.as<int>() + 1, b->stream));
                jobs.clear();
            }
        }
    }
    TW_TRY(mark(2));
    // float LUTs (the LUT samplers and the plain path), one launch per frame
    for (int i = 0; i < count; ++i) {
        Engine& e = a.frames[i]->e;
        if (e.prm.path == TWDIC_PATH_FAST) {
            const int sampler = batch_sampler(b->tune, e);
            if (sampler == kSampLut) TW_TRY(prepare_target_for(e, sampler));
        } else {
            TW_TRY(e.prepare_target());
        }
    }
    TW_TRY(mark(3));
    // one launch per residency level and sampler (and per kMaxJobs frames): a
    // launch sizes shared memory for its largest subset, so frames whose
    // subsets allow more resident CTAs are not launched with larger ones
    struct IcOrder {
        int residency, sampler, frame;
    };
    std::vector<IcOrder> order;
    for (int i : fast_ic) {
        const Engine& e = a.frames[i]->e;
        IcgnTune t = b->tune;
        t.sampler = batch_sampler(b->tune, e);
        order.push_back(IcOrder{icgn_fast_residency(e.g, t), t.sampler, i});
    }
    std::stable_sort(order.begin(), order.end(), [](const IcOrder& x, const IcOrder& y) {
        return x.residency != y.residency ? x.residency > y.residency : x.sampler < y.sampler;
    });
    for (size_t k0 = 0; k0 < order.size();) {
        IcgnJobs J;
        J.njobs = 0;
        J.total = 0;
        IcgnTune tune = b->tune;
        tune.sampler = order[k0].sampler;
        size_t k = k0;
        for (; k < order.size() && J.njobs < kMaxJobs && order[k].residency == order[k0].residency &&
               order[k].sampler == order[k0].sampler;
             ++k) {
            const int i = order[k].frame;
            Engine& e = a.frames[i]->e;
            const FrameOut o = frame_out(e, a, i);
            IcgnJob& jb = J.job[J.njobs++];
            jb.g = e.g;
            jb.ref = e.d_ref.as<uint8_t>();
            jb.tar = e.d_tar.as<uint8_t>();
            jb.poi = e.d_poi.as<int2>();
            jb.stats = e.c_stat.as<float>();
            jb.hinv = e.c_chol64.as<double>();
            jb.rflag = e.c_flag64.as<uint8_t>();
            jb.table = tune.sampler == kSampWindow ? nullptr : e.d_lut.p;
            jb.grad = e.c_grad.as<float2>();
            jb.samples = e.c_samp.as<float4>();
            jb.u = o.u;
            jb.v = o.v;
            jb.p6 = o.p6;
            jb.iters = o.it;
            jb.flags = o.fl;
            jb.n = e.n;
            jb.begin = J.total;
            J.total += e.n;
        }
        k0 = k;
        TW_CUDA(launch_icgn_fast_jobs(J, b->d_work.as<int>(), tune, b->stream));
    }
    for (int i = 0; i < count; ++i) {
        Engine& e = a.frames[i]->e;
        if (e.prm.path == TWDIC_PATH_FAST) continue;
        const FrameOut o = frame_out(e, a, i);
        TW_TRY(e.icgn_solve(o.u, o.v, o.p6, o.it, o.fl));
    }
    TW_TRY(mark(4));
    if (timed) b->ph_recorded = true;
    return TWDIC_OK;
}

}  // namespace

extern "C" {

int twdic_batch_create(twdic_batch** out) {
    if (!out) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    std::unique_ptr<twdic_batch> b(new twdic_batch());
    TW_CUDA(cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking));
    b->stream = b->own_stream;
    TW_CUDA(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    for (auto& e : b->ph) TW_CUDA(cudaEventCreate(&e));
    TW_TRY(b->d_work.ensure(sizeof(int) * (2 + kMaxTcSegsScratch)));
    TW_TRY(b->d_err.ensure(sizeof(unsigned)));
    TW_CUDA(cudaMemset(b->d_err.p, 0, sizeof(unsigned)));
    b->tune.threads = 1024;
    b->tune.chunk = 32;
    b->tune.sampler = kSampNbhd;
    *out = b.release();
    return TWDIC_OK;
}

int twdic_batch_set_stream(twdic_batch* b, void* stream) {
    if (!b) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    // a captured graph may be launched into any stream: it stays valid
    b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
    return TWDIC_OK;
}

int twdic_batch_set_tuning(twdic_batch* b, int icgn_threads, int icgn_ctas_per_sm, int icgn_sampler) {
    if (!b) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    if (!valid_icgn_threads(icgn_threads))
        return fail(TWDIC_ERR_INVALID_ARG, "threads must be 32, 64, 128, 256, 512 or 1024");
    if (icgn_sampler < kSampWindow || icgn_sampler > kSampNbhd)
        return fail(TWDIC_ERR_INVALID_ARG, "sampler must be 0, 1 or 2");
    b->tune.threads = icgn_threads;
    b->tune.ctas_per_sm = icgn_ctas_per_sm;
    b->tune.sampler = icgn_sampler;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->key.clear();
    return TWDIC_OK;
}

int twdic_batch_set_icgn_layout(twdic_batch* b, int chunk) {
    if (!b) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    if (chunk < 0) return fail(TWDIC_ERR_INVALID_ARG, "chunk must be >= 0");
    b->tune.chunk = chunk;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->key.clear();
    return TWDIC_OK;
}

int twdic_batch_set_icgn_unroll(twdic_batch* b, int unroll) {
    if (!b) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    if (unroll != 2 && unroll != 4 && unroll != 8) return fail(TWDIC_ERR_INVALID_ARG, "unroll must be 2, 4 or 8");
    b->tune.unroll = unroll;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
    b->key.clear();
    return TWDIC_OK;
}

int twdic_batch_set_graph(twdic_batch* b, int enable) {
    if (!b) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle");
    b->use_graph = enable != 0;
    return TWDIC_OK;
}

int twdic_batch_process(twdic_batch* b, int32_t count, twdic_frame* const* frames, const uint8_t* const* tars,
                        const int32_t* strides, int mem_in, float* const* u, float* const* v, float* const* zncc,
                        float* const* p6, int32_t* const* iters, uint8_t* const* flags, int mem_out,
                        int32_t* replayed) {
    if (!b || !frames || !tars || !u || !v) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    if (count < 1) return fail(TWDIC_ERR_INVALID_ARG, "count must be >= 1");
    TW_TRY(check_mem(mem_in));
    TW_TRY(check_mem(mem_out));
    if (replayed) *replayed = 0;
    for (int i = 0; i < count; ++i) {
        if (!frames[i] || !tars[i] || !u[i] || !v[i]) return fail(TWDIC_ERR_INVALID_ARG, "NULL frame %d argument", i);
        if (!frames[i]->e.have_ref) return fail(TWDIC_ERR_STATE, "frame %d has no reference image", i);
        for (int k = 0; k < i; ++k)
            if (frames[k] == frames[i]) return fail(TWDIC_ERR_INVALID_ARG, "frame %d appears twice in the batch", i);
    }
    const BatchArgs a{count, frames, tars, strides, mem_in, u, v, zncc, p6, iters, flags, mem_out};
    // order after earlier work on each frame's own stream (reference uploads)
    std::vector<cudaStream_t> saved(count);
    for (int i = 0; i < count; ++i) {
        Engine& e = frames[i]->e;
        saved[i] = e.stream;
        if (e.stream != b->stream) {
            TW_CUDA(cudaEventRecord(e.ev_sync, e.stream));
            TW_CUDA(cudaStreamWaitEvent(b->stream, e.ev_sync, 0));
        }
    }
    auto restore = [&]() {
        for (int i = 0; i < count; ++i) frames[i]->e.stream = saved[i];
    };
    // graph replay: same frames and arrays, device-resident, caches built
    const bool graphable = b->use_graph && mem_in == TWDIC_MEM_DEVICE && mem_out == TWDIC_MEM_DEVICE;
    std::vector<uintptr_t> key;
    bool caches_ok = true;
    if (graphable) {
        key.push_back((uintptr_t)count);
        for (int i = 0; i < count; ++i) {
            const Engine& e = frames[i]->e;
            caches_ok = caches_ok && e.cache_valid;
            // tensor-core FFT-CC frames read the reference spectra
            if (e.prm.path == TWDIC_PATH_FAST && e.fftcc_tune.use_tc && !e.guess && fftcc_tc_supported(e.g))
                caches_ok = caches_ok && e.fspec_valid;
            // the frame's own settings that batch_enqueue reads, then its arrays
            for (uintptr_t x : {(uintptr_t)frames[i], (uintptr_t)e.guess, (uintptr_t)e.interp,
                                (uintptr_t)e.fftcc_tune.use_tc, (uintptr_t)tars[i],
                                (uintptr_t)(strides ? strides[i] : 0),
                                (uintptr_t)u[i], (uintptr_t)v[i], (uintptr_t)(zncc ? zncc[i] : nullptr),
                                (uintptr_t)(p6 ? p6[i] : nullptr), (uintptr_t)(iters ? iters[i] : nullptr),
                                (uintptr_t)(flags ? flags[i] : nullptr)})
                key.push_back(x);
        }
    }
    int rc = TWDIC_OK;
    if (graphable && caches_ok && b->exec && key == b->key) {
        for (int i = 0; i < count; ++i) frames[i]->e.have_tar = true;
        cudaError_t e = cudaGraphLaunch(b->exec, b->stream);
        if (e != cudaSuccess) rc = fail(TWDIC_ERR_CUDA, "cudaGraphLaunch: %s", cudaGetErrorString(e));
        if (replayed && rc == TWDIC_OK) *replayed = 1;
    } else {
        rc = batch_enqueue(b, a);
        if (rc == TWDIC_OK && graphable) {
            // record the same call into a graph for the next identical call
            if (b->exec) cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
            b->key.clear();
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                const int rc2 = batch_enqueue(b, a);
                e = cudaStreamEndCapture(b->stream, &graph);
                if (rc2 == TWDIC_OK && e == cudaSuccess && graph) {
                    if (cudaGraphInstantiate(&b->exec, graph, 0) == cudaSuccess) b->key = key;
                    else b->exec = nullptr;
                }
                if (graph) cudaGraphDestroy(graph);
            }
            cudaGetLastError();  // a failed capture leaves the batch ungraphed, not broken
        }
    }
    restore();
    if (rc != TWDIC_OK) return rc;
    // later work on each frame's own stream waits for the batch
    TW_CUDA(cudaEventRecord(b->done, b->stream));
    for (int i = 0; i < count; ++i)
        if (frames[i]->e.stream != b->stream) TW_CUDA(cudaStreamWaitEvent(frames[i]->e.stream, b->done, 0));
    if (mem_out == TWDIC_MEM_HOST) {
        for (int i = 0; i < count; ++i) {
            Engine& e = frames[i]->e;
            const FrameOut o = frame_out(e, a, i);
            const size_t n = (size_t)e.n;
            TW_TRY(copy_out(u[i], o.u, 4 * n, mem_out, b->stream));
            TW_TRY(copy_out(v[i], o.v, 4 * n, mem_out, b->stream));
            if (zncc) TW_TRY(copy_out(zncc[i], o.z, 4 * n, mem_out, b->stream));
            if (p6) TW_TRY(copy_out(p6[i], o.p6, 24 * n, mem_out, b->stream));
            if (iters) TW_TRY(copy_out(iters[i], o.it, 4 * n, mem_out, b->stream));
            if (flags) TW_TRY(copy_out(flags[i], o.fl, n, mem_out, b->stream));
        }
        unsigned h = 0;
        TW_CUDA(cudaMemcpyAsync(&h, b->d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
        TW_CUDA(cudaStreamSynchronize(b->stream));
        if (h & kErrTimeout) {
            cudaMemsetAsync(b->d_err.p, 0, sizeof(unsigned), b->stream);
            return fail(TWDIC_ERR_TIMEOUT, "a bounded device-side wait gave up");
        }
    }
    return TWDIC_OK;
}

int twdic_batch_phase_times(twdic_batch* b, float* t4) {
    if (!b || !t4) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    if (!b->ph_recorded) return fail(TWDIC_ERR_STATE, "no batch call has run without a graph");
    TW_CUDA(cudaEventSynchronize(b->ph[4]));
    for (int k = 0; k < 4; ++k) TW_CUDA(cudaEventElapsedTime(&t4[k], b->ph[k], b->ph[k + 1]));
    return TWDIC_OK;
}

int twdic_batch_destroy(twdic_batch* b) {
    delete b;
    return TWDIC_OK;
}

}  // extern "C"

// ------------------------------------------------------------ tracking ----
// The reference's per-camera loop (FFTCCTWorkerThread::processFrameFFTCC /
// processFrameFFTCC_ICGN, TW/TW_Core/fftcctworkerthread.cpp:219-330,
// :399-481): frame k (counted from 1) with (k - 1) % interval == 0 becomes the
// reference; at such a frame after the first, the last frame's displacements
// are accumulated and every POI moves by their truncation; every frame runs
// FFT-CC (and IC-GN) at the current POIs against the current reference.
struct twdic_tracker {
    Engine e;
    int interval = 50;
    int with_icgn = 1;
    int64_t frame = 0;
    DevBuf d_acc_u, d_acc_v, d_last_u, d_last_v;
};

extern "C" {

int twdic_tracker_create(const twdic_params* p, int32_t refresh_interval, int32_t with_icgn, twdic_tracker** out) {
    if (!out) return fail(TWDIC_ERR_INVALID_ARG, "NULL handle output");
    *out = nullptr;
    if (refresh_interval < 1) return fail(TWDIC_ERR_INVALID_ARG, "refresh_interval must be >= 1");
    std::unique_ptr<twdic_tracker> t(new (std::nothrow) twdic_tracker);
    if (!t) return fail(TWDIC_ERR_NO_MEMORY, "host allocation failed");
    TW_TRY(engine_grid_init(t->e, p, true));
    t->interval = refresh_interval;
    t->with_icgn = with_icgn ? 1 : 0;
    const size_t b = sizeof(float) * (size_t)t->e.n;
    TW_TRY(t->d_acc_u.ensure(b));
    TW_TRY(t->d_acc_v.ensure(b));
    TW_TRY(t->d_last_u.ensure(b));
    TW_TRY(t->d_last_v.ensure(b));
    TW_CUDA(cudaMemsetAsync(t->d_acc_u.p, 0, b, t->e.stream));
    TW_CUDA(cudaMemsetAsync(t->d_acc_v.p, 0, b, t->e.stream));
    TW_CUDA(cudaStreamSynchronize(t->e.stream));
    *out = t.release();
    return TWDIC_OK;
}

int twdic_tracker_num_pois(const twdic_tracker* t, int32_t* n) {
    if (!t || !n) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    *n = t->e.n;
    return TWDIC_OK;
}

int twdic_tracker_process(twdic_tracker* t, const uint8_t* img, int32_t stride, int mem_in, float* u, float* v,
                          float* acc_u, float* acc_v, int32_t* poi_yx, uint8_t* flags, int mem_out) {
    if (!t || !img) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    TW_TRY(check_mem(mem_in));
    TW_TRY(check_mem(mem_out));
    Engine& e = t->e;
    const size_t n = (size_t)e.n;
    t->frame += 1;
    if ((t->frame - 1) % t->interval == 0) {
        if (t->frame > t->interval) {
            const Geom& g = e.g;
            TW_CUDA(launch_track_update(e.d_poi.as<int2>(), t->d_last_u.as<float>(), t->d_last_v.as<float>(),
                                        t->d_acc_u.as<float>(), t->d_acc_v.as<float>(), e.n, g.sy + g.ry,
                                        g.sy + g.rh - 1 - g.ry, g.sx + g.rx, g.sx + g.rw - 1 - g.rx, e.stream));
        }
        TW_TRY(e.set_ref(img, stride, mem_in));  // also drops the per-reference cache (the POIs moved)
    }
    TW_TRY(e.set_tar(img, stride, mem_in));
    float* du = t->d_last_u.as<float>();
    float* dv = t->d_last_v.as<float>();
    TW_CUDA(cudaMemsetAsync(du, 0, 4 * n, e.stream));
    TW_CUDA(cudaMemsetAsync(dv, 0, 4 * n, e.stream));
    TW_CUDA(cudaMemsetAsync(e.d_zncc.p, 0, 4 * n, e.stream));
    TW_CUDA(cudaMemsetAsync(e.d_iters.p, 0, 4 * n, e.stream));
    TW_TRY(e.ensure_cache(nullptr));
    TW_TRY(e.fftcc(du, dv, e.d_zncc.as<float>(), e.d_fst.as<uint8_t>()));
    if (t->with_icgn) {
        TW_TRY(e.icgn(du, dv, e.d_p6.as<float>(), e.d_iters.as<int>(), e.d_flags.as<uint8_t>()));
    } else {
        TW_CUDA(cudaMemsetAsync(e.d_flags.p, 0, n, e.stream));
    }
    TW_TRY(copy_out(u, du, 4 * n, mem_out, e.stream));
    TW_TRY(copy_out(v, dv, 4 * n, mem_out, e.stream));
    TW_TRY(copy_out(acc_u, t->d_acc_u.p, 4 * n, mem_out, e.stream));
    TW_TRY(copy_out(acc_v, t->d_acc_v.p, 4 * n, mem_out, e.stream));
    TW_TRY(copy_out(poi_yx, e.d_poi.p, 8 * n, mem_out, e.stream));
    TW_TRY(copy_out(flags, t->with_icgn ? e.d_flags.p : e.d_fst.p, n, mem_out, e.stream));
    if (mem_out == TWDIC_MEM_HOST) return e.check_err();
    return TWDIC_OK;
}

int twdic_tracker_colormap(twdic_tracker* t, uint32_t* tex_u, uint32_t* tex_v, float min_u, float max_u,
                           float min_v, float max_v, int mem) {
    if (!t || !tex_u || !tex_v) return fail(TWDIC_ERR_INVALID_ARG, "NULL argument");
    TW_TRY(check_mem(mem));
    if (!(max_u > min_u) || !(max_v > min_v)) return fail(TWDIC_ERR_INVALID_ARG, "colour range must be non-empty");
    Engine& e = t->e;
    const size_t px = (size_t)e.g.rw * e.g.rh;
    uint32_t* du = tex_u;
    uint32_t* dv = tex_v;
    DevBuf tmp;
    if (mem == TWDIC_MEM_HOST) {
        // draw into device copies of the caller's images, then copy back
        TW_TRY(tmp.ensure(8 * px));
        du = tmp.as<uint32_t>();
        dv = du + px;
        TW_CUDA(cudaMemcpyAsync(du, tex_u, 4 * px, cudaMemcpyHostToDevice, e.stream));
        TW_CUDA(cudaMemcpyAsync(dv, tex_v, 4 * px, cudaMemcpyHostToDevice, e.stream));
    }
    TW_CUDA(launch_colormap(du, dv, e.d_poi.as<int2>(), t->d_last_u.as<float>(), t->d_last_v.as<float>(),
                            t->d_acc_u.as<float>(), t->d_acc_v.as<float>(), e.n, e.g, min_u, max_u, min_v, max_v,
                            e.stream));
    if (mem == TWDIC_MEM_HOST) {
        TW_CUDA(cudaMemcpyAsync(tex_u, du, 4 * px, cudaMemcpyDeviceToHost, e.stream));
        TW_CUDA(cudaMemcpyAsync(tex_v, dv, 4 * px, cudaMemcpyDeviceToHost, e.stream));
        TW_CUDA(cudaStreamSynchronize(e.stream));
    }
    return TWDIC_OK;
}

int twdic_tracker_destroy(twdic_tracker* t) {
    delete t;
    return TWDIC_OK;
}

}  // extern "C"
