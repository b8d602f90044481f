// Kernel launchers of the DIC hot path (internal to libtwdic).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "dic_common.cuh"

namespace twdic {

// Target samplers of the fast IC-GN kernel.
enum IcgnSampler {
    kSampWindow = 0,  // staged target window in shared memory, Catmull-Rom
    kSampLut = 1,     // per-frame float bicubic LUT (64 B per ROI pixel), Horner
    kSampNbhd = 2,    // per-frame 4x4 byte neighbourhood table (16 B per ROI pixel), Catmull-Rom
    kSampNbhdBs = 3,  // the same table over every ROI pixel, the reference's B-spline interpolant
};

// Launch shape of the fast IC-GN kernel, chosen by the autotuner.
struct IcgnTune {
    int threads = 128;    // 32, 64, 128 or 256 threads per CTA (one POI per CTA at a time)
    int ctas_per_sm = 0;  // persistent CTAs per SM (0 = occupancy limit)
    int sampler = kSampWindow;  // needs no per-frame table
    // > 0: one POI per warp, the CTA's warps walking runs of `chunk`
    // consecutive POIs over the per-reference gradient image (threads 128 to
    // 1024, a table sampler); 0: one POI per CTA
    int chunk = 0;
    int unroll = 8;  // sample-loop unrolling of the one-POI-per-warp kernel (2, 4 or 8)
};

// Image pairs (jobs) of one batched launch: each job has its own geometry,
// images, POI set, reference cache and outputs.  The table is a kernel
// parameter (__grid_constant__).
constexpr int kMaxJobs = 32;

struct IcgnJob {
    Geom g;
    const uint8_t* ref;
    const uint8_t* tar;
    const int2* poi;
    const float* stats;   // 16 floats per POI (launch_ref_precompute_fast)
    const double* hinv;   // 21 doubles per POI
    const uint8_t* rflag;
    const void* table;    // per-frame target table of the sampler (or null: window)
    const __half2* grad = nullptr;  // per-reference gradient image, rw x rh (or null: staged per POI)
    float* u;
    float* v;
    float* p6;
    int* iters;
    uint8_t* flags;
    int n;      // POIs of the job
    int begin;  // first global POI index of the job
};
struct IcgnJobs {
    int njobs = 0;
    int total = 0;  // POIs of all jobs
    IcgnJob job[kMaxJobs];
};

// Launch shape of the tensor-core FFT-CC kernel.
struct FftccTune {
    int use_tc = 1;          // 0: FP32 SIMT DFT kernel
    int groups = 0;          // tensor-core kernel: 128-thread groups per CTA (0 = as many as fit, up to 4)
    int pois_per_group = 0;  // POIs per group batch (0 = the most the tiles hold)
    int twiddle_lo = 0;      // 1: FP16 hi + lo twiddles (two MMAs per product), 0: hi only
};

// ---- plain FP32 path (kernels_plain.cu)
// tw: twiddle table, tw[k] = exp(-2 pi i k / 2rx) for k < 64, then the same for 2ry
cudaError_t launch_fftcc_plain(const Geom& g, const uint8_t* ref, const uint8_t* tar, const int2* poi, int n,
                               const float2* tw, float* u, float* v, float* zncc, uint8_t* status, cudaStream_t st);
cudaError_t launch_ref_precompute_plain(const Geom& g, const uint8_t* ref, const int2* poi, int n, float* subR,
                                        float2* sd, float* chol, float* refnorm, uint8_t* rflag, cudaStream_t st);
cudaError_t launch_bicubic_lut(const Geom& g, const uint8_t* tar, float4* lut, cudaStream_t st);
// B-spline coefficient LUT of the target, same layout (kernels_plain.cu)
cudaError_t launch_bspline_lut(const Geom& g, const uint8_t* tar, float4* lut, cudaStream_t st);
// 4x4 byte neighbourhoods of every ROI pixel of the target (kernels_icgn_fast.cu);
// full: the last ROI row and column too, bytes outside the image zero (the
// B-spline sampler), otherwise those entries are zero (the bicubic samplers)
cudaError_t launch_nbhd_table(const Geom& g, const uint8_t* tar, uint4* table, cudaStream_t st, bool full = false);
cudaError_t launch_icgn_plain(const Geom& g, const uint8_t* tar, const int2* poi, int n, const float* subR,
                              const float2* sd, const float* chol, const float* refnorm, const uint8_t* rflag,
                              const float4* lut, float* u, float* v, float* p6, int* iters, uint8_t* flags,
                              cudaStream_t st);

// ---- fast IC-GN (kernels_icgn_fast.cu)
// stats: 16 floats per POI (mean, norm, sum SD_k [6], sum SD_k (R - mean) [6], pad);
// chol: 21 doubles per POI, the packed symmetric inverse Hessian formed in FP64
// from its Cholesky factor.  Two launches on st: k_ref_sums (subset sums, the
// FP32 Hessian staged in chol) then k_ref_factor (FP64 factorization in place).
cudaError_t launch_ref_precompute_fast(const Geom& g, const uint8_t* ref, const int2* poi, int n, float* stats,
                                       double* chol, uint8_t* rflag, cudaStream_t st);
cudaError_t launch_icgn_fast(const Geom& g, const uint8_t* ref, const uint8_t* tar, const int2* poi, int n,
                             const float* stats, const double* chol, const uint8_t* rflag, const void* table,
                             int* work, float* u, float* v, float* p6, int* iters, uint8_t* flags,
                             const IcgnTune& tune, cudaStream_t st, const __half2* grad = nullptr);
// Per-reference gradient image (R_x, R_y) of the ROI, half2, rw x rh (kernels_icgn_fast.cu)
cudaError_t launch_ref_grad(const Geom& g, const uint8_t* ref, __half2* grad, cudaStream_t st);
int icgn_fast_window(const Geom& g);
// CTAs per SM the fast IC-GN kernel can keep resident for this geometry and
// launch shape (shared memory, registers, the 32-CTA limit): jobs batched
// into one launch should share it, since the launch sizes shared memory for
// its largest subset
int icgn_fast_residency(const Geom& g, const IcgnTune& tune);
// all jobs of the table in one persistent launch
cudaError_t launch_icgn_fast_jobs(const IcgnJobs& jobs, int* work, const IcgnTune& tune, cudaStream_t st);

// ---- tensor-core FFT-CC (kernels_fftcc_tc.cu)
// err: error flags; work: one int of scratch (the batch counter, zeroed by the launcher)
cudaError_t launch_fftcc_tc(const Geom& g, const uint8_t* ref, const uint8_t* tar, const int2* poi, int n,
                            float* u, float* v, float* zncc, uint8_t* status, unsigned* err, int* work,
                            const FftccTune& tune, cudaStream_t st);
// One image pair of a batched tensor-core FFT-CC launch (all jobs share rx = ry).
struct FftccJob {
    Geom g;
    const uint8_t* ref;
    const uint8_t* tar;
    const int2* poi;
    int n;
    float* u;
    float* v;
    float* zncc;
    uint8_t* status;
};
cudaError_t launch_fftcc_tc_jobs(const FftccJob* jobs, int njobs, const FftccTune& tune, unsigned* err, int* work,
                                 cudaStream_t st);
bool fftcc_tc_supported(const Geom& g);

// ---- tracking loop (kernels_track.cu)
// Copy n device (y, x) pairs into dst; *changed |= 1 when any pair differed
// (the caller zeroes it first)
cudaError_t launch_poi_refresh(const int32_t* src, int2* dst, int n, int* changed, cudaStream_t st);
cudaError_t launch_track_update(int2* poi, const float* u, const float* v, float* acc_u, float* acc_v, int n,
                                int lo_y, int hi_y, int lo_x, int hi_x, cudaStream_t st);
cudaError_t launch_colormap(uint32_t* tex_u, uint32_t* tex_v, const int2* poi, const float* u, const float* v,
                            const float* acc_u, const float* acc_v, int n, const Geom& g, float min_u, float max_u,
                            float min_v, float max_v, cudaStream_t st);

}  // namespace twdic
