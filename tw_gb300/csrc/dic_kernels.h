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

// Image pairs (jobs) of one batched IC-GN launch: each job has its own
// geometry, images, POI set, reference cache and outputs.  The table is a
// kernel parameter (__grid_constant__, at most 32 KB).
constexpr int kMaxJobs = 128;

struct IcgnJob {
    Geom g;
    const uint8_t* ref;
    const uint8_t* tar;
    const int2* poi;
    const float* stats;   // 16 floats per POI (launch_ref_precompute_fast)
    const double* hinv;   // 21 doubles per POI
    const uint8_t* rflag;
    const void* table;    // per-frame target table of the sampler (or null: window)
    const float2* grad = nullptr;  // per-reference gradient image, rw x rh (or null: staged per POI)
    const float4* samples = nullptr;  // subset sample table (launch_sample_table)
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
static_assert(sizeof(IcgnJobs) < 32000, "IC-GN job table exceeds the kernel parameter limit");

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
// One frame of a batch's preparation launch (kernels_icgn_fast.cu): its
// neighbourhood table (table null: none) and the output arrays set to zero
// (null: left alone), n entries each.
struct PrepJob {
    Geom g;
    const uint8_t* tar;
    uint4* table;
    int full;            // the B-spline form of the table
    float* zero_f[3];    // u, v, zncc
    int* zero_i;         // iteration counters
    int n;
    long long px_begin;  // first table item of the frame
    long long z_begin;   // first zeroing item of the frame
};
constexpr int kMaxPrepJobs = 128;
struct PrepJobs {
    int njobs = 0;
    long long px_total = 0, z_total = 0;
    PrepJob job[kMaxPrepJobs];
};
static_assert(sizeof(PrepJobs) < 32000, "preparation table exceeds the kernel parameter limit");
cudaError_t launch_batch_prepare(const PrepJobs& jobs, cudaStream_t st);
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
                             const IcgnTune& tune, cudaStream_t st, const float2* grad = nullptr,
                             const float4* samples = nullptr);
// The samples of a (2 rx + 1) x (2 ry + 1) subset in the reference's order
// (row by row): entry k = (dx, dy) as floats, then the column and row
// within the subset as int bits (kernels_icgn_fast.cu)
cudaError_t launch_sample_table(int rx, int ry, float4* out, cudaStream_t st);
// Per-reference gradient image (R_x, R_y) of the ROI, float2, rw x rh (kernels_icgn_fast.cu)
cudaError_t launch_ref_grad(const Geom& g, const uint8_t* ref, float2* grad, cudaStream_t st);
int icgn_fast_window(const Geom& g);
// CTAs per SM the fast IC-GN kernel can keep resident for this geometry and
// launch shape (shared memory, registers, the 32-CTA limit): jobs batched
// into one launch should share it, since the launch sizes shared memory for
// its largest subset
int icgn_fast_residency(const Geom& g, const IcgnTune& tune);
// all jobs of the table in one persistent launch
cudaError_t launch_icgn_fast_jobs(const IcgnJobs& jobs, int* work, const IcgnTune& tune, cudaStream_t st);

// ---- tensor-core FFT-CC (kernels_fftcc_tc.cu)
// The TMA descriptors of an image pair live in device memory (kTcMapsBytes,
// 128-byte aligned), kept by the frame handle that owns the images: encoded on
// the host by fftcc_tc_encode_maps for a launch shape (window size and
// tuning; the key tells when a re-encoding is due) and copied by the caller.
constexpr size_t kTcMapsBytes = 512;
struct TcMapInfo {
    uint64_t key;  // fftcc_tc_maps_key of the shape encoded for
    int uw;        // width of the one-row boxes (0: not used)
    int utoff;     // offset of the target's one-row box in a group's window region
};
uint64_t fftcc_tc_maps_key(const Geom& g, const FftccTune& tune);
bool fftcc_tc_encode_maps(const Geom& g, const uint8_t* ref, const uint8_t* tar, const FftccTune& tune,
                          void* host_buf, TcMapInfo* info);
// err: error flags; work: scratch -- one int (one window size) or kMaxTcSegsScratch
// ints (several), zeroed by the launcher
// The reference windows' spectra are cached per reference: fspec [n][N/2+1][FS]
// FP16 (Re, Im) pairs with FS = N rounded up to 4 (fftcc_tc_spectrum_bytes),
// fsum [n] the windows' (sum f, sum f^2).  ref = true runs the per-reference
// pass that writes them; ref = false the per-frame FFT-CC that reads them.
cudaError_t launch_fftcc_tc(const Geom& g, const uint8_t* ref_img, const uint8_t* tar_img, const void* maps,
                            uint64_t map_key, int uw, int utoff, uint32_t* fspec, int2* fsum, const int2* poi, int n, float* u, float* v, float* zncc, uint8_t* status,
                            unsigned* err, int* work, const FftccTune& tune, cudaStream_t st, bool ref = false);
size_t fftcc_tc_spectrum_bytes(const Geom& g, int n);
// One image pair of a batched tensor-core FFT-CC launch.  Jobs of one window
// size share one k_fftcc_tc launch; jobs of several window sizes (up to 32)
// share one k_fftcc_tc_seg launch.
constexpr int kMaxTcJobsPerLaunch = 128;
constexpr int kMaxTcSegsScratch = 32;
struct FftccJob {
    Geom g;
    const void* maps;  // device TMA descriptors (fftcc_tc_encode_maps)
    uint64_t map_key;
    int uw, utoff;
    const uint8_t* ref;  // the images the maps describe
    const uint8_t* tar;
    uint32_t* fspec;  // the job's cached reference spectra (launch_fftcc_tc)
    int2* fsum;
    const int2* poi;
    int n;
    float* u;
    float* v;
    float* zncc;
    uint8_t* status;
};
cudaError_t launch_fftcc_tc_jobs(const FftccJob* jobs, int njobs, const FftccTune& tune, unsigned* err, int* work,
                                 cudaStream_t st, bool ref = false);
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
