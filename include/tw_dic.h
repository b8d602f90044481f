/*
 * tw_dic.h -- C ABI of the GB300 (sm_103a) 2D DIC hot path: integer-pixel
 * FFT cross-correlation (FFT-CC) followed by first-order IC-GN sub-pixel
 * registration with bicubic interpolation.
 *
 * Drop-in boundary for TW_Engine's FFT-CC and IC-GN classes.  Each entry
 * point names the reference interface it replaces (paths relative to the
 * TWANG006/TW project root).  Conventions:
 *   - every function returns an int status, TWDIC_OK (0) on success and a
 *     negative TWDIC_ERR_* value otherwise; nothing calls exit() or throws
 *     across the ABI (the reference's checkCudaErrors exits the process,
 *     TW/TW_Engine/helper_cuda.h:965-995);
 *   - images are 8-bit gray, row-major, `stride` bytes per row (the reference
 *     copies rows*cols bytes of a contiguous cv::Mat, so stride == width
 *     there, TW/TW_Engine/TW_paDIC_cuFFTCC2D.cu:281-287);
 *   - POI positions are int32 (y, x) pairs, x fastest, as the reference's
 *     iPOIXY arrays (TW/TW_Engine/TW_utils.cpp:29-49);
 *   - a `mem` argument says whether a pointer is host (TWDIC_MEM_HOST) or
 *     device (TWDIC_MEM_DEVICE) memory; host buffers are staged through the
 *     handle's device buffers on the handle's stream;
 *   - caller-owned buffers throughout: handles never free memory they did
 *     not allocate (the reference's cuICGN2D destructor frees borrowed
 *     pointers, TW/TW_Engine/TW_paDIC_cuICGN2D.cu:719-729; this ABI does not).
 *   - handles are not thread-safe (neither are the reference's objects);
 *     distinct handles may be used from distinct threads.
 */
#ifndef TW_DIC_H
#define TW_DIC_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define TWDIC_API __attribute__((visibility("default")))
#else
#define TWDIC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define TWDIC_ABI_VERSION 2

/* status codes */
#define TWDIC_OK 0
#define TWDIC_ERR_INVALID_ARG (-1)  /* bad pointer, size or enum value */
#define TWDIC_ERR_NO_POI (-2)       /* "Number of POIs is below 0!" (TW_paDIC_FFTCC2D.cpp:88-94 via cuFFTCC2D ctor) */
#define TWDIC_ERR_BORDER (-3)       /* ROI leaves no one-pixel image border (TW_utils.cpp:254-257, :615-619) */
#define TWDIC_ERR_STATE (-4)        /* call order: e.g. compute before a reference image was set */
#define TWDIC_ERR_CUDA (-5)         /* a CUDA runtime call failed; see twdic_last_error() */
#define TWDIC_ERR_NO_MEMORY (-6)    /* device allocation failed or the HBM budget would be exceeded */
#define TWDIC_ERR_UNSUPPORTED (-7)  /* parameter outside the library's limits (e.g. subset radius > 31) */
#define TWDIC_ERR_TIMEOUT (-8)      /* a bounded device-side wait gave up */
#define TWDIC_ERR_BUSY (-9)         /* a serving stream's queue is full: the frame was dropped */
#define TWDIC_PENDING 1             /* twdic_poll: the frame is not done yet (not an error) */

#define TWDIC_MEM_HOST 0
#define TWDIC_MEM_DEVICE 1

/* Compute path.  PLAIN is the straightforward FP32 SIMT path (one CTA per
 * POI, per-reference steepest-descent images and per-frame bicubic LUT in
 * HBM).  FAST is the tensor-core / staged-window path (FP16 hi/lo DFT GEMMs on
 * tcgen05, FP64 Cholesky, on-chip interpolation). */
#define TWDIC_PATH_PLAIN 0
#define TWDIC_PATH_FAST 1

/* ICGN2DFlag (TW/TW_Engine/TW_paDIC.h:74-81) */
#define TWDIC_ICGN_SUCCESS 0
#define TWDIC_ICGN_DARK_SUBSET 1
#define TWDIC_ICGN_SINGULAR_HESSIAN 2
#define TWDIC_ICGN_SINGULAR_WARP 3
#define TWDIC_ICGN_OUT_OF_ROI 4

/* FFT-CC per-POI status */
#define TWDIC_FFTCC_OK 0
#define TWDIC_FFTCC_DARK_SUBSET 1 /* outputs of this POI are left untouched (TW_paDIC_FFTCC2D_CPU.cpp:272-275) */

/* Constructor parameters.  Field meaning follows the reference constructors:
 * Fftcc2D(imgW, imgH, startX, startY, roiW, roiH, subsetX, subsetY, gridX,
 * gridY, marginX, marginY) (TW/TW_Engine/TW_paDIC_FFTCC2D.h:38-43) and
 * ICGN2D_CPU/cuICGN2D(..., iNumIterations, fDeltaP, ...)
 * (TW/TW_Engine/TW_paDIC_ICGN2D_CPU.h:23-44, TW_paDIC_cuICGN2D.h:14-22). */
typedef struct twdic_params {
  int32_t img_width, img_height;  /* whole image */
  int32_t start_x, start_y;       /* ROI top-left */
  int32_t roi_width, roi_height;
  int32_t subset_x, subset_y;     /* half sizes r: FFT window 2r, IC-GN subset 2r+1 */
  int32_t grid_space_x, grid_space_y;
  int32_t margin_x, margin_y;
  int32_t max_iterations;         /* IC-GN iteration cap (callers use 20) */
  float delta_p;                  /* IC-GN convergence threshold on the scaled ||dP|| (callers use 0.001) */
  int32_t path;                   /* TWDIC_PATH_* */
} twdic_params;

/* Last error message of the calling thread (never NULL). */
TWDIC_API const char* twdic_last_error(void);
TWDIC_API int twdic_abi_version(void);

/* Number of POIs for a parameter set: NX = floor((roiW - 2 rX - 2 mX) / gX) + 1
 * (Fftcc2D::recomputeNumPOI, TW/TW_Engine/TW_paDIC_FFTCC2D.cpp:88-94). */
TWDIC_API int twdic_num_pois(const twdic_params* p, int32_t* num_x, int32_t* num_y);

/* POI grid (ComputePOIPositions_s/_m, TW/TW_Engine/TW_utils.cpp:29-94;
 * cuComputePOIPositions, TW/TW_Engine/TW_cuUtils.cu:83-134).  Host output,
 * num_x*num_y (y, x) pairs. */
TWDIC_API int twdic_poi_positions(const twdic_params* p, int32_t* poi_yx);

/* ------------------------------------------------------------- FFT-CC --- */
typedef struct twdic_fftcc twdic_fftcc;

/* cuFFTCC2D(imgW, imgH, roiW, roiH, startX, startY, ...) / Fftcc2D_CPU ctor
 * (TW/TW_Engine/TW_paDIC_cuFFTCC2D.cu:193-210, TW_paDIC_FFTCC2D_CPU.cpp:8-79)
 * plus cuInitializeFFTCC's allocations (TW_paDIC_cuFFTCC2D.cu:464-548). */
TWDIC_API int twdic_fftcc_create(const twdic_params* p, twdic_fftcc** out);
/* GetNumPOIsX / GetNumPOIsY (TW/TW_Engine/TW_paDIC_FFTCC2D.h:99-101) */
TWDIC_API int twdic_fftcc_num_pois(const twdic_fftcc* h, int32_t* num_x, int32_t* num_y);
/* The handle's device POI array (g_cuHandle.m_d_iPOIXY): copies it out. */
TWDIC_API int twdic_fftcc_poi_positions(const twdic_fftcc* h, int32_t* poi_yx, int mem);
/* ResetRefImg (TW/TW_Engine/TW_paDIC_cuFFTCC2D.cu:679-685) */
TWDIC_API int twdic_fftcc_reset_ref(twdic_fftcc* h, const uint8_t* img, int32_t stride, int mem);
/* SetTarImg (TW/TW_Engine/TW_paDIC_cuFFTCC2D.cu:687-693) */
TWDIC_API int twdic_fftcc_set_tar(twdic_fftcc* h, const uint8_t* img, int32_t stride, int mem);
/* ComputeFFTCC / cuComputeFFTCC on the current target
 * (TW/TW_Engine/TW_paDIC_cuFFTCC2D.cu:334-431, :550-647; CPU semantics of
 * TW_paDIC_FFTCC2D_CPU.cpp:222-326).  u, v, zncc: num_pois floats each.
 * status (may be NULL): num_pois bytes of TWDIC_FFTCC_*. */
TWDIC_API int twdic_fftcc_compute(twdic_fftcc* h, float* u, float* v, float* zncc, uint8_t* status, int mem);
/* DestroyFFTCC / cuDestroyFFTCC (TW/TW_Engine/TW_paDIC_cuFFTCC2D.cu:433-461, :649-677) */
TWDIC_API int twdic_fftcc_destroy(twdic_fftcc* h);

/* -------------------------------------------------------------- IC-GN --- */
typedef struct twdic_icgn twdic_icgn;

/* cuICGN2D(imgW, imgH, startX, startY, roiW, roiH, subsetX, subsetY,
 * numberX, numberY, iNumIterations, fDeltaP, Iflag) + prepare()
 * (TW/TW_Engine/TW_paDIC_cuICGN2D.cu:694-768); ICGN2D_CPU ctor
 * (TW_paDIC_ICGN2D_CPU.cpp:13-34).  num_x*num_y is the POI count of every
 * compute call. */
TWDIC_API int twdic_icgn_create(const twdic_params* p, int32_t num_x, int32_t num_y, twdic_icgn** out);
/* ResetRefImg / cuInitialize (TW/TW_Engine/TW_paDIC_cuICGN2D.cu:770-795;
 * TW_paDIC_ICGN2D_CPU.cpp:66-70).  The per-reference precompute runs on the
 * next compute call, and again on any later call whose POI contents differ
 * from the previous call's (host or device POIs alike: a device POI array is
 * read afresh on every call, so it may be rewritten in place between calls). */
TWDIC_API int twdic_icgn_reset_ref(twdic_icgn* h, const uint8_t* img, int32_t stride, int mem);
/* cuCompute (TW/TW_Engine/TW_paDIC_cuICGN2D.cu:811-968) with the CPU path's
 * semantics ICGN2D_Algorithm (TW_paDIC_ICGN2D_CPU.cpp:77-132, :481-925).
 *   tar     target image (mem_in)
 *   poi_yx  num_pois (y, x) pairs (mem_in)
 *   u, v    in/out: FFT-CC guesses in, sub-pixel displacements out (mem_out)
 *   p6      out (may be NULL): num_pois x (u, ux, uy, v, vx, vy)
 *   iters   in/out (may be NULL): iteration counter per POI; left unchanged
 *           for POIs that stop before their first solve, as the reference
 *   flags   out (may be NULL): TWDIC_ICGN_* per POI */
TWDIC_API int twdic_icgn_compute(twdic_icgn* h, const uint8_t* tar, int32_t stride, const int32_t* poi_yx, int mem_in,
                       float* u, float* v, float* p6, int32_t* iters, uint8_t* flags, int mem_out);
/* cuFinalize + destructor (TW/TW_Engine/TW_paDIC_cuICGN2D.cu:970-989) */
TWDIC_API int twdic_icgn_destroy(twdic_icgn* h);

/* --------------------------------------------------- fused frame path --- */
/* One frame of FFTCCTWorkerThread::processFrameFFTCC_ICGN's DIC work
 * (TW/TW_Core/fftcctworkerthread.cpp:399-481): cuComputeFFTCC then
 * cuICGN2D::cuCompute on the same target, with the reference cached. */
typedef struct twdic_frame twdic_frame;
TWDIC_API int twdic_frame_create(const twdic_params* p, twdic_frame** out);
TWDIC_API int twdic_frame_num_pois(const twdic_frame* h, int32_t* num_x, int32_t* num_y);
TWDIC_API int twdic_frame_poi_positions(const twdic_frame* h, int32_t* poi_yx, int mem);
TWDIC_API int twdic_frame_set_reference(twdic_frame* h, const uint8_t* img, int32_t stride, int mem);
/* Outputs (any may be NULL except u, v): zncc from FFT-CC, the IC-GN
 * deformation p6, iteration counts and flags. */
TWDIC_API int twdic_frame_process(twdic_frame* h, const uint8_t* tar, int32_t stride, int mem_in, float* u, float* v,
                        float* zncc, float* p6, int32_t* iters, uint8_t* flags, int mem_out);
/* Bind a handle to a CUDA stream (cudaStream_t passed as void*; NULL = the
 * handle's own stream).  All work of later calls is ordered on it. */
TWDIC_API int twdic_frame_set_stream(twdic_frame* h, void* stream);
/* Device time of the phases of the last process call, in milliseconds:
 * t[0] target upload, t[1] FFT-CC, t[2] target preparation, t[3] IC-GN,
 * t[4] result download, t[5] per-reference precompute (0 when cached). */
TWDIC_API int twdic_frame_phase_times(const twdic_frame* h, float* t6);
TWDIC_API int twdic_frame_destroy(twdic_frame* h);
/* The interpolation and gradient tables of the frame's current images, for
 * inspection, copied to host memory (dst: host floats).  The reference keeps
 * these as members of its IC-GN classes (ICGN2D_CPU::m_fRx, m_fRy,
 * m_fInterpolation, TW/TW_Engine/TW_paDIC_ICGN2D_CPU.h:113-125; cuICGN2D's
 * device buffers in GPUHandle_ICGN, TW/TW_Engine/TW_paDIC.h:40-70).
 *   TWDIC_TABLE_BICUBIC_LUT    roi_h x roi_w x 4 x 4: the target's bicubic LUT
 *       (BicubicCoefficients_s, TW/TW_Engine/TW_utils.cpp:604-700), [y][x][k][n]
 *       the coefficient of fy^k fx^n, last ROI row and column zero
 *   TWDIC_TABLE_BSPLINE_LUT    the same for the B-spline LUT
 *       (BicubicSplineCoefficients_s, TW_utils.cpp:521-602)
 *   TWDIC_TABLE_REF_GRADIENT   roi_h x roi_w x 2: (R_x, R_y) of the reference
 *       over the ROI, central differences (GradientXY_2Images_s,
 *       TW_utils.cpp:232-305), as the fast path keeps them (halves of
 *       integers below 128, exact in FP32)
 *   TWDIC_TABLE_SUBSET_GRADIENT num_pois x S x 2 (S = subset pixels, row
 *       major): (R_x, R_y) of every POI's subset as the plain path's
 *       per-reference cache keeps them (plain path handles only)
 * The LUTs need a target (a processed frame), the gradients a reference. */
#define TWDIC_TABLE_BICUBIC_LUT 0
#define TWDIC_TABLE_BSPLINE_LUT 1
#define TWDIC_TABLE_REF_GRADIENT 2
#define TWDIC_TABLE_SUBSET_GRADIENT 3
TWDIC_API int twdic_frame_table(twdic_frame* h, int which, float* dst);

/* IC-GN target interpolation, ICGN2DInterpolationFLag (TW/TW_Engine/TW_paDIC.h:89-93),
 * the Iflag of the ICGN2D_CPU / cuICGN2D constructors (TW_paDIC_ICGN2D_CPU.h:23-44):
 * TWDIC_INTERP_BICUBIC, the Hermite bicubic LUT (BicubicCoefficients_s,
 * TW_utils.cpp:604-700; the default), or TWDIC_INTERP_BSPLINE, the bicubic
 * B-spline LUT (BicubicSplineCoefficients_s, TW_utils.cpp:521-602; every ROI
 * pixel has coefficients, image pixels outside the image read as 0).  The fast
 * path evaluates either from the 16-byte neighbourhood table (the default
 * sampler) or from the coefficient LUT (sampler 1). */
#define TWDIC_INTERP_BICUBIC 0
#define TWDIC_INTERP_BSPLINE 1
TWDIC_API int twdic_icgn_set_interpolation(twdic_icgn* h, int mode);
TWDIC_API int twdic_frame_set_interpolation(twdic_frame* h, int mode);

/* Launch-shape tuning of a frame handle (no counterpart in the reference;
 * set by the autotuner).  icgn_threads: 32, 64, 128 or 256 threads per IC-GN CTA;
 * icgn_ctas_per_sm: persistent CTAs per SM (0 = occupancy limit);
 * icgn_sampler: target interpolation of the fast IC-GN, 0 = staged window,
 * 1 = per-frame bicubic coefficient LUT, 2 = per-frame 4x4 neighbourhood
 * table; fftcc_use_tc: 1 = tensor-core FFT-CC when available. */
TWDIC_API int twdic_frame_set_tuning(twdic_frame* h, int icgn_threads, int icgn_ctas_per_sm, int icgn_sampler,
                                     int fftcc_use_tc);
/* IC-GN work layout of the fast path.  chunk = 0: one POI per CTA (threads
 * 32 to 256).  chunk > 0: one POI per warp; the warps of a CTA (threads 128
 * to 1024, a table sampler) take POIs from runs of `chunk` consecutive POIs,
 * so the subsets in flight on an SM overlap and are re-read from L1, and the
 * reference gradients come from a per-reference image (8 B per ROI pixel). */
TWDIC_API int twdic_frame_set_icgn_layout(twdic_frame* h, int chunk);
/* Initial guesses of a frame handle in batched calls (twdic_batch_process and
 * the server): mode 0 (default) runs FFT-CC and starts IC-GN from its integer
 * displacements, as FFTCCTWorkerThread::processFrameFFTCC_ICGN does; mode 1
 * skips FFT-CC and starts IC-GN from the u, v arrays passed in (in/out, as
 * cuICGN2D::cuCompute's U, V), e.g. the previous frame's displacements of a
 * camera stream; ZNCC is then not written. */
TWDIC_API int twdic_frame_set_guess_mode(twdic_frame* h, int mode);
/* Unrolling of the IC-GN sample loop (2, 4 or 8; default 8) for the one-POI-per-warp
 * layout with 1024-thread CTAs (other shapes unroll by 4). */
TWDIC_API int twdic_frame_set_icgn_unroll(twdic_frame* h, int unroll);

/* FFT-CC tile of a frame handle: use_tc (tensor-core kernel), groups (0 = as
 * many 128-thread groups per CTA as fit, 1 to 5 = at most that many),
 * pois_per_group (POIs per group batch, 0 = the most the tiles hold).  No
 * reference counterpart. */
TWDIC_API int twdic_frame_set_fftcc_tuning(twdic_frame* h, int use_tc, int groups, int pois_per_group);
/* Twiddle precision of the tensor-core FFT-CC: hi_lo = 1 splits every twiddle
 * into FP16 hi + lo parts (two MMAs per product), 0 (the default) keeps the hi
 * part only.  The integer displacement and ZNCC are exact either way (the
 * candidates of the approximate surface are re-evaluated in integers); the
 * split only narrows the approximate surface's error (largest measured at a
 * candidate on a 2048x2048 frame, 41x41 subsets: 4.7e-4 with the split,
 * 8.9e-4 without, in ZNCC units, against a candidate window of 0.01). */
TWDIC_API int twdic_frame_set_fftcc_twiddles(twdic_frame* h, int hi_lo);

typedef struct {
    int32_t icgn_threads, icgn_ctas_per_sm, icgn_sampler;
    int32_t fftcc_use_tc, fftcc_groups, fftcc_pois_per_group;
    float fftcc_ms, icgn_ms; /* phase times of the chosen shapes (target preparation included in icgn_ms) */
    int32_t from_cache;      /* 1: read from the cache file, not measured */
    int32_t icgn_chunk;      /* IC-GN work layout (twdic_frame_set_icgn_layout) */
    int32_t icgn_unroll;     /* IC-GN sample-loop unrolling (twdic_frame_set_icgn_unroll) */
} twdic_tuning;
TWDIC_API int twdic_frame_get_tuning(const twdic_frame* h, twdic_tuning* out);
/* Autotuner (no reference counterpart): times the FFT-CC tile shapes and the
 * IC-GN launch shapes, samplers and sample-loop unrolling on this handle's reference and the given
 * target (one warm-up and three timed frames each, median), keeps the fastest
 * and returns it.  cache_path (may be NULL): a text file of earlier choices
 * keyed by GPU name, SM count and every geometry parameter; a hit is applied
 * without timing, a new choice is appended. */
TWDIC_API int twdic_frame_autotune(twdic_frame* h, const uint8_t* tar, int32_t stride, int mem,
                                   const char* cache_path, twdic_tuning* out);

/* ------------------------------------------- IC-GN without allocation --- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory when they run IC-GN: a real-time camera loop whose frame deadline
 * cannot absorb cudaMalloc's implicit device-wide synchronisation or an
 * out-of-memory failure mid-stream, or an application whose device memory is
 * budgeted up front by another allocator.  Runs the fast IC-GN path
 * (per-reference precompute, then the persistent IC-GN kernel) for one
 * target frame, with every buffer supplied by the caller and the path's
 * scratch (per-POI reference cache and work counter) held in a fixed-size
 * static device array inside the library: no cudaMalloc, cudaFree or
 * allocating library call.
 *   - at most TWDIC_NOALLOC_MAX_POIS POIs per call (larger counts return
 *     TWDIC_ERR_UNSUPPORTED); the array takes about 46 MB on every GPU that
 *     loads the library, until the process exits;
 *   - all pointers are device pointers: images as in twdic_icgn_compute
 *     (pitch = img_width), poi_yx 8-byte aligned, u/v/iters in-out, p6 and
 *     flags out, all num_pois long; the work is queued on `stream`
 *     (cudaStream_t as void*, NULL = legacy default stream) and the call
 *     returns without synchronising;
 *   - the bicubic interpolation (TWDIC_INTERP_BICUBIC), sampled from the
 *     target image itself (no per-frame table);
 *   - the reference precompute is redone on every call (no cache survives
 *     between calls); the array keeps the last call's contents, and the parts
 *     that must start at zero are cleared on the stream by each call;
 *   - every call shares the one array: calls whose GPU work overlaps (other
 *     streams, other host threads) race and corrupt each other's results --
 *     serialise them;
 *   - the parameters are checked as twdic_icgn_create checks them; the
 *     path must be TWDIC_PATH_FAST (TWDIC_ERR_UNSUPPORTED otherwise);
 *   - the first call on a device resolves the array's device address
 *     (cudaGetSymbolAddress, which may load the library's module on that
 *     device); make that first call before any stream capture.  The address
 *     is resolved again when another context is current on the device;
 *     cudaDeviceReset between calls is not supported (the new primary
 *     context may not be told apart from the old one). */
#define TWDIC_NOALLOC_MAX_POIS 196608
TWDIC_API int twdic_icgn_compute_noalloc(const twdic_params* p, const uint8_t* d_ref, const uint8_t* d_tar,
                                         const int32_t* d_poi_yx, int32_t num_pois, float* d_u, float* d_v,
                                         float* d_p6, int32_t* d_iters, uint8_t* d_flags, void* stream);

/* ---- batches (no reference counterpart) ----
 * Several frame handles' targets in one set of launches: one launch builds
 * every frame's per-frame table and zeroes its outputs, the fast-path frames
 * share one tensor-core FFT-CC launch (all window sizes) and one persistent
 * IC-GN launch (per interpolant; up to 128 frames per launch, larger batches
 * take several).  Image pairs and POI sets may differ
 * in size.  Results equal those of twdic_frame_process on each frame.  Each
 * frame appears at most once per call; frames must live on the current
 * device.  The batch's IC-GN launch shape (set_tuning) applies to all its
 * fast-path frames.
 *
 * Graph mode (set_graph(1)): a call with device inputs and outputs whose
 * frames and arrays equal the previous call's replays a CUDA graph captured
 * from that call (one cudaGraphLaunch; `*replayed` = 1).  Inputs are read
 * from the same device arrays, so the caller refreshes their contents
 * between calls. */
typedef struct twdic_batch twdic_batch;
TWDIC_API int twdic_batch_create(twdic_batch** out);
TWDIC_API int twdic_batch_set_stream(twdic_batch* b, void* stream);
TWDIC_API int twdic_batch_set_tuning(twdic_batch* b, int icgn_threads, int icgn_ctas_per_sm, int icgn_sampler);
/* IC-GN work layout of the batch's launches (twdic_frame_set_icgn_layout). */
TWDIC_API int twdic_batch_set_icgn_layout(twdic_batch* b, int chunk);
/* IC-GN sample-loop unrolling of the batch's launches (twdic_frame_set_icgn_unroll). */
TWDIC_API int twdic_batch_set_icgn_unroll(twdic_batch* b, int unroll);
TWDIC_API int twdic_batch_set_graph(twdic_batch* b, int enable);
/* Arrays of `count` entries; zncc, p6, iters, flags (the arrays) may be NULL,
 * strides may be NULL (contiguous images); replayed may be NULL. */
TWDIC_API int twdic_batch_process(twdic_batch* b, int32_t count, twdic_frame* const* frames,
                                  const uint8_t* const* tars, const int32_t* strides, int mem_in, float* const* u,
                                  float* const* v, float* const* zncc, float* const* p6, int32_t* const* iters,
                                  uint8_t* const* flags, int mem_out, int32_t* replayed);
/* Device time of the phases of the last batch call that ran without a graph
 * (the first of a graph-mode pair, or any call with graphs off), in
 * milliseconds: t[0] target copies and the preparation launch (tables,
 * zeroed outputs), t[1] FFT-CC, t[2] float LUTs (LUT sampler and plain
 * frames only), t[3] IC-GN. */
TWDIC_API int twdic_batch_phase_times(twdic_batch* b, float* t4);
TWDIC_API int twdic_batch_destroy(twdic_batch* b);

/* Device memory a frame handle with these parameters holds after its first
 * frame (fast path: images, POIs, outputs, per-reference cache, target
 * table; plain path likewise), rounded to allocation granules.  Host-only. */
TWDIC_API int twdic_frame_device_bytes(const twdic_params* p, uint64_t* bytes);

/* ---- serving (no reference counterpart) ----
 * Several camera streams of possibly different sizes.  Each stream keeps its
 * reference precompute and per-frame tables on the device; a stream is
 * admitted only while the device memory of all admitted streams stays within
 * hbm_budget_bytes (0 = 90 % of the free memory at creation).  twdic_submit
 * copies a target into one of the stream's queue_depth pinned slots, or drops
 * it with TWDIC_ERR_BUSY when all are taken (the reference's bounded frame
 * queue).  A scheduler thread batches the next pending frame of idle streams
 * (up to max_batch) into one twdic_batch launch on a free lane (CUDA stream,
 * up to `lanes` batches in flight), so frames that arrive while others are on
 * the GPU join the next batch.  By default (mix_sizes = 0) the frames are
 * taken in order of expected finish (submit time plus an estimate of the
 * frame's device time from its POI count) and a batch holds only frames
 * within a factor of two of its first frame's POI count; with mix_sizes = 1,
 * oldest first and any sizes.  Results equal
 * twdic_frame_process on the same frame.  twdic_poll returns TWDIC_PENDING
 * until the frame is done (wait = 1 blocks), then copies the results out and
 * frees the slot; latency_ms is submit-to-done.  A ticket is read once: a
 * second twdic_poll on it fails with TWDIC_ERR_INVALID_ARG (read) or
 * TWDIC_ERR_STATE (being read).  twdic_server_remove_stream waits for the
 * stream's batch in flight and for twdic_submit / twdic_poll copies into or
 * out of its slots, then drops its pending frames; a twdic_poll waiting on
 * one of them returns TWDIC_ERR_STATE. */
typedef struct twdic_server twdic_server;
typedef struct {
    uint64_t hbm_budget_bytes;
    int32_t max_batch;    /* 1..32 frames per batched launch */
    int32_t queue_depth;  /* 1..64 pending frames per stream */
    int32_t lanes;        /* 1..4 batches in flight */
    int32_t use_graph;    /* replay CUDA graphs when a stream mix repeats */
    int32_t start_paused; /* 1: hold frames until twdic_server_resume */
    int32_t icgn_threads; /* fast IC-GN launch shape (0 = default) */
    int32_t icgn_sampler; /* fast IC-GN target sampler when icgn_threads > 0 */
    int32_t mix_sizes;    /* 0 (default): a batch holds the oldest pending frame and the frames whose
                             POI count is within a factor of two of it; 1: frames of any size */
} twdic_server_config;
typedef struct {
    uint64_t submitted, completed, dropped, batches, batched_frames, graph_replays;
    uint64_t committed_bytes, budget_bytes;
    int32_t streams;
    double p50_ms, p99_ms, max_ms; /* submit-to-done latency over completed frames */
    uint64_t max_batch_formed;     /* frames in the largest batch launched */
    int32_t peak_lanes_in_flight;  /* most batches launched and not yet retired at one time */
    int32_t peak_device_batches;   /* most batches running on the device at one time */
    double device_busy_ms;         /* device time with a batch running (union of the batches'
                                      intervals, timed by CUDA events on their lanes) */
    double device_overlap_ms;      /* device time with two or more batches running */
} twdic_server_counters;
TWDIC_API int twdic_server_create(const twdic_server_config* cfg, twdic_server** out);
TWDIC_API int twdic_server_add_stream(twdic_server* s, const twdic_params* p, int32_t* stream_id);
TWDIC_API int twdic_server_remove_stream(twdic_server* s, int32_t stream_id);
TWDIC_API int twdic_server_set_reference(twdic_server* s, int32_t stream_id, const uint8_t* img, int32_t stride);
TWDIC_API int twdic_submit(twdic_server* s, int32_t stream_id, const uint8_t* tar, int32_t stride,
                           uint64_t* ticket);
TWDIC_API int twdic_poll(twdic_server* s, uint64_t ticket, int32_t wait, float* u, float* v, float* zncc,
                         float* p6, int32_t* iters, uint8_t* flags, double* latency_ms);
TWDIC_API int twdic_server_resume(twdic_server* s);
TWDIC_API int twdic_server_stats(twdic_server* s, twdic_server_counters* out);
/* One camera stream's statistics (FFTCCTWorkerThread::updateFPS,
 * TW/TW_Core/fftcctworkerthread.cpp:574-605): frames completed and dropped,
 * submit-to-done latency percentiles, and the reference's average processing
 * rate -- the integer mean of 1000 / (integer milliseconds between two
 * completed frames) over the last 32 frames, refreshed every 32 frames (0
 * until the first 32). */
typedef struct {
    uint64_t completed, dropped;
    int32_t average_fps;
    double p50_ms, p99_ms;
} twdic_stream_stats;
TWDIC_API int twdic_server_stream_stats(twdic_server* s, int32_t stream_id, twdic_stream_stats* out);
/* Last-frame guesses for one camera stream: mode 1 keeps each frame's
 * displacements on the device and starts the next frame's IC-GN from them,
 * skipping FFT-CC (ZNCC is not written); the first frame after
 * twdic_server_set_reference runs FFT-CC.  Mode 0 (default): FFT-CC every
 * frame, the reference's behaviour. */
TWDIC_API int twdic_server_set_stream_guess(twdic_server* s, int32_t stream_id, int mode);
TWDIC_API int twdic_server_destroy(twdic_server* s);

/* ---- tracking loop (FFTCCTWorkerThread::processFrameFFTCC /
 * processFrameFFTCC_ICGN, TW/TW_Core/fftcctworkerthread.cpp:219-330, :399-481;
 * TW/TW_Core/cuda_utils.cu:109-240) ----
 * One camera's frame sequence.  Frame k (counted from 1) with
 * (k - 1) % refresh_interval == 0 becomes the reference (the reference uses
 * 50); at such a frame after the first, the last frame's displacements are
 * added to the accumulated ones (cuAccumulateUV) and every POI moves by their
 * truncation, y += int(v), x += int(u) (cuUpdatePOIpos), held so that its
 * subset stays in the ROI.  Every frame runs FFT-CC, and IC-GN when
 * with_icgn, at the current POIs against the current reference.
 *   u, v        this frame's displacement at the current POIs (n floats each)
 *   acc_u/v     accumulated displacement of the current POIs (total = acc + u)
 *   poi_yx      current POI positions, (y, x) pairs
 *   flags       IC-GN flags (FFT-CC status without IC-GN)
 * Any output may be NULL. */
typedef struct twdic_tracker twdic_tracker;
TWDIC_API int twdic_tracker_create(const twdic_params* p, int32_t refresh_interval, int32_t with_icgn,
                                   twdic_tracker** out);
TWDIC_API int twdic_tracker_num_pois(const twdic_tracker* t, int32_t* n);
TWDIC_API int twdic_tracker_process(twdic_tracker* t, const uint8_t* img, int32_t stride, int mem_in, float* u,
                                    float* v, float* acc_u, float* acc_v, int32_t* poi_yx, uint8_t* flags,
                                    int mem_out);
/* constructTextImageFixedMinMax (TW/TW_Core/cuda_utils.cu:109-172) after the
 * last process call: each POI is drawn at its displayed position (current
 * POI + truncated displacement, cuAccumulatePOI) as a 3x3 block coloured by
 * its total displacement clamped to [min, max], into two ROI-sized RGBA
 * images (uint32, red in the lowest byte; a 256-entry jet map).  Pixels not
 * drawn keep their contents; pixels outside the ROI are skipped. */
TWDIC_API int twdic_tracker_colormap(twdic_tracker* t, uint32_t* tex_u, uint32_t* tex_v, float min_u, float max_u,
                                     float min_v, float max_v, int mem);
TWDIC_API int twdic_tracker_destroy(twdic_tracker* t);

#ifdef __cplusplus
}
#endif

#endif /* TW_DIC_H */
