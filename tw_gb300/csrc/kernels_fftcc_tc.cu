// Tensor-core FFT-CC: the per-POI 2D DFTs of Fftcc2D_CPU::ComputeFFTCC
// (TW_paDIC_FFTCC2D_CPU.cpp:222-326) as batched GEMMs on tcgen05.
//
// For an N x N window (N = 2r, no padding of the data: the correlation stays
// circular as in the reference), with w = exp(-2 pi i / N):
//   stage 1  Y[kx][y]  = sum_x f[y][x] w^(kx x)          kx <= N/2 (real input)
//   stage 2  F[kx][ky] = sum_y Y[kx][y] w^(ky y)
//   cross    C = conj(F) G / (||f-mean|| ||g-mean||), C[0][0] = 0 (mean removal)
//   stage 3  conj(Z[kx][v]) = sum_ky conj(C[kx][ky]) w^(ky v)   (the forward
//            matrices serve the inverse transform through the conjugate)
//   stage 4  c[v][u]  = sum_kx weight(kx) Re(Z[kx][v] w^(-kx u))  (c2r)
// so that c[v][u] is the correlation at the shift (u, v) = (x, y).  Stage 1
// runs along the window rows, which are contiguous in memory.
// Every stage is D[128 x n] += A[128 x k] B[k x n] with the data as A
// (rows = window rows / spectrum rows of several POIs, K-major in shared
// memory) and constant twiddle matrices as B (K-major), FP16 operands, FP32
// accumulators in tensor memory.  Twiddles are single FP16 by default, or
// split hi + lo (two MMAs per product); the data operands are single FP16.
// The resulting surface is accurate to ~1e-3 in ZNCC units, so the integer
// peak is then decided exactly: every shift within kCandZncc of the
// approximate maximum is re-evaluated as the exact integer correlation
// sum_x f(x) g(x + k) (whose order is the order of the mean-subtracted
// correlation), with the reference's first-maximum rule.
// ZNCC is the quotient of the exact integer sums, evaluated in FP32.
//
// Up to five groups of 128 threads (one warpgroup each, each with the TMEM
// columns of its widest accumulator: 96 up to N = 48, then 128, so five groups
// there and four above) per CTA, one CTA per SM, persistent over batches of
// POIs; thread 0
// of a group issues its MMAs, completion is signalled through an mbarrier
// (bounded wait), the epilogues read TMEM with tcgen05.ld.  The reference
// windows' spectra are computed once per reference (the per-reference pass)
// and read back by the per-frame pass, which transforms the target windows
// only.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <climits>
#include <cmath>
#include <memory>
#include <mutex>
#include <map>
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "dic_common.cuh"
#include "dic_kernels.h"

namespace twdic {

namespace {

constexpr int kThreads = 128;
constexpr int kCandChunk = 128;   // exact re-evaluations per pass (all POIs of a group batch)
constexpr int kMaxPB = 8;         // POIs per batch (upper bound)
constexpr int kMaxGroups = 5;     // 128-thread groups per CTA (upper bound; window sizes up to 48)
constexpr int kSegGroups = 4;     // groups per CTA of the larger windows and of the segmented kernel
// Candidate window of the approximate correlation surface, in ZNCC units.
// The exact peak lies within twice the surface's error of the approximate
// maximum; the largest error measured at any evaluated candidate on the
// 2048x2048 / r = 20 workload (155,236 POIs, FP16 operands, FP32
// accumulation) is 8.9e-4 with single FP16 twiddles and 4.7e-4 with hi + lo
// twiddles, so 0.01 keeps a margin of five or more.
constexpr float kCandZncc = 0.01f;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kTmemCols = 128;  // TMEM columns a group may use (its stride is the shape's tcols)
constexpr unsigned kWaitLimit = 1u << 24;

// The tensor maps of one image pair: boxes [N rows][uw bytes] holding the
// windows of a batch whose POIs lie on one POI row.
struct alignas(128) TcMaps {
    CUtensorMap ref_u, tar_u;
};
constexpr int kMaxTcJobs = kMaxTcJobsPerLaunch;  // image pairs per launch
constexpr int kMaxTcSegs = kMaxTcSegsScratch;    // window sizes per launch (N = 8 .. 64, even)

struct TcShape {
    int N, H, HP, NP, PB, tiles1, K4, groups;
    int tcols;      // TMEM columns per group (96 or 128): the widest accumulator of the four stages
    int uw, utoff;  // one-row boxes: width (0: none for this geometry) and the target box's offset
    int win_bytes;  // a group's window region
    int tiles4;  // 128-row tiles of the surface (stage 4)
    int FS;      // complex values per cached spectrum row: N rounded up to 4
    int NW4;  // 32-bit words per window row in the exact re-evaluation
    int lo;   // 1: twiddles as FP16 hi + lo (two MMAs per product), 0: hi only
    // shared twiddle tables
    int off_b1h, off_b1l, off_c2h, off_c2l, off_s2h, off_s2l, off_b4h, off_b4l, tab_bytes;
    // single-FP16 twiddles: the stage-2/3 matrices with K = (x, part) interleaved,
    // rows kx: [cos, sin] (real part of the product) and [-sin, cos] (imaginary)
    int off_w2re, off_w2im;
    // per-group operand regions, relative to the group's base
    int off_a13, off_a2, off_a4, off_win, group_bytes;
    // row-contiguous operands A2, A4 (row r at 16 r, 8-column chunk c at c lbo):
    // chunk strides, the chunks without data that the MMAs read [z lo, z hi)
    int lbo2, lbo4, z2lo, z2hi, z4lo, z4hi;
    int z2part, z4part;  // the first zeroed chunk holds data too
    int z4early;         // A4's zeroed chunks lie past A3: zeroed in epilogue 2
    int ks2;  // K steps (16) of stages 2 and 3: the data columns only
    int k3w;  // K width of A3's layout
    int smem_bytes;
};

// One image pair (job) of a launch: its images (TMA tensor maps in device
// memory, kept by the frame handle), POIs and outputs.  A launch's jobs are
// ordered by window size; a segment is a run of jobs of one window size.
struct TcJob {
    const TcMaps* maps;  // device copy of the job's tensor maps
    const uint8_t* ref;  // the images (windows of batches off one POI row are read from here)
    const uint8_t* tar;
    uint32_t* fspec;     // reference spectra [n][H][FS] FP16 pairs (per-reference cache)
    int2* fsum;          // reference windows' (sum f, sum f^2) [n]
    int uw;              // width of the one-row boxes (0: not used for this job)
    int utoff;           // offset of the target box in the window region (128-byte aligned)
    Geom g;
    const int2* poi;
    float* u;
    float* v;
    float* zncc;
    uint8_t* status;
    int n;            // POIs of the job
    int batch_begin;  // first batch index of the job within its segment
};
struct TcJobs {
    int njobs;
    int nbatch;  // batches of all jobs (one window size) or of the first segment
    TcJob job[kMaxTcJobs];
};
// A segment of a mixed-size launch: its shape, twiddle tables and jobs
// [job_lo, job_hi); CTAs [cta_begin, next segment's cta_begin) start on it.
struct TcSeg {
    TcShape s;
    const uint4* tables;
    int job_lo, job_hi;
    int nbatch;
    int shape;  // index of (NP, HP) in kTcShapes
    int cta_begin;
};
struct TcSegs {
    int nseg;
    TcSeg seg[kMaxTcSegs];
};
static_assert(sizeof(TcJobs) + sizeof(TcSegs) + 64 < 32000, "kernel parameters exceed the 32 KB limit");

struct PeakScratch {
    int cand[kCandChunk];
    int candS[kCandChunk];
};

__host__ __device__ __forceinline__ int kmaj(int r, int k, int K) {  // LBO 128 B, SBO 16*K B
    return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// ------------------------------------------------------------ PTX glue ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    // no-swizzle K-major descriptor: start>>4 [0,14), LBO>>4 [16,30), SBO>>4 [32,46), version 1 at bit 46
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__host__ __device__ constexpr uint32_t idesc_f16(int n, bool neg_b) {
    // kind::f16: D f32 (bit 4), A = B = f16, both K-major, N>>3 at bit 17, M>>4 at bit 24
    return (1u << 4) | ((neg_b ? 1u : 0u) << 14) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: returns false (and leaves the caller to abort) after kWaitLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (unsigned i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// 2D TMA box load (x must be a multiple of 16 bytes) completing on `bar`
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
// named barrier over the 128 threads of one group
__device__ __forceinline__ void group_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
__device__ __forceinline__ int group_sync_or(int id, int v) {
    int r;
    asm volatile("{\n .reg .pred p, q;\n setp.ne.s32 p, %2, 0;\n bar.red.or.pred q, %1, 128, p;\n selp.s32 %0, 1, 0, q;\n}\n"
                 : "=r"(r) : "r"(id), "r"(v) : "memory");
    return r;
}

// FP16 pair of two bytes of w (PRMT selector 0x4140: bytes 0, 1; 0x4342:
// bytes 2, 3): the halves 0x64bb are 1024 + bb, less 1024 exactly
__device__ __forceinline__ uint32_t bytes_h2(uint32_t w, uint32_t sel) {
    const uint32_t b = __byte_perm(w, 0x64646464u, sel);
    uint32_t r;
    asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(b), "r"(0x64006400u));
    return r;
}
// one aligned 32-bit word of shared memory
__device__ __forceinline__ uint32_t lds_u32(uint32_t a) {
    uint32_t v;
    asm("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a));
    return v;
}
// sum_{i < len} f[i] g[i] of two byte runs at any shared-memory addresses:
// aligned words, one load and one funnel shift per word of each run (the
// words past a run's end, up to 7 bytes, lie in the same region)
__device__ __forceinline__ unsigned dot_bytes_s(uint32_t fa, uint32_t ga, int len, unsigned acc) {
    const uint32_t fal = fa & ~3u, fsh = (fa & 3) * 8;
    const uint32_t gal = ga & ~3u, gsh = (ga & 3) * 8;
    uint32_t fp = lds_u32(fal), gp = lds_u32(gal);
    int i = 0;
#pragma unroll 4
    for (; i + 4 <= len; i += 4) {
        const uint32_t fn = lds_u32(fal + i + 4), gn = lds_u32(gal + i + 4);
        acc = __dp4a(__funnelshift_r(fp, fn, fsh), __funnelshift_r(gp, gn, gsh), acc);
        fp = fn;
        gp = gn;
    }
    if (i < len) {  // 1 to 3 bytes left
        const uint32_t fn = lds_u32(fal + i + 4), gn = lds_u32(gal + i + 4);
        const uint32_t m = 0xffffffffu >> (8 * (4 - (len - i)));
        acc = __dp4a(__funnelshift_r(fp, fn, fsh) & m, __funnelshift_r(gp, gn, gsh), acc);
    }
    return acc;
}
// 4 bytes from any shared-memory byte pointer derived from the dynamic
// shared buffer (two aligned words, funnel shift)
__device__ __forceinline__ uint32_t ld_unaligned_p(const uint8_t* a) {
    const unsigned mis = (unsigned)(reinterpret_cast<uintptr_t>(a) & 3);
    const uint32_t* w = reinterpret_cast<const uint32_t*>(a - mis);
    return __funnelshift_r(w[0], w[1], mis * 8u);
}
// order-preserving map of FP32 to unsigned, and back
__device__ __forceinline__ uint32_t f32_ord(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float f32_unord(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}

__device__ __forceinline__ uint32_t pack2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ void st_half(uint8_t* p, float v) { *reinterpret_cast<__half*>(p) = __float2half_rn(v); }

// ----------------------------------------------------------------- kernel --
// Each 128-thread group of a CTA runs its own batches (own operand region,
// TMEM columns, mbarriers and named barrier) and the groups share the twiddle
// tables, so one group's load and MMA latency overlaps other groups'
// epilogues.  A group's GEMM operands A1, A2, A3, A4 and its peak scratch
// share one region: each is written only after the MMA that reads the
// previous one has completed.

// Shared state of a CTA's groups (static shared memory).
struct TcCta {
    uint64_t mbar_mma[kMaxGroups];
    uint64_t mbar_tma[kMaxGroups][2];  // one per window slot
    uint32_t tmem_slot;
    int seg;
    int wsum[kMaxGroups][2 * kMaxPB][2];
    float sscale[kMaxGroups][kMaxPB];
    int sdark[kMaxGroups][kMaxPB];
    int cbase[kMaxGroups][kMaxPB];      // first candidate slot of each POI
    int cend[kMaxGroups][kMaxPB];       // one past its last
    int wtot[kMaxGroups][2][4];         // candidates per warp and surface tile
    uint32_t smaxv[kMaxGroups][kMaxPB];  // ordered value of the approximate peak
    // per window slot (a group's batch in work and the next one, staged
    // while the first runs): POIs, each window's (0, 0) (staged box or the
    // image), the windows' row stride, 1 when they are the staged boxes
    int2 spoi[kMaxGroups][2][kMaxPB];
    const uint8_t* wptr[kMaxGroups][2][2 * kMaxPB];
    int wrs[kMaxGroups][2];
    int wsm[kMaxGroups][2];
    int snext[kMaxGroups];
};

// The tensor maps of jobs [lo, hi): visible to the tensor-map proxy (they
// were written to device memory by copies) and prefetched.  Thread 0 of each
// group issues the group's TMA copies, so each such thread fences.
__device__ __forceinline__ void tc_acquire_maps(const TcJobs& J, int lo, int hi) {
    for (int j = lo; j < hi; ++j) {
        const TcMaps* m = J.job[j].maps;
        const CUtensorMap* mm[2] = {&m->ref_u, &m->tar_u};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                             reinterpret_cast<uint64_t>(mm[k]))
                         : "memory");
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(mm[k])) : "memory");
        }
    }
}

// The twiddle tables of one window size into the start of shared memory
// (every thread of the CTA takes part; the caller synchronises).
__device__ __forceinline__ void tc_load_tables(uint8_t* sm, const uint4* __restrict__ tables, int bytes) {
    uint4* dst = reinterpret_cast<uint4*>(sm);
    for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) dst[i] = tables[i];
    fence_async_smem();
}

// The batches of one group over jobs [job_lo, job_hi) of J, which share the
// window size of shape s: batch indices [first, nbatch) -- the group's first
// batch, then the next free one from `counter` plus `counter_base`, drawn by
// thread 0 one batch ahead.  The windows are double-buffered: while a batch
// runs, the next one's POIs are loaded and its windows are staged into the
// other slot (after the batch's stage-1 MMAs are issued), so a batch starts
// on windows already in shared memory.
// phase / tphase: the parities of the group's MMA mbarrier and of its two
// TMA mbarriers (bits 0 and 1), carried across calls.  Returns false after a
// bounded wait gave up (err set).
// REF: the per-reference pass -- stages 1 and 2 of the reference windows,
// whose spectra (scaled by sqrt(n2) / ||f - mean f||, FP16 pairs) and integer
// sums go to the job's cache.  Otherwise the per-frame pass: stages 1 and 2 of
// the target windows only, the reference spectra read from that cache.
// Zeros in the chunks of A4 (rows [0, rows)) that hold stage-4 K columns
// past the data.
__device__ __forceinline__ void zero_a4_padding(uint8_t* a4, const TcShape& s, int rows, int t) {
    for (int c = s.z4lo; c < s.z4hi; ++c)
        for (int r = t; r < rows; r += 128)
            *reinterpret_cast<uint4*>(a4 + c * s.lbo4 + r * 16) = make_uint4(0, 0, 0, 0);
}

template <int NP, int HP, bool MULTI, bool LO, bool REF>
__device__ __forceinline__ bool tc_group_batches(const TcJobs& J, const TcShape& s, int job_lo, int job_hi,
                                                 int nbatch, int first, int* counter, int counter_base,
                                                 unsigned* err, TcCta& cs, uint8_t* sm, uint32_t& phase,
                                                 uint32_t& tphase) {
    const int grp = threadIdx.x >> 7;
    const int t = threadIdx.x & 127, warp = t >> 5, lane = t & 31;
    const int bar_id = 1 + grp;
    const int N = s.N, H = s.H, PB = s.PB, K4 = s.K4;
    const int n2 = N * N;
    constexpr int K1 = NP;
    uint8_t* gbase = sm + s.tab_bytes + grp * s.group_bytes;
    // window slots 0 and 1, win_bytes apart: the two one-row TMA boxes,
    // reference at 0, target at utoff
    uint8_t* wwin = gbase + s.off_win;
    PeakScratch* ps = reinterpret_cast<PeakScratch*>(gbase + s.off_a13);
    uint64_t* mbar = &cs.mbar_mma[grp];
    const uint32_t tm = cs.tmem_slot + grp * s.tcols;
    const uint32_t tm_warp = tm + ((uint32_t)(warp * 32) << 16);
    const uint32_t gaddr = smem_u32(gbase);
    const uint32_t sbase = smem_u32(sm);
    const int FS = s.FS;  // cached spectrum: complex values per (POI, ky) row
    // the job (image pair, POI set) of a batch: batches of job j are
    // [batch_begin_j, batch_begin_j + ceil(n_j / PB))
    auto job_of = [&](int bt) {
        int jx = job_lo;
        if (MULTI) {
            while (jx + 1 < job_hi && bt >= J.job[jx + 1].batch_begin) ++jx;
        }
        return jx;
    };
    // POI t of a batch (t < PB), (-1, -1) past the job's POIs
    auto batch_poi = [&](int bt) {
        const TcJob& jx = J.job[job_of(bt)];
        const int bx0 = (bt - jx.batch_begin) * PB;
        return bx0 + t < jx.n ? jx.poi[bx0 + t] : make_int2(-1, -1);
    };
    // warp 1 (all its lanes): a batch's windows into slot sl2, its POIs
    // being in that slot.  When the POIs lie on one POI row, one [N][uw] TMA
    // box per image holds all the windows (x aligned down to 16 bytes);
    // otherwise (a batch across POI rows, POIs off the grid) the windows are
    // read from the images in global memory.  The per-frame pass also sends
    // the batch's cached reference spectra towards L2 (epilogue 2 reads them).
    // Warp 1 works while thread 0 issues the MMAs.
    auto stage_windows = [&](int bt, int sl2) {
        const TcJob& jx = J.job[job_of(bt)];
        const Geom& gx = jx.g;
        uint8_t* wbuf = wwin + sl2 * s.win_bytes;
        uint64_t* tb = &cs.mbar_tma[grp][sl2];
        const int2 pyx = lane < PB ? cs.spoi[grp][sl2][lane] : make_int2(-1, -1);
        const bool v = pyx.x >= 0;
        const int ymin = __reduce_min_sync(kFull, v ? pyx.x : INT_MAX);
        const int ymax = __reduce_max_sync(kFull, v ? pyx.x : INT_MIN);
        const int xmin = __reduce_min_sync(kFull, v ? pyx.y : INT_MAX);
        const int xmax = __reduce_max_sync(kFull, v ? pyx.y : INT_MIN);
        const int xau = (xmin - gx.rx) & ~15;
        const bool uni = jx.uw > 0 && ymin == ymax && xmax - gx.rx + N - xau <= jx.uw;
        if (lane == 0) {
            fence_async_smem();  // the slot's earlier generic reads come before the copies' writes
            if (uni) {
                const int y0 = ymin - gx.ry;
                mbar_expect_tx(tb, (uint32_t)(2 * N * jx.uw));
                tma_load_2d(wbuf, &jx.maps->ref_u, xau, y0, tb);
                tma_load_2d(wbuf + jx.utoff, &jx.maps->tar_u, xau, y0, tb);
            } else {
                mbar_expect_tx(tb, 0u);  // completes the phase: nothing to load
            }
            cs.wrs[grp][sl2] = uni ? jx.uw : gx.pitch;
            cs.wsm[grp][sl2] = uni ? 1 : 0;
            if (!REF) {
                const int bx0 = (bt - jx.batch_begin) * PB;
                const int np = min(PB, jx.n - bx0);
                asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(
                                 reinterpret_cast<uint64_t>(jx.fspec + (size_t)bx0 * H * FS)),
                             "r"((uint32_t)(np * H * FS * 4))
                             : "memory");
            }
        }
        if (lane < PB) {
            if (uni) {
                const int xo = v ? pyx.y - gx.rx - xau : 0;
                cs.wptr[grp][sl2][2 * lane] = wbuf + xo;
                cs.wptr[grp][sl2][2 * lane + 1] = wbuf + jx.utoff + xo;
            } else {
                const size_t o = v ? (size_t)(pyx.x - gx.ry) * gx.pitch + (pyx.y - gx.rx) : 0;
                cs.wptr[grp][sl2][2 * lane] = jx.ref + o;
                cs.wptr[grp][sl2][2 * lane + 1] = jx.tar + o;
            }
        }
    };
    // a bounded wait gave up: the error flag, and thread 0 lets the next
    // batch's copies (when staged) land before the group returns
    auto abort_group = [&](bool pending, int sl2) {
        if (t == 0) {
            atomicOr(err, kErrTimeout);
            if (pending) mbar_wait(&cs.mbar_tma[grp][sl2], (tphase >> sl2) & 1u);
        }
    };
    // prologue: the first batch staged in slot 0, the batch after it drawn
    // (published after a barrier: the caller's threads may still be reading
    // the first batch from snext)
    int cur = first, sl = 0, nxt = 0;
    if (cur >= nbatch) return true;
    if (t < PB) cs.spoi[grp][0][t] = batch_poi(cur);
    if (t == 0) nxt = counter_base + atomicAdd(counter, 1);
    group_sync(bar_id);
    if (warp == 1) stage_windows(cur, 0);
    if (t == 0) cs.snext[grp] = nxt;
    group_sync(bar_id);
    int nb = cs.snext[grp];
    while (cur < nbatch) {
        const int jj = job_of(cur);
        const TcJob& jb = J.job[jj];
        const Geom& g = jb.g;
        const int n_job = jb.n;
        const int b0 = (cur - jb.batch_begin) * PB;
        const bool have_next = nb < nbatch;
        // loads in flight through the window wait and the A1 build: the next
        // batch's POIs, this batch's reference window sums (per-frame pass)
        int2 npoi = make_int2(-1, -1), fsum = make_int2(0, 0);
        if (t < PB) {
            if (have_next) npoi = batch_poi(nb);
            if (!REF && b0 + t < n_job) fsum = jb.fsum[b0 + t];
        }
        if (t == 0) nxt = have_next ? counter_base + atomicAdd(counter, 1) : nbatch;  // the batch after nb
        if (t < 2 * kMaxPB * 2) (&cs.wsum[grp][0][0])[t] = 0;
        if (t < PB) cs.smaxv[grp][t] = 0u;
        // this batch's windows (staged one batch earlier)
        bool ok = mbar_wait(&cs.mbar_tma[grp][sl], (tphase >> sl) & 1u);
        tphase ^= 1u << sl;
        if (group_sync_or(bar_id, !ok)) { abort_group(false, sl ^ 1); return false; }

        // ---- phase L2: windows -> A1, exact FP16: row (POI, window row y),
        // K = window column x; the reference windows in the per-reference
        // pass, the target windows in the per-frame pass.  A thread reads its
        // row as aligned 32-bit words (one funnel shift per word for the
        // window's byte offset), makes FP16 of the bytes by PRMT (the half
        // 0x64bb is 1024 + bb) and one packed subtraction, and sums the bytes
        // and their squares by DP4A; integer sums per window by segmented
        // warp reductions.  Rows past the batch's windows are not written
        // (the rows of D1 they give are never read).
        for (int rr = t; rr < s.tiles1 * 128; rr += 128) {
            const int pw = rr / N, y = rr - pw * N;
            const int wi = 2 * pw + (REF ? 0 : 1);
            const bool inb = pw < PB;
            const bool data = inb && cs.spoi[grp][sl][pw].x >= 0;
            unsigned su = 0u, sq = 0u;
            if (inb) {
                const uint8_t* src = data ? cs.wptr[grp][sl][wi] + y * cs.wrs[grp][sl] : wwin;
                const unsigned sh = 8u * (unsigned)(reinterpret_cast<uintptr_t>(src) & 3);
                const uint32_t* ws = reinterpret_cast<const uint32_t*>(src - (sh >> 3));
                uint8_t* a1 = gbase + s.off_a13 + (rr >> 7) * (128 * K1 * 2) + kmaj(rr & 127, 0, K1);
                uint32_t lo = data ? ws[0] : 0u;
#pragma unroll
                for (int c = 0; c < K1 / 8; ++c) {
                    uint32_t w[2];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int j = 2 * c + h;  // bytes x = 4 j .. 4 j + 3
                        w[h] = 0u;
                        if (data && 4 * j < N) {
                            const uint32_t hi = ws[j + 1];
                            w[h] = __funnelshift_r(lo, hi, sh);
                            lo = hi;
                            if (4 * j + 4 > N) w[h] &= 0xffffffffu >> (8 * (4 * j + 4 - N));
                        }
                    }
                    su = __dp4a(w[0], 0x01010101u, su);
                    su = __dp4a(w[1], 0x01010101u, su);
                    sq = __dp4a(w[0], w[0], sq);
                    sq = __dp4a(w[1], w[1], sq);
                    *reinterpret_cast<uint4*>(a1 + c * 128) =
                        make_uint4(bytes_h2(w[0], 0x4140u), bytes_h2(w[0], 0x4342u), bytes_h2(w[1], 0x4140u),
                                   bytes_h2(w[1], 0x4342u));
                }
            }
            const int key = data ? wi : -1;
            const unsigned seg = __match_any_sync(kFull, key);
            const int gs = __reduce_add_sync(seg, (int)su), gq = __reduce_add_sync(seg, (int)sq);
            if (data && lane == __ffs(seg) - 1) {
                atomicAdd(&cs.wsum[grp][wi][0], gs);
                atomicAdd(&cs.wsum[grp][wi][1], gq);
            }
        }
        if (t < PB) {
            cs.spoi[grp][sl ^ 1][t] = npoi;  // the next batch's POIs, for its staging below
            if (!REF && b0 + t < n_job) {
                cs.wsum[grp][2 * t][0] = fsum.x;
                cs.wsum[grp][2 * t][1] = fsum.y;
            }
        }
        fence_async_smem();
        group_sync(bar_id);
        const bool pending = have_next;  // from here the next batch's copies may be in flight

        // ---- stage 1: D1[(w,y)][(part,kx)] = A1 * B1 (the real DFT along x)
        if (t == 0) {
            tc_fence_after();
            for (int tile = 0; tile < s.tiles1; ++tile) {
                const uint32_t a0 = gaddr + s.off_a13 + tile * (128 * K1 * 2);
                for (int kk = 0; kk < K1 / 16; ++kk) {
                    const uint64_t a = sdesc(a0 + kk * 256, 128, 16 * K1);
                    const uint64_t bh = sdesc(sbase + s.off_b1h + kk * 256, 128, 16 * K1);
                    const uint64_t bl = sdesc(sbase + s.off_b1l + kk * 256, 128, 16 * K1);
                    mma_f16(tm + tile * 2 * HP, a, bh, idesc_f16(2 * HP, false), kk > 0);
                    if (LO) mma_f16(tm + tile * 2 * HP, a, bl, idesc_f16(2 * HP, false), 1);
                }
            }
            mma_commit(mbar);
        }
        if (warp == 1 && have_next) stage_windows(nb, sl ^ 1);  // slot sl ^ 1 was last read by the previous batch
        // per-POI normalisation while the MMAs run: nf = n sum (f - mean)^2 =
        // n sum f^2 - (sum f)^2, exact in integers (likewise ng); the scale of
        // the cached reference spectrum is sqrt(n) / sqrt(nf), of the target's
        // sqrt(n) / sqrt(ng), so the cross power is n / sqrt(nf ng) conj(F) G
        if (t < PB) {
            const int wf = 2 * t, wg = 2 * t + 1;
            const long long numf = (long long)n2 * cs.wsum[grp][wf][1] - (long long)cs.wsum[grp][wf][0] * cs.wsum[grp][wf][0];
            const long long numg = (long long)n2 * cs.wsum[grp][wg][1] - (long long)cs.wsum[grp][wg][0] * cs.wsum[grp][wg][0];
            const bool dark = b0 + t >= n_job || numf == 0 || (!REF && numg == 0);
            cs.sdark[grp][t] = dark ? 1 : 0;
            cs.sscale[grp][t] = dark ? 0.f : sqrtf((float)n2) * rsqrtf((float)(REF ? numf : numg));
        }
        ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        if (group_sync_or(bar_id, !ok)) { abort_group(pending, sl ^ 1); return false; }
        tc_fence_after();

        // ---- epilogue 1: D1 -> A2 (rows (p, kx); K = (y, part) interleaved
        // with single twiddles, so that a row's Re and Im of one y are one
        // 32-bit store; K = (part, y) with split ones), FP16.  A2 is
        // row-contiguous per 8-column chunk: a thread's rows (p, kx),
        // kx = 0 .. H-1, are 16 bytes apart.  Columns of the stage-2 K past
        // the data are zero: the chunks they lie in are zeroed row by row
        // first (a chunk holding data too, only when N % 4 = 2, then waits
        // for the zeros before its data).  A2 overwrites A1 (the region is
        // shared; stage 1 has completed).
        {
            const int LB2 = s.lbo2;
            uint8_t* a2 = gbase + s.off_a2;
            const int rows = PB * H;
            for (int c = s.z2lo; c < s.z2hi; ++c)
                for (int r = t; r < rows; r += 128) {
                    *reinterpret_cast<uint4*>(a2 + c * LB2 + r * 16) = make_uint4(0, 0, 0, 0);
                    if (LO) *reinterpret_cast<uint4*>(a2 + (NP / 8 + c) * LB2 + r * 16) = make_uint4(0, 0, 0, 0);
                }
            if (s.z2part) group_sync(bar_id);
            for (int tile = 0; tile < s.tiles1; ++tile) {
                const int rr = tile * 128 + t;
                const int p = rr / N, y = rr - p * N;
                const bool data = p < PB;
                uint8_t* rowp = a2 + (data ? p * H : 0) * 16 +
                                (LO ? (y >> 3) * LB2 + (y & 7) * 2 : (y >> 2) * LB2 + (y & 3) * 4);
                uint8_t* rowi = a2 + (data ? p * H : 0) * 16 + ((NP + y) >> 3) * LB2 + ((NP + y) & 7) * 2;
                // TMEM reads three 8-column chunks at a time, one wait each
#pragma unroll
                for (int cb = 0; cb < HP; cb += 24) {
                    float dre[24], dim[24];
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        if (cb + 8 * q < HP) {
                            tmem_ld8(tm_warp + tile * 2 * HP + cb + 8 * q, dre + 8 * q);
                            tmem_ld8(tm_warp + tile * 2 * HP + HP + cb + 8 * q, dim + 8 * q);
                        }
                    }
                    tmem_ld_wait();
                    if (data) {
#pragma unroll
                        for (int j = 0; j < 24; ++j) {
                            const int ky = cb + j;
                            if (ky < HP && ky < H) {
                                if (LO) {
                                    st_half(rowp + ky * 16, dre[j]);
                                    st_half(rowi + ky * 16, dim[j]);
                                } else {
                                    *reinterpret_cast<uint32_t*>(rowp + ky * 16) = pack2(dre[j], dim[j]);
                                }
                            }
                        }
                    }
                }
            }
        }
        tc_fence_before();
        fence_async_smem();
        group_sync(bar_id);

        // ---- stage 2: F = Y * W (rows (p,kx); columns Re ky | Im ky), K
        // steps over the data columns only
        if (t == 0) {
            tc_fence_after();
            const int LB2 = s.lbo2;
            const uint32_t a2 = gaddr + s.off_a2;
            if (!LO) {
                // K = (y, part) interleaved: one MMA per output part and K step
                for (int kk = 0; kk < s.ks2; ++kk) {
                    const uint64_t a = sdesc(a2 + 2 * kk * LB2, LB2, 128);
                    const uint64_t wr = sdesc(sbase + s.off_w2re + kk * 256, 128, 32 * NP);
                    const uint64_t wi = sdesc(sbase + s.off_w2im + kk * 256, 128, 32 * NP);
                    mma_f16(tm, a, wr, idesc_f16(NP, false), kk > 0);       // Re = Yr cos + Yi sin
                    mma_f16(tm + NP, a, wi, idesc_f16(NP, false), kk > 0);  // Im = -Yr sin + Yi cos
                }
            }
            for (int kk = 0; LO && kk < s.ks2; ++kk) {
                const uint64_t ar = sdesc(a2 + 2 * kk * LB2, LB2, 128);
                const uint64_t ai = sdesc(a2 + (NP / 8 + 2 * kk) * LB2, LB2, 128);
                const uint64_t ch = sdesc(sbase + s.off_c2h + kk * 256, 128, 16 * NP);
                const uint64_t cl = sdesc(sbase + s.off_c2l + kk * 256, 128, 16 * NP);
                const uint64_t sh = sdesc(sbase + s.off_s2h + kk * 256, 128, 16 * NP);
                const uint64_t sl = sdesc(sbase + s.off_s2l + kk * 256, 128, 16 * NP);
                const uint32_t acc = kk > 0;
                mma_f16(tm, ar, ch, idesc_f16(NP, false), acc);  // Re = Yr cos + Yi sin
                if (LO) mma_f16(tm, ar, cl, idesc_f16(NP, false), 1);
                mma_f16(tm, ai, sh, idesc_f16(NP, false), 1);
                if (LO) mma_f16(tm, ai, sl, idesc_f16(NP, false), 1);
                mma_f16(tm + NP, ar, sh, idesc_f16(NP, true), acc);  // Im = -Yr sin + Yi cos
                if (LO) mma_f16(tm + NP, ar, sl, idesc_f16(NP, true), 1);
                mma_f16(tm + NP, ai, ch, idesc_f16(NP, false), 1);
                if (LO) mma_f16(tm + NP, ai, cl, idesc_f16(NP, false), 1);
            }
            mma_commit(mbar);
        }
        // row t of the spectra is (p, kx); in the per-frame pass the cached
        // reference row is read from L2 while stage 2 runs (with split
        // twiddles chunk by chunk in epilogue 2: registers)
        const bool rowv2 = t < PB * H;
        const int p2 = rowv2 ? t / H : 0, ky2 = rowv2 ? t - p2 * H : 0;
        const bool live2 = rowv2 && !REF && !cs.sdark[grp][p2];
        const uint4* frow = reinterpret_cast<const uint4*>(jb.fspec + ((size_t)(live2 ? b0 + p2 : 0) * H + ky2) * FS);
        uint4 fr[LO ? 1 : NP / 4];
        if (!REF && !LO) {
#pragma unroll
            for (int i = 0; i < (LO ? 1 : NP / 4); ++i)
                fr[i] = (live2 && 4 * i < FS) ? __ldg(frow + i) : make_uint4(0u, 0u, 0u, 0u);
        }
        ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        if (group_sync_or(bar_id, !ok)) { abort_group(pending, sl ^ 1); return false; }
        tc_fence_after();

        if (REF) {
            // ---- the reference spectra to the cache: row (p, kx) of FS FP16
            // pairs (Re, Im), scaled by sqrt(n2) / ||f - mean f|| (zero for a
            // dark subset), ky >= N zero; then the windows' integer sums
            const bool live = rowv2 && b0 + p2 < n_job;
            const float sc = live ? cs.sscale[grp][p2] : 0.f;
            uint4* dst = reinterpret_cast<uint4*>(jb.fspec + ((size_t)(live ? b0 + p2 : 0) * H + ky2) * FS);
#pragma unroll
            for (int c = 0; c < NP; c += 8) {
                float re[8], im[8];
                tmem_ld8(tm_warp + c, re);
                tmem_ld8(tm_warp + NP + c, im);
                tmem_ld_wait();
                uint32_t w[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) w[i] = (c + i < N) ? pack2(re[i] * sc, im[i] * sc) : 0u;
                if (live && c < FS) {
                    dst[c >> 2] = make_uint4(w[0], w[1], w[2], w[3]);
                    if (c + 8 <= FS) dst[(c >> 2) + 1] = make_uint4(w[4], w[5], w[6], w[7]);
                }
            }
            if (t < PB && b0 + t < n_job) jb.fsum[b0 + t] = make_int2(cs.wsum[grp][2 * t][0], cs.wsum[grp][2 * t][1]);
            tc_fence_before();
            if (t == 0) cs.snext[grp] = nxt;
            group_sync(bar_id);
            cur = nb;
            nb = cs.snext[grp];
            sl ^= 1;
            continue;
        }

        // ---- epilogue 2: cross power C = conj(F) G * scale -> A3 = conj(C),
        // F the cached reference spectrum, G the target's from TMEM; row t of
        // A3 is (p, kx) = t.  Columns ky >= N within the stage-3 K are zero;
        // rows past the data are not written (the rows of D3 they give are
        // never read)
        {
            if (s.z4early) zero_a4_padding(gbase + s.off_a4, s, PB * N, t);
            const float sc = live2 ? cs.sscale[grp][p2] : 0.f;
            const int K3 = s.k3w;
            uint8_t* a3 = gbase + s.off_a13;
#pragma unroll
            for (int c = 0; c < NP; c += 8) {
                if (c >= N) break;  // past the data (split twiddles: zero chunks below)
                float gr[8], gi[8];
                tmem_ld8(tm_warp + c, gr);
                tmem_ld8(tm_warp + NP + c, gi);
                tmem_ld_wait();
                uint4 fa, fb;
                if (LO) {
                    fa = (live2 && c < FS) ? __ldg(frow + (c >> 2)) : make_uint4(0u, 0u, 0u, 0u);
                    fb = (live2 && c + 8 <= FS) ? __ldg(frow + (c >> 2) + 1) : make_uint4(0u, 0u, 0u, 0u);
                } else {
                    fa = fr[LO ? 0 : c >> 2];
                    fb = fr[LO ? 0 : (c >> 2) + 1];
                }
                const uint32_t fw[8] = {fa.x, fa.y, fa.z, fa.w, fb.x, fb.y, fb.z, fb.w};
                float br[8], bi[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&fw[i]));
                    const int kx = c + i;
                    float cr = (f.x * gr[i] + f.y * gi[i]) * sc;
                    float ci = (f.x * gi[i] - f.y * gr[i]) * sc;
                    if (kx >= N || (ky2 == 0 && kx == 0)) { cr = 0.f; ci = 0.f; }
                    br[i] = cr;
                    bi[i] = -ci;  // conj(C) feeds the forward matrices of stage 3
                }
                if (rowv2) {
                    uint4 q;
                    if (LO) {  // K = (part, ky)
                        q.x = pack2(br[0], br[1]); q.y = pack2(br[2], br[3]);
                        q.z = pack2(br[4], br[5]); q.w = pack2(br[6], br[7]);
                        *reinterpret_cast<uint4*>(a3 + kmaj(t, c, K3)) = q;
                        q.x = pack2(bi[0], bi[1]); q.y = pack2(bi[2], bi[3]);
                        q.z = pack2(bi[4], bi[5]); q.w = pack2(bi[6], bi[7]);
                        *reinterpret_cast<uint4*>(a3 + kmaj(t, NP + c, K3)) = q;
                    } else {  // K = (ky, part) interleaved
                        q.x = pack2(br[0], bi[0]); q.y = pack2(br[1], bi[1]);
                        q.z = pack2(br[2], bi[2]); q.w = pack2(br[3], bi[3]);
                        *reinterpret_cast<uint4*>(a3 + kmaj(t, 2 * c, K3)) = q;
                        q.x = pack2(br[4], bi[4]); q.y = pack2(br[5], bi[5]);
                        q.z = pack2(br[6], bi[6]); q.w = pack2(br[7], bi[7]);
                        *reinterpret_cast<uint4*>(a3 + kmaj(t, 2 * c + 8, K3)) = q;
                    }
                }
            }
            // split twiddles: whole chunks of each part block past the data
            // within the stage-3 K
            if (LO && rowv2) {
                for (int c = (N + 7) & ~7; c < 16 * s.ks2; c += 8) {
                    *reinterpret_cast<uint4*>(a3 + kmaj(t, c, K3)) = make_uint4(0, 0, 0, 0);
                    *reinterpret_cast<uint4*>(a3 + kmaj(t, NP + c, K3)) = make_uint4(0, 0, 0, 0);
                }
            }
        }
        tc_fence_before();
        fence_async_smem();
        group_sync(bar_id);

        // ---- stage 3: conj(Z) = conj(C) * W (rows (p,kx); columns Re v | Im v)
        if (t == 0) {
            tc_fence_after();
            const int K3 = s.k3w;
            if (!LO) {
                for (int kk = 0; kk < s.ks2; ++kk) {
                    const uint64_t a = sdesc(gaddr + s.off_a13 + kk * 256, 128, 16 * K3);
                    const uint64_t wr = sdesc(sbase + s.off_w2re + kk * 256, 128, 32 * NP);
                    const uint64_t wi = sdesc(sbase + s.off_w2im + kk * 256, 128, 32 * NP);
                    mma_f16(tm, a, wr, idesc_f16(NP, false), kk > 0);
                    mma_f16(tm + NP, a, wi, idesc_f16(NP, false), kk > 0);
                }
            }
            for (int kk = 0; LO && kk < s.ks2; ++kk) {
                const uint64_t ar = sdesc(gaddr + s.off_a13 + kk * 256, 128, 16 * K3);
                const uint64_t ai = sdesc(gaddr + s.off_a13 + (NP / 8 + 2 * kk) * 128, 128, 16 * K3);
                const uint64_t ch = sdesc(sbase + s.off_c2h + kk * 256, 128, 16 * NP);
                const uint64_t cl = sdesc(sbase + s.off_c2l + kk * 256, 128, 16 * NP);
                const uint64_t sh = sdesc(sbase + s.off_s2h + kk * 256, 128, 16 * NP);
                const uint64_t sl = sdesc(sbase + s.off_s2l + kk * 256, 128, 16 * NP);
                const uint32_t acc = kk > 0;
                mma_f16(tm, ar, ch, idesc_f16(NP, false), acc);
                if (LO) mma_f16(tm, ar, cl, idesc_f16(NP, false), 1);
                mma_f16(tm, ai, sh, idesc_f16(NP, false), 1);
                if (LO) mma_f16(tm, ai, sl, idesc_f16(NP, false), 1);
                mma_f16(tm + NP, ar, sh, idesc_f16(NP, true), acc);
                if (LO) mma_f16(tm + NP, ar, sl, idesc_f16(NP, true), 1);
                mma_f16(tm + NP, ai, ch, idesc_f16(NP, false), 1);
                if (LO) mma_f16(tm + NP, ai, cl, idesc_f16(NP, false), 1);
            }
            mma_commit(mbar);
        }
        ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        if (group_sync_or(bar_id, !ok)) { abort_group(pending, sl ^ 1); return false; }
        tc_fence_after();

        // ---- epilogue 3: D3 -> A4 (rows (p, v), K = (kx, part) interleaved:
        // k = 2 kx + part, so a POI row's Re and Im of one kx are one 32-bit
        // store), c2r weights folded in.  A4 is row-contiguous per chunk like
        // A2: a thread's rows (p, v), v = 0 .. N-1, are 16 bytes apart.  The
        // chunks holding columns past the data are zeroed first: in
        // epilogue 2 when A3 does not reach them, else here, and a chunk
        // holding data too then waits for the zeros.  A4 overwrites A3
        // (stage 3 has completed)
        {
            const int LB4 = s.lbo4;
            uint8_t* a4 = gbase + s.off_a4;
            if (!s.z4early) {
                zero_a4_padding(a4, s, PB * N, t);
                if (s.z4part) group_sync(bar_id);
            }
            const bool rowv = t < PB * H;
            const int p = rowv ? t / H : 0, ky = rowv ? t - (t / H) * H : 0;
            const float wgt = (ky == 0 || 2 * ky == N) ? 1.f : 2.f;
            uint8_t* rowp = a4 + (p * N) * 16 + (ky >> 2) * LB4 + (ky & 3) * 4;
            // TMEM reads three 8-column chunks at a time, one wait each
            // (columns N .. NP-1 are padding)
#pragma unroll
            for (int cb = 0; cb < NP; cb += 24) {
                if (cb >= N) break;
                float re[24], im[24];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    if (cb + 8 * q < NP) {
                        tmem_ld8(tm_warp + cb + 8 * q, re + 8 * q);
                        tmem_ld8(tm_warp + NP + cb + 8 * q, im + 8 * q);
                    }
                }
                tmem_ld_wait();
                if (rowv) {
#pragma unroll
                    for (int j = 0; j < 24; ++j) {
                        const int x = cb + j;
                        if (x < NP && x < N) {
                            // Zi = -D_i
                            *reinterpret_cast<uint32_t*>(rowp + x * 16) = pack2(wgt * re[j], -wgt * im[j]);
                        }
                    }
                }
            }
        }
        tc_fence_before();
        fence_async_smem();
        group_sync(bar_id);

        // ---- stage 4: c[(p,v)][u] = A4 * B4 (the c2r inverse along kx)
        if (t == 0) {
            tc_fence_after();
            const int LB4 = s.lbo4;
            for (int tile = 0; tile < s.tiles4; ++tile) {
                for (int kk = 0; kk < K4 / 16; ++kk) {
                    const uint64_t a = sdesc(gaddr + s.off_a4 + tile * 2048 + 2 * kk * LB4, LB4, 128);
                    const uint64_t bh = sdesc(sbase + s.off_b4h + kk * 256, 128, 16 * K4);
                    const uint64_t bl = sdesc(sbase + s.off_b4l + kk * 256, 128, 16 * K4);
                    mma_f16(tm + tile * NP, a, bh, idesc_f16(NP, false), kk > 0);
                    if (LO) mma_f16(tm + tile * NP, a, bl, idesc_f16(NP, false), 1);
                }
            }
            mma_commit(mbar);
        }
        ok = mbar_wait(mbar, phase);
        phase ^= 1u;
        if (group_sync_or(bar_id, !ok)) { abort_group(pending, sl ^ 1); return false; }
        tc_fence_after();

        // ---- epilogue 4: approximate peak, candidates, exact re-evaluation
        // (scratch in the shared operand region, which stage 4 has finished
        // reading; the surface stays in TMEM and is read twice in chunks).
        // Thread t holds surface row R = 128 k + t of tile k (R = p N + v:
        // POI p, y shift v, the values over the x shift u in the row's TMEM
        // columns)
        const int ntile = s.tiles4;
        if (t < kCandChunk) ps->candS[t] = 0;
        // approximate peak value per POI: each thread's maximum over y of its
        // rows, then a segmented warp reduction and one shared atomic per warp
        // segment, tile by tile
        float bvk[2] = {-3.4e38f, -3.4e38f};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (k >= ntile) break;
            const int R = 128 * k + t;
            const bool rowv = R < PB * N;
            const int p4 = rowv ? R / N : 0;
            const bool live = rowv && !cs.sdark[grp][p4];
            float bv = -3.4e38f;
#pragma unroll
            for (int y0 = 0; y0 < NP; y0 += 8) {
                if (y0 >= N) break;  // padding columns
                float cv[8];
                tmem_ld8(tm_warp + k * NP + y0, cv);
                tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (live && y0 + j < N && cv[j] > bv) bv = cv[j];
            }
            const unsigned seg = __match_any_sync(kFull, live ? p4 : -1);
            const uint32_t ov = __reduce_max_sync(seg, f32_ord(bv));
            if (live && lane == __ffs(seg) - 1) atomicMax(&cs.smaxv[grp][p4], ov);
            bvk[k] = bv;
        }
        group_sync(bar_id);
        // candidates: every shift within kCandZncc (ZNCC units; the surface is
        // N^2 ZNCC) of the approximate peak, the peak itself included, as one
        // bit per y of each row; a warp with no such row skips the second read
        uint64_t cmk[2] = {0ull, 0ull};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (k >= ntile) break;
            const int R = 128 * k + t;
            const bool rowv = R < PB * N;
            const int p4 = rowv ? R / N : 0;
            const bool live = rowv && !cs.sdark[grp][p4];
            const float th = live ? f32_unord(cs.smaxv[grp][p4]) - kCandZncc * (float)n2 : 3.4e38f;
            if (__any_sync(kFull, live && bvk[k] >= th)) {
                uint64_t m = 0ull;
#pragma unroll
                for (int y0 = 0; y0 < NP; y0 += 8) {
                    if (y0 >= N) break;  // padding columns
                    float cv[8];
                    tmem_ld8(tm_warp + k * NP + y0, cv);
                    tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        if (live && y0 + j < N && cv[j] >= th) m |= 1ull << (y0 + j);
                }
                cmk[k] = m;
            }
        }
        tc_fence_before();
        // candidate slots in row order (R, then y) by group-wide exclusive
        // scans of the per-row counts, tile 0 first; a POI's rows are
        // consecutive, so POI p owns the slots [cbase[p], cend[p])
        int exk[2] = {0, 0}, cnk[2] = {0, 0}, ink[2] = {0, 0};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            cnk[k] = __popcll(cmk[k]);
            int incl = cnk[k];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int up = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += up;
            }
            ink[k] = incl;
            if (lane == 31) cs.wtot[grp][k][warp] = incl;
        }
        group_sync(bar_id);
        int total = 0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            int wpre = 0, tk = 0;
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const int tw = cs.wtot[grp][k][w];
                wpre += (w < warp) ? tw : 0;
                tk += tw;
            }
            exk[k] = total + wpre + ink[k] - cnk[k];
            total += tk;
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (k >= ntile) break;
            const int R = 128 * k + t;
            if (R < PB * N) {
                const int p4 = R / N, x4 = R - p4 * N;
                if (x4 == 0) cs.cbase[grp][p4] = exk[k];
                if (x4 == N - 1) cs.cend[grp][p4] = exk[k] + cnk[k];
            }
        }
        // exact integer correlation of every candidate, kCandChunk slots at a
        // time (any number of candidates: a broad or periodic surface only
        // takes more chunks), read from the windows: tasks (slot, row) over
        // the group's threads, four products per DP4A, one shared atomic per
        // task (windows read from the images: lanes walk the words of their
        // row in a lane-rotated order).  Thread t < PB keeps POI t's best candidate: the
        // largest exact sum, the smallest index among equal sums (the
        // reference's first maximum), whatever the chunking.
        int best_s = INT_MIN, best_i = 0;
        for (int lo = 0; lo < total; lo += kCandChunk) {
            if (lo > 0) {
                group_sync(bar_id);  // the previous chunk's sums have been read
                if (t < kCandChunk) ps->candS[t] = 0;
            }
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (cnk[k] > 0 && exk[k] < lo + kCandChunk && exk[k] + cnk[k] > lo) {
                    const int R = 128 * k + t;
                    const int p4 = R / N, x4 = R - p4 * N;
                    uint64_t m = cmk[k];
                    for (int q = exk[k]; m != 0; ++q) {
                        const int y = __ffsll((long long)m) - 1;
                        m &= m - 1;
                        // POI, y shift v (the row x4), x shift u (the bit y)
                        if (q >= lo && q < lo + kCandChunk) ps->cand[q - lo] = (p4 << 16) | (x4 << 8) | y;
                    }
                }
            }
            group_sync(bar_id);
            const int nc = min(total - lo, kCandChunk);
            {
                const int NW4 = s.NW4;
                const uint32_t tail = (N & 3) ? (0xffffffffu >> (8 * (4 - (N & 3)))) : 0xffffffffu;
                const int rot = lane % NW4;
                const int rs = cs.wrs[grp][sl];
                const bool wsm = cs.wsm[grp][sl] != 0;
                // task (c, y) = y nc + c for thread t, stepped by 128: a
                // warp's lanes take the candidates of one row side by side
                // (windows of different POIs: their rows fall in different
                // banks), one shared atomic per task
                const int dy = 128 / nc, dc = 128 - dy * nc;
                int y = t / nc, c = t - (t / nc) * nc;
                for (; y < N;) {
                    unsigned acc0 = 0u, acc1 = 0u;
                    {
                        const int code = ps->cand[c];
                        const int p = code >> 16, ky = (code >> 8) & 0xff, kx = code & 0xff;
                        int yy = y + ky;
                        if (yy >= N) yy -= N;
                        int j = rot;
                        if (wsm) {
                            // the staged boxes: the circular row product as
                            // two linear segments, f[0, N - kx) g[kx, N) and
                            // f[N - kx, N) g[0, kx)
                            const uint32_t fb = smem_u32(cs.wptr[grp][sl][2 * p]) + y * rs;
                            const uint32_t gb = smem_u32(cs.wptr[grp][sl][2 * p + 1]) + yy * rs;
                            acc0 = dot_bytes_s(fb, gb + kx, N - kx, acc0);
                            acc1 = dot_bytes_s(fb + N - kx, gb, kx, acc1);
                        } else {
                            const uint8_t* fb = cs.wptr[grp][sl][2 * p] + y * rs;
                            const uint8_t* gb = cs.wptr[grp][sl][2 * p + 1] + yy * rs;
                            const uint32_t g0 = ld_unaligned_p(gb);
#pragma unroll 2
                            for (int jj = 0; jj < NW4; ++jj) {
                                uint32_t fw = ld_unaligned_p(fb + 4 * j);
                                if (j == NW4 - 1) fw &= tail;
                                int a = kx + 4 * j;
                                if (a >= N) a -= N;
                                uint32_t gw = ld_unaligned_p(gb + a);
                                if (a + 4 > N) {
                                    const int nlo = N - a;
                                    gw = (gw & (0xffffffffu >> (8 * (4 - nlo)))) | (g0 << (8 * nlo));
                                }
                                if (jj & 1) acc1 = __dp4a(fw, gw, acc1);
                                else acc0 = __dp4a(fw, gw, acc0);
                                if (++j == NW4) j = 0;
                            }
                        }
                    }
                    atomicAdd(&ps->candS[c], (int)(acc0 + acc1));
                    c += dc;
                    y += dy;
                    if (c >= nc) {
                        c -= nc;
                        ++y;
                    }
                }
            }
            group_sync(bar_id);
            if (t < PB && !cs.sdark[grp][t]) {
                const int a = max(cs.cbase[grp][t], lo), b = min(cs.cend[grp][t], lo + kCandChunk);
                for (int k = a; k < b; ++k) {
                    const int code = ps->cand[k - lo];
                    const int sc = ps->candS[k - lo], id = ((code >> 8) & 0xff) * N + (code & 0xff);
                    if (sc > best_s || (sc == best_s && id < best_i)) {
                        best_s = sc;
                        best_i = id;
                    }
                }
            }
        }
        if (t < PB && b0 + t < n_job) {
            const int gp = b0 + t;
            float* u = jb.u;
            float* v = jb.v;
            float* zncc = jb.zncc;
            uint8_t* status = jb.status;
            if (cs.sdark[grp][t]) {
                status[gp] = 1;  // dark subset: outputs untouched (TW_paDIC_FFTCC2D_CPU.cpp:272-275)
            } else {
                int iu = best_i % N, iv = best_i / N;
                if (iu > g.rx) iu -= N;
                if (iv > g.ry) iv -= N;
                const long long sf = cs.wsum[grp][2 * t][0], sg = cs.wsum[grp][2 * t + 1][0];
                const long long numf = (long long)n2 * cs.wsum[grp][2 * t][1] - sf * sf;
                const long long numg = (long long)n2 * cs.wsum[grp][2 * t + 1][1] - sg * sg;
                // exact integer numerator and norms; the quotient in FP32
                // (relative error below 5e-7: GB300's FP64 divide and square
                // root are slow)
                const long long cnum = (long long)n2 * best_s - sf * sg;
                u[gp] = (float)iu;
                v[gp] = (float)iv;
                zncc[gp] = (float)cnum * rsqrtf((float)numf) * rsqrtf((float)numg);
                status[gp] = 0;
            }
        }
        if (t == 0) cs.snext[grp] = nxt;
        group_sync(bar_id);
        cur = nb;
        nb = cs.snext[grp];
        sl ^= 1;
    }
    return true;
}

// TMEM columns and mbarriers of the CTA's groups; false (err set, TMEM
// freed) when the dynamic shared memory is not 128-byte aligned, which the
// TMA destinations need.  Ends with a CTA barrier.
__device__ __forceinline__ bool tc_setup(TcCta& cs, uint8_t* sm, int groups, uint32_t tmem_cols, unsigned* err) {
    if (threadIdx.x < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&cs.tmem_slot)),
                     "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < groups; ++k) {
            mbar_init(&cs.mbar_mma[k]);
            mbar_init(&cs.mbar_tma[k][0]);
            mbar_init(&cs.mbar_tma[k][1]);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (smem_u32(sm) & 127u) {
        if (threadIdx.x == 0) atomicOr(err, kErrTimeout);
        if (threadIdx.x < 32)
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(cs.tmem_slot),
                         "r"(tmem_cols));
        return false;
    }
    return true;
}

__device__ __forceinline__ void tc_teardown(TcCta& cs, uint32_t tmem_cols) {
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(cs.tmem_slot),
                     "r"(tmem_cols));
}

// One window size: blockDim = 128 * s.groups (up to five).  The first batch
// of every group by position, then the next free one from the launch-wide
// counter, which evens out the groups' finishing times.
template <int NP, int HP, bool MULTI, bool LO, bool REF>
__global__ void __launch_bounds__(NP <= 48 ? 128 * kMaxGroups : 128 * kSegGroups, 1) k_fftcc_tc(const __grid_constant__ TcJobs J, TcShape s,
                                                                 const uint4* __restrict__ tables, unsigned* err,
                                                                 int* work) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ TcCta cs;
    const int grp = threadIdx.x >> 7;
    uint32_t tmem_cols = 32u;  // the groups' columns, allocated as a power of two
    while (tmem_cols < (uint32_t)(s.groups * s.tcols)) tmem_cols <<= 1;
    tc_load_tables(sm, tables, s.tab_bytes);
    if ((threadIdx.x & 127) == 0) tc_acquire_maps(J, 0, J.njobs);
    if (!tc_setup(cs, sm, s.groups, tmem_cols, err)) return;
    uint32_t phase = 0, tphase = 0;
    tc_group_batches<NP, HP, MULTI, LO, REF>(J, s, 0, J.njobs, J.nbatch, blockIdx.x * s.groups + grp, work,
                                        gridDim.x * s.groups, err, cs, sm, phase, tphase);
    tc_teardown(cs, tmem_cols);
}

// The (NP, HP) instantiations of the body: NP = window size rounded up to
// 16, HP = N / 2 + 1 rounded up to 8.
constexpr int kTcShapes[8][2] = {{16, 8}, {16, 16}, {32, 16}, {32, 24}, {48, 24}, {48, 32}, {64, 32}, {64, 40}};

template <bool LO>
__device__ __forceinline__ bool tc_run_segment(const TcJobs& J, const TcSeg& sg, int* counter, unsigned* err,
                                               TcCta& cs, uint8_t* sm, uint32_t& phase, uint32_t& tphase) {
    const int grp = threadIdx.x >> 7;
    if (grp >= sg.s.groups) return true;  // this segment's shared memory holds fewer groups
    // every batch, the first included, from the segment's counter
    if ((threadIdx.x & 127) == 0) cs.snext[grp] = atomicAdd(counter, 1);
    group_sync(1 + grp);
    const int first = cs.snext[grp];
#define TWDIC_TC_SEG(K)                                                                                     \
    case K:                                                                                                  \
        return tc_group_batches<kTcShapes[K][0], kTcShapes[K][1], true, LO, false>(J, sg.s, sg.job_lo,       \
                                                                            sg.job_hi, sg.nbatch, first,     \
                                                                            counter, 0, err, cs, sm, phase,  \
                                                                            tphase);
    switch (sg.shape) {
        TWDIC_TC_SEG(0)
        TWDIC_TC_SEG(1)
        TWDIC_TC_SEG(2)
        TWDIC_TC_SEG(3)
        TWDIC_TC_SEG(4)
        TWDIC_TC_SEG(5)
        TWDIC_TC_SEG(6)
        TWDIC_TC_SEG(7)
        default:
            return true;
    }
#undef TWDIC_TC_SEG
}

// Several window sizes in one persistent launch (blockDim = 512, four groups
// at most): jobs grouped into segments by window size.  A CTA starts on the
// segment its index falls in (CTAs are spread over segments in proportion to
// their work), loads that window size's twiddle tables, and its groups take
// the segment's batches from the segment's counter; when they run out, the
// CTA moves to the next segment with batches left, until none has.
template <bool LO>
__global__ void __launch_bounds__(128 * kSegGroups, 1) k_fftcc_tc_seg(const __grid_constant__ TcJobs J,
                                                                     const __grid_constant__ TcSegs S,
                                                                     unsigned* err, int* counters) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ TcCta cs;
    constexpr uint32_t tmem_cols = 512u;
    if (!tc_setup(cs, sm, kSegGroups, tmem_cols, err)) return;
    if ((threadIdx.x & 127) == 0) tc_acquire_maps(J, 0, J.njobs);
    int seg = 0;
    while (seg + 1 < S.nseg && (int)blockIdx.x >= S.seg[seg + 1].cta_begin) ++seg;
    uint32_t phase = 0, tphase = 0;
    for (;;) {
        const TcSeg& sg = S.seg[seg];
        tc_load_tables(sm, sg.tables, sg.s.tab_bytes);
        __syncthreads();
        const bool ok = tc_run_segment<LO>(J, sg, counters + seg, err, cs, sm, phase, tphase);
        // every group is done with this segment's tables; the next segment
        // with batches left (the counters only grow)
        if (threadIdx.x == 0) {
            int next = -1;
            for (int d = 1; ok && d <= S.nseg; ++d) {
                const int c = (seg + d) % S.nseg;
                if (atomicAdd(counters + c, 0) < S.seg[c].nbatch) {
                    next = c;
                    break;
                }
            }
            cs.seg = next;
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        seg = cs.seg;
        if (seg < 0) break;
    }
    tc_teardown(cs, tmem_cols);
}

// ----------------------------------------------------------- host side ----
int round_up(int x, int m) { return (x + m - 1) / m * m; }

bool make_shape(const Geom& g, const FftccTune& tune, TcShape& s) {
    if (g.rx != g.ry) return false;
    const int N = 2 * g.rx;
    if (N < 8 || N > 64) return false;
    s.N = N;
    s.H = N / 2 + 1;
    s.HP = round_up(s.H, 8);
    s.NP = round_up(N, 16);
    // POIs per batch: the (POI, ky) rows of stages 2 and 3 fill one 128-row
    // tile; the (POI, x) rows of stages 1 and 4 take up to two, each with its
    // own TMEM columns (2 HP at stage 1, NP at stage 4) within the group's 128
    int pb = std::min(128 / s.H, kMaxPB);
    if (tune.pois_per_group > 0) pb = std::min(pb, tune.pois_per_group);  // tuned batch size
    int tiles = 0;
    for (; pb >= 1; --pb) {
        tiles = (pb * N + 127) / 128;
        if (tiles <= 2 && tiles * 2 * s.HP <= kTmemCols && tiles * s.NP <= kTmemCols) break;
    }
    if (pb < 1 || 2 * s.NP > kTmemCols || 2 * s.HP > 80) return false;
    s.PB = pb;
    s.tiles1 = tiles;
    s.tiles4 = tiles;
    s.K4 = 2 * s.HP;
    s.FS = round_up(N, 4);
    const int K1 = s.NP, N1 = 2 * s.HP, NP = s.NP, K4 = s.K4;
    s.lo = tune.twiddle_lo ? 1 : 0;
    int o = 0;
    s.off_b1l = s.off_c2h = s.off_c2l = s.off_s2h = s.off_s2l = s.off_b4l = s.off_w2re = s.off_w2im = 0;
    s.off_b1h = o; o += N1 * K1 * 2;
    if (s.lo) {
        s.off_b1l = o; o += N1 * K1 * 2;
        s.off_c2h = o; o += NP * NP * 2;
        s.off_c2l = o; o += NP * NP * 2;
        s.off_s2h = o; o += NP * NP * 2;
        s.off_s2l = o; o += NP * NP * 2;
    } else {
        s.off_w2re = o; o += NP * 2 * NP * 2;
        s.off_w2im = o; o += NP * 2 * NP * 2;
    }
    s.off_b4h = o; o += NP * K4 * 2;
    if (s.lo) { s.off_b4l = o; o += NP * K4 * 2; }
    s.tab_bytes = round_up(o, 1024);
    o = s.tab_bytes;
    // per-group regions: one operand region shared by A1, A2, A3, A4 and the
    // peak scratch, then the windows
    s.NW4 = (N + 3) / 4;
    // stages 2 and 3 take K over the data columns only: (y, part) interleaved
    // 2N with single twiddles, N per part block with split ones
    s.ks2 = s.lo ? (N + 15) / 16 : (2 * N + 15) / 16;
    s.k3w = s.lo ? 2 * NP : 16 * s.ks2;
    // A2 [<= 128 rows], A4 [tiles4 x 128 rows]: chunk strides of 16 (rows + 1)
    // bytes put one row's chunks in distinct banks
    s.lbo2 = 16 * (128 + 1);
    s.lbo4 = 16 * (s.tiles4 * 128 + 1);
    s.z2lo = s.lo ? N / 8 : 2 * N / 8;
    s.z2hi = 2 * s.ks2;
    s.z2part = (s.lo ? N % 8 : 2 * N % 8) != 0 && s.z2lo < s.z2hi;
    s.z4lo = 2 * s.H / 8;
    s.z4hi = K4 / 8;
    s.z4part = 2 * s.H % 8 != 0 && s.z4lo < s.z4hi;
    const int a1 = s.tiles1 * 128 * K1 * 2;
    const int a2 = (s.lo ? NP / 8 + 2 * s.ks2 : 2 * s.ks2) * s.lbo2;
    const int a3 = 128 * s.k3w * 2;
    const int a4 = (K4 / 8) * s.lbo4;
    s.z4early = a3 <= s.z4lo * s.lbo4;
    const int region = round_up(std::max(std::max(a1, a2), std::max(std::max(a3, a4), (int)sizeof(PeakScratch))),
                                128);
    s.off_a13 = 0;
    s.off_a2 = 0;
    s.off_a4 = 0;
    // windows: the batch's two one-row boxes (PB windows at the grid step
    // apart, x aligned down to 16 bytes, at most 256 bytes wide), the target's
    // 128-byte aligned; 16 spare bytes keep the 8-byte reads of
    // ld_unaligned_p inside the region
    s.uw = round_up((pb - 1) * g.grid_x + N + 15, 16);
    if (g.grid_x <= 0 || s.uw > 256) s.uw = 0;
    s.utoff = round_up(N * s.uw, 128);
    s.win_bytes = round_up(s.utoff + N * s.uw + 16, 128);
    s.off_win = region;
    s.group_bytes = round_up(region + 2 * s.win_bytes, 1024);  // two window slots
    // 227 KB per CTA, less the static state (the dynamic part starts 1024-byte aligned)
    const int limit = 227 * 1024 - round_up((int)sizeof(TcCta), 1024);
    // TMEM: each group's widest accumulator (stage 1: tiles x 2 HP, stages 2
    // and 3: 2 NP, stage 4: tiles x NP), 96 columns up to N = 48, so five
    // groups share the 512 columns there, four above
    s.tcols = round_up(std::max(std::max(s.tiles1 * 2 * s.HP, s.tiles4 * s.NP), 2 * s.NP), 32);
    s.groups = std::min(std::min(kMaxGroups, 512 / s.tcols), (limit - o) / s.group_bytes);
    if (tune.groups > 0) s.groups = std::min(s.groups, tune.groups);  // tuned group count
    if (s.groups < 1) return false;
    s.smem_bytes = o + s.groups * s.group_bytes;
    return s.smem_bytes <= limit;
}

// Twiddle matrices B1, C2, S2, B4 (hi and lo FP16) in the no-swizzle K-major
// layout the kernel's descriptors expect, computed in double.
std::vector<uint8_t> make_tables(const TcShape& s) {
    std::vector<uint8_t> blob(s.tab_bytes, 0);
    const int N = s.N, H = s.H, HP = s.HP, NP = s.NP, K1 = s.NP, K4 = s.K4;
    const double two_pi = 6.283185307179586476925286766559;
    // the hi part (and with split twiddles the lo part) of entry (r, k)
    auto put = [&](int off_h, int off_l, int r, int k, int K, double val) {
        const __half h = __double2half(val);
        std::memcpy(&blob[off_h + kmaj(r, k, K)], &h, 2);
        if (s.lo) {
            const __half l = __double2half(val - (double)__half2float(h));
            std::memcpy(&blob[off_l + kmaj(r, k, K)], &l, 2);
        }
    };
    auto put1 = [&](int off, int r, int k, int K, double val) {
        const __half h = __double2half(val);
        std::memcpy(&blob[off + kmaj(r, k, K)], &h, 2);
    };
    auto ang = [&](int a, int b) { return two_pi * (double)((long long)a * b % N) / N; };
    for (int ky = 0; ky < H; ++ky)
        for (int y = 0; y < N; ++y) {
            put(s.off_b1h, s.off_b1l, ky, y, K1, std::cos(ang(ky, y)));        // Re part row
            put(s.off_b1h, s.off_b1l, HP + ky, y, K1, -std::sin(ang(ky, y)));  // Im part row
            put(s.off_b4h, s.off_b4l, y, 2 * ky, K4, std::cos(ang(ky, y)));       // K = (ky, part) interleaved
            put(s.off_b4h, s.off_b4l, y, 2 * ky + 1, K4, -std::sin(ang(ky, y)));
        }
    for (int kx = 0; kx < N; ++kx)
        for (int x = 0; x < N; ++x) {
            if (s.lo) {
                put(s.off_c2h, s.off_c2l, kx, x, NP, std::cos(ang(kx, x)));
                put(s.off_s2h, s.off_s2l, kx, x, NP, std::sin(ang(kx, x)));
            } else {
                put1(s.off_w2re, kx, 2 * x, 2 * NP, std::cos(ang(kx, x)));
                put1(s.off_w2re, kx, 2 * x + 1, 2 * NP, std::sin(ang(kx, x)));
                put1(s.off_w2im, kx, 2 * x, 2 * NP, -std::sin(ang(kx, x)));
                put1(s.off_w2im, kx, 2 * x + 1, 2 * NP, std::cos(ang(kx, x)));
            }
        }
    return blob;
}

// Twiddle tables per (device, N), built once per process and kept for its
// lifetime (a few tens of KB each), so that launches after the first never
// allocate: a launch captured into a CUDA graph must not.
struct TablesCache {
    std::mutex mu;
    std::map<std::pair<int, int>, uint4*> dev;  // (device, 2 N + lo)
};
TablesCache& tables_cache() {
    static TablesCache* c = new TablesCache();  // never destroyed: may outlive the CUDA context
    return *c;
}

cudaError_t tables_for(const TcShape& s, const uint4** out) {
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return e;
    TablesCache& c = tables_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    const int key = 2 * s.N + s.lo;
    auto it = c.dev.find({device, key});
    if (it != c.dev.end()) {
        *out = it->second;
        return cudaSuccess;
    }
    std::vector<uint8_t> blob = make_tables(s);
    uint4* d = nullptr;
    e = cudaMalloc(&d, blob.size());
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(d, blob.data(), blob.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return e;
    }
    c.dev[{device, key}] = d;
    *out = d;
    return cudaSuccess;
}

}  // namespace

bool fftcc_tc_supported(const Geom& g) {
    TcShape s;
    return (g.pitch % 16) == 0 && make_shape(g, FftccTune{}, s);
}

namespace {

// cuTensorMapEncodeTiled, resolved once through the runtime (no link-time
// dependency on libcuda)
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// 8-bit image as a 2D tensor (x = column, y = row) read in boxes of
// box_w x N bytes; reads outside the image are zero-filled
bool image_map(CUtensorMap* m, const Geom& g, const uint8_t* img, const TcShape& s, int box_w) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)g.img_w, (cuuint64_t)g.img_h};
    const cuuint64_t strides[1] = {(cuuint64_t)g.pitch};
    const cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)s.N};
    const cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<uint8_t*>(img), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

static_assert(sizeof(TcMaps) <= kTcMapsBytes, "TcMaps larger than its buffer");

uint64_t fftcc_tc_maps_key(const Geom& g, const FftccTune& tune) {
    TcShape s;
    if (!make_shape(g, tune, s)) return 0;
    return 1ull | ((uint64_t)s.PB << 8) | ((uint64_t)s.N << 16) | ((uint64_t)s.uw << 24) | ((uint64_t)s.utoff << 40);
}

bool fftcc_tc_encode_maps(const Geom& g, const uint8_t* ref, const uint8_t* tar, const FftccTune& tune,
                          void* host_buf, TcMapInfo* info) {
    TcShape s;
    if (!make_shape(g, tune, s)) return false;
    if ((g.pitch % 16) != 0 || (reinterpret_cast<uintptr_t>(ref) & 15) || (reinterpret_cast<uintptr_t>(tar) & 15) ||
        (reinterpret_cast<uintptr_t>(host_buf) & 127))
        return false;
    TcMaps* m = new (host_buf) TcMaps();
    int uw = s.uw, utoff = s.utoff;
    if (uw > 0 && (!image_map(&m->ref_u, g, ref, s, uw) || !image_map(&m->tar_u, g, tar, s, uw))) return false;
    if (uw == 0) {
        utoff = 0;
        std::memset(m, 0, sizeof(TcMaps));  // never read
    }
    info->key = fftcc_tc_maps_key(g, tune);
    info->uw = uw;
    info->utoff = utoff;
    return true;
}

namespace {

// A job of the kernels' table from a launcher job, whose maps must have been
// encoded for this launch's shape.
bool fill_job(TcJob& o, const FftccJob& in, const FftccTune& tune, const TcShape& launch) {
    if (!in.maps || (reinterpret_cast<uintptr_t>(in.maps) & 127) || in.map_key != fftcc_tc_maps_key(in.g, tune))
        return false;
    if (!in.fspec || !in.fsum) return false;
    o.maps = static_cast<const TcMaps*>(in.maps);
    o.fspec = in.fspec;
    o.fsum = in.fsum;
    o.ref = in.ref;
    o.tar = in.tar;
    o.uw = in.uw;
    o.utoff = in.utoff;
    // the one-row boxes only where they fit this launch's window region
    // (a job of a mixed-size launch may have another grid step than the one
    // the segment's shape was made for); otherwise the windows come from the images
    if (o.uw > 0 && (o.utoff + launch.N * o.uw + 16 > launch.win_bytes || in.g.rx * 2 != launch.N)) o.uw = 0;
    o.g = in.g;
    o.poi = in.poi;
    o.u = in.u;
    o.v = in.v;
    o.zncc = in.zncc;
    o.status = in.status;
    o.n = in.n;
    return true;
}

int shape_index(const TcShape& s) {
    for (int k = 0; k < 8; ++k)
        if (kTcShapes[k][0] == s.NP && kTcShapes[k][1] == s.HP) return k;
    return -1;
}

// Jobs of several window sizes in one k_fftcc_tc_seg launch.  counters:
// kMaxTcSegs ints of scratch.
cudaError_t launch_segments(const FftccJob* jobs, int njobs, const FftccTune& tune, unsigned* err, int* counters,
                            cudaStream_t st) {
    // jobs grouped by window size (stable)
    std::vector<int> order(njobs);
    for (int j = 0; j < njobs; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return jobs[a].g.rx < jobs[b].g.rx; });
    std::unique_ptr<TcJobs> J(new TcJobs());
    std::unique_ptr<TcSegs> S(new TcSegs());
    J->njobs = njobs;
    S->nseg = 0;
    std::vector<double> work;
    int smem = 0;
    for (int k = 0; k < njobs; ++k) {
        const FftccJob& in = jobs[order[k]];
        if (S->nseg == 0 || in.g.rx != J->job[S->seg[S->nseg - 1].job_lo].g.rx) {
            if (S->nseg == kMaxTcSegs) return cudaErrorInvalidValue;
            TcSeg& sg = S->seg[S->nseg++];
            // at most kSegGroups groups: the segmented kernel holds every window
            // size's code, and 128 registers keep it free of spills
            FftccTune ts = tune;
            if (ts.groups == 0 || ts.groups > kSegGroups) ts.groups = kSegGroups;
            if (!make_shape(in.g, ts, sg.s)) return cudaErrorNotSupported;
            sg.shape = shape_index(sg.s);
            if (sg.shape < 0) return cudaErrorNotSupported;
            cudaError_t e = tables_for(sg.s, &sg.tables);
            if (e != cudaSuccess) return e;
            sg.job_lo = k;
            sg.nbatch = 0;
            smem = std::max(smem, sg.s.smem_bytes);
            work.push_back(0.0);
        }
        TcSeg& sg = S->seg[S->nseg - 1];
        if (in.g.rx != in.g.ry) return cudaErrorInvalidValue;
        TcJob& o = J->job[k];
        if (!fill_job(o, in, tune, sg.s)) return cudaErrorInvalidValue;
        o.batch_begin = sg.nbatch;
        const int nb = (in.n + sg.s.PB - 1) / sg.s.PB;
        sg.nbatch += nb;
        sg.job_hi = k + 1;
        work.back() += (double)nb * sg.s.N * sg.s.N;
    }
    J->nbatch = S->seg[0].nbatch;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // CTAs spread over the segments in proportion to their work (batches x N^2)
    double total = 0.0;
    for (double w : work) total += w;
    if (total <= 0.0) return cudaSuccess;
    double acc = 0.0;
    for (int k = 0; k < S->nseg; ++k) {
        S->seg[k].cta_begin = (int)(acc / total * sms + 0.5);
        acc += work[k];
    }
    auto kern = tune.twiddle_lo ? k_fftcc_tc_seg<true> : k_fftcc_tc_seg<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(counters, 0, sizeof(int) * kMaxTcSegs, st);
    if (e != cudaSuccess) return e;
    kern<<<sms, kThreads * kSegGroups, smem, st>>>(*J, *S, err, counters);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fftcc_tc_jobs(const FftccJob* jobs, int njobs, const FftccTune& tune, unsigned* err, int* work,
                                 cudaStream_t st, bool ref) {
    // the per-reference pass runs with single twiddles whatever the tuning
    // (its spectra are rounded to FP16 when cached)
    FftccTune tn = tune;
    if (ref) tn.twiddle_lo = 0;
    if (njobs < 1 || njobs > kMaxTcJobs) return cudaErrorInvalidValue;
    for (int j = 1; j < njobs; ++j)
        if (jobs[j].g.rx != jobs[0].g.rx || jobs[j].g.ry != jobs[0].g.ry) {
            if (ref) return cudaErrorInvalidValue;  // the per-reference pass runs one window size per launch
            return launch_segments(jobs, njobs, tune, err, work, st);  // several window sizes
        }
    TcShape s;
    if (!make_shape(jobs[0].g, tn, s)) return cudaErrorNotSupported;
    std::unique_ptr<TcJobs> J(new TcJobs());
    J->njobs = njobs;
    int nb = 0;
    for (int j = 0; j < njobs; ++j) {
        TcJob& o = J->job[j];
        if (!fill_job(o, jobs[j], tn, s)) return cudaErrorInvalidValue;
        o.batch_begin = nb;
        nb += (jobs[j].n + s.PB - 1) / s.PB;
    }
    J->nbatch = nb;
    if (nb == 0) return cudaSuccess;
    const uint4* tables = nullptr;
    {
        cudaError_t e = tables_for(s, &tables);
        if (e != cudaSuccess) return e;
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void (*kern)(const TcJobs, TcShape, const uint4*, unsigned*, int*) = nullptr;
    const bool multi = njobs > 1;
#define TWDIC_TC_CASE(NPV, HPV)                                                                          \
    case NPV * 100 + HPV:                                                                                \
        if (ref)                                                                                         \
            kern = multi ? k_fftcc_tc<NPV, HPV, true, false, true> : k_fftcc_tc<NPV, HPV, false, false, true>; \
        else if (s.lo)                                                                                   \
            kern = multi ? k_fftcc_tc<NPV, HPV, true, true, false> : k_fftcc_tc<NPV, HPV, false, true, false>; \
        else                                                                                             \
            kern = multi ? k_fftcc_tc<NPV, HPV, true, false, false>                                      \
                         : k_fftcc_tc<NPV, HPV, false, false, false>;                                    \
        break;
    switch (s.NP * 100 + s.HP) {
        TWDIC_TC_CASE(16, 8)
        TWDIC_TC_CASE(16, 16)
        TWDIC_TC_CASE(32, 16)
        TWDIC_TC_CASE(32, 24)
        TWDIC_TC_CASE(48, 24)
        TWDIC_TC_CASE(48, 32)
        TWDIC_TC_CASE(64, 32)
        TWDIC_TC_CASE(64, 40)
        default: return cudaErrorNotSupported;
    }
#undef TWDIC_TC_CASE
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, s.smem_bytes);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (e != cudaSuccess) return e;
    // one CTA per SM holds two groups when shared memory allows; with one
    // group, two CTAs share an SM when they fit
    const int threads = kThreads * s.groups;
    int occ = 1;
    if (s.groups == 1 && 2 * (s.smem_bytes + 2048) <= 228 * 1024) occ = 2;
    const int grid = std::max(1, std::min(sms * occ, (nb + s.groups - 1) / s.groups));
    e = cudaMemsetAsync(work, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    kern<<<grid, threads, s.smem_bytes, st>>>(*J, s, tables, err, work);
    return cudaGetLastError();
}

cudaError_t launch_fftcc_tc(const Geom& g, const uint8_t* ref_img, const uint8_t* tar_img, const void* maps,
                            uint64_t map_key, int uw, int utoff, uint32_t* fspec, int2* fsum, const int2* poi, int n, float* u, float* v, float* zncc, uint8_t* status,
                            unsigned* err, int* work, const FftccTune& tune, cudaStream_t st, bool ref) {
    if (n <= 0) return cudaSuccess;
    FftccJob job{g, maps, map_key, uw, utoff, ref_img, tar_img, fspec, fsum, poi, n, u, v, zncc, status};
    return launch_fftcc_tc_jobs(&job, 1, tune, err, work, st, ref);
}

size_t fftcc_tc_spectrum_bytes(const Geom& g, int n) {
    const int N = 2 * g.rx;
    return (size_t)n * (N / 2 + 1) * round_up(N, 4) * 4;
}

}  // namespace twdic
