// Serving loop over several camera streams (no reference counterpart; the
// reference's capture -> FFT-CC -> IC-GN worker threads, fftcctworkerthread.cpp
// and icgnworkerthread.cpp, process one camera with one frame in flight).
//
// Each stream owns a frame handle (its reference cache and per-frame tables
// stay on the device), a ring of pinned host slots for submitted targets and
// their results, and device staging arrays.  A stream is admitted only if
// its device memory fits the server's HBM budget.  A submit to a full ring is
// dropped (the reference's bounded frame queue drops when full,
// TW_Concurrent_Buffer.cpp).  One scheduler thread batches the oldest pending
// frame of every idle stream (by default only frames within a factor of two
// of the oldest one's POI count) into one twdic_batch launch on a free lane
// (CUDA stream): frames that arrive while batches are on the GPU are taken by
// the next free lane, so several batches overlap on the device.  Each batch's
// device interval is timed by events on its lane.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/tw_dic.h"

namespace twdic {
void set_error_message(const char* msg);  // capi.cu
}

namespace {

using Clock = std::chrono::steady_clock;

int fail_msg(int code, const char* msg) {
    twdic::set_error_message(msg);
    return code;
}

enum SlotState { kFree = 0, kFilling, kQueued, kInFlight, kDone, kFailed, kReading };

struct Slot {
    uint64_t ticket = 0;
    int state = kFree;
    int rc = TWDIC_OK;
    Clock::time_point t_submit, t_done;
    void* h_block = nullptr;  // pinned: target, then u, v, zncc, p6, iters, flags
    uint8_t* h_tar = nullptr;
    float *h_u = nullptr, *h_v = nullptr, *h_z = nullptr, *h_p6 = nullptr;
    int32_t* h_it = nullptr;
    uint8_t* h_fl = nullptr;
};

struct CamStream {
    int id = 0;
    twdic_params prm{};
    twdic_frame* frame = nullptr;
    int n = 0;
    size_t img_bytes = 0;
    uint64_t bytes = 0;  // committed against the budget
    std::vector<Slot> slots;
    std::deque<int> queue;  // slot indices, oldest first
    bool busy = false;      // a frame of this stream is in a batch in flight
    bool has_ref = false;
    // guesses: 1 = after a completed frame of the current reference, IC-GN starts
    // from the last displacements (still in d_u, d_v) and FFT-CC is skipped
    int guess_mode = 0;
    bool has_guess = false;
    void* d_block = nullptr;
    uint8_t* d_tar = nullptr;
    float *d_u = nullptr, *d_v = nullptr, *d_z = nullptr, *d_p6 = nullptr;
    int32_t* d_it = nullptr;
    uint8_t* d_fl = nullptr;
    // per-stream statistics: counters, latencies, and the processing rate of
    // FFTCCTWorkerThread::updateFPS (TW/TW_Core/fftcctworkerthread.cpp:574-605)
    uint64_t completed = 0, dropped = 0;
    std::vector<double> lat_ms;
    bool has_done = false;
    Clock::time_point last_done;
    std::deque<int> fps_q;  // instantaneous rates, at most kFpsWindow
    int fps_samples = 0, fps_avg = 0;
};

// PROCESSING_FPS_STAT_QUEUE_LENGTH (TW/TW_Core/Structures.h:26)
constexpr int kFpsWindow = 32;

// updateFPS: the rate 1000 / elapsed (integer milliseconds between two
// completed frames of the stream, integer division) joins a queue of at most
// kFpsWindow values; every kFpsWindow samples, once the queue is full, the
// average is their integer mean and the sample count restarts.
void fps_update(CamStream& cs, int elapsed_ms) {
    if (elapsed_ms > 0) {
        cs.fps_q.push_back(1000 / elapsed_ms);
        cs.fps_samples += 1;
    }
    if ((int)cs.fps_q.size() > kFpsWindow) cs.fps_q.pop_front();
    if ((int)cs.fps_q.size() == kFpsWindow && cs.fps_samples == kFpsWindow) {
        int sum = 0;
        while (!cs.fps_q.empty()) {
            sum += cs.fps_q.front();
            cs.fps_q.pop_front();
        }
        cs.fps_avg = sum / kFpsWindow;
        cs.fps_samples = 0;
    }
}

struct Lane {
    cudaStream_t st = nullptr;
    cudaEvent_t start = nullptr;  // recorded when the lane's stream reaches the batch (timing)
    cudaEvent_t done = nullptr;   // after the batch's result copies (timing)
    bool busy = false;
    int rc = TWDIC_OK;
    std::vector<std::pair<int, int>> work;  // (stream id, slot)
};

// Expected device time of a frame for the scheduler's ordering: a fixed part
// and a part per POI (about what a 31x31-subset frame takes on GB300).
constexpr int64_t kServiceNs = 200000;
constexpr int64_t kServiceNsPerPoi = 30;

// Device-side interval of one batch, milliseconds after the server's base event.
struct Interval {
    float t0, t1;
};
constexpr size_t kMaxIntervals = 1 << 20;

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace

struct twdic_server {
    twdic_server_config cfg{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_sched, cv_done;
    std::map<int, std::unique_ptr<CamStream>> streams;
    std::vector<Lane> lanes;
    std::map<std::vector<int>, twdic_batch*> batches;  // one per stream mix (its graph)
    std::deque<std::vector<int>> batch_order;
    std::map<uint64_t, std::pair<int, int>> tickets;
    uint64_t next_ticket = 1;
    int next_id = 0;
    uint64_t committed = 0;
    bool stop = false;
    bool paused = false;
    std::thread worker;
    uint64_t submitted = 0, completed = 0, dropped = 0, nbatches = 0, batched_frames = 0, replays = 0;
    uint64_t max_batch_formed = 0;  // frames in the largest batch launched
    int32_t peak_lanes = 0;         // most batches in flight at one time (host view)
    std::vector<double> lat_ms;
    cudaEvent_t base = nullptr;     // time origin of the batch intervals
    std::vector<Interval> intervals;
};

namespace {

constexpr int kMaxMixes = 64;

void free_stream_buffers(CamStream& s) {
    for (Slot& sl : s.slots)
        if (sl.h_block) cudaFreeHost(sl.h_block);
    s.slots.clear();
    if (s.d_block) cudaFree(s.d_block);
    s.d_block = nullptr;
    if (s.frame) twdic_frame_destroy(s.frame);
    s.frame = nullptr;
}

// Output layout of one slot / staging block for n POIs after the target.
size_t outputs_bytes(int n) { return align256(4 * (size_t)n) * 3 + align256(24 * (size_t)n) + align256(4 * (size_t)n) +
                                     align256((size_t)n); }

template <typename F>
void carve(uint8_t* base, size_t img_bytes, int n, F&& set) {
    uint8_t* p = base;
    uint8_t* tar = p;
    p += align256(img_bytes);
    float* u = reinterpret_cast<float*>(p);
    p += align256(4 * (size_t)n);
    float* v = reinterpret_cast<float*>(p);
    p += align256(4 * (size_t)n);
    float* z = reinterpret_cast<float*>(p);
    p += align256(4 * (size_t)n);
    float* p6 = reinterpret_cast<float*>(p);
    p += align256(24 * (size_t)n);
    int32_t* it = reinterpret_cast<int32_t*>(p);
    p += align256(4 * (size_t)n);
    uint8_t* fl = p;
    set(tar, u, v, z, p6, it, fl);
}

twdic_batch* batch_for(twdic_server* s, const std::vector<int>& mix) {
    auto it = s->batches.find(mix);
    if (it != s->batches.end()) return it->second;
    twdic_batch* b = nullptr;
    if (twdic_batch_create(&b) != TWDIC_OK) return nullptr;
    twdic_batch_set_graph(b, s->cfg.use_graph);
    if (s->cfg.icgn_threads > 0)
        twdic_batch_set_tuning(b, s->cfg.icgn_threads, 0, s->cfg.icgn_sampler);
    if ((int)s->batches.size() >= kMaxMixes) {
        auto old = s->batch_order.front();
        s->batch_order.pop_front();
        twdic_batch_destroy(s->batches[old]);
        s->batches.erase(old);
    }
    s->batches[mix] = b;
    s->batch_order.push_back(mix);
    return b;
}

void drop_batches_with(twdic_server* s, int stream_id) {
    for (auto it = s->batches.begin(); it != s->batches.end();) {
        if (std::find(it->first.begin(), it->first.end(), stream_id) != it->first.end()) {
            twdic_batch_destroy(it->second);
            s->batch_order.erase(std::find(s->batch_order.begin(), s->batch_order.end(), it->first));
            it = s->batches.erase(it);
        } else {
            ++it;
        }
    }
}

// Enqueue one batch on a free lane (called with the lock held).
int launch_batch(twdic_server* s, Lane& lane, std::vector<CamStream*>& picked) {
    std::vector<int> mix;
    for (CamStream* cs : picked) mix.push_back(cs->id);
    std::sort(mix.begin(), mix.end());
    lane.work.clear();
    const int k = (int)picked.size();
    std::vector<twdic_frame*> frames(k);
    std::vector<const uint8_t*> tars(k);
    std::vector<float*> u(k), v(k), z(k), p6(k);
    std::vector<int32_t*> it(k);
    std::vector<uint8_t*> fl(k);
    int rc = TWDIC_OK;
    if (cudaEventRecord(lane.start, lane.st) != cudaSuccess) rc = fail_msg(TWDIC_ERR_CUDA, "event record failed");
    for (int i = 0; i < k; ++i) {
        CamStream* cs = picked[i];
        const int si = cs->queue.front();
        cs->queue.pop_front();
        Slot& sl = cs->slots[si];
        sl.state = kInFlight;
        cs->busy = true;
        lane.work.emplace_back(cs->id, si);
        frames[i] = cs->frame;
        if (rc == TWDIC_OK) rc = twdic_frame_set_guess_mode(cs->frame, cs->guess_mode && cs->has_guess ? 1 : 0);
        tars[i] = cs->d_tar;
        u[i] = cs->d_u;
        v[i] = cs->d_v;
        z[i] = cs->d_z;
        p6[i] = cs->d_p6;
        it[i] = cs->d_it;
        fl[i] = cs->d_fl;
        if (cudaMemcpyAsync(cs->d_tar, sl.h_tar, cs->img_bytes, cudaMemcpyHostToDevice, lane.st) != cudaSuccess)
            rc = fail_msg(TWDIC_ERR_CUDA, "target upload failed");
    }
    twdic_batch* b = rc == TWDIC_OK ? batch_for(s, mix) : nullptr;
    if (rc == TWDIC_OK && !b) rc = fail_msg(TWDIC_ERR_CUDA, "batch creation failed");
    int32_t replayed = 0;
    if (rc == TWDIC_OK) rc = twdic_batch_set_stream(b, lane.st);
    if (rc == TWDIC_OK)
        rc = twdic_batch_process(b, k, frames.data(), tars.data(), nullptr, TWDIC_MEM_DEVICE, u.data(), v.data(),
                                 z.data(), p6.data(), it.data(), fl.data(), TWDIC_MEM_DEVICE, &replayed);
    for (int i = 0; i < k && rc == TWDIC_OK; ++i) {
        CamStream* cs = picked[i];
        Slot& sl = cs->slots[lane.work[i].second];
        const size_t n = (size_t)cs->n;
        const cudaMemcpyKind d2h = cudaMemcpyDeviceToHost;
        if (cudaMemcpyAsync(sl.h_u, cs->d_u, 4 * n, d2h, lane.st) != cudaSuccess ||
            cudaMemcpyAsync(sl.h_v, cs->d_v, 4 * n, d2h, lane.st) != cudaSuccess ||
            cudaMemcpyAsync(sl.h_z, cs->d_z, 4 * n, d2h, lane.st) != cudaSuccess ||
            cudaMemcpyAsync(sl.h_p6, cs->d_p6, 24 * n, d2h, lane.st) != cudaSuccess ||
            cudaMemcpyAsync(sl.h_it, cs->d_it, 4 * n, d2h, lane.st) != cudaSuccess ||
            cudaMemcpyAsync(sl.h_fl, cs->d_fl, n, d2h, lane.st) != cudaSuccess)
            rc = fail_msg(TWDIC_ERR_CUDA, "result download failed");
    }
    if (cudaEventRecord(lane.done, lane.st) != cudaSuccess && rc == TWDIC_OK)
        rc = fail_msg(TWDIC_ERR_CUDA, "event record failed");
    lane.busy = true;
    lane.rc = rc;
    s->nbatches += 1;
    s->batched_frames += (uint64_t)k;
    s->replays += replayed ? 1 : 0;
    s->max_batch_formed = std::max(s->max_batch_formed, (uint64_t)k);
    int in_flight = 0;
    for (const Lane& l : s->lanes) in_flight += l.busy ? 1 : 0;
    s->peak_lanes = std::max(s->peak_lanes, in_flight);
    return rc;
}

// Mark the frames of a finished lane done (lock held).
void retire(twdic_server* s, Lane& lane) {
    const Clock::time_point now = Clock::now();
    if (lane.rc == TWDIC_OK && s->intervals.size() < kMaxIntervals) {
        float a = 0.f, b = 0.f;
        if (cudaEventElapsedTime(&a, s->base, lane.start) == cudaSuccess &&
            cudaEventElapsedTime(&b, s->base, lane.done) == cudaSuccess)
            s->intervals.push_back({a, b});
    }
    for (auto& w : lane.work) {
        auto it = s->streams.find(w.first);
        if (it == s->streams.end()) continue;
        CamStream& cs = *it->second;
        Slot& sl = cs.slots[w.second];
        sl.t_done = now;
        sl.rc = lane.rc;
        sl.state = lane.rc == TWDIC_OK ? kDone : kFailed;
        cs.busy = false;
        if (lane.rc == TWDIC_OK) {
            const double ms = std::chrono::duration<double, std::milli>(sl.t_done - sl.t_submit).count();
            s->completed += 1;
            s->lat_ms.push_back(ms);
            cs.completed += 1;
            cs.lat_ms.push_back(ms);
            cs.has_guess = true;
            if (cs.has_done)
                fps_update(cs, (int)std::chrono::duration_cast<std::chrono::milliseconds>(now - cs.last_done).count());
            cs.has_done = true;
            cs.last_done = now;
        }
    }
    lane.work.clear();
    lane.busy = false;
}

void worker_main(twdic_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        bool progressed = false;
        bool any_busy = false;
        for (Lane& lane : s->lanes) {
            if (!lane.busy) continue;
            const cudaError_t q = cudaEventQuery(lane.done);
            if (q == cudaSuccess || q != cudaErrorNotReady) {
                if (q != cudaSuccess && lane.rc == TWDIC_OK) lane.rc = TWDIC_ERR_CUDA;
                retire(s, lane);
                progressed = true;
            } else {
                any_busy = true;
            }
        }
        if (progressed) s->cv_done.notify_all();
        if (s->stop && !any_busy) break;
        if (!s->stop && !s->paused) {
            for (Lane& lane : s->lanes) {
                if (lane.busy) continue;
                // the next pending frame of every idle stream
                std::vector<CamStream*> ready;
                for (auto& kv : s->streams) {
                    CamStream& cs = *kv.second;
                    if (!cs.busy && cs.has_ref && !cs.queue.empty()) ready.push_back(&cs);
                }
                if (ready.empty()) break;
                if (s->cfg.mix_sizes) {
                    // oldest pending frame first
                    std::sort(ready.begin(), ready.end(), [](CamStream* a, CamStream* b) {
                        return a->slots[a->queue.front()].t_submit < b->slots[b->queue.front()].t_submit;
                    });
                } else {
                    // earliest expected finish first: submit time plus an estimate
                    // of the frame's device time from its POI count, so that a small
                    // frame is not queued behind a much larger one submitted just
                    // before it, while a large frame still ages to the front
                    auto key = [](CamStream* c) {
                        return c->slots[c->queue.front()].t_submit +
                               std::chrono::nanoseconds(kServiceNs + kServiceNsPerPoi * (int64_t)c->n);
                    };
                    std::sort(ready.begin(), ready.end(), [&](CamStream* a, CamStream* b) { return key(a) < key(b); });
                    // size-aware: the first frame and the frames whose POI count is
                    // within a factor of two of it, so that a small frame does not
                    // wait for a much larger one in the same batch (the others take
                    // the next free lane)
                    const int n0 = ready.front()->n;
                    std::vector<CamStream*> same;
                    for (CamStream* cs : ready)
                        if (2 * (int64_t)cs->n >= n0 && cs->n <= 2 * (int64_t)n0) same.push_back(cs);
                    ready.swap(same);
                }
                if ((int)ready.size() > s->cfg.max_batch) ready.resize(s->cfg.max_batch);
                launch_batch(s, lane, ready);
                progressed = true;
                any_busy = true;
            }
        }
        if (!progressed) {
            if (any_busy)
                s->cv_sched.wait_for(lk, std::chrono::microseconds(50));
            else
                s->cv_sched.wait(lk);
        }
    }
}

}  // namespace

extern "C" {

int twdic_server_create(const twdic_server_config* cfg, twdic_server** out) {
    if (!cfg || !out) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (cfg->max_batch < 1 || cfg->max_batch > 32) return fail_msg(TWDIC_ERR_INVALID_ARG, "max_batch must be 1..32");
    if (cfg->queue_depth < 1 || cfg->queue_depth > 64)
        return fail_msg(TWDIC_ERR_INVALID_ARG, "queue_depth must be 1..64");
    if (cfg->lanes < 1 || cfg->lanes > 4) return fail_msg(TWDIC_ERR_INVALID_ARG, "lanes must be 1..4");
    std::unique_ptr<twdic_server> s(new twdic_server());
    s->cfg = *cfg;
    if (cudaGetDevice(&s->device) != cudaSuccess) return fail_msg(TWDIC_ERR_CUDA, "no CUDA device");
    if (s->cfg.hbm_budget_bytes == 0) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return fail_msg(TWDIC_ERR_CUDA, "cudaMemGetInfo failed");
        s->cfg.hbm_budget_bytes = (uint64_t)(free_b * 0.9);
    }
    s->paused = cfg->start_paused != 0;
    s->lanes.resize(cfg->lanes);
    for (Lane& l : s->lanes) {
        if (cudaStreamCreateWithFlags(&l.st, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&l.start) != cudaSuccess || cudaEventCreate(&l.done) != cudaSuccess)
            return fail_msg(TWDIC_ERR_CUDA, "lane stream creation failed");
    }
    if (cudaEventCreate(&s->base) != cudaSuccess || cudaEventRecord(s->base, s->lanes[0].st) != cudaSuccess ||
        cudaEventSynchronize(s->base) != cudaSuccess)
        return fail_msg(TWDIC_ERR_CUDA, "base event failed");
    twdic_server* raw = s.get();
    s->worker = std::thread(worker_main, raw);
    *out = s.release();
    return TWDIC_OK;
}

int twdic_server_add_stream(twdic_server* s, const twdic_params* p, int32_t* stream_id) {
    if (!s || !p || !stream_id) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL argument");
    uint64_t est = 0;
    int rc = twdic_frame_device_bytes(p, &est);
    if (rc != TWDIC_OK) return rc;
    int32_t nx = 0, ny = 0;
    rc = twdic_num_pois(p, &nx, &ny);
    if (rc != TWDIC_OK) return rc;
    const int n = nx * ny;
    const size_t img = (size_t)p->img_width * p->img_height;
    const size_t dev_bytes = align256(img) + outputs_bytes(n);
    est += (dev_bytes + (2ull << 20) - 1) / (2ull << 20) * (2ull << 20);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->committed + est > s->cfg.hbm_budget_bytes) {
            char buf[200];
            snprintf(buf, sizeof(buf), "HBM budget: stream needs %llu bytes, %llu of %llu committed",
                     (unsigned long long)est, (unsigned long long)s->committed,
                     (unsigned long long)s->cfg.hbm_budget_bytes);
            return fail_msg(TWDIC_ERR_NO_MEMORY, buf);
        }
        s->committed += est;  // reserved while the stream is set up
    }
    std::unique_ptr<CamStream> cs(new CamStream());
    cs->prm = *p;
    cs->n = n;
    cs->img_bytes = img;
    cs->bytes = est;
    auto undo = [&](int code) {
        free_stream_buffers(*cs);
        std::lock_guard<std::mutex> lk(s->mu);
        s->committed -= est;
        return code;
    };
    rc = twdic_frame_create(p, &cs->frame);
    if (rc != TWDIC_OK) return undo(rc);
    if (cudaMalloc(&cs->d_block, dev_bytes) != cudaSuccess) return undo(fail_msg(TWDIC_ERR_NO_MEMORY, "cudaMalloc failed"));
    carve(static_cast<uint8_t*>(cs->d_block), img, n,
          [&](uint8_t* t, float* u, float* v, float* z, float* p6, int32_t* it, uint8_t* fl) {
              cs->d_tar = t; cs->d_u = u; cs->d_v = v; cs->d_z = z; cs->d_p6 = p6; cs->d_it = it; cs->d_fl = fl;
          });
    cs->slots.resize(s->cfg.queue_depth);
    for (Slot& sl : cs->slots) {
        if (cudaMallocHost(&sl.h_block, dev_bytes) != cudaSuccess)
            return undo(fail_msg(TWDIC_ERR_NO_MEMORY, "cudaMallocHost failed"));
        carve(static_cast<uint8_t*>(sl.h_block), img, n,
              [&](uint8_t* t, float* u, float* v, float* z, float* p6, int32_t* it, uint8_t* fl) {
                  sl.h_tar = t; sl.h_u = u; sl.h_v = v; sl.h_z = z; sl.h_p6 = p6; sl.h_it = it; sl.h_fl = fl;
              });
    }
    std::lock_guard<std::mutex> lk(s->mu);
    cs->id = s->next_id++;
    *stream_id = cs->id;
    s->streams[cs->id] = std::move(cs);
    return TWDIC_OK;
}

int twdic_server_remove_stream(twdic_server* s, int32_t stream_id) {
    if (!s) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL handle");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->streams.find(stream_id);
    if (it == s->streams.end()) return fail_msg(TWDIC_ERR_INVALID_ARG, "unknown stream id");
    // no batch of the stream in flight, no twdic_submit copying into its
    // slots and no twdic_poll copying out of them
    s->cv_done.wait(lk, [&] {
        if (it->second->busy) return false;
        for (const Slot& sl : it->second->slots)
            if (sl.state == kFilling || sl.state == kReading) return false;
        return true;
    });
    CamStream& cs = *it->second;
    for (Slot& sl : cs.slots)
        if (sl.ticket) s->tickets.erase(sl.ticket);
    drop_batches_with(s, stream_id);
    s->committed -= cs.bytes;
    free_stream_buffers(cs);
    s->streams.erase(it);
    lk.unlock();
    s->cv_done.notify_all();  // calls waiting on the removed stream's tickets
    return TWDIC_OK;
}

int twdic_server_set_reference(twdic_server* s, int32_t stream_id, const uint8_t* img, int32_t stride) {
    if (!s || !img) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->streams.find(stream_id);
    if (it == s->streams.end()) return fail_msg(TWDIC_ERR_INVALID_ARG, "unknown stream id");
    s->cv_done.wait(lk, [&] { return !it->second->busy; });
    CamStream& cs = *it->second;
    const int rc = twdic_frame_set_reference(cs.frame, img, stride, TWDIC_MEM_HOST);
    if (rc == TWDIC_OK) {
        cs.has_ref = true;
        cs.has_guess = false;  // the next frame starts from FFT-CC again
    }
    lk.unlock();
    s->cv_sched.notify_all();
    return rc;
}

int twdic_submit(twdic_server* s, int32_t stream_id, const uint8_t* tar, int32_t stride, uint64_t* ticket) {
    if (!s || !tar || !ticket) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->streams.find(stream_id);
    if (it == s->streams.end()) return fail_msg(TWDIC_ERR_INVALID_ARG, "unknown stream id");
    CamStream& cs = *it->second;
    if (stride == 0) stride = cs.prm.img_width;
    if (stride < cs.prm.img_width) return fail_msg(TWDIC_ERR_INVALID_ARG, "stride < width");
    int si = -1;
    for (int i = 0; i < (int)cs.slots.size(); ++i)
        if (cs.slots[i].state == kFree) { si = i; break; }
    s->submitted += 1;
    if (si < 0) {
        s->dropped += 1;
        cs.dropped += 1;
        return fail_msg(TWDIC_ERR_BUSY, "stream queue full: frame dropped");
    }
    Slot& sl = cs.slots[si];
    sl.state = kFilling;
    sl.ticket = s->next_ticket++;
    sl.t_submit = Clock::now();
    *ticket = sl.ticket;
    s->tickets[sl.ticket] = {stream_id, si};
    lk.unlock();
    const int w = cs.prm.img_width, h = cs.prm.img_height;
    if (stride == w) {
        std::memcpy(sl.h_tar, tar, (size_t)w * h);
    } else {
        for (int y = 0; y < h; ++y) std::memcpy(sl.h_tar + (size_t)y * w, tar + (size_t)y * stride, w);
    }
    lk.lock();
    sl.state = kQueued;
    cs.queue.push_back(si);
    lk.unlock();
    s->cv_sched.notify_all();
    s->cv_done.notify_all();  // a twdic_server_remove_stream waiting for this copy
    return TWDIC_OK;
}

int twdic_poll(twdic_server* s, uint64_t ticket, int32_t wait, float* u, float* v, float* zncc, float* p6,
               int32_t* iters, uint8_t* flags, double* latency_ms) {
    if (!s) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL handle");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail_msg(TWDIC_ERR_INVALID_ARG, "unknown ticket");
    const int sid = it->second.first, si = it->second.second;
    CamStream* cs = s->streams.at(sid).get();
    Slot* sl = &cs->slots[si];
    if (sl->state == kReading) return fail_msg(TWDIC_ERR_STATE, "ticket is being read by another call");
    if (sl->state != kDone && sl->state != kFailed) {
        if (!wait) return TWDIC_PENDING;
        // the ticket leaves the table when its stream is removed or another
        // call reads it; the slot is not touched after that
        auto gone = [&] { return s->tickets.find(ticket) == s->tickets.end(); };
        s->cv_done.wait(lk, [&] { return s->stop || gone() || sl->state == kDone || sl->state == kFailed; });
        if (gone()) return fail_msg(TWDIC_ERR_STATE, "ticket taken by another call or its stream removed");
        if (sl->state != kDone && sl->state != kFailed) return fail_msg(TWDIC_ERR_STATE, "server stopped");
    }
    const int rc = sl->rc;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(sl->t_done - sl->t_submit).count();
    sl->state = kReading;
    lk.unlock();
    const size_t n = (size_t)cs->n;
    if (rc == TWDIC_OK) {
        if (u) std::memcpy(u, sl->h_u, 4 * n);
        if (v) std::memcpy(v, sl->h_v, 4 * n);
        if (zncc) std::memcpy(zncc, sl->h_z, 4 * n);
        if (p6) std::memcpy(p6, sl->h_p6, 24 * n);
        if (iters) std::memcpy(iters, sl->h_it, 4 * n);
        if (flags) std::memcpy(flags, sl->h_fl, n);
    }
    lk.lock();
    s->tickets.erase(ticket);
    sl->ticket = 0;
    sl->state = kFree;
    lk.unlock();
    s->cv_done.notify_all();  // other calls waiting on this ticket
    return rc == TWDIC_OK ? TWDIC_OK : fail_msg(rc, "the batch holding this frame failed");
}

int twdic_server_resume(twdic_server* s) {
    if (!s) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL handle");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->paused = false;
    }
    s->cv_sched.notify_all();
    return TWDIC_OK;
}

int twdic_server_stats(twdic_server* s, twdic_server_counters* out) {
    if (!s || !out) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->dropped = s->dropped;
    out->batches = s->nbatches;
    out->batched_frames = s->batched_frames;
    out->graph_replays = s->replays;
    out->committed_bytes = s->committed;
    out->budget_bytes = s->cfg.hbm_budget_bytes;
    out->streams = (int32_t)s->streams.size();
    out->max_batch_formed = s->max_batch_formed;
    out->peak_lanes_in_flight = s->peak_lanes;
    // device time: union of the batches' intervals, the part of it covered by
    // two or more batches at once, and the most batches running at one time
    if (!s->intervals.empty()) {
        std::vector<std::pair<float, int>> ev;
        ev.reserve(2 * s->intervals.size());
        for (const Interval& iv : s->intervals) {
            ev.push_back({iv.t0, +1});
            ev.push_back({iv.t1, -1});
        }
        std::sort(ev.begin(), ev.end(), [](const std::pair<float, int>& a, const std::pair<float, int>& b) {
            return a.first < b.first || (a.first == b.first && a.second < b.second);
        });
        int active = 0, peak = 0;
        double busy = 0.0, overlap = 0.0;
        for (size_t i = 0; i < ev.size(); ++i) {
            if (i > 0) {
                const double dt = (double)ev[i].first - (double)ev[i - 1].first;
                if (active >= 1) busy += dt;
                if (active >= 2) overlap += dt;
            }
            active += ev[i].second;
            peak = std::max(peak, active);
        }
        out->device_busy_ms = busy;
        out->device_overlap_ms = overlap;
        out->peak_device_batches = peak;
    }
    if (!s->lat_ms.empty()) {
        std::vector<double> l = s->lat_ms;
        std::sort(l.begin(), l.end());
        auto q = [&](double f) { return l[std::min(l.size() - 1, (size_t)(f * (l.size() - 1) + 0.5))]; };
        out->p50_ms = q(0.50);
        out->p99_ms = q(0.99);
        out->max_ms = l.back();
    }
    return TWDIC_OK;
}

int twdic_server_set_stream_guess(twdic_server* s, int32_t stream_id, int mode) {
    if (!s) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL argument");
    if (mode != 0 && mode != 1) return fail_msg(TWDIC_ERR_INVALID_ARG, "guess mode must be 0 or 1");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->streams.find(stream_id);
    if (it == s->streams.end()) return fail_msg(TWDIC_ERR_INVALID_ARG, "unknown stream id");
    it->second->guess_mode = mode;
    return TWDIC_OK;
}

int twdic_server_stream_stats(twdic_server* s, int32_t stream_id, twdic_stream_stats* out) {
    if (!s || !out) return fail_msg(TWDIC_ERR_INVALID_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->streams.find(stream_id);
    if (it == s->streams.end()) return fail_msg(TWDIC_ERR_INVALID_ARG, "unknown stream id");
    const CamStream& cs = *it->second;
    std::memset(out, 0, sizeof(*out));
    out->completed = cs.completed;
    out->dropped = cs.dropped;
    out->average_fps = cs.fps_avg;
    if (!cs.lat_ms.empty()) {
        std::vector<double> l = cs.lat_ms;
        std::sort(l.begin(), l.end());
        auto q = [&](double f) { return l[std::min(l.size() - 1, (size_t)(f * (l.size() - 1) + 0.5))]; };
        out->p50_ms = q(0.50);
        out->p99_ms = q(0.99);
    }
    return TWDIC_OK;
}

int twdic_server_destroy(twdic_server* s) {
    if (!s) return TWDIC_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_sched.notify_all();
    s->cv_done.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (auto& kv : s->batches) twdic_batch_destroy(kv.second);
    s->batches.clear();
    for (auto& kv : s->streams) free_stream_buffers(*kv.second);
    s->streams.clear();
    for (Lane& l : s->lanes) {
        if (l.start) cudaEventDestroy(l.start);
        if (l.done) cudaEventDestroy(l.done);
        if (l.st) cudaStreamDestroy(l.st);
    }
    if (s->base) cudaEventDestroy(s->base);
    delete s;
    return TWDIC_OK;
}

}  // extern "C"
