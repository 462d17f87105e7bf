// astc_server.cu -- continuous-batching request server over the encoder.
//
// Worker loop (one thread per server):
//   1. retire: every busy slot whose event has completed releases its
//      requests' pool memory and marks them done;
//   2. admit + launch: for every free slot, take queued requests in arrival
//      order while their input + output fit in the free pool memory and the
//      batch has room; copy them in (2-D copies, so requests may point into
//      larger images), encode (one astc_batch graph launch, or one plain
//      kernel per request in per-request mode), copy the blocks out, record
//      the slot's event;
//   3. otherwise sleep on a condition variable for at most 50 us (a submit
//      wakes it at once).
// The pool is one device allocation with a first-fit free list (256-byte
// granules, neighbours coalesced on free).  No device code waits on the
// host; every host wait (request wait, destroy) is either bounded by the
// caller's timeout or waits on CUDA events of work already launched.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "astc_internal.h"

namespace astc {
namespace {

using Clock = std::chrono::steady_clock;

constexpr size_t kGranule = 256;

size_t round_up(size_t n) { return (n + kGranule - 1) & ~(kGranule - 1); }

class FirstFit {
public:
    void reset(size_t size) {
        free_.clear();
        free_[0] = size;
        total_ = size;
    }
    // returns the offset or SIZE_MAX
    size_t alloc(size_t n) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            const size_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > n) free_[off + n] = len - n;
            return off;
        }
        return SIZE_MAX;
    }
    void release(size_t off, size_t n) {
        auto it = free_.emplace(off, n).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t total() const { return total_; }

private:
    std::map<size_t, size_t> free_;
    size_t total_ = 0;
};

enum ReqState { kQueued = 0, kAdmitted = 1, kDone = 2 };

struct Req {
    uint64_t id = 0;
    astc_request r{};
    size_t pitch = 0, in_bytes = 0, out_bytes = 0, off = 0, need = 0;
    bool out_direct = false;        // blocks written straight into pinned host memory
    Clock::time_point t_submit, t_admit, t_done;
    int state = kQueued;
    astc_status status = ASTC_OK;
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    cudaEvent_t t_start = nullptr, t_end = nullptr;   // timing: the slot's work on the device
    astc_batch* batch = nullptr;
    std::vector<Req*> reqs;
    bool busy = false;
};

double us_since(Clock::time_point t0, Clock::time_point t) {
    return std::chrono::duration<double, std::micro>(t - t0).count();
}

// One retired slot launch: its device interval (ms after the server's
// reference event) and how many requests it carried.
struct Interval {
    float start_ms, end_ms;
    int requests;
};

// A server that is never asked to reset its statistics keeps the record of
// its most recent 2^20 launches (16 MiB) and drops older halves.
constexpr size_t kMaxIntervals = size_t(1) << 20;

}  // namespace
}  // namespace astc

using namespace astc;

struct astc_server {
    astc_server_config cfg{};
    int device = 0;
    uint8_t* d_pool = nullptr;
    FirstFit pool;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
    uint64_t next_id = 1;
    bool stop = false;
    std::thread worker;
    Clock::time_point t0 = Clock::now();
    std::string worker_error;
    cudaEvent_t t0_event = nullptr;          // device clock origin of the intervals
    std::vector<Interval> intervals;         // retired launches since the last reset (the
                                             // most recent kMaxIntervals of them)
};

namespace {

// Issues one slot's copies, encode and event.  Called without the lock.
cudaError_t launch_slot(astc_server* s, Slot& slot) {
    cudaError_t e = cudaEventRecord(slot.t_start, slot.stream);
    if (e != cudaSuccess) return e;
    std::vector<astc_batch_item> items;
    items.reserve(slot.reqs.size());
    for (Req* q : slot.reqs) {
        uint8_t* d_in = s->d_pool + q->off;
        uint8_t* d_out = d_in + round_up(q->in_bytes);
        const size_t row = (size_t)q->r.width * 4;
        // requests in host memory the device reaches in place (pinned, or
        // pageable where the device reads the host's page tables) are read and
        // written there (zero-copy); the pool space stays reserved, so
        // admission by memory behaves the same for every request
        const void* in_view = host_device_view(q->r.rgba8).ptr;
        void* out_view = const_cast<void*>(host_device_view(q->r.out).ptr);
        q->out_direct = out_view && reinterpret_cast<uintptr_t>(out_view) % 16 == 0;
        astc_batch_item it;
        if (in_view && reinterpret_cast<uintptr_t>(in_view) % 4 == 0 && q->pitch % 4 == 0) {
            it.rgba8 = static_cast<const uint8_t*>(in_view);
            it.row_pitch = q->pitch;
        } else {
            e = cudaMemcpy2DAsync(d_in, row, q->r.rgba8, q->pitch, row, q->r.height, cudaMemcpyHostToDevice,
                                  slot.stream);
            if (e != cudaSuccess) return e;
            it.rgba8 = d_in;
            it.row_pitch = row;
        }
        if (q->out_direct) d_out = static_cast<uint8_t*>(out_view);
        it.width = q->r.width;
        it.height = q->r.height;
        it.block_dim = q->r.block_dim;
        it.has_alpha = q->r.has_alpha;
        it.is_normal = q->r.is_normal;
        it.srgb = q->r.srgb;
        it.border = q->r.border;
        it.out = d_out;
        items.push_back(it);
    }
    if (s->cfg.mode == ASTC_SERVE_BATCHED) {
        const astc_status st = astc_batch_encode_quality(slot.batch, items.data(), (int)items.size(),
                                                         s->cfg.precision, s->cfg.quality, slot.stream);
        if (st != ASTC_OK) return cudaErrorUnknown;
    } else {
        for (const astc_batch_item& it : items) {
            EncodeJob j;
            j.in = it.rgba8;
            j.pitch = it.row_pitch;
            j.width = it.width;
            j.height = it.height;
            j.block_dim = it.block_dim;
            j.has_alpha = it.has_alpha;
            j.is_normal = it.is_normal;
            j.srgb = it.srgb;
            j.border = it.border;
            j.precision = s->cfg.precision;
            j.quality = s->cfg.quality;
            j.out = it.out;
            e = s->cfg.quality != ASTC_QUALITY_FAST           ? launch_encode_search(j, slot.stream)
                : s->cfg.precision == ASTC_PRECISION_HALF2 ? launch_encode_h2(j, slot.stream)
                                                           : launch_encode(j, slot.stream);
            if (e != cudaSuccess) return e;
        }
    }
    for (Req* q : slot.reqs) {
        if (q->out_direct) continue;
        const uint8_t* d_out = s->d_pool + q->off + round_up(q->in_bytes);
        e = cudaMemcpyAsync(q->r.out, d_out, q->out_bytes, cudaMemcpyDeviceToHost, slot.stream);
        if (e != cudaSuccess) return e;
    }
    if ((e = cudaEventRecord(slot.t_end, slot.stream)) != cudaSuccess) return e;
    return cudaEventRecord(slot.done, slot.stream);
}

void worker_main(astc_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        bool progress = false;
        // 1. retire finished slots
        for (Slot& slot : s->slots) {
            if (!slot.busy) continue;
            const cudaError_t q = cudaEventQuery(slot.done);
            if (q == cudaErrorNotReady) continue;
            const Clock::time_point now = Clock::now();
            for (Req* r : slot.reqs) {
                s->pool.release(r->off, r->need);
                r->state = kDone;
                r->t_done = now;
                if (q != cudaSuccess) r->status = ASTC_ERR_CUDA;
            }
            if (q != cudaSuccess) {
                s->worker_error = cudaGetErrorString(q);
                cudaGetLastError();
            } else {
                float a = 0.0f, b = 0.0f;
                if (cudaEventElapsedTime(&a, s->t0_event, slot.t_start) == cudaSuccess &&
                    cudaEventElapsedTime(&b, s->t0_event, slot.t_end) == cudaSuccess) {
                    if (s->intervals.size() >= kMaxIntervals)
                        s->intervals.erase(s->intervals.begin(), s->intervals.begin() + kMaxIntervals / 2);
                    s->intervals.push_back({a, b, (int)slot.reqs.size()});
                }
                cudaGetLastError();
            }
            slot.reqs.clear();
            slot.busy = false;
            progress = true;
        }
        if (progress) s->cv_done.notify_all();
        // 2. admit and launch into free slots
        for (Slot& slot : s->slots) {
            if (slot.busy || s->queue.empty()) continue;
            const int cap = s->cfg.mode == ASTC_SERVE_BATCHED ? s->cfg.max_batch : 1;
            while (!s->queue.empty() && (int)slot.reqs.size() < cap) {
                Req* r = s->queue.front();
                const size_t off = s->pool.alloc(r->need);
                if (off == SIZE_MAX) break;                  // wait for memory to free up
                s->queue.pop_front();
                r->off = off;
                r->state = kAdmitted;
                r->t_admit = Clock::now();
                slot.reqs.push_back(r);
            }
            if (slot.reqs.empty()) break;                    // head request does not fit yet
            slot.busy = true;
            lk.unlock();
            const cudaError_t e = launch_slot(s, slot);
            lk.lock();
            if (e != cudaSuccess) {
                s->worker_error = cudaGetErrorString(e);
                cudaGetLastError();
                const Clock::time_point now = Clock::now();
                cudaStreamSynchronize(slot.stream);          // work already issued on the slot
                for (Req* r : slot.reqs) {
                    s->pool.release(r->off, r->need);
                    r->state = kDone;
                    r->status = ASTC_ERR_CUDA;
                    r->t_done = now;
                }
                slot.reqs.clear();
                slot.busy = false;
                s->cv_done.notify_all();
            }
            progress = true;
        }
        bool any_busy = false;
        for (Slot& slot : s->slots) any_busy |= slot.busy;
        if (s->stop && s->queue.empty() && !any_busy) break;
        if (!progress) s->cv_work.wait_for(lk, std::chrono::microseconds(50));
    }
}

}  // namespace

extern "C" {

astc_status astc_server_create(const astc_server_config* cfg, astc_server** out) {
    if (!cfg || !out) return set_error(ASTC_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (cfg->pool_bytes < (1u << 20)) return set_error(ASTC_ERR_INVALID_ARG, "pool_bytes must be >= 1 MiB");
    if (cfg->inflight < 1 || cfg->inflight > 16) return set_error(ASTC_ERR_INVALID_ARG, "inflight must be 1..16");
    if (cfg->max_batch < 1 || cfg->max_batch > 65536)
        return set_error(ASTC_ERR_INVALID_ARG, "max_batch must be 1..65536");
    if (cfg->precision != ASTC_PRECISION_FP32 && cfg->precision != ASTC_PRECISION_HALF2)
        return set_error(ASTC_ERR_INVALID_ARG, "bad precision");
    if (cfg->mode != ASTC_SERVE_BATCHED && cfg->mode != ASTC_SERVE_PER_REQUEST)
        return set_error(ASTC_ERR_INVALID_ARG, "bad mode");
    if (cfg->quality < ASTC_QUALITY_FAST || cfg->quality > ASTC_QUALITY_THREE_PARTITIONS)
        return set_error(ASTC_ERR_INVALID_ARG, "bad quality");
    if (cfg->quality != ASTC_QUALITY_FAST && cfg->precision != ASTC_PRECISION_FP32)
        return set_error(ASTC_ERR_UNSUPPORTED, "the quality modes are FP32 only");
    std::unique_ptr<astc_server> s(new (std::nothrow) astc_server());
    if (!s) return set_error(ASTC_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->cfg = *cfg;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    s->cfg.pool_bytes &= ~(kGranule - 1);
    if ((e = cudaMalloc(reinterpret_cast<void**>(&s->d_pool), s->cfg.pool_bytes)) != cudaSuccess)
        return cuda_error(e, "cudaMalloc of the staging pool");
    s->pool.reset(s->cfg.pool_bytes);
    s->slots.resize(cfg->inflight);
    astc_status st = ASTC_OK;
    for (Slot& slot : s->slots) {
        if ((e = cudaStreamCreateWithFlags(&slot.stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&slot.done, cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventCreate(&slot.t_start)) != cudaSuccess || (e = cudaEventCreate(&slot.t_end)) != cudaSuccess) {
            st = cuda_error(e, "stream/event creation");
            break;
        }
        if (cfg->mode == ASTC_SERVE_BATCHED &&
            (st = astc_batch_create(cfg->max_batch, (long long)(s->cfg.pool_bytes / 16), &slot.batch)) != ASTC_OK)
            break;
    }
    if (st == ASTC_OK) {
        if ((e = cudaEventCreate(&s->t0_event)) != cudaSuccess ||
            (e = cudaEventRecord(s->t0_event, s->slots[0].stream)) != cudaSuccess ||
            (e = cudaEventSynchronize(s->t0_event)) != cudaSuccess)
            st = cuda_error(e, "reference event");
    }
    if (st != ASTC_OK) {
        astc_server_destroy(s.release());
        return st;
    }
    astc_server* raw = s.get();
    raw->worker = std::thread(worker_main, raw);
    *out = s.release();
    return ASTC_OK;
}

astc_status astc_server_submit(astc_server* s, const astc_request* r, uint64_t* ticket) {
    if (!s || !r || !ticket) return set_error(ASTC_ERR_INVALID_ARG, "NULL argument");
    if (!r->rgba8 || !r->out) return set_error(ASTC_ERR_INVALID_ARG, "rgba8 and out must be non-NULL");
    if (r->block_dim != 4 && r->block_dim != 6) return set_error(ASTC_ERR_INVALID_ARG, "block_dim must be 4 or 6");
    if (r->width <= 0 || r->height <= 0 || r->width > 0xFFFFFF || r->height > 0xFFFFFF)
        return set_error(ASTC_ERR_INVALID_ARG, "bad request size");
    if (r->border != ASTC_BORDER_ZERO && r->border != ASTC_BORDER_CLAMP)
        return set_error(ASTC_ERR_INVALID_ARG, "bad border");
    const size_t pitch = r->row_pitch ? r->row_pitch : (size_t)r->width * 4;
    if (pitch < (size_t)r->width * 4) return set_error(ASTC_ERR_INVALID_ARG, "row_pitch < 4 * width");
    auto q = std::make_unique<Req>();
    q->r = *r;
    q->pitch = pitch;
    q->in_bytes = (size_t)r->width * r->height * 4;
    q->out_bytes = astc_encoded_size(r->width, r->height, r->block_dim);
    q->need = round_up(q->in_bytes) + round_up(q->out_bytes);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return set_error(ASTC_ERR_CANCELLED, "server is shutting down");
    if (q->need > s->pool.total())
        return set_error(ASTC_ERR_BUSY, "request is larger than the staging pool");
    q->id = s->next_id++;
    q->t_submit = Clock::now();
    *ticket = q->id;
    s->queue.push_back(q.get());
    s->reqs.emplace(q->id, std::move(q));
    s->cv_work.notify_one();
    return ASTC_OK;
}

astc_status astc_server_wait(astc_server* s, uint64_t ticket, int timeout_ms, astc_request_stats* stats) {
    if (!s) return set_error(ASTC_ERR_INVALID_ARG, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(ASTC_ERR_INVALID_ARG, "unknown ticket");
    Req* r = it->second.get();
    auto done = [&] { return r->state == kDone; };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, done);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
        return set_error(ASTC_ERR_TIMEOUT, "request not finished within the timeout");
    }
    if (stats) {
        stats->submit_us = us_since(s->t0, r->t_submit);
        stats->admit_us = r->status == ASTC_ERR_CANCELLED ? stats->submit_us : us_since(s->t0, r->t_admit);
        stats->done_us = us_since(s->t0, r->t_done);
        stats->status = r->status;
    }
    const astc_status st = r->status;
    s->reqs.erase(it);
    if (st != ASTC_OK)
        return set_error(st, st == ASTC_ERR_CANCELLED ? "request was cancelled" : "request failed: " + s->worker_error);
    return ASTC_OK;
}

astc_status astc_server_cancel(astc_server* s, uint64_t ticket) {
    if (!s) return set_error(ASTC_ERR_INVALID_ARG, "NULL server");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error(ASTC_ERR_INVALID_ARG, "unknown ticket");
    Req* r = it->second.get();
    if (r->state != kQueued) return set_error(ASTC_ERR_BUSY, "request already admitted");
    s->queue.erase(std::find(s->queue.begin(), s->queue.end(), r));
    r->state = kDone;
    r->status = ASTC_ERR_CANCELLED;
    r->t_done = Clock::now();
    s->cv_done.notify_all();
    return ASTC_OK;
}

astc_status astc_server_replay(astc_server* s, const astc_request* reqs, const double* arrival_us, int n,
                               double* latency_us, double* wall_s) {
    if (!s || (n > 0 && (!reqs || !arrival_us || !latency_us))) return set_error(ASTC_ERR_INVALID_ARG, "NULL argument");
    std::vector<uint64_t> tickets(n);
    const Clock::time_point start = Clock::now() + std::chrono::milliseconds(1);
    for (int i = 0; i < n; ++i) {
        const Clock::time_point due = start + std::chrono::nanoseconds((long long)(arrival_us[i] * 1000.0));
        while (Clock::now() < due) {
            if (due - Clock::now() > std::chrono::microseconds(200)) std::this_thread::sleep_for(std::chrono::microseconds(100));
        }
        const astc_status st = astc_server_submit(s, &reqs[i], &tickets[i]);
        if (st != ASTC_OK) {
            for (int k = 0; k < i; ++k) astc_server_wait(s, tickets[k], -1, nullptr);
            return st;
        }
    }
    Clock::time_point last = start;
    astc_status first_err = ASTC_OK;
    for (int i = 0; i < n; ++i) {
        astc_request_stats st{};
        const astc_status rc = astc_server_wait(s, tickets[i], -1, &st);
        if (rc != ASTC_OK && first_err == ASTC_OK) first_err = rc;
        const Clock::time_point due = start + std::chrono::nanoseconds((long long)(arrival_us[i] * 1000.0));
        const double due_us = us_since(s->t0, due);
        latency_us[i] = st.done_us - due_us;
        const Clock::time_point done = s->t0 + std::chrono::nanoseconds((long long)(st.done_us * 1000.0));
        if (done > last) last = done;
    }
    if (wall_s) *wall_s = std::chrono::duration<double>(last - start).count();
    return first_err;
}

astc_status astc_server_get_stats(astc_server* s, int reset, astc_server_stats* out) {
    if (!s || !out) return set_error(ASTC_ERR_INVALID_ARG, "NULL argument");
    std::vector<Interval> iv;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        iv = s->intervals;
        if (reset) s->intervals.clear();
    }
    memset(out, 0, sizeof(*out));
    out->launches = (long long)iv.size();
    if (iv.empty()) return ASTC_OK;
    // sweep over the interval ends: time with >= 1 and >= 2 slots on the device
    std::vector<std::pair<double, int>> ev;
    ev.reserve(2 * iv.size());
    double first = 1e300, last = -1e300;
    for (const Interval& v : iv) {
        out->requests += v.requests;
        out->max_requests_per_launch = std::max(out->max_requests_per_launch, v.requests);
        const double a = v.start_ms * 1e-3, b = std::max(v.start_ms, v.end_ms) * 1e-3;
        out->device_slot_s += b - a;
        ev.push_back({a, +1});
        ev.push_back({b, -1});
        first = std::min(first, a);
        last = std::max(last, b);
    }
    std::sort(ev.begin(), ev.end());
    int depth = 0;
    double prev = ev.front().first;
    for (const auto& p : ev) {
        const double dt = p.first - prev;
        if (depth >= 1) out->device_busy_s += dt;
        if (depth >= 2) out->device_overlap_s += dt;
        depth += p.second;
        prev = p.first;
    }
    out->device_span_s = last - first;
    return ASTC_OK;
}

astc_status astc_server_destroy(astc_server* s) {
    if (!s) return ASTC_OK;
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cv_work.notify_all();
        s->worker.join();
    }
    int cur = 0;
    const bool have = cudaGetDevice(&cur) == cudaSuccess;
    cudaSetDevice(s->device);
    for (Slot& slot : s->slots) {
        if (slot.stream) cudaStreamSynchronize(slot.stream);
        if (slot.batch) astc_batch_destroy(slot.batch);
        if (slot.done) cudaEventDestroy(slot.done);
        if (slot.t_start) cudaEventDestroy(slot.t_start);
        if (slot.t_end) cudaEventDestroy(slot.t_end);
        if (slot.stream) cudaStreamDestroy(slot.stream);
    }
    if (s->t0_event) cudaEventDestroy(s->t0_event);
    if (s->d_pool) cudaFree(s->d_pool);
    if (have) cudaSetDevice(cur);
    cudaGetLastError();
    delete s;
    return ASTC_OK;
}

}  // extern "C"
