// Request server: continuous batching of adaptive PIV requests on one device.
// Declarations: include/qlpiv.h (qlpiv_server_*).
//
// The reference processes one frame pair per job and host thread (S/jobs/LocalPIVOpenCLGpuJob.java,
// jobs pooled by S/jobs/OpenClGpuManager.java:121-148).  Here a device-owner thread keeps up to
// `slots` requests on the GPU at once, each on its own stream with its own adaptive plan, so the
// kernels of requests of different sizes and schedules overlap on the device:
//
//   submit (any thread)   checks the request, copies both frames into pinned staging (a first-fit
//                         arena), queues it;
//   owner thread          admits queued requests first-fit while their device memory (the plan
//                         estimate) fits the HBM budget and a slot is free; a slot whose cached
//                         plan matches the request reuses it; idle slots' cached plans are dropped
//                         when memory is short; device memory comes from a stream-ordered pool,
//                         so no allocation synchronises the device;
//   completion            a host callback after the result download wakes the owner, which copies
//                         the results into the caller's buffers and marks the ticket done;
//   poll (any thread)     waits for its ticket.
//
// A request's work is exactly the qlpiv_piv_adaptive sequence for its pair, so its result does
// not depend on what else is in flight.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "qlpiv_handle.h"
#include "qlpiv_internal.h"

namespace qlpiv {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// First-fit allocator over one pinned host block (offsets in 256-byte units of alignment).
class PinnedArena {
  public:
    cudaError_t init(size_t bytes) {
        cap_ = (bytes + 255) & ~(size_t)255;
        cudaError_t e = cudaHostAlloc(&base_, cap_, cudaHostAllocPortable);
        if (e != cudaSuccess) {
            base_ = nullptr;
            return e;
        }
        free_[0] = cap_;
        return cudaSuccess;
    }
    void release() {
        if (base_) cudaFreeHost(base_);
        base_ = nullptr;
        free_.clear();
    }
    size_t capacity() const { return cap_; }
    // nullptr when no free block is large enough
    char *alloc(size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t off = it->first, len = it->second;
            free_.erase(it);
            if (len > bytes) free_[off + bytes] = len - bytes;
            return base_ + off;
        }
        return nullptr;
    }
    void free(char *p, size_t bytes) {
        if (!p) return;
        bytes = (bytes + 255) & ~(size_t)255;
        size_t off = (size_t)(p - base_);
        auto next = free_.lower_bound(off);
        if (next != free_.end() && off + bytes == next->first) {  // merge with the following block
            bytes += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {  // merge with the preceding block
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += bytes;
                return;
            }
        }
        free_[off] = bytes;
    }

  private:
    char *base_ = nullptr;
    size_t cap_ = 0;
    std::map<size_t, size_t> free_;  // offset -> length
};

struct Request {
    uint64_t ticket = 0;
    qlpiv_adaptive_desc desc{};
    int pixel_type = 0, height = 0, width = 0, tiles_i = 0, tiles_j = 0;
    size_t dev_bytes = 0;
    char *stage_in = nullptr, *stage_out = nullptr;  // pinned: frames A, B (packed rows); results u, v
    size_t in_bytes = 0, out_bytes = 0;
    float *out_u = nullptr, *out_v = nullptr;        // caller's buffers
    qlpiv_status status = QLPIV_OK;
    std::string error;
    bool done = false;
    Clock::time_point t_submit, t_admit, t_done;
};

struct Slot {
    qlpiv_handle *h = nullptr;
    Request *req = nullptr;
    bool finished = false;           // set by the stream callback
    size_t held = 0;                 // device bytes of the cached plan (estimate)
    qlpiv_adaptive_desc key{};       // what the cached plan was built for
    int key_pt = -1, key_h = 0, key_w = 0;
};

}  // namespace
}  // namespace qlpiv

using namespace qlpiv;

struct qlpiv_server {
    int device = 0;
    size_t budget = 0;
    int submit_timeout_ms = 10000;
    cudaMemPool_t pool = nullptr;
    PinnedArena arena;
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cv_owner, cv_done, cv_staging;
    std::deque<Request *> pending;
    std::unordered_map<uint64_t, Request *> reqs;
    uint64_t next_ticket = 1;
    bool stop = false;
    bool wake = false;
    int64_t submitted = 0, completed = 0, failed = 0;
    std::thread owner;
};

namespace {

struct SlotDone {
    qlpiv_server *s;
    int slot;
};

void CUDART_CB on_slot_done(void *p) {
    SlotDone *d = static_cast<SlotDone *>(p);
    {
        std::lock_guard<std::mutex> lk(d->s->mu);
        d->s->slots[d->slot].finished = true;
        d->s->wake = true;
    }
    d->s->cv_owner.notify_one();
    delete d;
}

size_t held_total(const qlpiv_server *s) {
    size_t t = 0;
    for (const Slot &sl : s->slots) t += sl.held;
    return t;
}

bool same_key(const Slot &sl, const Request *r) {
    return sl.key_pt == r->pixel_type && sl.key_h == r->height && sl.key_w == r->width &&
           std::memcmp(&sl.key, &r->desc, sizeof(r->desc)) == 0;
}

void finish(qlpiv_server *s, Request *r, qlpiv_status st, const std::string &msg) {
    r->status = st;
    r->error = msg;
    r->done = true;
    r->t_done = Clock::now();
    if (st == QLPIV_OK) s->completed++;
    else s->failed++;
    s->arena.free(r->stage_in, r->in_bytes);
    s->arena.free(r->stage_out, r->out_bytes);
    r->stage_in = r->stage_out = nullptr;
    s->cv_staging.notify_all();
    s->cv_done.notify_all();
}

// Picks a free slot for r and makes room in the budget; -1 when r cannot start now.
int choose_slot(qlpiv_server *s, const Request *r) {
    int best = -1;
    for (int k = 0; k < (int)s->slots.size(); k++) {
        const Slot &sl = s->slots[k];
        if (sl.req) continue;
        if (same_key(sl, r)) return k;  // its plan is reused: no new memory
        if (best < 0 || sl.held > s->slots[best].held) best = k;
    }
    if (best < 0) return -1;
    size_t need = held_total(s) - s->slots[best].held + r->dev_bytes;
    // drop idle slots' cached plans while the budget is short
    for (int k = 0; k < (int)s->slots.size() && need > s->budget; k++) {
        Slot &sl = s->slots[k];
        if (k == best || sl.req || sl.held == 0) continue;
        drop_plan(sl.h);
        need -= sl.held;
        sl.held = 0;
        sl.key_pt = -1;
    }
    return need <= s->budget ? best : -1;
}

void owner_loop(qlpiv_server *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        // completions
        for (int k = 0; k < (int)s->slots.size(); k++) {
            Slot &sl = s->slots[k];
            if (!sl.req) continue;
            const cudaError_t e = cudaStreamQuery(sl.h->stream);
            if (!sl.finished && e == cudaErrorNotReady) continue;
            Request *r = sl.req;
            sl.req = nullptr;
            sl.finished = false;
            if (e != cudaSuccess && e != cudaErrorNotReady) {
                finish(s, r, QLPIV_E_CUDA, std::string("device error: ") + cudaGetErrorString(e));
                continue;
            }
            const size_t n = (size_t)r->tiles_i * r->tiles_j;
            std::memcpy(r->out_u, r->stage_out, sizeof(float) * n);
            std::memcpy(r->out_v, r->stage_out + sizeof(float) * n, sizeof(float) * n);
            finish(s, r, QLPIV_OK, "");
        }
        // admissions, first fit in arrival order
        for (auto it = s->pending.begin(); it != s->pending.end() && !s->stop;) {
            Request *r = *it;
            const int k = choose_slot(s, r);
            if (k < 0) {
                ++it;
                continue;
            }
            it = s->pending.erase(it);
            Slot &sl = s->slots[k];
            sl.req = r;
            sl.finished = false;
            r->t_admit = Clock::now();
            const bool reuse = same_key(sl, r);
            if (!reuse) {
                sl.held = r->dev_bytes;
                sl.key = r->desc;
                sl.key_pt = r->pixel_type;
                sl.key_h = r->height;
                sl.key_w = r->width;
            }
            // queue the request's work without holding the lock (only this thread uses the slot)
            lk.unlock();
            qlpiv_status st;
            std::string msg;
            {
                AsyncAllocScope scope(s->pool, sl.h->stream);
                const size_t n = (size_t)r->tiles_i * r->tiles_j;
                const size_t img = (size_t)r->height * r->width * pixel_bytes(r->pixel_type);
                float *ou = reinterpret_cast<float *>(r->stage_out);
                st = queue_adaptive_pinned(sl.h, &r->desc, r->pixel_type, r->height, r->width, r->stage_in,
                                           r->stage_in + ((img + 255) & ~(size_t)255), r->width, ou, ou + n);
                if (st == QLPIV_OK) {
                    SlotDone *d = new SlotDone{s, k};
                    const cudaError_t e = cudaLaunchHostFunc(sl.h->stream, on_slot_done, d);
                    if (e != cudaSuccess) {
                        delete d;
                        st = cuda_fail(e, "completion callback");
                    }
                }
                if (st != QLPIV_OK) msg = qlpiv_last_error();
            }
            lk.lock();
            if (st != QLPIV_OK) {
                sl.req = nullptr;
                drop_plan(sl.h);
                sl.held = 0;
                sl.key_pt = -1;
                finish(s, r, st, msg);
            }
        }
        bool busy = false;
        for (const Slot &sl : s->slots) busy = busy || sl.req != nullptr;
        if (s->stop && !busy) break;
        if (!s->wake) {
            // callbacks wake the loop; the timeout also catches a stream that failed before them
            s->cv_owner.wait_for(lk, std::chrono::milliseconds(busy ? 5 : 100));
        }
        s->wake = false;
    }
}

}  // namespace

extern "C" {

qlpiv_status qlpiv_adaptive_plan_bytes(const qlpiv_adaptive_desc *desc, int pixel_type, int height, int width,
                                       int pairs, int64_t *bytes) {
    if (!desc || !bytes || pairs <= 0) return fail(QLPIV_E_ARG, "NULL argument or pairs <= 0");
    int n = 0;
    qlpiv_grid g[16];
    qlpiv_status st = qlpiv_adaptive_levels(desc, height, width, &n, g, 16);
    if (st != QLPIV_OK) return st;
    if (pixel_type != QLPIV_PIX_U8 && pixel_type != QLPIV_PIX_U16)
        return fail(QLPIV_E_ARG, "adaptive PIV takes u8 or u16 images");
    const size_t b = plan_device_bytes(desc, pixel_type, height, width, pairs);
    if (b == 0) return fail(QLPIV_E_SHAPE, "image too small for the schedule");
    *bytes = (int64_t)b;
    return QLPIV_OK;
}

qlpiv_status qlpiv_server_create(const qlpiv_server_params *params, qlpiv_server **out) {
    if (!out) return fail(QLPIV_E_ARG, "output pointer is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return fail(QLPIV_E_NO_DEVICE, "no CUDA device (%s)", cudaGetErrorString(e));
    const int dev = params ? params->device : 0;
    if (dev < 0 || dev >= ndev) return fail(QLPIV_E_ARG, "device %d out of range", dev);
    const int nslots = params && params->slots > 0 ? params->slots : 16;
    if (nslots > 256) return fail(QLPIV_E_ARG, "at most 256 slots");
    DeviceScope ds(dev);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    qlpiv_server *s = new qlpiv_server();
    s->device = dev;
    s->submit_timeout_ms = params && params->submit_timeout_ms > 0 ? params->submit_timeout_ms : 10000;
    size_t free_b = 0, total_b = 0;
    if ((e = cudaMemGetInfo(&free_b, &total_b)) != cudaSuccess) {
        delete s;
        return cuda_fail(e, "cudaMemGetInfo");
    }
    s->budget = params && params->hbm_budget > 0 ? (size_t)params->hbm_budget : (size_t)(0.8 * (double)free_b);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    if ((e = cudaMemPoolCreate(&s->pool, &props)) != cudaSuccess) {
        delete s;
        return cuda_fail(e, "memory pool");
    }
    uint64_t keep = s->budget;  // freed blocks stay in the pool up to the budget
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    const size_t staging = params && params->staging_bytes > 0 ? (size_t)params->staging_bytes : ((size_t)1 << 30);
    if ((e = s->arena.init(staging)) != cudaSuccess) {
        cudaMemPoolDestroy(s->pool);
        delete s;
        return cuda_fail(e, "pinned staging");
    }
    s->slots.resize(nslots);
    for (Slot &sl : s->slots) {
        qlpiv_params hp{};
        hp.device = dev;
        qlpiv_status st = qlpiv_create(&hp, &sl.h);
        if (st != QLPIV_OK) {
            for (Slot &o : s->slots)
                if (o.h) qlpiv_destroy(o.h);
            s->arena.release();
            cudaMemPoolDestroy(s->pool);
            delete s;
            return st;
        }
    }
    s->owner = std::thread(owner_loop, s);
    *out = s;
    return QLPIV_OK;
}

qlpiv_status qlpiv_server_destroy(qlpiv_server *s) {
    if (!s) return QLPIV_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->wake = true;
        for (Request *r : s->pending) finish(s, r, QLPIV_E_CANCELLED, "server destroyed");
        s->pending.clear();
    }
    s->cv_owner.notify_all();
    if (s->owner.joinable()) s->owner.join();
    DeviceScope ds(s->device);
    for (Slot &sl : s->slots) {
        if (!sl.h) continue;
        drop_plan(sl.h);
        qlpiv_destroy(sl.h);
    }
    for (auto &kv : s->reqs) delete kv.second;
    s->arena.release();
    if (s->pool) cudaMemPoolDestroy(s->pool);
    delete s;
    return QLPIV_OK;
}

qlpiv_status qlpiv_submit(qlpiv_server *s, const qlpiv_request *rq, uint64_t *ticket) {
    if (!s || !rq || !ticket || !rq->schedule || !rq->img_a || !rq->img_b || !rq->out_u || !rq->out_v)
        return fail(QLPIV_E_ARG, "NULL argument");
    if (rq->pixel_type != QLPIV_PIX_U8 && rq->pixel_type != QLPIV_PIX_U16)
        return fail(QLPIV_E_ARG, "adaptive PIV takes u8 or u16 images");
    if (rq->height <= 0 || rq->width <= 0 || rq->pitch < rq->width)
        return fail(QLPIV_E_SHAPE, "image %d x %d, pitch %lld", rq->height, rq->width, (long long)rq->pitch);
    int n = 0;
    qlpiv_grid g[16];
    qlpiv_status st = qlpiv_adaptive_levels(rq->schedule, rq->height, rq->width, &n, g, 16);
    if (st != QLPIV_OK) return st;
    int64_t dev_bytes = 0;
    if ((st = qlpiv_adaptive_plan_bytes(rq->schedule, rq->pixel_type, rq->height, rq->width, 1, &dev_bytes)) !=
        QLPIV_OK)
        return st;
    Request *r = new Request();
    r->desc = *rq->schedule;
    r->pixel_type = rq->pixel_type;
    r->height = rq->height;
    r->width = rq->width;
    r->tiles_i = g[n - 1].tiles_i;
    r->tiles_j = g[n - 1].tiles_j;
    r->dev_bytes = (size_t)dev_bytes;
    r->out_u = rq->out_u;
    r->out_v = rq->out_v;
    const size_t pb = pixel_bytes(rq->pixel_type), row = (size_t)rq->width * pb, img = row * rq->height;
    const size_t img_al = (img + 255) & ~(size_t)255;
    r->in_bytes = 2 * img_al;
    r->out_bytes = sizeof(float) * 2 * (size_t)r->tiles_i * r->tiles_j;
    if (r->dev_bytes > s->budget || r->in_bytes + r->out_bytes > s->arena.capacity()) {
        delete r;
        return fail(QLPIV_E_OOM, "request needs %zu device bytes (budget %zu) and %zu staging bytes",
                    (size_t)dev_bytes, s->budget, (size_t)(2 * img_al));
    }
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop) {
        delete r;
        return fail(QLPIV_E_CANCELLED, "server is shutting down");
    }
    const auto deadline = Clock::now() + std::chrono::milliseconds(s->submit_timeout_ms);
    for (;;) {
        r->stage_in = s->arena.alloc(r->in_bytes);
        if (r->stage_in) {
            r->stage_out = s->arena.alloc(r->out_bytes);
            if (r->stage_out) break;
            s->arena.free(r->stage_in, r->in_bytes);
            r->stage_in = nullptr;
        }
        if (s->cv_staging.wait_until(lk, deadline) == std::cv_status::timeout) {
            delete r;
            return fail(QLPIV_E_TIMEOUT, "pinned staging stayed full for %d ms", s->submit_timeout_ms);
        }
    }
    char *a = r->stage_in, *b = r->stage_in + img_al;
    lk.unlock();  // the copy into staging runs in the caller's thread, unlocked
    const char *sa = static_cast<const char *>(rq->img_a), *sb = static_cast<const char *>(rq->img_b);
    const size_t src_row = (size_t)rq->pitch * pb;
    for (int y = 0; y < rq->height; y++) {
        std::memcpy(a + y * row, sa + y * src_row, row);
        std::memcpy(b + y * row, sb + y * src_row, row);
    }
    lk.lock();
    r->t_submit = Clock::now();
    r->ticket = s->next_ticket++;
    s->reqs[r->ticket] = r;
    s->pending.push_back(r);
    s->submitted++;
    s->wake = true;
    *ticket = r->ticket;
    lk.unlock();
    s->cv_owner.notify_one();
    return QLPIV_OK;
}

qlpiv_status qlpiv_poll(qlpiv_server *s, uint64_t ticket, qlpiv_result *result, int timeout_ms) {
    if (!s || !result) return fail(QLPIV_E_ARG, "NULL argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return fail(QLPIV_E_ARG, "unknown ticket %llu", (unsigned long long)ticket);
    Request *r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        return QLPIV_E_TIMEOUT;
    result->status = r->status;
    result->tiles_i = r->tiles_i;
    result->tiles_j = r->tiles_j;
    const bool admitted = r->t_admit.time_since_epoch().count() != 0;
    result->queue_ms = admitted ? ms_between(r->t_submit, r->t_admit) : ms_between(r->t_submit, r->t_done);
    result->device_ms = admitted ? ms_between(r->t_admit, r->t_done) : 0.0;
    result->total_ms = ms_between(r->t_submit, r->t_done);
    const qlpiv_status st = r->status;
    const std::string msg = r->error;
    s->reqs.erase(it);
    delete r;
    if (st != QLPIV_OK) fail(st, "%s", msg.c_str());  // the request's message for qlpiv_last_error
    return QLPIV_OK;
}

qlpiv_status qlpiv_server_stats_read(qlpiv_server *s, qlpiv_server_stats *st) {
    if (!s || !st) return fail(QLPIV_E_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(st, 0, sizeof(*st));
    st->submitted = s->submitted;
    st->completed = s->completed;
    st->failed = s->failed;
    st->pending = (int64_t)s->pending.size();
    for (const Slot &sl : s->slots) st->in_flight += sl.req ? 1 : 0;
    st->device_bytes_in_flight = (int64_t)held_total(s);
    st->hbm_budget = (int64_t)s->budget;
    return QLPIV_OK;
}

}  // extern "C"
