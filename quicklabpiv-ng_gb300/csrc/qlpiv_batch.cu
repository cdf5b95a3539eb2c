// Mixed batch plan: many frame pairs of uneven sizes, each with its own IA size and overlap, as
// one flattened work list per IA size, autotuned and captured in one CUDA graph.
// Declarations: include/qlpiv.h (qlpiv_mixed_plan_*).
//
// The reference correlates one pair and one IA size per job (S/jobs/LocalPIVOpenCLGpuJob.java, one
// job per thread, OpenClGpuManager.java:121-148).  Here every pair's level-0 grid
// (AdaptiveInterAreaStrategySuperPosition, as qlpiv_grid_superposition) is appended to the work
// list of its IA size; the plan launches K1 once per size, each launch on its own branch of the
// graph so the sizes run concurrently, and the graph is replayed per batch (schedule
// QLPIV_SCHEDULE_PER_SIZE); or IA 16, 32 and 64 in one persistent launch that drains the three
// work lists (qlpiv_xcorr_mixed.cu) beside the IA-128 launch (QLPIV_SCHEDULE_PERSISTENT).  The
// autotuner times each size's launch over its real work list with 1, 2, 4, 8, 16 and 32 waves of
// resident CTAs and keeps the fastest, then times both schedules over the whole batch and keeps
// the faster.  Vectors come out size-major (16, 32, 64, 128) and pair-contiguous inside a size.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "qlpiv_adaptive.h"
#include "qlpiv_handle.h"
#include "qlpiv_internal.h"
#include "qlpiv_xcorr.cuh"
#include "qlpiv_xcorr_launch.h"

using namespace qlpiv;

namespace {

constexpr int kNumSizes = 4;
constexpr int kSizes[kNumSizes] = {16, 32, 64, 128};

struct Group {
    int n = 0;
    long count = 0, out_offset = 0;
    DevBuf work;       // frame index, a_top, a_left (int32, count each)
    int waves = 0;
    cudaStream_t side = nullptr;
    cudaEvent_t done = nullptr;
};

}  // namespace

struct qlpiv_mixed_plan {
    int device = 0, pixel_type = 0, num_pairs = 0;
    qlpiv_pass_desc tmpl{};
    DevBuf frames, out;
    Group groups[kNumSizes];
    std::vector<int64_t> pair_offset;
    std::vector<int32_t> tiles_ij;
    int64_t total = 0;
    int schedule = QLPIV_SCHEDULE_PER_SIZE;
    DevBuf next;  // the persistent launch's work counters
    cudaStream_t mixed_side = nullptr;
    cudaEvent_t mixed_done = nullptr;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

IaJob group_job(const qlpiv_mixed_plan *p, const Group &g) {
    IaJob job{};
    const int32_t *w = g.work.as<int32_t>();
    job.frames = p->frames.as<qlpiv_frame>();
    job.frame_idx = w;
    job.num_frames = p->num_pairs;
    job.a_top = job.b_top = w + g.count;
    job.a_left = job.b_left = w + 2 * g.count;
    job.count = g.count;
    job.norm_mode = p->tmpl.norm_mode;
    job.max_mode = p->tmpl.max_mode;
    job.fixed_max_a = p->tmpl.fixed_max_a;
    job.fixed_max_b = p->tmpl.fixed_max_b;
    job.subpix = p->tmpl.subpix_mode;
    job.subpix_pixels = p->tmpl.subpix_mode >= QLPIV_SUBPIX_GAUSS_LM ? p->tmpl.subpix_pixels : 0;
    job.subpix_iters = p->tmpl.subpix_iterations;
    job.out = p->out.as<qlpiv_vector>() + g.out_offset;
    job.waves = g.waves;
    return job;
}

// The persistent launch covers IA 16, 32 and 64 (IA 128 keeps its own launch).
bool persistent_supported(const qlpiv_mixed_plan *p) {
    bool any = false;
    for (int k = 0; k < 3; k++) {
        const Group &g = p->groups[k];
        if (g.count == 0) continue;
        any = true;
        if (!mixed_kernel_supported(group_job(p, g))) return false;
    }
    return any;
}

// Queues one batch on s with the given schedule: every launch on its own branch forked from s,
// joined back into s (also the body of the captured graph).
cudaError_t enqueue(qlpiv_mixed_plan *p, cudaStream_t s, int num_sms, int schedule) {
    cudaError_t e = cudaEventRecord(p->fork, s);
    for (Group &g : p->groups) {
        if (g.count == 0 || e != cudaSuccess) continue;
        if (schedule == QLPIV_SCHEDULE_PERSISTENT && g.n != 128) continue;
        if ((e = cudaStreamWaitEvent(g.side, p->fork, 0)) != cudaSuccess) break;
        IaJob job = group_job(p, g);
        if ((e = launch_xcorr(job, g.n, p->pixel_type, g.side, num_sms)) != cudaSuccess) break;
        if ((e = cudaEventRecord(g.done, g.side)) != cudaSuccess) break;
        if ((e = cudaStreamWaitEvent(s, g.done, 0)) != cudaSuccess) break;
    }
    if (e == cudaSuccess && schedule == QLPIV_SCHEDULE_PERSISTENT) {
        MixedJob mj{};
        const int order[3] = {2, 1, 0};  // IA 64, 32, 16
        for (int k = 0; k < 3; k++) mj.job[k] = group_job(p, p->groups[order[k]]);
        mj.next = p->next.as<unsigned>();
        if ((e = cudaStreamWaitEvent(p->mixed_side, p->fork, 0)) == cudaSuccess &&
            (e = launch_k1_mixed(mj, p->pixel_type, p->mixed_side, num_sms)) == cudaSuccess &&
            (e = cudaEventRecord(p->mixed_done, p->mixed_side)) == cudaSuccess)
            e = cudaStreamWaitEvent(s, p->mixed_done, 0);
    }
    return e;
}

void release(qlpiv_mixed_plan *p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->fork) cudaEventDestroy(p->fork);
    if (p->mixed_side) cudaStreamDestroy(p->mixed_side);
    if (p->mixed_done) cudaEventDestroy(p->mixed_done);
    p->next.release();
    for (Group &g : p->groups) {
        if (g.side) cudaStreamDestroy(g.side);
        if (g.done) cudaEventDestroy(g.done);
        g.work.release();
    }
    p->frames.release();
    p->out.release();
    delete p;
}

}  // namespace

extern "C" {

qlpiv_status qlpiv_mixed_plan_create(qlpiv_handle *h, const qlpiv_pass_desc *tmpl, int pixel_type, int num_pairs,
                                     const qlpiv_frame *frames, const int32_t *ia_size, const float *overlap_factor,
                                     int autotune, qlpiv_mixed_plan **out) {
    if (!h || !tmpl || !frames || !ia_size || !overlap_factor || !out) return fail(QLPIV_E_ARG, "NULL argument");
    *out = nullptr;
    if (num_pairs <= 0) return fail(QLPIV_E_ARG, "num_pairs must be positive");
    if (pixel_type != QLPIV_PIX_U8 && pixel_type != QLPIV_PIX_U16 && pixel_type != QLPIV_PIX_F32)
        return fail(QLPIV_E_ARG, "unknown pixel type %d", pixel_type);
    if (tmpl->num_peaks != 0) return fail(QLPIV_E_ARG, "mixed batches run FindMaximumFromCenter (num_peaks 0)");
    if (qlpiv_status st = check_subpix(tmpl->subpix_mode, tmpl->subpix_pixels, tmpl->subpix_iterations)) return st;
    if (tmpl->max_mode == QLPIV_MAX_GIVEN) return fail(QLPIV_E_ARG, "given tile maxima need the tile entry points");
    qlpiv_mixed_plan *p = new qlpiv_mixed_plan();
    p->device = h->device;
    p->pixel_type = pixel_type;
    p->num_pairs = num_pairs;
    p->tmpl = *tmpl;
    // per size: the flattened work lists (pairs in order, tiles row-major)
    std::vector<int32_t> lists[kNumSizes][3];
    std::vector<int> pair_group(num_pairs);
    std::vector<long> pair_first(num_pairs);
    p->tiles_ij.resize(2 * (size_t)num_pairs);
    const int margins[4] = {0, 0, 0, 0};
    for (int q = 0; q < num_pairs; q++) {
        const qlpiv_frame &f = frames[q];
        int gi = -1;
        for (int k = 0; k < kNumSizes; k++)
            if (ia_size[q] == kSizes[k]) gi = k;
        if (gi < 0) {
            release(p);
            return fail(QLPIV_E_SHAPE, "pair %d: IA size %d is not supported (16, 32, 64, 128)", q, ia_size[q]);
        }
        if (!f.img_a || !f.img_b || f.height <= 0 || f.width <= 0 || f.pitch < f.width) {
            release(p);
            return fail(QLPIV_E_SHAPE, "pair %d: NULL image or bad geometry", q);
        }
        qlpiv_grid g{};
        if (grid_superposition(f.height, f.width, margins, ia_size[q], 0, overlap_factor[q], &g, nullptr, nullptr,
                               0) < -1 ||
            g.tiles_i <= 0 || g.tiles_j <= 0) {
            release(p);
            return fail(QLPIV_E_SHAPE, "pair %d: image %d x %d too small for IA %d", q, f.height, f.width, ia_size[q]);
        }
        std::vector<int32_t> tops(g.tiles_i), lefts(g.tiles_j);
        grid_superposition(f.height, f.width, margins, ia_size[q], 0, overlap_factor[q], &g, tops.data(),
                           lefts.data(), 1 << 30);
        pair_group[q] = gi;
        pair_first[q] = (long)lists[gi][0].size();
        p->tiles_ij[2 * q] = g.tiles_i;
        p->tiles_ij[2 * q + 1] = g.tiles_j;
        for (int i = 0; i < g.tiles_i; i++)
            for (int j = 0; j < g.tiles_j; j++) {
                lists[gi][0].push_back(q);
                lists[gi][1].push_back(tops[i]);
                lists[gi][2].push_back(lefts[j]);
            }
    }
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    cudaStream_t s = h->stream;
    cudaError_t e;
    long off = 0;
    for (int k = 0; k < kNumSizes; k++) {
        Group &g = p->groups[k];
        g.n = kSizes[k];
        g.count = (long)lists[k][0].size();
        g.out_offset = off;
        off += g.count;
    }
    p->total = off;
    p->pair_offset.resize(num_pairs + 1);
    for (int q = 0; q < num_pairs; q++) p->pair_offset[q] = p->groups[pair_group[q]].out_offset + pair_first[q];
    p->pair_offset[num_pairs] = p->total;
    if ((e = p->frames.ensure(sizeof(qlpiv_frame) * num_pairs)) != cudaSuccess ||
        (e = p->out.ensure(sizeof(qlpiv_vector) * (size_t)(p->total > 0 ? p->total : 1))) != cudaSuccess ||
        (e = cudaMemcpyAsync(p->frames.p, frames, sizeof(qlpiv_frame) * num_pairs, cudaMemcpyHostToDevice, s)) !=
            cudaSuccess ||
        (e = cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming)) != cudaSuccess) {
        release(p);
        return cuda_fail(e, "mixed plan buffers");
    }
    for (Group &g : p->groups) {
        if (g.count == 0) continue;
        const int k = (int)(&g - p->groups);
        if ((e = g.work.ensure(sizeof(int32_t) * 3 * g.count)) != cudaSuccess ||
            (e = cudaStreamCreateWithFlags(&g.side, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming)) != cudaSuccess) {
            release(p);
            return cuda_fail(e, "mixed plan group");
        }
        for (int a = 0; a < 3; a++)
            if ((e = cudaMemcpyAsync(g.work.as<int32_t>() + a * g.count, lists[k][a].data(), sizeof(int32_t) * g.count,
                                     cudaMemcpyHostToDevice, s)) != cudaSuccess) {
                release(p);
                return cuda_fail(e, "work list upload");
            }
    }
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) {  // the host lists die at return
        release(p);
        return cuda_fail(e, "mixed plan upload");
    }
    // autotune the waves of each size on its own work list (also the launches' first-use set-up,
    // which must not happen inside the capture)
    const bool tune = autotune == QLPIV_AUTOTUNE_ON;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    for (Group &g : p->groups) {
        if (g.count == 0) continue;
        const int cands[6] = {1, 2, 4, 8, 16, 32};
        float best = 1e30f;
        int best_w = 8;
        for (int c = 0; c < (tune ? 6 : 1); c++) {
            g.waves = tune ? cands[c] : 0;
            IaJob job = group_job(p, g);
            if ((e = launch_xcorr(job, g.n, pixel_type, s, h->num_sms)) != cudaSuccess) break;  // warm-up
            cudaEventRecord(t0, s);
            for (int r = 0; r < 3 && e == cudaSuccess; r++) e = launch_xcorr(job, g.n, pixel_type, s, h->num_sms);
            cudaEventRecord(t1, s);
            if (e != cudaSuccess || (e = cudaEventSynchronize(t1)) != cudaSuccess) break;
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, t0, t1);
            if (ms < best) {
                best = ms;
                best_w = g.waves;
            }
        }
        if (e != cudaSuccess) break;
        g.waves = tune ? best_w : 0;
    }
    // the schedule: per-size launches, or the persistent launch (timed over the whole batch)
    if (e == cudaSuccess && autotune != QLPIV_AUTOTUNE_OFF && persistent_supported(p)) {
        if ((e = p->next.ensure(4 * sizeof(unsigned))) == cudaSuccess &&
            (e = cudaStreamCreateWithFlags(&p->mixed_side, cudaStreamNonBlocking)) == cudaSuccess)
            e = cudaEventCreateWithFlags(&p->mixed_done, cudaEventDisableTiming);
        float ms_sched[2] = {1e30f, 1e30f};
        for (int sc = 0; sc < 2 && e == cudaSuccess; sc++) {
            if (!tune && sc != QLPIV_SCHEDULE_PERSISTENT) continue;
            if ((e = enqueue(p, s, h->num_sms, sc)) != cudaSuccess) break;  // warm-up
            cudaEventRecord(t0, s);
            for (int r = 0; r < 3 && e == cudaSuccess; r++) e = enqueue(p, s, h->num_sms, sc);
            cudaEventRecord(t1, s);
            if (e != cudaSuccess || (e = cudaEventSynchronize(t1)) != cudaSuccess) break;
            cudaEventElapsedTime(&ms_sched[sc], t0, t1);
        }
        if (e == cudaSuccess)
            p->schedule = ms_sched[QLPIV_SCHEDULE_PERSISTENT] < ms_sched[QLPIV_SCHEDULE_PER_SIZE]
                              ? QLPIV_SCHEDULE_PERSISTENT
                              : QLPIV_SCHEDULE_PER_SIZE;
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (e != cudaSuccess) {
        release(p);
        return cuda_fail(e, "autotune");
    }
    // capture: fork one branch per launch from the handle's stream, join back
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        release(p);
        return cuda_fail(e, "graph capture");
    }
    cudaError_t ce = enqueue(p, s, h->num_sms, p->schedule);
    e = cudaStreamEndCapture(s, &p->graph);
    if (ce != cudaSuccess || e != cudaSuccess ||
        (e = cudaGraphInstantiate(&p->exec, p->graph, 0)) != cudaSuccess) {
        release(p);
        return cuda_fail(ce != cudaSuccess ? ce : e, "graph capture");
    }
    *out = p;
    return QLPIV_OK;
}

qlpiv_status qlpiv_mixed_plan_info(const qlpiv_mixed_plan *p, int64_t *total_vectors, int64_t *pair_offset,
                                   int32_t *tiles_ij, int32_t *waves) {
    if (!p) return fail(QLPIV_E_ARG, "plan is NULL");
    if (total_vectors) *total_vectors = p->total;
    if (pair_offset) std::memcpy(pair_offset, p->pair_offset.data(), sizeof(int64_t) * (p->num_pairs + 1));
    if (tiles_ij) std::memcpy(tiles_ij, p->tiles_ij.data(), sizeof(int32_t) * 2 * p->num_pairs);
    if (waves)
        for (int k = 0; k < kNumSizes; k++) waves[k] = p->groups[k].waves;
    return QLPIV_OK;
}

qlpiv_status qlpiv_mixed_plan_schedule(const qlpiv_mixed_plan *p, int32_t *schedule) {
    if (!p || !schedule) return fail(QLPIV_E_ARG, "NULL argument");
    *schedule = p->schedule;
    return QLPIV_OK;
}

qlpiv_status qlpiv_mixed_plan_run(qlpiv_handle *h, qlpiv_mixed_plan *p, qlpiv_vector **device_out) {
    if (!h || !p) return fail(QLPIV_E_ARG, "NULL argument");
    if (h->device != p->device) return fail(QLPIV_E_ARG, "plan belongs to device %d", p->device);
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    const cudaError_t e = cudaGraphLaunch(p->exec, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "graph launch");
    for (const Group &g : p->groups)
        h->launches += g.count > 0 && (p->schedule == QLPIV_SCHEDULE_PER_SIZE || g.n == 128) ? 1 : 0;
    if (p->schedule == QLPIV_SCHEDULE_PERSISTENT) h->launches += 1;
    if (device_out) *device_out = p->out.as<qlpiv_vector>();
    return QLPIV_OK;
}

qlpiv_status qlpiv_mixed_plan_download(qlpiv_handle *h, qlpiv_mixed_plan *p, qlpiv_vector *host_out) {
    if (!h || !p || !host_out) return fail(QLPIV_E_ARG, "NULL argument");
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    cudaError_t e;
    if ((e = cudaMemcpyAsync(host_out, p->out.p, sizeof(qlpiv_vector) * p->total, cudaMemcpyDeviceToHost,
                             h->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(h->stream)) != cudaSuccess)
        return cuda_fail(e, "mixed plan download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_mixed_plan_destroy(qlpiv_mixed_plan *p) {
    if (!p) return QLPIV_OK;
    DeviceScope ds(p->device);
    release(p);
    return QLPIV_OK;
}

}  // extern "C"
