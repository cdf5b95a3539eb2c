// Adaptive batch: frame pairs of uneven sizes, each with its own adaptive schedule, replayed from
// one captured CUDA graph.  Declarations: include/qlpiv.h (qlpiv_adaptive_batch_*).
//
// The reference runs one adaptive job per frame pair and host thread (S/jobs/LocalPIVOpenCLGpuJob.java
// :188-411, pooled by S/jobs/OpenClGpuManager.java:121-148).  Here the pairs that share frame size,
// pixel type and schedule form a group; a group runs the device adaptive loop of
// qlpiv_piv_adaptive_device over all its pairs (every level one flattened work list, warping,
// validation and inheritance for the whole group) on its own stream, and the groups are branches of
// one graph forked from and joined into the caller's handle stream, so groups of different sizes and
// schedules overlap on the device.  A pair's displacements are those qlpiv_piv_adaptive gives for it
// alone.
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "qlpiv_handle.h"
#include "qlpiv_internal.h"

using namespace qlpiv;

namespace {

struct BatchGroup {
    qlpiv_handle *h = nullptr;  // own stream and adaptive plan
    qlpiv_adaptive_desc desc{};
    int height = 0, width = 0, pairs = 0, tiles = 0;  // tiles: last level's tiles per pair
    long out_offset = 0;                              // in the batch's outputs
    DevBuf table;                                     // the group's device frame table
    cudaEvent_t done = nullptr;
};

}  // namespace

struct qlpiv_adaptive_batch {
    int device = 0, pixel_type = 0, num_pairs = 0;
    std::vector<BatchGroup> groups;
    std::vector<int64_t> pair_offset;
    std::vector<int32_t> tiles_ij;
    int64_t total = 0;
    DevBuf out_u, out_v;
    cudaEvent_t fork = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

void release(qlpiv_adaptive_batch *b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->fork) cudaEventDestroy(b->fork);
    for (BatchGroup &g : b->groups) {
        g.table.release();
        if (g.done) cudaEventDestroy(g.done);
        if (g.h) qlpiv_destroy(g.h);
    }
    b->out_u.release();
    b->out_v.release();
    delete b;
}

// Queues every group's adaptive loop on its own stream, forked from and joined into s.
qlpiv_status enqueue(qlpiv_adaptive_batch *b, cudaStream_t s) {
    cudaError_t e = cudaEventRecord(b->fork, s);
    if (e != cudaSuccess) return cuda_fail(e, "batch fork");
    for (BatchGroup &g : b->groups) {
        if ((e = cudaStreamWaitEvent(g.h->stream, b->fork, 0)) != cudaSuccess) return cuda_fail(e, "batch fork");
        const qlpiv_status st = qlpiv_piv_adaptive_device(g.h, &g.desc, b->pixel_type, g.height, g.width, g.pairs,
                                                          g.table.as<qlpiv_frame>(), b->out_u.as<float>() + g.out_offset,
                                                          b->out_v.as<float>() + g.out_offset);
        if (st != QLPIV_OK) return st;
        if ((e = cudaEventRecord(g.done, g.h->stream)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(s, g.done, 0)) != cudaSuccess)
            return cuda_fail(e, "batch join");
    }
    return QLPIV_OK;
}

}  // namespace

extern "C" {

qlpiv_status qlpiv_adaptive_batch_create(qlpiv_handle *h, int pixel_type, int num_pairs, const qlpiv_frame *frames,
                                         const qlpiv_adaptive_desc *schedules, int num_schedules,
                                         const int32_t *schedule_of_pair, qlpiv_adaptive_batch **out) {
    if (!h || !frames || !schedules || !schedule_of_pair || !out) return fail(QLPIV_E_ARG, "NULL argument");
    *out = nullptr;
    if (num_pairs <= 0 || num_schedules <= 0) return fail(QLPIV_E_ARG, "num_pairs and num_schedules must be positive");
    if (pixel_type != QLPIV_PIX_U8 && pixel_type != QLPIV_PIX_U16)
        return fail(QLPIV_E_ARG, "adaptive PIV takes u8 or u16 images");
    // group the pairs by (height, width, schedule), in order of first appearance
    std::map<std::tuple<int, int, int>, int> key_group;
    std::vector<std::vector<int>> members;
    std::vector<std::tuple<int, int, int>> keys;
    for (int q = 0; q < num_pairs; q++) {
        const qlpiv_frame &f = frames[q];
        const int si = schedule_of_pair[q];
        if (si < 0 || si >= num_schedules) return fail(QLPIV_E_ARG, "pair %d: schedule %d out of range", q, si);
        if (!f.img_a || !f.img_b || f.height <= 0 || f.width <= 0 || f.pitch < f.width)
            return fail(QLPIV_E_SHAPE, "pair %d: NULL image or bad geometry", q);
        const auto key = std::make_tuple(f.height, f.width, si);
        auto it = key_group.find(key);
        if (it == key_group.end()) {
            it = key_group.emplace(key, (int)members.size()).first;
            members.emplace_back();
            keys.push_back(key);
        }
        members[it->second].push_back(q);
    }
    qlpiv_adaptive_batch *b = new qlpiv_adaptive_batch();
    b->device = h->device;
    b->pixel_type = pixel_type;
    b->num_pairs = num_pairs;
    b->pair_offset.assign(num_pairs + 1, 0);
    b->tiles_ij.assign(2 * (size_t)num_pairs, 0);
    b->groups.resize(members.size());
    long off = 0;
    for (size_t k = 0; k < members.size(); k++) {
        BatchGroup &g = b->groups[k];
        g.height = std::get<0>(keys[k]);
        g.width = std::get<1>(keys[k]);
        g.desc = schedules[std::get<2>(keys[k])];
        g.pairs = (int)members[k].size();
        int n = 0;
        qlpiv_grid grids[16];
        qlpiv_status st = qlpiv_adaptive_levels(&g.desc, g.height, g.width, &n, grids, 16);
        if (st != QLPIV_OK) {
            release(b);
            return st;
        }
        g.tiles = grids[n - 1].tiles_i * grids[n - 1].tiles_j;
        g.out_offset = off;
        for (int m = 0; m < g.pairs; m++) {
            const int q = members[k][m];
            b->pair_offset[q] = off + (long)m * g.tiles;
            b->tiles_ij[2 * q] = grids[n - 1].tiles_i;
            b->tiles_ij[2 * q + 1] = grids[n - 1].tiles_j;
        }
        off += (long)g.pairs * g.tiles;
    }
    b->total = off;
    b->pair_offset[num_pairs] = off;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) {
        release(b);
        return cuda_fail(ds.err, "cudaSetDevice");
    }
    cudaStream_t s = h->stream;
    cudaError_t e;
    if ((e = b->out_u.ensure(sizeof(float) * (size_t)b->total)) != cudaSuccess ||
        (e = b->out_v.ensure(sizeof(float) * (size_t)b->total)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess) {
        release(b);
        return cuda_fail(e, "adaptive batch buffers");
    }
    for (size_t k = 0; k < b->groups.size(); k++) {
        BatchGroup &g = b->groups[k];
        qlpiv_params hp{};
        hp.device = h->device;
        qlpiv_status st = qlpiv_create(&hp, &g.h);
        if (st != QLPIV_OK) {
            release(b);
            return st;
        }
        std::vector<qlpiv_frame> t(g.pairs);
        for (int m = 0; m < g.pairs; m++) t[m] = frames[members[k][m]];
        if ((e = cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming)) != cudaSuccess ||
            (e = g.table.ensure(sizeof(qlpiv_frame) * g.pairs)) != cudaSuccess ||
            (e = cudaMemcpy(g.table.p, t.data(), sizeof(qlpiv_frame) * g.pairs, cudaMemcpyHostToDevice)) !=
                cudaSuccess) {
            release(b);
            return cuda_fail(e, "adaptive batch group");
        }
    }
    // one run outside the capture builds the groups' plans and the kernels' first-use set-up
    qlpiv_status st = enqueue(b, s);
    if (st == QLPIV_OK && (e = cudaStreamSynchronize(s)) != cudaSuccess) st = cuda_fail(e, "adaptive batch warm-up");
    if (st != QLPIV_OK) {
        release(b);
        return st;
    }
    if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        release(b);
        return cuda_fail(e, "graph capture");
    }
    st = enqueue(b, s);
    e = cudaStreamEndCapture(s, &b->graph);
    if (st != QLPIV_OK || e != cudaSuccess || (e = cudaGraphInstantiate(&b->exec, b->graph, 0)) != cudaSuccess) {
        release(b);
        return st != QLPIV_OK ? st : cuda_fail(e, "graph capture");
    }
    *out = b;
    return QLPIV_OK;
}

qlpiv_status qlpiv_adaptive_batch_info(const qlpiv_adaptive_batch *b, int64_t *total_tiles, int64_t *pair_offset,
                                       int32_t *tiles_ij, int32_t *groups) {
    if (!b) return fail(QLPIV_E_ARG, "batch is NULL");
    if (total_tiles) *total_tiles = b->total;
    if (pair_offset) std::memcpy(pair_offset, b->pair_offset.data(), sizeof(int64_t) * (b->num_pairs + 1));
    if (tiles_ij) std::memcpy(tiles_ij, b->tiles_ij.data(), sizeof(int32_t) * 2 * b->num_pairs);
    if (groups) *groups = (int32_t)b->groups.size();
    return QLPIV_OK;
}

qlpiv_status qlpiv_adaptive_batch_run(qlpiv_handle *h, qlpiv_adaptive_batch *b, float **device_u, float **device_v) {
    if (!h || !b) return fail(QLPIV_E_ARG, "NULL argument");
    if (h->device != b->device) return fail(QLPIV_E_ARG, "batch belongs to device %d", b->device);
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    const cudaError_t e = cudaGraphLaunch(b->exec, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "graph launch");
    h->launches += 1;
    if (device_u) *device_u = b->out_u.as<float>();
    if (device_v) *device_v = b->out_v.as<float>();
    return QLPIV_OK;
}

qlpiv_status qlpiv_adaptive_batch_download(qlpiv_handle *h, qlpiv_adaptive_batch *b, float *host_u, float *host_v) {
    if (!h || !b || !host_u || !host_v) return fail(QLPIV_E_ARG, "NULL argument");
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    cudaError_t e;
    const size_t bytes = sizeof(float) * (size_t)b->total;
    if ((e = cudaMemcpyAsync(host_u, b->out_u.p, bytes, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(host_v, b->out_v.p, bytes, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(h->stream)) != cudaSuccess)
        return cuda_fail(e, "adaptive batch download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_adaptive_batch_destroy(qlpiv_adaptive_batch *b) {
    if (!b) return QLPIV_OK;
    DeviceScope ds(b->device);
    release(b);
    return QLPIV_OK;
}

}  // extern "C"
