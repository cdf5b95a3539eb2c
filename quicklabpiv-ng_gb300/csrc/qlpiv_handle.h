// Handle internals shared by the host translation units of libqlpiv_gpu.so.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <vector>

#include "qlpiv.h"

namespace qlpiv {

qlpiv_status fail(qlpiv_status st, const char *fmt, ...);
qlpiv_status cuda_fail(cudaError_t e, const char *what);

// Stream-ordered allocation for the buffers a thread creates while an AsyncAllocScope is
// active (the request server: no device-wide synchronisation from cudaMalloc / cudaFree while
// other requests run).
struct AsyncAlloc {
    cudaMemPool_t pool = nullptr;
    cudaStream_t stream = nullptr;
};
AsyncAlloc &async_alloc_tls();
struct AsyncAllocScope {
    AsyncAlloc saved;
    AsyncAllocScope(cudaMemPool_t pool, cudaStream_t stream) : saved(async_alloc_tls()) {
        async_alloc_tls() = AsyncAlloc{pool, stream};
    }
    ~AsyncAllocScope() { async_alloc_tls() = saved; }
};

// Device buffer that only grows.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaStream_t astream = nullptr;  // set when allocated from a pool: freed in that stream's order
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        release();
        size_t want = bytes < 256 ? 256 : bytes;
        const AsyncAlloc &aa = async_alloc_tls();
        cudaError_t e;
        if (aa.pool) {
            e = cudaMallocFromPoolAsync(&p, want, aa.pool, aa.stream);
            if (e == cudaSuccess) astream = aa.stream;
        } else {
            e = cudaMalloc(&p, want);
        }
        if (e == cudaSuccess) cap = want;
        else p = nullptr;
        return e;
    }
    void release() {
        if (p) {
            if (astream) cudaFreeAsync(p, astream);
            else cudaFree(p);
        }
        p = nullptr;
        cap = 0;
        astream = nullptr;
    }
    template <typename T>
    T *as() const {
        return reinterpret_cast<T *>(p);
    }
};

// Makes a device current for the calling thread and restores the previous one on
// scope exit.
struct DeviceScope {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceScope(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

struct AdaptivePlan;
void destroy_plan(AdaptivePlan *p);

// One pending stage timing (events recorded, not yet read back).
struct StageEvent {
    std::string stage;
    int level, ia_side;
    long launches, items;
    cudaEvent_t begin, end;
};

struct StageTotal {
    std::string stage;
    int level, ia_side;
    long launches, items;
    double ms;
};

}  // namespace qlpiv

struct qlpiv_handle {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;       // stream work is queued on
    cudaStream_t own_stream = nullptr;   // the handle's own non-blocking stream
    std::mutex mu;
    long launches = 0;
    qlpiv::DevBuf tiles_a, tiles_b, max_a, max_b, origins, vectors, planes, frames;
    qlpiv::DevBuf scratch[12];           // stage test hooks
    // batched multi-peak replay of the tile / frame pass entry points (one stream: one set):
    // batches, their claim bitmask (zeroed when allocated) and the retry list
    qlpiv::DevBuf mp_batch, mp_slots, mp_retry;
    long mp_units = 0;
    qlpiv::AdaptivePlan *plan = nullptr; // cached adaptive PIV plan
    bool profiling = false;
    std::vector<qlpiv::StageEvent> prof_pending;
    std::vector<qlpiv::StageTotal> prof_totals;
};
