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

// Device buffer that only grows.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
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
    qlpiv::AdaptivePlan *plan = nullptr; // cached adaptive PIV plan
    bool profiling = false;
    std::vector<qlpiv::StageEvent> prof_pending;
    std::vector<qlpiv::StageTotal> prof_totals;
};
