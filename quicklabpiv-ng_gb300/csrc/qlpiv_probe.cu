// Instrumentation: live FP32 FMA throughput of the device, the compute roofline
// denominator for the FFT kernels (MEASURED_PEAKS-style figure for SIMT FP32).
#include <cuda_runtime.h>

#include "qlpiv.h"
#include "qlpiv_div.cuh"
#include "qlpiv_internal.h"
#include "qlpiv_logdf.cuh"

namespace {

__global__ void __launch_bounds__(256) fma_probe(float *out, int iters, float a, float b) {
    // 8 independent FMA chains per thread keep the pipes busy
    float x0 = threadIdx.x, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
    float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 1.2345f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" qlpiv_status qlpiv_measure_fp32_peak(int device, double *tflops) {
    if (!tflops) return QLPIV_E_ARG;
    *tflops = 0.0;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return QLPIV_E_NO_DEVICE;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float *out = nullptr;
    const int blocks = sms * 8, threads = 256, iters = 4096;
    qlpiv_status st = QLPIV_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) {
        st = QLPIV_E_OOM;
    } else if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        st = QLPIV_E_CUDA;
    } else {
        float best_ms = 1e30f;
        for (int rep = 0; rep < 4; rep++) {
            cudaEventRecord(e0);
            fma_probe<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
            cudaEventRecord(e1);
            if (cudaEventSynchronize(e1) != cudaSuccess) { st = QLPIV_E_CUDA; break; }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms < best_ms) best_ms = ms;
        }
        if (st == QLPIV_OK) {
            const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
            *tflops = flops / (best_ms * 1e-3) / 1e12;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (out) cudaFree(out);
    cudaSetDevice(prev);
    return st;
}

// Instrumentation: the fit's float-pair logarithm (qlpiv_logdf.cuh) beside CUDA's double log for
// n host floats, so that its error bound can be checked on the device.
namespace {
__global__ void log_probe(const float *x, long n, const float4 *tab, double *mine, double *ref) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const qlpiv::fpair p = qlpiv::log_fpair(x[k], tab);
    mine[k] = (double)p.hi + (double)p.lo;
    ref[k] = log((double)x[k]);
}
}  // namespace

extern "C" qlpiv_status qlpiv_probe_log(int device, const float *x, long n, double *mine, double *ref) {
    if (!x || !mine || !ref || n < 0) return QLPIV_E_ARG;
    for (long k = 0; k < n; k++)
        if (!(x[k] >= 1.17549435e-38f && x[k] < 3.4e38f)) return QLPIV_E_ARG;  // positive normal floats
    if (n == 0) return QLPIV_OK;
    if (cudaSetDevice(device) != cudaSuccess) return QLPIV_E_NO_DEVICE;
    const qlpiv::cplx *tw = nullptr;
    if (qlpiv::ensure_twiddles(device, &tw) != cudaSuccess) return QLPIV_E_CUDA;
    float *dx = nullptr;
    double *dm = nullptr, *dr = nullptr;
    qlpiv_status st = QLPIV_OK;
    if (cudaMalloc(&dx, sizeof(float) * n) != cudaSuccess || cudaMalloc(&dm, sizeof(double) * n) != cudaSuccess ||
        cudaMalloc(&dr, sizeof(double) * n) != cudaSuccess) {
        st = QLPIV_E_OOM;
    } else if (cudaMemcpy(dx, x, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
        st = QLPIV_E_CUDA;
    } else {
        log_probe<<<(unsigned)((n + 255) / 256), 256>>>(dx, n, qlpiv::log_table(device), dm, dr);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(mine, dm, sizeof(double) * n, cudaMemcpyDeviceToHost) !=
                                                     cudaSuccess ||
            cudaMemcpy(ref, dr, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = QLPIV_E_CUDA;
    }
    cudaFree(dx);
    cudaFree(dm);
    cudaFree(dr);
    return st;
}

// Instrumentation: the tile normalisation's division (qlpiv_div.cuh) against IEEE division over
// every integer v in [0, 65535] and divisor m in [1, 65535]; counts the quotients that differ.
namespace {
__global__ void division_probe(unsigned long long *mismatches) {
    const int m = blockIdx.x + 1;  // divisor 1..65535
    const float fm = (float)m, rm = __frcp_rn(fm);
    unsigned long long bad = 0;
    for (int v = threadIdx.x; v < 65536; v += blockDim.x) {
        const float fv = (float)v;
        if (__float_as_uint(qlpiv::div_int(fv, fm, rm)) != __float_as_uint(__fdiv_rn(fv, fm))) bad++;
    }
    if (bad) atomicAdd(mismatches, bad);
}
}  // namespace

extern "C" qlpiv_status qlpiv_probe_division(int device, int64_t *mismatches) {
    if (!mismatches) return QLPIV_E_ARG;
    *mismatches = -1;
    if (cudaSetDevice(device) != cudaSuccess) return QLPIV_E_NO_DEVICE;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return QLPIV_E_OOM;
    qlpiv_status st = QLPIV_OK;
    unsigned long long h = 0;
    if (cudaMemset(d, 0, sizeof(*d)) != cudaSuccess) st = QLPIV_E_CUDA;
    if (st == QLPIV_OK) {
        division_probe<<<65535, 256>>>(d);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
            st = QLPIV_E_CUDA;
    }
    cudaFree(d);
    if (st == QLPIV_OK) *mismatches = (int64_t)h;
    return st;
}
