// Internal declarations shared by the CUDA translation units of libqlpiv_gpu.so.
#pragma once
#include <cuda_runtime.h>

#include "qlpiv.h"

namespace qlpiv {

struct IaJob;
struct cplx;

constexpr int kMaxDevices = 64;

// Uploads the FFT twiddle tables to device `dev` (the current device) once.
cudaError_t ensure_twiddles(int dev, const cplx **table);

// K1 fused FFT-PIV over job.count IAs of side n on `stream`.
cudaError_t launch_xcorr(const IaJob &job, int n, int pixel_type, cudaStream_t stream, int num_sms);
bool xcorr_size_supported(int n);
// FindMaximumMultiPeaks settings the kernel supports for IA side n (records fit on chip).
bool multipeak_supported(int n, int num_peaks, int peak_kernel);

inline size_t pixel_bytes(int pixel_type) {
    return pixel_type == QLPIV_PIX_U8 ? 1 : (pixel_type == QLPIV_PIX_U16 ? 2 : 4);
}

}  // namespace qlpiv
