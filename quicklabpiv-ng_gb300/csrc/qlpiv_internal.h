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
// log_fpair table of `dev` (valid after ensure_twiddles on that device).
const float4 *log_table(int dev);

// K1 fused FFT-PIV over job.count IAs of side n on `stream`; *nlaunch (optional): kernels queued.
cudaError_t launch_xcorr(const IaJob &job, int n, int pixel_type, cudaStream_t stream, int num_sms,
                         int *nlaunch = nullptr);
bool xcorr_size_supported(int n);
// Device bytes of the batched multi-peak replay buffer (IaJob.mp_batch) for a launch site on a GPU
// with num_sms SMs; *units = IaJob.mp_batch_units.  The slot bitmask (IaJob.mp_slots, zeroed once;
// every launch leaves it zero) takes xcorr_batch_slot_bytes(units); the retry list (IaJob.mp_retry)
// 1 + count ints.
size_t xcorr_batch_bytes(int num_sms, long *units);
size_t xcorr_batch_slot_bytes(long units);
// FindMaximumMultiPeaks settings the kernel supports for IA side n (records fit on chip).
bool multipeak_supported(int n, int num_peaks, int peak_kernel);

// Request-server helpers (qlpiv_pipeline.cu): admission estimate of an adaptive plan's device
// memory; the adaptive loop of one pinned host pair queued without waiting; dropping a plan.
size_t plan_device_bytes(const qlpiv_adaptive_desc *d, int pixel_type, int height, int width, int pairs);
qlpiv_status queue_adaptive_pinned(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int pixel_type, int height,
                                   int width, const void *img_a, const void *img_b, long pitch, float *out_u,
                                   float *out_v);
void drop_plan(qlpiv_handle *h);

// Sub-pixel mode settings (qlpiv_capi.cu): QLPIV_OK or QLPIV_E_ARG with the message set.
qlpiv_status check_subpix(int mode, int pixels, int iterations);

// Tile.accumulateDisplacement / replaceDisplacement under NoOutOfBoundClipping
// (S/iareas/Tile.java:103-136,156-189): false when the tile of side n at (top, left), moved by the
// rounded displacement (FastMath.round: floor(x + 0.5f)), fails the reference's test
// top + ru < 0, top + n + ru >= h, left + rv < 0, left + n + rv >= w.  n == 0 means clipping is
// allowed and nothing is refused.  Float compares of small integers, as in the reference.
__host__ __device__ __forceinline__ bool tile_inside(int n, int h, int w, int top, int left, float u, float v) {
    if (n == 0) return true;
    const float ru = floorf(u + 0.5f), rv = floorf(v + 0.5f);
    return !((float)top + ru < 0.0f || (float)(top + n) + ru >= (float)h || (float)left + rv < 0.0f ||
             (float)(left + n) + rv >= (float)w);
}

inline size_t pixel_bytes(int pixel_type) {
    return pixel_type == QLPIV_PIX_U8 ? 1 : (pixel_type == QLPIV_PIX_U16 ? 2 : 4);
}

}  // namespace qlpiv
