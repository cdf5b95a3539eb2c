// K1 launch helpers shared by the per-size translation units (qlpiv_xcorr{16,32,64,128}.cu),
// which compile in parallel; qlpiv_xcorr.cu holds the device tables and the dispatch.
#pragma once
#include <mutex>

#include "qlpiv_internal.h"
#include "qlpiv_xcorr.cuh"

namespace qlpiv {

constexpr int kMultiWaves16 = 2;

inline int twiddle_offset(int m) { return m == 32 ? 0 : (m == 64 ? 32 : (m == 128 ? 96 : 224)); }

// Default waves of resident CTAs (IA 16: warps) per launch in multi-peak mode, per IA size.  With
// the batched list replay a unit replays its IAs 32 at a time, so fewer waves fill more batches;
// measured on the headline adaptive workload (pass times in ms at 2 / 4 / 8 / 16 / 32 waves):
// IA 16 18.63 / 18.74 / 19.0 / 19.40 / 20.10; IA 32 (8 / 16 / 32) 17.68 / 17.61 / 17.75;
// IA 64 (8 / 16 / 32) 18.69 / 18.62 / 18.60.
template <int N>
constexpr int multi_waves() {
    return N == 16 ? kMultiWaves16 : (N == 32 ? 16 : 32);
}

constexpr size_t kSubpixSmem = sizeof(float) * 32 * 2 * kMaxSubpixPixels;

// The batched multi-peak replay (mp_batched) applies to the job and its buffers were given.
inline bool batch_eligible(const IaJob &job) {
    return job.mp_batch != nullptr && job.mp_slots != nullptr && job.mp_retry != nullptr && job.mp_batch_units > 0 &&
           job.ia_list == nullptr && job.num_peaks >= 1 && job.num_peaks <= 4 &&
           (job.subpix == QLPIV_SUBPIX_NONE || job.subpix == QLPIV_SUBPIX_GAUSS3);
}

// Batched launch: the retry count is zeroed before the main launch; the IAs it flags run again
// through the per-IA path in a second launch of `retry_grid` units over the device list.
template <typename Launch>
inline cudaError_t launch_batched(const IaJob &j, long grid, long retry_grid, cudaStream_t stream, Launch launch,
                                  int *nlaunch) {
    cudaError_t e = cudaMemsetAsync(j.mp_retry, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    if ((e = launch(j, grid)) != cudaSuccess) return e;
    IaJob r = j;
    r.mp_batch = nullptr;
    r.ia_list = j.mp_retry;
    if ((e = launch(r, retry_grid)) != cudaSuccess) return e;
    if (nlaunch) *nlaunch = 2;
    return cudaSuccess;
}


// Per-size launchers (pixel type and the P-point instantiation chosen inside).
cudaError_t launch_k1_16(const IaJob &job, int pixel_type, cudaStream_t stream, int num_sms, int *nlaunch);
cudaError_t launch_k1_32(const IaJob &job, int pixel_type, cudaStream_t stream, int num_sms, int *nlaunch);
cudaError_t launch_k1_64(const IaJob &job, int pixel_type, cudaStream_t stream, int num_sms, int *nlaunch);
cudaError_t launch_k1_128(const IaJob &job, int pixel_type, cudaStream_t stream, int num_sms, int *nlaunch);

// The persistent mixed-size K1 (qlpiv_xcorr_mixed.cu): job[0..2] = the IA 64, 32 and 16 work
// lists (count 0: none), next = 3 device counters (zeroed by the launch).  One CTA per SM.
struct MixedJob {
    IaJob job[3];
    unsigned *next;
};
bool mixed_kernel_supported(const IaJob &tmpl);
cudaError_t launch_k1_mixed(const MixedJob &mj, int pixel_type, cudaStream_t stream, int num_sms);

// Calls L<Pix, PP>::run(job, args...) for the job's pixel type and sub-pixel stencil mode.
template <template <typename, bool> class L, typename... A>
cudaError_t dispatch_pix(const IaJob &job, int pixel_type, A... args) {
    const bool pp = job.subpix_pixels > 0;
    switch (pixel_type) {
        case QLPIV_PIX_U8: return pp ? L<uint8_t, true>::run(job, args...) : L<uint8_t, false>::run(job, args...);
        case QLPIV_PIX_U16: return pp ? L<uint16_t, true>::run(job, args...) : L<uint16_t, false>::run(job, args...);
        case QLPIV_PIX_F32: return pp ? L<float, true>::run(job, args...) : L<float, false>::run(job, args...);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace qlpiv
