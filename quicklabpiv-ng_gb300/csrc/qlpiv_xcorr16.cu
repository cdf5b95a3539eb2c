// K1 for IA 16: the warp-per-IA kernel (qlpiv_xcorr_warp.cuh), every pixel type.
#include <cstdlib>
#include <mutex>

#include "qlpiv_xcorr_launch.h"
#include "qlpiv_xcorr_warp.cuh"

namespace qlpiv {

// IA 16: one warp per IA, w16::kWarps warps per CTA, `waves` waves of resident CTAs.
template <typename Pix, bool PP>
static cudaError_t launch_warp16(const IaJob &job, cudaStream_t stream, int num_sms, int *nlaunch) {
    static std::mutex mu;
    static int blocks_per_sm[kMaxDevices] = {0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    const size_t base = w16::kWarps * w16::kWarpSmemAligned;
    int bps;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (blocks_per_sm[dev] == 0) {
            e = cudaFuncSetAttribute(xcorr16_warp_kernel<Pix, PP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(base + w16::kWarps * kSubpixSmem));
            if (e == cudaSuccess && !PP)
                e = cudaFuncSetAttribute(xcorr16_warp_kernel<Pix, PP, !PP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(base + w16::kWarps * kSubpixSmem));
            if (e != cudaSuccess) return e;
            int b = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, xcorr16_warp_kernel<Pix, PP, false>, w16::kThreads,
                                                              base);
            if (e != cudaSuccess) return e;
            blocks_per_sm[dev] = b < 1 ? 1 : b;
        }
        bps = blocks_per_sm[dev];
    }
    const cplx *tw = nullptr;
    if ((e = ensure_twiddles(dev, &tw)) != cudaSuccess) return e;
    IaJob j = job;
    j.twiddles = tw + twiddle_offset(32);
    j.log_tab = log_table(dev);
    long grid = (long)num_sms * bps * (job.waves > 0 ? job.waves : (job.num_peaks > 0 ? multi_waves<16>() : 8));
    const long need = (job.count + w16::kWarps - 1) / w16::kWarps;
    if (grid > need) grid = need;
    if (grid < 1) return cudaSuccess;
    const size_t smem = base + (j.subpix_pixels > 0 ? w16::kWarps * sizeof(float) * 32 * 2 * j.subpix_pixels : 0);
    // the batched main launch runs the BATCH instantiation (P-point fits are never batched), the
    // retry launch the per-IA one
    auto launch = [&](const IaJob &jj, long g) {
        if (!PP && jj.mp_batch != nullptr)
            xcorr16_warp_kernel<Pix, PP, !PP><<<(unsigned)g, w16::kThreads, smem, stream>>>(jj);
        else
            xcorr16_warp_kernel<Pix, PP, false><<<(unsigned)g, w16::kThreads, smem, stream>>>(jj);
        return cudaGetLastError();
    };
    // the batched replay needs a batch for every resident warp
    if (batch_eligible(job) && (long)num_sms * bps * w16::kWarps <= job.mp_batch_units)
        return launch_batched(j, grid, (long)num_sms * bps, stream, launch, nlaunch);
    j.mp_batch = nullptr;
    return launch(j, grid);
}


template <typename Pix, bool PP>
struct Launch16 {
    static cudaError_t run(const IaJob &job, cudaStream_t stream, int num_sms, int *nlaunch) {
        return launch_warp16<Pix, PP>(job, stream, num_sms, nlaunch);
    }
};

cudaError_t launch_k1_16(const IaJob &job, int pixel_type, cudaStream_t stream, int num_sms, int *nlaunch) {
    return dispatch_pix<Launch16>(job, pixel_type, stream, num_sms, nlaunch);
}

}  // namespace qlpiv
