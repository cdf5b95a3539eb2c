// K1 for IA 32: the CTA-per-IA kernel (qlpiv_xcorr.cuh), every pixel type.
#include <cstdlib>
#include <mutex>

#include "qlpiv_xcorr_launch.h"

namespace qlpiv {

template <int N, typename Pix, bool PP>
static cudaError_t launch_one(const IaJob &job, cudaStream_t stream, int num_sms, int *nlaunch) {
    using S = XcorrShape<N>;
    // The shared-memory opt-in is a per-device attribute of the function: set it once
    // per (instantiation, device).
    static std::mutex mu;
    static int blocks_per_sm[kMaxDevices] = {0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    int bps;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (blocks_per_sm[dev] == 0) {
            e = cudaFuncSetAttribute(xcorr_kernel<N, Pix, PP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(S::SMEM + kSubpixSmem));
            if (e != cudaSuccess) return e;
            int b = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, xcorr_kernel<N, Pix, PP>, S::T, S::SMEM);
            if (e != cudaSuccess) return e;
            blocks_per_sm[dev] = b < 1 ? 1 : b;
        }
        bps = blocks_per_sm[dev];
    }
    const cplx *tw = nullptr;
    if ((e = ensure_twiddles(dev, &tw)) != cudaSuccess) return e;
    IaJob j = job;
    j.twiddles = tw + twiddle_offset(S::M);
    j.log_tab = log_table(dev);
    // every CTA loops over IAs; eight waves of CTAs balance the single-peak kernel best, the
    // multi-peak ones multi_waves<N>() (qlpiv_xcorr_launch.h)
    long grid = (long)num_sms * bps * (job.waves > 0 ? job.waves : (job.num_peaks > 0 ? multi_waves<32>() : 8));
    if (grid > job.count) grid = job.count;
    if (grid < 1) return cudaSuccess;
    // P-point sub-pixel stencils: 2 P floats per queued fit after the fixed layout
    const size_t smem = S::SMEM + (j.subpix_pixels > 0 ? sizeof(float) * 32 * 2 * j.subpix_pixels : 0);
    auto launch = [&](const IaJob &jj, long g) {
        xcorr_kernel<N, Pix, PP><<<(unsigned)g, S::T, smem, stream>>>(jj);
        return cudaGetLastError();
    };
    // the batched replay needs a batch for every resident CTA
    if (batch_eligible(job) && (long)num_sms * bps <= job.mp_batch_units)
        return launch_batched(j, grid, (long)num_sms * bps, stream, launch, nlaunch);
    j.mp_batch = nullptr;
    return launch(j, grid);
}


template <typename Pix, bool PP>
struct Launch32 {
    static cudaError_t run(const IaJob &job, cudaStream_t stream, int num_sms, int *nlaunch) {
        return launch_one<32, Pix, PP>(job, stream, num_sms, nlaunch);
    }
};

cudaError_t launch_k1_32(const IaJob &job, int pixel_type, cudaStream_t stream, int num_sms, int *nlaunch) {
    return dispatch_pix<Launch32>(job, pixel_type, stream, num_sms, nlaunch);
}

}  // namespace qlpiv
