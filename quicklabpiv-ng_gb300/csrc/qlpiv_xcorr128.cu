// K1 for IA 128: the two-CTA cluster kernel (qlpiv_xcorr_pair.cuh), every pixel type.
#include <cstdlib>
#include <mutex>

#include "qlpiv_xcorr_launch.h"
#include "qlpiv_xcorr_pair.cuh"

namespace qlpiv {

// IA 128: one cluster of two CTAs per IA, one CTA per SM; `waves` clusters per SM pair.
template <typename Pix, bool PP>
static cudaError_t launch_pair(const IaJob &job, cudaStream_t stream, int num_sms, int * /*nlaunch*/) {
    static std::mutex mu;
    static bool ready[kMaxDevices] = {false};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!ready[dev]) {
            e = cudaFuncSetAttribute(xcorr_pair_kernel<Pix, PP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(PairShape::SMEM + kSubpixSmem));
            if (e != cudaSuccess) return e;
            ready[dev] = true;
        }
    }
    const cplx *tw = nullptr;
    if ((e = ensure_twiddles(dev, &tw)) != cudaSuccess) return e;
    IaJob j = job;
    j.twiddles = tw + twiddle_offset(256);
    j.log_tab = log_table(dev);
    j.mp_batch = nullptr;
    // multi-peak mode: one resident wave (the fit queue fills between flushes), as K1
    long grid = (long)(num_sms & ~1) * (job.waves > 0 ? job.waves : (job.num_peaks > 0 ? 1 : 4));
    if (grid > 2 * job.count) grid = 2 * job.count;
    if (grid < 2) return cudaSuccess;
    if (job.num_peaks > 0) {
        // one (2N-1)^2 plane per cluster, kept per device and grown on demand
        static float *planes[kMaxDevices] = {nullptr};
        static long capacity[kMaxDevices] = {0};
        std::lock_guard<std::mutex> lock(mu);
        const long need = grid / 2 * (long)PairShape::D * PairShape::D;
        if (capacity[dev] < need) {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            if ((e = cudaStreamIsCapturing(stream, &cs)) != cudaSuccess) return e;
            if (cs != cudaStreamCaptureStatusNone) return cudaErrorStreamCaptureUnsupported;
            if (planes[dev] != nullptr && (e = cudaFree(planes[dev])) != cudaSuccess) return e;
            planes[dev] = nullptr;
            capacity[dev] = 0;
            if ((e = cudaMalloc(&planes[dev], sizeof(float) * need)) != cudaSuccess) return e;
            capacity[dev] = need;
        }
        j.mp_planes = planes[dev];
    }
    const size_t smem = PairShape::SMEM + (j.subpix_pixels > 0 ? sizeof(float) * 32 * 2 * j.subpix_pixels : 0);
    xcorr_pair_kernel<Pix, PP><<<(unsigned)grid, PairShape::T, smem, stream>>>(j);
    return cudaGetLastError();
}


template <typename Pix, bool PP>
struct Launch128 {
    static cudaError_t run(const IaJob &job, cudaStream_t stream, int num_sms, int *nlaunch) {
        return launch_pair<Pix, PP>(job, stream, num_sms, nlaunch);
    }
};

cudaError_t launch_k1_128(const IaJob &job, int pixel_type, cudaStream_t stream, int num_sms, int *nlaunch) {
    return dispatch_pix<Launch128>(job, pixel_type, stream, num_sms, nlaunch);
}

}  // namespace qlpiv
