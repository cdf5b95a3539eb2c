// K1 instantiations (IA side x pixel type) and their launcher.
#include <mutex>

#include "qlpiv_internal.h"
#include "qlpiv_xcorr.cuh"

namespace qlpiv {

template <int N, typename Pix>
static cudaError_t launch_one(const IaJob &job, cudaStream_t stream, int num_sms) {
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
            e = cudaFuncSetAttribute(xcorr_kernel<N, Pix>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
            if (e != cudaSuccess) return e;
            int b = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, xcorr_kernel<N, Pix>, S::T, S::SMEM);
            if (e != cudaSuccess) return e;
            blocks_per_sm[dev] = b < 1 ? 1 : b;
        }
        bps = blocks_per_sm[dev];
    }
    long grid = (long)num_sms * bps * 8;
    if (grid > job.count) grid = job.count;
    if (grid < 1) return cudaSuccess;
    xcorr_kernel<N, Pix><<<(unsigned)grid, S::T, S::SMEM, stream>>>(job);
    return cudaGetLastError();
}

template <typename Pix>
static cudaError_t launch_pix(const IaJob &job, int n, cudaStream_t stream, int num_sms) {
    switch (n) {
        case 16: return launch_one<16, Pix>(job, stream, num_sms);
        case 32: return launch_one<32, Pix>(job, stream, num_sms);
        case 64: return launch_one<64, Pix>(job, stream, num_sms);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_xcorr(const IaJob &job, int n, int pixel_type, cudaStream_t stream, int num_sms) {
    switch (pixel_type) {
        case QLPIV_PIX_U8: return launch_pix<uint8_t>(job, n, stream, num_sms);
        case QLPIV_PIX_U16: return launch_pix<uint16_t>(job, n, stream, num_sms);
        case QLPIV_PIX_F32: return launch_pix<float>(job, n, stream, num_sms);
        default: return cudaErrorInvalidValue;
    }
}

bool xcorr_size_supported(int n) { return n == 16 || n == 32 || n == 64; }

}  // namespace qlpiv
