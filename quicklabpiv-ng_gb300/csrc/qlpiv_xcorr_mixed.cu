// K1 over a mixed-size work list in one persistent launch: IA 64, 32 and 16 work lists drained by
// every CTA from per-size counters, largest IAs first, with the per-IA bodies of the per-size
// kernels (xcorr_cta_ia, xcorr16_warp_ia), so every vector is the one the per-size kernel writes.
//
// One CTA of 512 threads per SM works, in turn, on
//   IA 64: one IA at a time with all 512 threads (the IA-64 kernel's group);
//   IA 32: two IAs at a time, one per 256-thread half, each half synchronised by its own named
//          barrier (bar.sync 1 / 2, 256 threads);
//   IA 16: sixteen IAs at a time, one per warp, IAs claimed four at a time.
// A CTA moves to the next size when the counter of the current one runs out, so the sizes overlap
// across CTAs and the tail of one size is filled by the next.  Shared memory is the largest of
// the three layouts (sixteen warp blocks of the IA-16 kernel), registers up to 128 (the IA-16
// body's), so one CTA is resident per SM: half the warps the IA-32 / IA-64 kernels keep resident.
// FindMaximumFromCenter with the 3-point (or no) sub-pixel fit only; IA 128 (a two-CTA cluster)
// runs in its own launch.
#include <mutex>

#include "qlpiv_xcorr_launch.h"
#include "qlpiv_xcorr_warp.cuh"

namespace qlpiv {

namespace {

constexpr int kMixThreads = 512;
constexpr unsigned kChunk16 = 4;  // IA-16 IAs claimed per counter update
constexpr size_t kHalf32 = (XcorrShape<32>::SMEM + 15) & ~(size_t)15;
constexpr size_t kWarpBlocks = 16 * w16::kWarpSmemAligned;
constexpr size_t kMixSmem16 = kWarpBlocks + 16 * sizeof(float) * 32 * 2;
constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t kMixSmem = cmax(cmax(XcorrShape<64>::SMEM, 2 * kHalf32), kMixSmem16);
static_assert(kMixSmem <= 227 * 1024, "mixed K1 layout exceeds the shared memory of one CTA");

template <typename Pix>
__global__ void __launch_bounds__(kMixThreads, 1) xcorr_mixed_kernel(MixedJob mj) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ unsigned s_next[2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // ---- IA 64: the CTA works on one IA ----
    if (mj.job[0].count > 0) {
        const IaJob &job = mj.job[0];
        using S = XcorrShape<64>;
        const CtaSmem<64> sm = cta_smem<64>(smem_raw);
        for (int e = tid; e < S::M; e += kMixThreads) sm.tw[e] = job.twiddles[e];
        int qn = 0, nb = 0;
        for (;;) {
            if (tid == 0) s_next[0] = atomicAdd(&mj.next[0], 1u);
            __syncthreads();
            const long k = s_next[0];
            if (k >= job.count) break;
            xcorr_cta_ia<64, Pix, false, false>(job, k, sm, tid, 0, qn, nullptr, nb);
        }
        if (qn > 0 && warp == 0) fit_flush<S::D, false>(sm.fitq, sm.fitv, qn, lane, job);
        __syncthreads();
    }

    // ---- IA 32: each 256-thread half works on its own IA ----
    if (mj.job[1].count > 0) {
        const IaJob &job = mj.job[1];
        using S = XcorrShape<32>;
        const int half = tid >> 8, ht = tid & 255, bar = 1 + half;
        const CtaSmem<32> sm = cta_smem<32>(smem_raw + half * kHalf32);
        for (int e = ht; e < S::M; e += 256) sm.tw[e] = job.twiddles[e];
        int qn = 0, nb = 0;
        for (;;) {
            if (ht == 0) s_next[half] = atomicAdd(&mj.next[1], 1u);
            bar_sync<256, true>(bar);
            const long k = s_next[half];
            if (k >= job.count) break;
            xcorr_cta_ia<32, Pix, false, true>(job, k, sm, ht, bar, qn, nullptr, nb);
        }
        if (qn > 0 && (ht >> 5) == 0) fit_flush<S::D, false>(sm.fitq, sm.fitv, qn, lane, job);
        __syncthreads();
    }

    // ---- IA 16: each warp works on its own IAs ----
    if (mj.job[2].count > 0) {
        const IaJob &job = mj.job[2];
        const w16::WarpSmem sm = w16::warp_smem(smem_raw, warp);
        float *fitv = reinterpret_cast<float *>(smem_raw + kWarpBlocks) + warp * 32 * 2;
        int qn = 0, nb = 0;
        for (;;) {
            unsigned k0 = 0;
            if (lane == 0) k0 = atomicAdd(&mj.next[2], kChunk16);
            k0 = __shfl_sync(0xffffffffu, k0, 0);
            if ((long)k0 >= job.count) break;
            const long kend = (long)k0 + kChunk16 < job.count ? (long)k0 + kChunk16 : job.count;
            for (long k = k0; k < kend; k++) xcorr16_warp_ia<Pix, false, false>(job, k, sm, fitv, lane, qn, nullptr, nb);
        }
        if (qn > 0) fit_flush<w16::D, false>(sm.fitq, fitv, qn, lane, job);
    }
}

template <typename Pix>
cudaError_t launch_mixed_pix(const MixedJob &mj, cudaStream_t stream, int num_sms) {
    static std::mutex mu;
    static bool ready[kMaxDevices] = {false};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!ready[dev]) {
            if ((e = cudaFuncSetAttribute(xcorr_mixed_kernel<Pix>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)kMixSmem)) != cudaSuccess)
                return e;
            int b = 0;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, xcorr_mixed_kernel<Pix>, kMixThreads,
                                                                   kMixSmem)) != cudaSuccess)
                return e;
            if (b < 1) return cudaErrorInvalidConfiguration;
            ready[dev] = true;
        }
    }
    const cplx *tw = nullptr;
    if ((e = ensure_twiddles(dev, &tw)) != cudaSuccess) return e;
    MixedJob m = mj;
    m.job[0].twiddles = tw + twiddle_offset(128);
    m.job[1].twiddles = tw + twiddle_offset(64);
    for (IaJob &j : m.job) j.log_tab = log_table(dev);
    if ((e = cudaMemsetAsync(m.next, 0, 3 * sizeof(unsigned), stream)) != cudaSuccess) return e;
    xcorr_mixed_kernel<Pix><<<(unsigned)num_sms, kMixThreads, kMixSmem, stream>>>(m);
    return cudaGetLastError();
}

}  // namespace

bool mixed_kernel_supported(const IaJob &tmpl) {
    return tmpl.num_peaks == 0 && tmpl.subpix_pixels == 0 && tmpl.mp_batch == nullptr && tmpl.ia_list == nullptr &&
           tmpl.planes == nullptr;
}

cudaError_t launch_k1_mixed(const MixedJob &mj, int pixel_type, cudaStream_t stream, int num_sms) {
    for (const IaJob &j : mj.job)
        if (j.count > 0 && !mixed_kernel_supported(j)) return cudaErrorInvalidValue;
    switch (pixel_type) {
        case QLPIV_PIX_U8: return launch_mixed_pix<uint8_t>(mj, stream, num_sms);
        case QLPIV_PIX_U16: return launch_mixed_pix<uint16_t>(mj, stream, num_sms);
        case QLPIV_PIX_F32: return launch_mixed_pix<float>(mj, stream, num_sms);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace qlpiv
