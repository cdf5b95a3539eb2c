// K1 instantiations (IA side x pixel type) and their launcher; IA 128 runs the two-CTA cluster
// variant (qlpiv_xcorr_pair.cuh).
#include <cmath>
#include <cstdlib>
#include <mutex>

#include "qlpiv_internal.h"
#include "qlpiv_xcorr.cuh"
#include "qlpiv_xcorr_pair.cuh"
#include "qlpiv_xcorr_warp.cuh"

namespace qlpiv {

// Twiddle tables exp(-2 pi i e / M) for M = 32, 64, 128, 256 (offsets 0, 32, 96, 224), filled
// once per device from the host (double precision, rounded to float).
static __device__ cplx g_twiddles[32 + 64 + 128 + 256];

static int twiddle_offset(int m) { return m == 32 ? 0 : (m == 64 ? 32 : (m == 128 ? 96 : 224)); }

// log_fpair table (qlpiv_logdf.cuh): {inv_k, -ln(inv_k) hi, -ln(inv_k) lo, 0}, inv_k = 1/(1 + k/64)
// rounded to float, k = 0..64; the logarithm of the float inv_k is taken in double.
static __device__ float4 g_logtab[65];
static const float4 *g_logtab_addr[kMaxDevices] = {nullptr};

const float4 *log_table(int dev) { return dev >= 0 && dev < kMaxDevices ? g_logtab_addr[dev] : nullptr; }

cudaError_t ensure_twiddles(int dev, const cplx **table) {
    static std::mutex mu;
    static const cplx *addr[kMaxDevices] = {nullptr};
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (addr[dev] == nullptr) {
        cplx host[32 + 64 + 128 + 256];
        for (int m : {32, 64, 128, 256})
            for (int e = 0; e < m; e++) {
                const double a = -2.0 * M_PI * (double)e / (double)m;
                host[twiddle_offset(m) + e] = cplx{(float)std::cos(a), (float)std::sin(a)};
            }
        cudaError_t err = cudaMemcpyToSymbol(g_twiddles, host, sizeof(host));
        if (err != cudaSuccess) return err;
        float4 lt[65];
        for (int k = 0; k <= 64; k++) {
            const float inv = (float)(1.0 / (1.0 + k / 64.0));
            const double v = -std::log((double)inv);
            const float hi = (float)v;
            lt[k] = make_float4(inv, hi, (float)(v - (double)hi), 0.0f);
        }
        if ((err = cudaMemcpyToSymbol(g_logtab, lt, sizeof(lt))) != cudaSuccess) return err;
        void *lp = nullptr;
        if ((err = cudaGetSymbolAddress(&lp, g_logtab)) != cudaSuccess) return err;
        g_logtab_addr[dev] = static_cast<const float4 *>(lp);
        void *p = nullptr;
        err = cudaGetSymbolAddress(&p, g_twiddles);
        if (err != cudaSuccess) return err;
        addr[dev] = static_cast<const cplx *>(p);
    }
    *table = addr[dev];
    return cudaSuccess;
}

// Default waves of resident CTAs per launch in multi-peak mode.  Measured on the headline adaptive
// workload (three multi-peak passes): 1 wave 558 frame-pairs/s, 4: 568, 16: 582, 32: 585, 64: 586.
constexpr int kMultiWaves = 32;

constexpr size_t kSubpixSmem = sizeof(float) * 32 * 2 * kMaxSubpixPixels;

// The batched multi-peak replay (mp_batched) applies to the job and its buffers were given.
static bool batch_eligible(const IaJob &job) {
    return job.mp_batch != nullptr && job.mp_slots != nullptr && job.mp_retry != nullptr && job.mp_batch_units > 0 &&
           job.ia_list == nullptr && job.num_peaks >= 1 && job.num_peaks <= 4 &&
           (job.subpix == QLPIV_SUBPIX_NONE || job.subpix == QLPIV_SUBPIX_GAUSS3);
}

// Batched launch: the retry count is zeroed before the main launch; the IAs it flags run again
// through the per-IA path in a second launch of `retry_grid` units over the device list.
template <typename Launch>
static cudaError_t launch_batched(const IaJob &j, long grid, long retry_grid, cudaStream_t stream, Launch launch,
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
    // every CTA loops over IAs; eight waves of CTAs balance the single-peak kernel best, 32 the
    // multi-peak one; the batched multi-peak replay runs one resident wave (a batch per CTA)
    long grid = (long)num_sms * bps * (job.waves > 0 ? job.waves : (job.num_peaks > 0 ? kMultiWaves : 8));
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
    long grid = (long)num_sms * bps * (job.waves > 0 ? job.waves : (job.num_peaks > 0 ? kMultiWaves : 8));
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
static cudaError_t launch_pix(const IaJob &job, int n, cudaStream_t stream, int num_sms, int *nlaunch) {
    switch (n) {
        case 16: return launch_warp16<Pix, PP>(job, stream, num_sms, nlaunch);
        case 32: return launch_one<32, Pix, PP>(job, stream, num_sms, nlaunch);
        case 64: return launch_one<64, Pix, PP>(job, stream, num_sms, nlaunch);
        case 128: return launch_pair<Pix, PP>(job, stream, num_sms, nlaunch);
        default: return cudaErrorInvalidValue;
    }
}

template <typename Pix>
static cudaError_t launch_pix(const IaJob &job, int n, cudaStream_t stream, int num_sms, int *nlaunch) {
    return job.subpix_pixels > 0 ? launch_pix<Pix, true>(job, n, stream, num_sms, nlaunch)
                                 : launch_pix<Pix, false>(job, n, stream, num_sms, nlaunch);
}

cudaError_t launch_xcorr(const IaJob &job, int n, int pixel_type, cudaStream_t stream, int num_sms, int *nlaunch) {
    if (nlaunch) *nlaunch = 1;
    switch (pixel_type) {
        case QLPIV_PIX_U8: return launch_pix<uint8_t>(job, n, stream, num_sms, nlaunch);
        case QLPIV_PIX_U16: return launch_pix<uint16_t>(job, n, stream, num_sms, nlaunch);
        case QLPIV_PIX_F32: return launch_pix<float>(job, n, stream, num_sms, nlaunch);
        default: return cudaErrorInvalidValue;
    }
}

bool xcorr_size_supported(int n) { return n == 16 || n == 32 || n == 64 || n == 128; }

// Resident batching units per SM at most (16 warps of the IA-16 kernel; the CTA kernels hold
// fewer CTAs).
constexpr long kMpUnitsPerSm = 16;
size_t xcorr_batch_bytes(int num_sms, long *units) {
    *units = kMpUnitsPerSm * num_sms;
    return sizeof(MpBatch) * (size_t)*units;
}
size_t xcorr_batch_slot_bytes(long units) { return sizeof(unsigned) * (size_t)((units + 31) / 32); }

template <int N>
static bool multipeak_fits_n(int kw) {
    return mp_stage_bytes(mp_geom(XcorrShape<N>::D, kw)) <= XcorrShape<N>::SCR_BYTES;
}

bool multipeak_supported(int n, int num_peaks, int peak_kernel) {
    if (num_peaks < 1 || num_peaks > QLPIV_MAX_PEAKS || peak_kernel < 2 || peak_kernel > 4096) return false;
    switch (n) {
        case 16: return multipeak_fits_n<16>(peak_kernel);
        case 32: return multipeak_fits_n<32>(peak_kernel);
        case 64: return multipeak_fits_n<64>(peak_kernel);
        // IA 128: the records are staged in rank 0's 64 column-pair regions
        case 128: return mp_stage_bytes(mp_geom(PairShape::D, peak_kernel)) <=
                         sizeof(cplx) * (size_t)PairShape::NR * PairShape::RP;
        default: return false;
    }
}

}  // namespace qlpiv
