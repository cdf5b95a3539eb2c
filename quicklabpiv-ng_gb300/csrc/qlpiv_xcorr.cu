// K1 device tables (twiddles, logarithm table) and the dispatch to the per-size launchers
// (qlpiv_xcorr{16,32,64,128}.cu).
#include <cmath>
#include <cstdlib>
#include <mutex>

#include "qlpiv_xcorr_launch.h"
#include "qlpiv_xcorr_pair.cuh"

namespace qlpiv {

// Twiddle tables exp(-2 pi i e / M) for M = 32, 64, 128, 256 (offsets 0, 32, 96, 224), filled
// once per device from the host (double precision, rounded to float).
static __device__ cplx g_twiddles[32 + 64 + 128 + 256];

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

cudaError_t launch_xcorr(const IaJob &job, int n, int pixel_type, cudaStream_t stream, int num_sms, int *nlaunch) {
    if (nlaunch) *nlaunch = 1;
    switch (n) {
        case 16: return launch_k1_16(job, pixel_type, stream, num_sms, nlaunch);
        case 32: return launch_k1_32(job, pixel_type, stream, num_sms, nlaunch);
        case 64: return launch_k1_64(job, pixel_type, stream, num_sms, nlaunch);
        case 128: return launch_k1_128(job, pixel_type, stream, num_sms, nlaunch);
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
