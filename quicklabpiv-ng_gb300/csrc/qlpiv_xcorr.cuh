// K1: fused FFT cross-correlation + integer peak + 3-point Gaussian sub-pixel fit,
// one CTA per interrogation area (IA) at a time, IA side N in {16, 32, 64}.
//
// Reference semantics (QuickLabPIV-ng, S/ = src/main/java/pt/quickLabPIV/):
//   tile max floored at 16         S/MatrixByte.java:16-33, S/MatrixInt16.java:21-38
//   v/max*16+1, A mirrored in re,  S/jobs/xcorr/FastRealFFTXCorr.java:44-68 (CPU: B by A's max)
//   B in im, zero padded to 2N     S/Matrix.java:175-181,282-288 (OpenCL job: own max)
//   Hermitian split + product      S/jobs/xcorr/FastRealFFTXCorr.java:70-116
//   (2N-1)^2 plane, shift N-1 = 0  S/jobs/xcorr/FastRealFFTXCorr.java:64-66
//   FindMaximumFromCenter          S/maximum/FindMaximumFromCenter.java:33-183
//   Gaussian1DPolynomial           S/interpolators/Gaussian1DPolynomialInterpolator.java:25-106
//   u = peakI - D/2, v = peakJ - D/2  S/maximum/MaxCrossResult.java:304-326
//
// Data flow inside the CTA (M = 2N, G = N/4 lanes per length-M transform):
//   1. every thread loads its share of the raw tile pixels (the exact pixels its
//      row transforms need), the CTA reduces the tile maxima;
//   2. row pass: the N non-zero rows of z = a' + i b' are transformed (upper half of
//      each row is zero) and scattered into N per-column-pair regions;
//   3. column task c transforms columns c and M-c (c = 0 pairs columns 0 and N),
//      forms P = F*G/M^2 with the mirror element fetched by warp shuffle, runs the
//      inverse column transform and stores q(., c) into its own region;
//   4. row-pair pass: rows 2p and 2p+1 of the Hermitian spectrum q are packed into
//      one complex inverse transform whose real/imaginary parts are the two
//      correlation rows; each lane scores its values with the reference's peak order
//      (value desc, distance to (N,N) asc, scan rank asc) and keeps the min floor;
//   5. CTA reduction of the peak key, then thread 0 fits the 3-point Gaussian from
//      the plane kept in shared memory and writes one 32-byte vector.
//   5'. multi-peak mode (FindMaximumMultiPeaks, S/maximum/FindMaximumMultiPeaks.java:42-162):
//      every thread reduces kw x kw cells of the plane to (max, position) records in
//      the reference's insertion order, with a per-32-record maximum; warp 0 then
//      replays the sorted, adjacency-suppressing list insertions
//      (S/util/SimpleFixedLengthFloatLinkedList.java:98-237), visiting only the records
//      that can change the list (all while it has room, otherwise those above its
//      minimum; whole 32-record chunks are skipped on their maximum), and queues one
//      fit per peak.
#pragma once
#include "qlpiv_fft.cuh"
#include "qlpiv_internal.h"
#include "qlpiv_logdf.cuh"
#include "qlpiv.h"
#include "qlpiv_subpix.cuh"

namespace qlpiv {

template <int N>
struct XcorrShape {
    static constexpr int M = 2 * N;
    static constexpr int D = M - 1;
    static constexpr int G = N / 4;                    // lanes per transform
    static constexpr int T = N == 16 ? 64 : (N == 32 ? 256 : 512);  // threads per CTA
    static constexpr int NG = T / G;                   // concurrent transforms
    static constexpr int ROUNDS = N / NG;              // tasks per group per phase
    // Shared-memory layouts (8-byte accesses of a 16-lane half-warp should touch 16 distinct bank
    // pairs).  Regions: slot s of a column-pair region at rslot(s), region pitch RP odd; FFT
    // exchanges in per-group buffers of pitch SP, layout L (qlpiv_fft.cuh).  N = 32: two groups
    // per half-warp, SP = 8 (mod 16) and the group-to-task maps below keep them on disjoint banks.
    static constexpr int L = N >= 32 ? 1 : 0;
    static constexpr int RP = N >= 32 ? M + 1 : M + M / 8 + 1;
    static constexpr int SP = N == 64 ? xbuf_size<M, 1>() : (N == 32 ? 72 : RP);
    static constexpr int MIN_BLOCKS = N == 16 ? 16 : (N == 32 ? 4 : 2);
    static constexpr size_t SCR_BYTES = sizeof(cplx) * (size_t)(NG * SP);
    static constexpr size_t SMEM = sizeof(cplx) * (size_t)(M + N * RP) + SCR_BYTES + 64 * sizeof(uint64_t) +
                                   32 * 56 /* fit queue */ + 256 /* multi-peak list */;
    __device__ static __forceinline__ int rslot(int s) { return N >= 32 ? s : pad8(s); }
    // Task of group grp in round r: the row of the row pass, the column pair of the column pass,
    // the row pair of the row-pair pass.  N = 32 (region pitch 65 = 1 mod 16): the two groups of a
    // half-warp take rows / columns 8 apart and row pairs 4 apart.  N = 64: the two groups of a
    // warp take row pairs 4 apart (their 4-byte plane stores land on disjoint banks).
    __device__ static __forceinline__ int task_row(int grp, int r) {
        return N == 32 ? ((grp >> 1) & 7) + 16 * (grp >> 4) + 8 * (grp & 1) : grp + NG * r;
    }
    __device__ static __forceinline__ int task_pair(int grp, int r) {
        return N >= 32 ? ((grp >> 1) & 3) + 8 * (grp >> 3) + 4 * (grp & 1) + NG * r : grp + NG * r;
    }
};

// FindMaximumMultiPeaks geometry of a d x d plane: slices = ceil(d / kw) per axis, the
// first `top` of them form the top/left half; records are visited slice by slice
// (row-major), four interleaved quadrant cells each.
struct MpGeom {
    int kw, top, nrec, nchunk;
};
__host__ __device__ inline MpGeom mp_geom(int d, int kw) {
    const int slices = (d + kw - 1) / kw;
    const int top = slices - slices / 2;
    const int nrec = 4 * top * top;
    return MpGeom{kw, top, nrec, (nrec + 31) / 32};
}
// Bytes of the per-IA record staging (values, positions, chunk maxima).
__host__ __device__ inline size_t mp_stage_bytes(const MpGeom &g) {
    return (size_t)g.nrec * 8 + (size_t)g.nchunk * 4;
}

template <typename Pix>
__device__ __forceinline__ float load_pix(const Pix *img, long pitch, int h, int w, int y, int x) {
    if ((unsigned)y >= (unsigned)h || (unsigned)x >= (unsigned)w) return 0.0f;
    return (float)__ldg(img + (long)y * pitch + x);
}

// Scan rank of cell (i, j) in FindMaximumFromCenter's visit order (first visit),
// centre c = N, h = N - 1.
__device__ __forceinline__ int peak_rank(int i, int j, int n) {
    const int c = n, h = n - 1;
    if (i == c && j == c) return 0;
    if (j == c) return i <= h ? 1 + 2 * (h - i) : 2 + 2 * (i - c);
    const int base1 = 1 + 2 * h;
    if (i == c) return j <= h ? base1 + 2 * (h - j) : base1 + 1 + 2 * (j - c);
    const int base2 = base1 + 2 * h;
    const bool top = i <= h, left = j <= h;
    const int a = top ? h - i : i - c;
    const int b = left ? h - j : j - c;
    const int q = top ? (left ? 0 : 2) : (left ? 1 : 3);
    return base2 + 4 * (a * h + b) + q;
}

__device__ __forceinline__ uint64_t peak_key(float v, int i, int j, int n) {
    if (!(v >= 0.0f)) return 0ull;  // negative or NaN never beats the running max of 0
    const uint32_t vb = __float_as_uint(v + 0.0f);
    const int di = i - n, dj = j - n;
    const uint32_t d2 = (uint32_t)(di * di + dj * dj);
    const uint32_t rk = (uint32_t)peak_rank(i, j, n);
    return ((uint64_t)vb << 32) | ((uint64_t)(0x7FFFu - d2) << 16) | (uint64_t)(0xFFFFu - rk);
}

struct IaJob {
    const void *img_a, *img_b;   // pixel planes (Pix), row pitch in elements
    long pitch_a, pitch_b;
    int h, w;
    const qlpiv_frame *frames;   // batched: per-IA frame table entry (NULL: img_a/img_b)
    const int *frame_idx;
    int num_frames;              // entries of `frames`: an IA whose index is outside [0, num_frames)
                                 // correlates two empty tiles instead of reading past the table
    const int *a_top, *a_left, *b_top, *b_left;  // per IA origins
    const float *max_a, *max_b;  // per IA maxima (max_mode == QLPIV_MAX_GIVEN)
    long count;
    int norm_mode, max_mode, subpix;  // subpix: qlpiv_subpix
    int subpix_pixels, subpix_iters;  // P-point interpolators: stencil pixels, Hongwei Guo iterations
    float fixed_max_a, fixed_max_b;
    qlpiv_vector *out;           // optional per-IA vectors (num_peaks per IA in multi-peak mode)
    float *planes;               // optional (2N-1)^2 planes per IA
    float *acc_u, *acc_v;        // optional: tile displacements += (u, v)  (Tile.accumulateDisplacement)
    const int *clip_top, *clip_left;  // NoOutOfBoundClipping of the accumulation: per IA tile origin,
    int clip_n, clip_h, clip_w;       //   tile side and image size (clip_n == 0: clipping allowed)
    int num_peaks;               // 0: FindMaximumFromCenter; k >= 1: FindMaximumMultiPeaks
    int peak_kernel;             // multi-peak cell width
    float2 *peak_uv;             // optional [count][k] displacement increments of every peak
    uint8_t *npeaks;             // optional [count] peaks found
    const cplx *twiddles;        // exp(-2 pi i e / M), e < M (device table, filled once per device)
    int waves;                   // grid = SMs x resident CTAs x waves; 0: the default per mode
    float *mp_planes;            // IA 128 multi-peak mode: one (2N-1)^2 plane per cluster (set by the launcher)
    const float4 *log_tab;       // log_fpair table (device, filled once per device with the twiddles)
    // batched multi-peak replay (NULL mp_batch: every IA replays its own list): mp_batch_units
    // batches, claimed by the resident warps (IA 16) or CTAs through the zeroed bitmask mp_slots;
    // IAs whose replay needs records that were not stored go to mp_retry ([0] count, then IAs)
    struct MpBatch *mp_batch;
    long mp_batch_units;
    unsigned *mp_slots;
    int *mp_retry;
    const int *ia_list;          // non-NULL: run IAs ia_list[1 .. 1 + ia_list[0]] instead of 0 .. count-1
};

// Integer peak and 3-point stencil of one IA, queued for the sub-pixel fit.
struct FitRec {
    long ia;
    int pi, pj, kind;   // kind: 0 fit, 1 no peak, 2 stencil off the plane, 3 no sub-pixel, 4 absent slot,
                        //       5 floor below the interpolator's limit
    int slot, npk;      // multi-peak: peak index (0 = largest) and peaks found
    float pv, mn, c0, yu, yd, xl, xr;
};
static_assert(sizeof(FitRec) == 56, "fit queue sizing");

// P-point interpolators on the stencils v (P values along I through the peak, then P along J):
// sub-pixel position, flags and (Hongwei Guo) peak value.  Out of line: the fits' double-precision
// working set stays out of K1's register allocation.
static __device__ __noinline__ void fit_ppoint(int mode, int P, int iters, int pi, int pj, const float *v, float *si,
                                        float *sj, float *pv, uint32_t *flags) {
    const float *vi = v, *vj = v + P;
    if (mode == QLPIV_SUBPIX_GAUSS_LM) {
        double m;
        if (sp_gauss_lm(vi, P, (double)pi, &m) && fabs(m - (double)pi) < 2.0) {
            *si = (float)m;
            *flags |= QLPIV_F_SUB_I;
        }
        if (sp_gauss_lm(vj, P, (double)pj, &m) && fabs(m - (double)pj) < 2.0) {
            *sj = (float)m;
            *flags |= QLPIV_F_SUB_J;
        }
        return;
    }
    float xs[kMaxSubpixPixels];
    float ym, ya, xm, xa;
    for (int k = 0; k < P; k++) xs[k] = (float)(pi - P / 2 + k);
    sp_hongwei_guo(xs, vi, P, iters, &ym, &ya);
    for (int k = 0; k < P; k++) xs[k] = (float)(pj - P / 2 + k);
    sp_hongwei_guo(xs, vj, P, iters, &xm, &xa);
    const bool yv = !(fabsf(__fsub_rn(ym, (float)pi)) > (float)P / 2.0f);
    const bool xv = !(fabsf(__fsub_rn(xm, (float)pj)) > (float)P / 2.0f);
    if (yv) { *si = ym; *flags |= QLPIV_F_SUB_I; }
    if (xv) { *sj = xm; *flags |= QLPIV_F_SUB_J; }
    if (yv) {
        *pv = ya;
        if (xv && xa > *pv) *pv = xa;
    } else if (xv) {
        *pv = xa;
    }
}

// Gaussian1DPolynomialInterpolator.interpolate (S/interpolators/Gaussian1DPolynomialInterpolator.java:25-106)
// for q[0..n): lane k handles record k, so the logarithms of 32 IAs share one
// warp instruction.  Called by one full warp.
template <int D, bool PP>
__device__ void fit_flush(const FitRec *q, const float *fitv, int n, int lane, const IaJob &job) {
    __syncwarp();
    if (lane < n) {
        const FitRec r = q[lane];
        float si = (float)r.pi, sj = (float)r.pj;
        float pv = r.pv;
        uint32_t flags = 0;
        if (r.kind == 1) {
            flags |= QLPIV_F_NO_PEAK;
        } else if (r.kind == 2) {
            flags |= QLPIV_F_EDGE;
        } else if (r.kind == 5) {
            flags |= QLPIV_F_FLOOR;
        } else if (PP && r.kind == 0 && job.subpix >= QLPIV_SUBPIX_GAUSS_LM) {
            if constexpr (PP)
                fit_ppoint(job.subpix, job.subpix_pixels, job.subpix_iters, r.pi, r.pj,
                           fitv + lane * 2 * job.subpix_pixels, &si, &sj, &pv, &flags);
        } else if (r.kind == 0) {
            const bool neg = r.c0 < 0.0f || r.yu < 0.0f || r.yd < 0.0f || r.xl < 0.0f || r.xr < 0.0f;
            const float y0 = r.yu + 1e-8f, y1 = r.c0 + 1e-8f, y2 = r.yd + 1e-8f;
            const float x0 = r.xl + 1e-8f, x1 = r.c0 + 1e-8f, x2 = r.xr + 1e-8f;
            float ti, tj;
            if (!neg) {
                // the reference's double logarithms, carried as float pairs (error < 1e-11)
                const fpair ly0 = log_fpair(y0, job.log_tab), ly1 = log_fpair(y1, job.log_tab),
                            ly2 = log_fpair(y2, job.log_tab);
                const fpair lx0 = log_fpair(x0, job.log_tab), lx1 = log_fpair(x1, job.log_tab),
                            lx2 = log_fpair(x2, job.log_tab);
                const fpair di = fp_add(fp_add(fp_scale2(ly0, 2.0f), fp_scale2(ly1, -4.0f)), fp_scale2(ly2, 2.0f));
                const fpair dj = fp_add(fp_add(fp_scale2(lx0, 2.0f), fp_scale2(lx1, -4.0f)), fp_scale2(lx2, 2.0f));
                const fpair ni = fp_add(ly0, fp_scale2(ly2, -1.0f)), nj = fp_add(lx0, fp_scale2(lx2, -1.0f));
                ti = __fadd_rn((float)r.pi, __fdiv_rn(fp_round(ni), fp_round(di)));
                tj = __fadd_rn((float)r.pj, __fdiv_rn(fp_round(nj), fp_round(dj)));
            } else {
                flags |= QLPIV_F_PARABOLIC;
                const float dy = __fadd_rn(__fadd_rn(__fmul_rn(2.0f, y0), -__fmul_rn(4.0f, y1)), __fmul_rn(2.0f, y2));
                const float dx = __fadd_rn(__fadd_rn(__fmul_rn(2.0f, x0), -__fmul_rn(4.0f, x1)), __fmul_rn(2.0f, x2));
                ti = __fadd_rn((float)r.pi, __fdiv_rn(y0 - y2, dy));
                tj = __fadd_rn((float)r.pj, __fdiv_rn(x0 - x2, dx));
            }
            if (isfinite(ti) && fabsf(ti - (float)r.pi) <= 1.0f) { si = ti; flags |= QLPIV_F_SUB_I; }
            if (isfinite(tj) && fabsf(tj - (float)r.pj) <= 1.0f) { sj = tj; flags |= QLPIV_F_SUB_J; }
        }
        qlpiv_vector o;
        o.u = si - (float)(D / 2);
        o.v = sj - (float)(D / 2);
        o.sub_i = si;
        o.sub_j = sj;
        o.peak_value = pv;
        o.min_floor = r.mn;
        o.peak_i = (int16_t)r.pi;
        o.peak_j = (int16_t)r.pj;
        o.flags = flags;
        if (r.kind == 4) {
            o = qlpiv_vector{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0, 0, QLPIV_F_ABSENT};
        }
        if (job.num_peaks == 0) {
            if (job.out != nullptr) job.out[r.ia] = o;
        } else {
            const long slot = r.ia * job.num_peaks + r.slot;
            if (job.out != nullptr) job.out[slot] = o;
            if (job.peak_uv != nullptr) job.peak_uv[slot] = make_float2(o.u, o.v);
            if (r.slot == 0 && job.npeaks != nullptr) job.npeaks[r.ia] = (uint8_t)r.npk;
        }
        if (job.acc_u != nullptr && r.slot == 0) {
            const float nu = job.acc_u[r.ia] + o.u, nv = job.acc_v[r.ia] + o.v;
            // an increment that would move the tile out of the image is dropped
            if (job.clip_n == 0 ||
                tile_inside(job.clip_n, job.clip_h, job.clip_w, job.clip_top[r.ia], job.clip_left[r.ia], nu, nv)) {
                job.acc_u[r.ia] = nu;
                job.acc_v[r.ia] = nv;
            }
        }
    }
    __syncwarp();
}

// SimpleFixedLengthFloatLinkedList.addInAscendOrder (S/util/SimpleFixedLengthFloatLinkedList.java:98-237)
// with the list held by one warp, entry r (ascending order) in lane r's registers.
// Called by the full warp with a warp-uniform candidate (v, i, j).  Entries smaller than v
// and adjacent to it are deleted, but only if v is inserted; v is refused next to an
// equal or larger entry, or when the list is full and v is not above its minimum;
// when the list overflows its smallest entry leaves.  Adjacent = squared distance below
// kd = (kw - 1) * kw (exact in float for plane coordinates).
struct WarpPeakList {
    float lv = 0.0f;
    int li = 0, lj = 0;
    int size = 0;       // warp-uniform
    __device__ __forceinline__ void insert(int lane, int k, float kd, float v, int i, int j) {
        const bool valid = lane < size;
        const bool less = valid && lv < v;
        const int di = i - li, dj = j - lj;
        const bool adj = valid && (float)(di * di + dj * dj) < kd;
        const int pos = __popc(__ballot_sync(0xffffffffu, less));
        if (size == k && pos == 0) return;
        if (__ballot_sync(0xffffffffu, valid && !less && adj) != 0u) return;
        const unsigned del = __ballot_sync(0xffffffffu, less && adj);
        const unsigned keep = ((1u << size) - 1u) & ~del;   // size <= 16
        const int ipos = pos - __popc(del);                 // deleted entries all lie below pos
        int nsize = size - __popc(del) + 1;
        const int drop = nsize > k ? 1 : 0;                 // only when nothing was deleted, ipos >= 1
        nsize -= drop;
        const int d = lane + drop;                          // this lane takes element d of the merged list
        int src = -1;
        if (d < ipos) src = (int)__fns(keep, 0, d + 1) ;
        else if (d > ipos) src = (int)__fns(keep, 0, d);
        const int sl = src < 0 ? 0 : (src & 31);
        const float sv = __shfl_sync(0xffffffffu, lv, sl);
        const int si = __shfl_sync(0xffffffffu, li, sl);
        const int sj = __shfl_sync(0xffffffffu, lj, sl);
        if (lane < nsize) {
            if (src < 0) { lv = v; li = i; lj = j; }
            else { lv = sv; li = si; lj = sj; }
        }
        size = nsize;
    }
    __device__ __forceinline__ float lowest() const { return __shfl_sync(0xffffffffu, lv, 0); }
    __device__ __forceinline__ void store(int lane, float *sv, int *si, int *sj) const {
        if (lane < size) { sv[lane] = lv; si[lane] = li; sj[lane] = lj; }
    }
};

// The same list for k <= KF held whole in every lane's registers (fully unrolled, no
// shuffles): every lane applies the same insertion to its own copy.
template <int KF>
struct RegPeakList {
    float lv[KF];
    int li[KF], lj[KF];
    int size = 0;
    __device__ __forceinline__ RegPeakList() {
#pragma unroll
        for (int r = 0; r < KF; r++) { lv[r] = 0.0f; li[r] = 0; lj[r] = 0; }
    }
    // entries [0, n) ascending; v goes to index pos (0 <= pos <= n < KF + drop); drop: the
    // smallest leaves afterwards
    __device__ __forceinline__ void place(int pos, int drop, float v, int i, int j) {
        float nv[KF];
        int ni[KF], nj[KF];
#pragma unroll
        for (int d = 0; d < KF; d++) {
            // merged element m = d + drop: lv[m] below pos, the new entry at pos, lv[m-1] above
            const int m = d + drop;
            const float a_v = (d + 1 < KF) ? lv[d + 1 < KF ? d + 1 : 0] : 0.0f;
            const int a_i = (d + 1 < KF) ? li[d + 1 < KF ? d + 1 : 0] : 0;
            const int a_j = (d + 1 < KF) ? lj[d + 1 < KF ? d + 1 : 0] : 0;
            const float lo_v = drop ? a_v : lv[d];              // lv[m]
            const int lo_i = drop ? a_i : li[d], lo_j = drop ? a_j : lj[d];
            const float hi_v = drop ? lv[d] : (d > 0 ? lv[d > 0 ? d - 1 : 0] : 0.0f);   // lv[m - 1]
            const int hi_i = drop ? li[d] : (d > 0 ? li[d > 0 ? d - 1 : 0] : 0);
            const int hi_j = drop ? lj[d] : (d > 0 ? lj[d > 0 ? d - 1 : 0] : 0);
            nv[d] = m < pos ? lo_v : (m == pos ? v : hi_v);
            ni[d] = m < pos ? lo_i : (m == pos ? i : hi_i);
            nj[d] = m < pos ? lo_j : (m == pos ? j : hi_j);
        }
#pragma unroll
        for (int d = 0; d < KF; d++) { lv[d] = nv[d]; li[d] = ni[d]; lj[d] = nj[d]; }
    }
    __device__ __forceinline__ void insert(int /*lane*/, int k, float kd, float v, int i, int j) {
        int pos = 0;
        bool refuse = false;
        unsigned del = 0u;
#pragma unroll
        for (int r = 0; r < KF; r++) {
            const bool valid = r < size;
            const bool less = valid && lv[r] < v;
            const int di = i - li[r], dj = j - lj[r];
            const bool adj = valid && (float)(di * di + dj * dj) < kd;
            pos += less ? 1 : 0;
            refuse = refuse || (valid && !less && adj);
            if (less && adj) del |= 1u << r;
        }
        if (size == k && pos == 0) return;
        if (refuse) return;
        if (del == 0u && size == k) {  // common: full, nothing adjacent -> the smallest leaves
            place(pos, 1, v, i, j);
            return;
        }
        if (del != 0u) {
            // rare: compact the survivors in place first (all deleted entries lie below pos);
            // survivor r moves down to slot w <= r
            int w = 0;
#pragma unroll
            for (int r = 0; r < KF; r++) {
                const bool surv = r < size && !((del >> r) & 1u);
#pragma unroll
                for (int q = 0; q <= r; q++) {
                    if (surv && w == q) {
                        lv[q] = lv[r];
                        li[q] = li[r];
                        lj[q] = lj[r];
                    }
                }
                w += surv ? 1 : 0;
            }
            const int nd = __popc(del);
            size -= nd;
            pos -= nd;
        }
        place(pos, 0, v, i, j);  // room for one more
        size++;
    }
    __device__ __forceinline__ float lowest() const { return lv[0]; }
    __device__ __forceinline__ void store(int lane, float *sv, int *si, int *sj) const {
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < KF; r++)
                if (r < size) { sv[r] = lv[r]; si[r] = li[r]; sj[r] = lj[r]; }
        }
    }
};

// Visits, in order, the records e >= e_begin with value >= floor_v that can change the
// list (all while it has room, otherwise those above its minimum), skipping whole
// 32-record chunks on their maximum.  With track set, remembers the list as it was before
// the last insertion that turned a full list into one with room (e_break = that record).
template <typename List>
__device__ void mp_visit(const MpGeom &gm, const float *recv, const int *recp, const float *chmax, int lane, int k,
                         float kd, int e_begin, float floor_v, List &lst, bool track, List &saved, int &e_break) {
    float lo = lst.size > 0 ? lst.lowest() : 0.0f;
    for (int c0 = (e_begin >> 5) & ~31; c0 < gm.nchunk; c0 += 32) {
        const int c = c0 + lane;
        const float cmx = c < gm.nchunk ? chmax[c] : 0.0f;
        unsigned todo = __ballot_sync(0xffffffffu, c < gm.nchunk && c >= (e_begin >> 5) && cmx >= floor_v);
        while (true) {
            const unsigned cmask = __ballot_sync(0xffffffffu, ((todo >> lane) & 1u) && (lst.size < k || cmx > lo));
            if (cmask == 0u) break;
            const int cl = __ffs(cmask) - 1;
            todo &= ~((2u << cl) - 1u);
            const int e = (c0 + cl) * 32 + lane;
            const bool in = e < gm.nrec && e >= e_begin;
            const float v = in ? recv[e] : 0.0f;
            const int pp = in ? recp[e] : 0;
            unsigned pend = __ballot_sync(0xffffffffu, in && v >= floor_v);
            while (true) {
                const unsigned cand = __ballot_sync(0xffffffffu, ((pend >> lane) & 1u) && (lst.size < k || v > lo));
                if (cand == 0u) break;
                const int src = __ffs(cand) - 1;
                pend &= ~((2u << src) - 1u);
                const float cv = __shfl_sync(0xffffffffu, v, src);
                int cp = __shfl_sync(0xffffffffu, pp, src);
                const int ce = (c0 + cl) * 32 + src;
                if (cp < 0) {  // stale position of the same quadrant, else (0, 0)
                    cp = 0;
                    for (int e2 = ce - 4; e2 >= 0; e2 -= 4)
                        if (recp[e2] >= 0) { cp = recp[e2]; break; }
                }
                if (track && lst.size == k) {
                    const List before = lst;
                    lst.insert(lane, k, kd, cv, cp >> 16, cp & 0xffff);
                    if (lst.size < k) {
                        saved = before;
                        e_break = ce;
                    }
                } else {
                    lst.insert(lane, k, kd, cv, cp >> 16, cp & 0xffff);
                }
                lo = lst.lowest();
            }
        }
    }
}

// Replays the insertions of the records (values recv, positions recp, -1 = stale) and
// returns the list size; the list is left in sv/si/sj (ascending).
//
// Records below a threshold t cannot change which entries >= t the list holds: run on
// the records >= t alone, the list always holds exactly the full run's entries >= t
// (an entry < t only ever leaves room or is evicted first, and is never needed to
// refuse or delete a record >= t).  So with t = the 4th largest chunk maximum the short
// run over the records >= t is the answer whenever it ends full; if it ended with room,
// the full run is resumed from the last point where the short run's list was full
// (both lists are equal there), or from the start if it never was.
template <typename List>
__device__ int mp_replay(const MpGeom &gm, const float *recv, const int *recp, const float *chmax, int lane, int k,
                         float kd, float *sv, int *si, int *sj) {
    // t: 4th largest chunk maximum (chunks lane, lane + 32, ... ; nchunk <= 128)
    float cm[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int c = lane + 32 * q;
        cm[q] = c < gm.nchunk ? chmax[c] : -1.0f;
    }
    float t = 0.0f;
    const int rounds = gm.nchunk < 4 ? gm.nchunk : 4;
    for (int r = 0; r < rounds; r++) {
        float lm = fmaxf(fmaxf(cm[0], cm[1]), fmaxf(cm[2], cm[3]));
        float wm = lm;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wm = fmaxf(wm, __shfl_xor_sync(0xffffffffu, wm, o));
        const int owner = __ffs(__ballot_sync(0xffffffffu, lm == wm)) - 1;
        if (lane == owner) {  // drop one occurrence
            if (cm[0] == wm) cm[0] = -1.0f;
            else if (cm[1] == wm) cm[1] = -1.0f;
            else if (cm[2] == wm) cm[2] = -1.0f;
            else cm[3] = -1.0f;
        }
        t = wm;
    }
    List lst, saved;
    int e_break = -1;
    if (t > 0.0f) {
        mp_visit<List>(gm, recv, recp, chmax, lane, k, kd, 0, t, lst, true, saved, e_break);
        if (lst.size < k) {
            if (e_break >= 0) {
                lst = saved;
                mp_visit<List>(gm, recv, recp, chmax, lane, k, kd, e_break, -3.402823466e38f, lst, false, saved,
                               e_break);
            } else {
                lst = List();
                mp_visit<List>(gm, recv, recp, chmax, lane, k, kd, 0, -3.402823466e38f, lst, false, saved, e_break);
            }
        }
    } else {
        mp_visit<List>(gm, recv, recp, chmax, lane, k, kd, 0, -3.402823466e38f, lst, false, saved, e_break);
    }
    lst.store(lane, sv, si, sj);
    __syncwarp();
    return lst.size;
}

// Cell maxima of the plane in record order (records e = 4 * slice + quadrant): strict >
// from 0, first in row-major order within the cell; position -1 = no positive value (the
// reference then reuses the quadrant's previous position).  Also the maximum of every
// 32 consecutive records.  KW = cell width, 0 = gm.kw at run time.  All threads.
template <int D, int T, int KW, typename Plane>
__device__ __forceinline__ void mp_cells(const MpGeom &gm, const Plane &P, float *recv, int *recp, float *chmax) {
    // T == 32: one warp works alone on its IA (the warp-per-IA kernel)
    const int lane = threadIdx.x & 31, warp = T == 32 ? 0 : (int)(threadIdx.x >> 5);
    const int kw = KW > 0 ? KW : gm.kw;
    // with a compile-time cell width the geometry is constant: no run-time division
    constexpr int kTop = KW > 0 ? ((D + KW - 1) / KW) - ((D + KW - 1) / KW) / 2 : 1;
    const int top = KW > 0 ? kTop : gm.top;
    const int nrec = KW > 0 ? 4 * kTop * kTop : gm.nrec;
    for (int base = warp * 32; base < nrec; base += T) {
        const int e = base + lane;
        float bv = 0.0f;
        if (e < nrec) {
            int bp = -1;
            const int sl = e >> 2, q = e & 3;
            const int ci = (KW > 0 ? sl / kTop : sl / top) + ((q & 2) ? top : 0);
            const int cj = (KW > 0 ? sl % kTop : sl % top) + ((q & 1) ? top : 0);
            const int i0 = ci * kw, j0 = cj * kw;
            if (KW > 0) {
#pragma unroll
                for (int a = 0; a < (KW > 0 ? KW : 1); a++) {
                    const int i = i0 + a;
#pragma unroll
                    for (int b = 0; b < (KW > 0 ? KW : 1); b++) {
                        const int j = j0 + b;
                        if (i < D && j < D) {
                            const float v = P(i, j);
                            if (v > bv) { bv = v; bp = (i << 16) | j; }
                        }
                    }
                }
            } else {
                for (int a = 0; a < kw; a++) {
                    const int i = i0 + a;
                    if (i >= D) break;
                    for (int b = 0; b < kw; b++) {
                        const int j = j0 + b;
                        if (j >= D) break;
                        const float v = P(i, j);
                        if (v > bv) { bv = v; bp = (i << 16) | j; }
                    }
                }
            }
            recv[e] = bv;
            recp[e] = bp;
        }
        float cm = bv;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cm = fmaxf(cm, __shfl_xor_sync(0xffffffffu, cm, o));
        if (lane == 0) chmax[base >> 5] = cm;
    }
}

// Sub-pixel stencil of record r (peak r.pi, r.pj already set): the kind, and the stencil values
// (3-point: in the record; P-point: 2P floats at fv, column then row, floor-lifted).
template <int D, typename Plane>
__device__ __forceinline__ void fit_stencil(FitRec &r, const IaJob &job, const Plane &P, float *fv) {
    r.kind = 0;
    if (!job.subpix) {
        r.kind = 3;
    } else if (r.pi == 0 && r.pj == 0) {
        r.kind = 1;
    } else if (job.subpix == QLPIV_SUBPIX_GAUSS3) {
        if (r.pi - 1 < 0 || r.pi + 1 >= D || r.pj - 1 < 0 || r.pj + 1 >= D) {
            r.kind = 2;
        } else {
            r.c0 = P(r.pi, r.pj);
            r.yu = P(r.pi - 1, r.pj);
            r.yd = P(r.pi + 1, r.pj);
            r.xl = P(r.pi, r.pj - 1);
            r.xr = P(r.pi, r.pj + 1);
        }
    } else {
        const int h = job.subpix_pixels / 2;
        const float lim = job.subpix == QLPIV_SUBPIX_GAUSS_LM ? -3.15f : -5.15f;
        if (r.pi - h < 0 || r.pi + h >= D || r.pj - h < 0 || r.pj + h >= D) {
            r.kind = 2;
        } else if (r.mn < lim) {
            r.kind = 5;  // the reference throws InterpolateException here
        } else {
            const float add = r.mn < 0.0f ? __fadd_rn(-r.mn, 1e-8f) : 0.0f;
            const int Pn = job.subpix_pixels;
            for (int k = 0; k < Pn; k++) {
                fv[k] = __fadd_rn(P(r.pi - h + k, r.pj), add);
                fv[Pn + k] = __fadd_rn(P(r.pi, r.pj - h + k), add);
            }
        }
    }
}

// FindMaximumMultiPeaks over a D x D plane read through P(i, j), by a CTA of T threads: the
// records are staged at `stage` (mp_stage_bytes), the list replayed by warp 0, one fit record
// queued per slot.
template <int T>
__device__ __forceinline__ void group_sync() {
    if constexpr (T == 32) __syncwarp();
    else __syncthreads();
}

template <int D, int T, typename Plane>
__device__ __forceinline__ void multipeak_core(const IaJob &job, long ia, float minf, const Plane &P, void *stage,
                                               uint64_t *red, FitRec *fitq, float *fitv, int qn, float *mp_lv,
                                               int *mp_li, int *mp_lj) {
    constexpr int NWARPS = T / 32;
    const int lane = threadIdx.x & 31, warp = T == 32 ? 0 : (int)(threadIdx.x >> 5);
    const int multi = job.num_peaks;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) minf = fminf(minf, __shfl_xor_sync(0xffffffffu, minf, o));
    group_sync<T>();  // plane complete; the FFT scratch is free for the records
    float *redf = reinterpret_cast<float *>(red);
    if (lane == 0) redf[warp] = minf;
    const MpGeom gm = mp_geom(D, job.peak_kernel);
    const int kw = gm.kw;
    float *recv = reinterpret_cast<float *>(stage);
    int *recp = reinterpret_cast<int *>(recv + gm.nrec);
    float *chmax = reinterpret_cast<float *>(recp + gm.nrec);
    // cell maxima: strict > from 0, first in row-major order; -1 = no positive
    // value (the reference then reuses the quadrant's previous position)
    if (kw == 3) {
        mp_cells<D, T, 3>(gm, P, recv, recp, chmax);
    } else {
        mp_cells<D, T, 0>(gm, P, recv, recp, chmax);
    }
    group_sync<T>();
    if (warp == 0) {
        float mn = lane < NWARPS ? redf[lane] : 3.402823466e38f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        const float kd = (float)((kw - 1) * kw);
        int size;
        switch (multi) {
            case 1: size = mp_replay<RegPeakList<1>>(gm, recv, recp, chmax, lane, 1, kd, mp_lv, mp_li, mp_lj); break;
            case 2: size = mp_replay<RegPeakList<2>>(gm, recv, recp, chmax, lane, 2, kd, mp_lv, mp_li, mp_lj); break;
            case 3: size = mp_replay<RegPeakList<3>>(gm, recv, recp, chmax, lane, 3, kd, mp_lv, mp_li, mp_lj); break;
            case 4: size = mp_replay<RegPeakList<4>>(gm, recv, recp, chmax, lane, 4, kd, mp_lv, mp_li, mp_lj); break;
            default: size = mp_replay<WarpPeakList>(gm, recv, recp, chmax, lane, multi, kd, mp_lv, mp_li, mp_lj);
        }
        // one fit record per slot, largest peak first
        if (lane < multi) {
            FitRec r;
            r.ia = ia;
            r.mn = mn;
            r.slot = lane;
            r.npk = size;
            r.pi = 0;
            r.pj = 0;
            r.pv = 0.0f;
            if (lane < size) {
                const int idx = size - 1 - lane;
                r.pi = mp_li[idx];
                r.pj = mp_lj[idx];
                r.pv = mp_lv[idx];
                fit_stencil<D>(r, job, P, fitv + (qn + lane) * 2 * job.subpix_pixels);
            } else {
                r.kind = 4;
            }
            fitq[qn + lane] = r;
        }
    }
}

// ---- Batched multi-peak replay ----
// The list replay of one IA is a short chain of dependent insertions (4 to 9 on the adaptive
// PIV planes) that a warp runs with every lane doing the same work.  Instead, the records the
// replay of an IA can reach are stored with the 3-point stencil at their position, kMpBatch
// IAs to a batch, and one warp replays the whole batch with one IA per lane.  Stored per IA:
// every record >= t, t = the 4th largest maximum of 32 consecutive records (the run over those
// records alone is exact whenever it ends with a full list, see mp_replay), and the last
// kMpTail records, from which the run resumes when its last full-to-room transition lies there.
// An IA whose replay needs records that were not stored (more than kMpCandMax of them, t == 0,
// or an earlier resume point) is flagged and run again through the per-IA path.  Used for
// k <= 4 peaks with the 3-point fit or none (the P-point stencils are not stored).
constexpr int kMpBatch = 32, kMpCandMax = 24, kMpTail = 8;
struct __align__(16) MpCand {
    float v;
    int code;  // record e << 14 | i << 7 | j (resolved position: planes of side <= 127)
    float c0, yu, yd, xl, xr, pad;
};
struct __align__(16) MpMeta {
    long ia;
    float mn, t;
    int n, retry;
    int pad[2];
};
struct MpBatch {
    MpMeta meta[kMpBatch];
    MpCand cand[kMpCandMax][kMpBatch];  // candidate-major: a lane's reads of one slot coalesce
};
static_assert(sizeof(MpCand) == 32 && sizeof(MpMeta) == 32, "batch layout");

__device__ __forceinline__ bool mp_batched(const IaJob &job) {
    return job.mp_batch != nullptr && job.num_peaks >= 1 && job.num_peaks <= 4 &&
           (job.subpix == QLPIV_SUBPIX_NONE || job.subpix == QLPIV_SUBPIX_GAUSS3);
}

// Claims a free batch (bit of the zeroed bitmask `slots`, `units` bits) for the calling warp or
// CTA, starting the search at word `hint`; -1 when a bounded search found none (the caller then
// replays per IA).  At most `units` warps / CTAs are resident, so one is normally free.
__device__ __forceinline__ int mp_claim(unsigned *slots, long units, int hint) {
    const int words = (int)((units + 31) / 32);
    for (int k = 0; k < 4 * words; k++) {
        const int w = (hint + k) % words;
        unsigned avail = ~*reinterpret_cast<volatile unsigned *>(slots + w);
        if (w == words - 1 && (units & 31) != 0) avail &= (1u << (units & 31)) - 1u;
        while (avail != 0u) {
            const unsigned bit = avail & (0u - avail);
            const unsigned old = atomicOr(slots + w, bit);
            if ((old & bit) == 0u) return w * 32 + (__ffs(bit) - 1);
            avail &= ~(old | bit);
        }
    }
    return -1;
}

// Returns batch s once its last replay is done.
__device__ __forceinline__ void mp_release(unsigned *slots, int s) {
    __threadfence();
    atomicAnd(slots + (s >> 5), ~(1u << (s & 31)));
}

// Stores IA `ia`'s reachable records (staged by mp_cells) as entry b of the batch.  One full warp.
template <int D, typename Plane>
__device__ void mp_extract(const MpGeom &gm, const Plane &P, const float *recv, const int *recp, const float *chmax,
                           int lane, long ia, float mn, MpBatch *bt, int b) {
    static_assert(D <= 127, "record positions are packed in 7 bits");
    // t: 4th largest chunk maximum; keys = float bits + 1 (records are >= +0), 0 = taken
    unsigned key[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int c = lane + 32 * q;
        key[q] = c < gm.nchunk ? __float_as_uint(chmax[c]) + 1u : 0u;
    }
    unsigned tk = 0u;
    const int rounds = gm.nchunk < 4 ? gm.nchunk : 4;
    for (int r = 0; r < rounds; r++) {
        const unsigned lm = max(max(key[0], key[1]), max(key[2], key[3]));
        const unsigned wm = __reduce_max_sync(0xffffffffu, lm);
        const int owner = __ffs(__ballot_sync(0xffffffffu, lm == wm)) - 1;
        if (lane == owner) {
            if (key[0] == wm) key[0] = 0u;
            else if (key[1] == wm) key[1] = 0u;
            else if (key[2] == wm) key[2] = 0u;
            else key[3] = 0u;
        }
        tk = wm;
    }
    const float t = __uint_as_float(tk - 1u);
    const bool ok = tk > 1u && t > 0.0f;
    const int tail = gm.nrec - kMpTail;
    const unsigned lt = (1u << lane) - 1u;
    int base = 0;
    if (ok) {
        for (int c0 = 0; c0 < gm.nchunk; c0 += 32) {
            const int c = c0 + lane;
            unsigned todo = __ballot_sync(0xffffffffu, c < gm.nchunk && (chmax[c] >= t || (c + 1) * 32 > tail));
            while (todo != 0u) {
                const int cl = __ffs(todo) - 1;
                todo &= todo - 1u;
                const int e = (c0 + cl) * 32 + lane;
                const float v = e < gm.nrec ? recv[e] : 0.0f;
                const bool take = e < gm.nrec && (v >= t || e >= tail);
                const unsigned mask = __ballot_sync(0xffffffffu, take);
                const int idx = base + __popc(mask & lt);
                if (take && idx < kMpCandMax) {
                    int pp = recp[e];
                    if (pp < 0) {  // stale: the quadrant's previous position, else (0, 0)
                        pp = 0;
                        for (int e2 = e - 4; e2 >= 0; e2 -= 4)
                            if (recp[e2] >= 0) { pp = recp[e2]; break; }
                    }
                    const int pi = pp >> 16, pj = pp & 0xffff;
                    MpCand cd;
                    cd.v = v;
                    cd.code = (e << 14) | (pi << 7) | pj;
                    cd.c0 = cd.yu = cd.yd = cd.xl = cd.xr = cd.pad = 0.0f;
                    if (pi >= 1 && pi <= D - 2 && pj >= 1 && pj <= D - 2) {
                        cd.c0 = P(pi, pj);
                        cd.yu = P(pi - 1, pj);
                        cd.yd = P(pi + 1, pj);
                        cd.xl = P(pi, pj - 1);
                        cd.xr = P(pi, pj + 1);
                    }
                    bt->cand[idx][b] = cd;
                }
                base += __popc(mask);
            }
        }
    }
    if (lane == 0) {
        MpMeta m;
        m.ia = ia;
        m.mn = mn;
        m.t = t;
        m.n = base < kMpCandMax ? base : kMpCandMax;
        m.retry = (!ok || base > kMpCandMax) ? 1 : 0;
        m.pad[0] = m.pad[1] = 0;
        bt->meta[b] = m;
    }
    __syncwarp();
}

// Lane b's replay of batch entry b (b < nb) into lst; true when the entry must be run again.
template <int K>
__device__ __forceinline__ bool mp_batch_replay(const MpBatch *bt, int b, int k, float kd, int nrec,
                                                RegPeakList<K> &lst, MpMeta &m) {
    m = bt->meta[b];
    if (m.retry) return true;
    RegPeakList<K> saved;
    int e_break = -1;
    float2 nx = m.n > 0 ? *reinterpret_cast<const float2 *>(&bt->cand[0][b]) : make_float2(0.0f, 0.0f);
    for (int s = 0; s < m.n; s++) {
        // (value, code) of entry s; entry s + 1's is on its way meanwhile
        const MpCand c{nx.x, __float_as_int(nx.y), 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        if (s + 1 < m.n) nx = *reinterpret_cast<const float2 *>(&bt->cand[s + 1][b]);
        if (!(c.v >= m.t)) continue;
        const int i = (c.code >> 7) & 127, j = c.code & 127;
        if (lst.size == k) {
            const RegPeakList<K> before = lst;
            lst.insert(0, k, kd, c.v, i, j);
            if (lst.size < k) {
                saved = before;
                e_break = c.code >> 14;
            }
        } else {
            lst.insert(0, k, kd, c.v, i, j);
        }
    }
    if (lst.size < k) {
        // resume at the last full-to-room transition: every record from there on must be stored
        if (e_break < 0 || e_break < nrec - kMpTail) return true;
        lst = saved;
        for (int s = 0; s < m.n; s++) {
            const float2 c = *reinterpret_cast<const float2 *>(&bt->cand[s][b]);
            const int code = __float_as_int(c.y);
            if ((code >> 14) >= e_break) lst.insert(0, k, kd, c.x, (code >> 7) & 127, code & 127);
        }
    }
    return false;
}

// Replays the nb entries of the batch (one per lane) and queues/flushes their fits, one peak
// slot per round through fitq; the entries to run again go to job.mp_retry.  One full warp;
// fitq must be empty.
template <int D, int K, bool PP>
__device__ void mp_batch_run_k(const MpBatch *bt, int nb, int lane, const IaJob &job, FitRec *fitq,
                                   const float *fitv) {
    const int k = job.num_peaks;
    const MpGeom gm = mp_geom(D, job.peak_kernel);
    const float kd = (float)((gm.kw - 1) * gm.kw);
    RegPeakList<K> lst;
    MpMeta m;
    bool retry = true;
    if (lane < nb) retry = mp_batch_replay<K>(bt, lane, k, kd, gm.nrec, lst, m);
    const bool emit = lane < nb && !retry;
    const unsigned em = __ballot_sync(0xffffffffu, emit);
    const int slot_q = __popc(em & ((1u << lane) - 1u));
    // stencils of the list entries: one pass over the stored records
    float4 sa[K];
    float sb[K];
#pragma unroll
    for (int q = 0; q < K; q++) { sa[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f); sb[q] = 0.0f; }
    if (emit) {
        unsigned found = 0u;
        for (int q2 = 0; q2 < m.n && found != (1u << lst.size) - 1u; q2++) {
            const float4 *c = reinterpret_cast<const float4 *>(&bt->cand[q2][lane]);
            const float4 h0 = c[0];
            const int code = __float_as_int(h0.y) & 0x3fff;
#pragma unroll
            for (int q = 0; q < K; q++) {
                if (q < lst.size && !((found >> q) & 1u) && code == ((lst.li[q] << 7) | lst.lj[q])) {
                    const float4 h1 = c[1];
                    sa[q] = make_float4(h0.z, h0.w, h1.x, h1.y);  // c0, yu, yd, xl
                    sb[q] = h1.z;                                 // xr
                    found |= 1u << q;
                }
            }
        }
    }
    for (int s = 0; s < k; s++) {
        if (emit) {
            FitRec r;
            r.ia = m.ia;
            r.mn = m.mn;
            r.slot = s;
            r.npk = lst.size;
            r.pi = 0;
            r.pj = 0;
            r.pv = 0.0f;
            r.c0 = r.yu = r.yd = r.xl = r.xr = 0.0f;
            r.kind = 4;
            int idx = lst.size - 1 - s;
            if (idx >= 0) {
                float pv = 0.0f;
                int pi = 0, pj = 0;
                float4 st = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                float sx = 0.0f;
#pragma unroll
                for (int q = 0; q < K; q++)
                    if (q == idx) { pv = lst.lv[q]; pi = lst.li[q]; pj = lst.lj[q]; st = sa[q]; sx = sb[q]; }
                r.pi = pi;
                r.pj = pj;
                r.pv = pv;
                if (!job.subpix) {
                    r.kind = 3;
                } else if (pi == 0 && pj == 0) {
                    r.kind = 1;
                } else if (pi - 1 < 0 || pi + 1 >= D || pj - 1 < 0 || pj + 1 >= D) {
                    r.kind = 2;
                } else {
                    r.kind = 0;
                    r.c0 = st.x;
                    r.yu = st.y;
                    r.yd = st.z;
                    r.xl = st.w;
                    r.xr = sx;
                }
            }
            fitq[slot_q] = r;
        }
        fit_flush<D, PP>(fitq, fitv, __popc(em), lane, job);
    }
    if (lane < nb && retry) {
        const int at = atomicAdd(job.mp_retry, 1);
        job.mp_retry[1 + at] = (int)m.ia;
    }
    __syncwarp();
}

// Out of line: it runs once per 32 IAs, and inlined it made every K1 pass slower (headline 875 ->
// 852 frame-pairs/s).
template <int D, bool PP>
__device__ __noinline__ void mp_batch_run(const MpBatch *bt, int nb, int lane, const IaJob &job, FitRec *fitq,
                                          const float *fitv) {
    switch (job.num_peaks) {
        case 1: mp_batch_run_k<D, 1, PP>(bt, nb, lane, job, fitq, fitv); break;
        case 2: mp_batch_run_k<D, 2, PP>(bt, nb, lane, job, fitq, fitv); break;
        case 3: mp_batch_run_k<D, 3, PP>(bt, nb, lane, job, fitq, fitv); break;
        default: mp_batch_run_k<D, 4, PP>(bt, nb, lane, job, fitq, fitv); break;
    }
}

// Step 5' in batched mode for one IA: every thread of the group stages the cell records (as
// multipeak_core), then warp 0 stores the reachable ones as entry b of the batch.  Inlined into
// every kernel: a call per IA saved registers around it and cost the IA-32 / IA-64 kernels 4-5 %
// in both single- and multi-peak passes (IA 64 multi-peak 18.43 -> 17.54 ms, single-peak
// 16.83 -> 16.06 ms on the headline frames).
template <int D, int T, typename Plane>
__device__ __forceinline__ void multipeak_stage(const IaJob &job, long ia, float minf, const Plane &P, void *stage,
                                                uint64_t *red, MpBatch *bt, int b) {
    constexpr int NWARPS = T / 32;
    const int lane = threadIdx.x & 31, warp = T == 32 ? 0 : (int)(threadIdx.x >> 5);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) minf = fminf(minf, __shfl_xor_sync(0xffffffffu, minf, o));
    group_sync<T>();
    float *redf = reinterpret_cast<float *>(red);
    if (lane == 0) redf[warp] = minf;
    const MpGeom gm = mp_geom(D, job.peak_kernel);
    float *recv = reinterpret_cast<float *>(stage);
    int *recp = reinterpret_cast<int *>(recv + gm.nrec);
    float *chmax = reinterpret_cast<float *>(recp + gm.nrec);
    if (gm.kw == 3) {
        mp_cells<D, T, 3>(gm, P, recv, recp, chmax);
    } else {
        mp_cells<D, T, 0>(gm, P, recv, recp, chmax);
    }
    group_sync<T>();
    if (warp == 0) {
        float mn = lane < NWARPS ? redf[lane] : 3.402823466e38f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mp_extract<D>(gm, P, recv, recp, chmax, lane, ia, mn, bt, b);
    }
}

// Step 5' of xcorr_kernel for one IA, per-IA list replay: the plane is in the column-pair regions,
// the records go to the FFT scratch, `multi` fit records are queued at fitq[qn..).  Called by every
// thread of the CTA.  Inlined: as a call it cost the IA-64 kernel 3 % (single-peak 16.05 -> 15.64
// ms with it inlined, batched multi-peak 17.52 -> 16.94 ms), the IA-32 kernel nothing.
template <int N>
__device__ __forceinline__ void multipeak_select(const IaJob &job, long ia, float minf, const float *regf, cplx *scr,
                                              uint64_t *red, FitRec *fitq, float *fitv, int qn, float *mp_lv,
                                              int *mp_li, int *mp_lj) {
    using S = XcorrShape<N>;
    constexpr int RP = S::RP;
    auto P = [&](int i, int j) -> float { return regf[2 * ((j >> 1) * RP + S::rslot(i)) + (j & 1)]; };
    multipeak_core<S::D, S::T>(job, ia, minf, P, scr, red, fitq, fitv, qn, mp_lv, mp_li, mp_lj);
}

// PP: the P-point sub-pixel interpolators are compiled in (their out-of-line double-precision
// fits cost the common instantiation registers even when unused).
// Shared memory of one group of the CTA kernel (the T threads that work on one IA): twiddles,
// column-pair regions, exchange buffers, reduction words, fit queue, multi-peak list, P-point
// stencils (2 P floats per queued fit at the end).
template <int N>
struct CtaSmem {
    cplx *tw, *reg, *scr;
    uint64_t *red;
    FitRec *fitq;
    float *mp_lv;
    int *mp_li, *mp_lj;
    float *fitv;
};
template <int N>
__device__ __forceinline__ CtaSmem<N> cta_smem(unsigned char *base) {
    using S = XcorrShape<N>;
    CtaSmem<N> sm;
    sm.tw = reinterpret_cast<cplx *>(base);
    sm.reg = sm.tw + S::M;                                      // N regions of RP complex
    sm.scr = sm.reg + N * S::RP;                                // NG exchange buffers of SP complex
    sm.red = reinterpret_cast<uint64_t *>(sm.scr + S::NG * S::SP);  // 64 words
    sm.fitq = reinterpret_cast<FitRec *>(sm.red + 64);          // 32 queued fits
    sm.mp_lv = reinterpret_cast<float *>(sm.fitq + 32);         // multi-peak list (ascending)
    sm.mp_li = reinterpret_cast<int *>(sm.mp_lv + QLPIV_MAX_PEAKS + 1);
    sm.mp_lj = sm.mp_li + QLPIV_MAX_PEAKS + 1;
    sm.fitv = reinterpret_cast<float *>(sm.mp_lj + QLPIV_MAX_PEAKS + 1);
    return sm;
}

// Barrier of a group of T threads: the whole CTA (NAMED false) or named barrier `bar` (the
// persistent mixed-size kernel runs two 256-thread groups per CTA).
template <int T, bool NAMED>
__device__ __forceinline__ void bar_sync(int bar) {
    if constexpr (NAMED) asm volatile("bar.sync %0, %1;" ::"r"(bar), "n"(T) : "memory");
    else __syncthreads();
}

// Steps 1-5 of the CTA kernel for IA `ia` by the T threads of one group (tid = 0..T-1): the fit
// records are queued at fitq[qn..) and flushed by the group's warp 0 every 32 (or, batched
// multi-peak, staged as entry nb of mpb).  Multi-peak modes need the whole CTA (NAMED false).
template <int N, typename Pix, bool PP, bool NAMED>
__device__ __forceinline__ void xcorr_cta_ia(const IaJob &job, long ia, const CtaSmem<N> &sm, int tid, int bar,
                                             int &qn, MpBatch *mpb, int &nb) {
    using S = XcorrShape<N>;
    constexpr int M = S::M, D = S::D, G = S::G, NG = S::NG, ROUNDS = S::ROUNDS, RP = S::RP, T = S::T;
    constexpr int L = S::L;
    cplx *const tw = sm.tw;
    cplx *const reg = sm.reg;
    cplx *const scr = sm.scr;
    cplx *const xb = scr + (tid / G) * S::SP;  // this group's exchange buffer
    uint64_t *const red = sm.red;
    FitRec *const fitq = sm.fitq;
    float *const fitv = sm.fitv;
    float *const mp_lv = sm.mp_lv;
    int *const mp_li = sm.mp_li;
    int *const mp_lj = sm.mp_lj;
    const int multi = NAMED ? 0 : job.num_peaks;  // 0: FindMaximumFromCenter
    const int KQ = multi > 0 ? multi : 1;         // fit records per IA
    const int g = tid % G;
    const int grp = tid / G;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    constexpr int NWARPS = T / 32;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    const int gbase = lane & ~(G - 1);
    const Pix *imgA, *imgB;
    long pitch_a, pitch_b;
    int img_h, img_w;
    if (job.frames != nullptr) {
        const int fi = job.frame_idx[ia];
        const qlpiv_frame fr = (unsigned)fi < (unsigned)job.num_frames ? job.frames[fi] : qlpiv_frame{};
        imgA = reinterpret_cast<const Pix *>(fr.img_a);
        imgB = reinterpret_cast<const Pix *>(fr.img_b);
        pitch_a = pitch_b = (long)fr.pitch;
        img_h = fr.height;
        img_w = fr.width;
    } else {
        imgA = reinterpret_cast<const Pix *>(job.img_a);
        imgB = reinterpret_cast<const Pix *>(job.img_b);
        pitch_a = job.pitch_a;
        pitch_b = job.pitch_b;
        img_h = job.h;
        img_w = job.w;
    }
    int at, al, bt, bl;
    if (job.a_top != nullptr) {
        at = job.a_top[ia]; al = job.a_left[ia];
        bt = job.b_top[ia]; bl = job.b_left[ia];
    } else {  // contiguous tiles: tile ia is rows [ia*N, ia*N + N) of an N-wide image
        at = bt = (int)(ia * N);
        al = bl = 0;
    }

    // ---- 1. raw tile pixels for this thread's row transforms ----
    float ra[ROUNDS][4], rb[ROUNDS][4];
    float mxa = 0.0f, mxb = 0.0f;
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int n1 = S::task_row(grp, r);
#pragma unroll
        for (int m = 0; m < 4; m++) {
            const int n2 = g + G * m;
            ra[r][m] = load_pix(imgA, pitch_a, img_h, img_w, at + (N - 1 - n1), al + (N - 1 - n2));
            rb[r][m] = load_pix(imgB, pitch_b, img_h, img_w, bt + n1, bl + n2);
            mxa = fmaxf(mxa, ra[r][m]);
            mxb = fmaxf(mxb, rb[r][m]);
        }
    }
    float maxA, maxB;
    if (job.max_mode == QLPIV_MAX_COMPUTE || job.max_mode == QLPIV_MAX_FIXED_A ||
        job.max_mode == QLPIV_MAX_FIXED_B) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mxa = fmaxf(mxa, __shfl_xor_sync(0xffffffffu, mxa, o));
            mxb = fmaxf(mxb, __shfl_xor_sync(0xffffffffu, mxb, o));
        }
        float *redf = reinterpret_cast<float *>(red);
        if (lane == 0) { redf[warp] = mxa; redf[32 + warp] = mxb; }
        bar_sync<T, NAMED>(bar);
        mxa = 0.0f; mxb = 0.0f;
#pragma unroll
        for (int k = 0; k < NWARPS; k++) { mxa = fmaxf(mxa, redf[k]); mxb = fmaxf(mxb, redf[32 + k]); }
        maxA = job.max_mode == QLPIV_MAX_FIXED_A ? job.fixed_max_a : fmaxf(mxa, 16.0f);
        maxB = job.max_mode == QLPIV_MAX_FIXED_B ? job.fixed_max_b : fmaxf(mxb, 16.0f);
    } else if (job.max_mode == QLPIV_MAX_GIVEN) {
        maxA = job.max_a[ia];
        maxB = job.max_b[ia];
    } else {
        maxA = job.fixed_max_a;
        maxB = job.fixed_max_b;
    }
    if (job.norm_mode == QLPIV_NORM_MAX_A) maxB = maxA;
    const bool normalize = job.norm_mode != QLPIV_NORM_NONE;

    // ---- 2. row pass ----
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int n1 = S::task_row(grp, r);
        cplx v[8];
#pragma unroll
        for (int m = 0; m < 4; m++) {
            float a = ra[r][m], b = rb[r][m];
            if (normalize) {
                // (v / max) * 16 + 1 with IEEE single operations, as in Java
                a = __fadd_rn(__fmul_rn(__fdiv_rn(a, maxA), 16.0f), 1.0f);
                b = __fadd_rn(__fmul_rn(__fdiv_rn(b, maxB), 16.0f), 1.0f);
            }
            v[m] = {a, b};
            v[m + 4] = {0.0f, 0.0f};
        }
        fft_group<M, false, L>(v, g, xb, tw);
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const int k2 = g + G * m;
            int region, slot;
            if (k2 == 0) { region = 0; slot = n1; }
            else if (k2 == N) { region = 0; slot = N + n1; }
            else if (k2 < N) { region = k2; slot = n1; }
            else { region = M - k2; slot = N + n1; }
            reg[region * RP + S::rslot(slot)] = v[m];
        }
    }
    bar_sync<T, NAMED>(bar);

    // ---- 3. column tasks ----
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int c = S::task_row(grp, r);
        cplx *rg = reg + c * RP;
        cplx z1[8], z2[8];
#pragma unroll
        for (int m = 0; m < 4; m++) {
            z1[m] = rg[S::rslot(g + G * m)];
            z2[m] = rg[S::rslot(N + g + G * m)];
            z1[m + 4] = {0.0f, 0.0f};
            z2[m + 4] = {0.0f, 0.0f};
        }
        fft_group<M, false, L>(z1, g, xb, tw);
        fft_group<M, false, L>(z2, g, xb, tw);
        // P(k1) = F*G/M^2, F = (Z1 + conj Zm)/2, G = (Z1 - conj Zm)/(2i), where Zm is the
        // mirror element Z(M-k1, M-c): held by lane (G-g)%G at m' = 7-m (g>0) or (8-m)%8.
        const int src = gbase + ((G - g) & (G - 1));
        const float scale = 0.5f * 0.5f / (float)(M * M);
        cplx p[8];
#pragma unroll
        for (int m = 0; m < 8; m++) {
            // c == 0: both columns are self-mirrored; otherwise the mirror is in z2
            const cplx s2 = (g == 0) ? z2[(8 - m) & 7] : z2[7 - m];
            const cplx s1 = (g == 0) ? z1[(8 - m) & 7] : z1[7 - m];
            cplx snd = (c == 0) ? s1 : s2;
            cplx zm;
            zm.x = __shfl_sync(0xffffffffu, snd.x, src);
            zm.y = __shfl_sync(0xffffffffu, snd.y, src);
            const cplx a = z1[m];
            // F*2 = (a.x + zm.x, a.y - zm.y);  G*2 = (a.y + zm.y, -(a.x - zm.x))
            const float fr = a.x + zm.x, fi = a.y - zm.y;
            const float gr = a.y + zm.y, gi = zm.x - a.x;
            p[m] = {(fr * gr - fi * gi) * scale, (fr * gi + fi * gr) * scale};
        }
        if (c == 0) {
            // second self-mirrored column (k2 = N): P_N packed as the imaginary part
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const cplx snd = (g == 0) ? z2[(8 - m) & 7] : z2[7 - m];
                cplx zm;
                zm.x = __shfl_sync(gmask, snd.x, src);
                zm.y = __shfl_sync(gmask, snd.y, src);
                const cplx a = z2[m];
                const float fr = a.x + zm.x, fi = a.y - zm.y;
                const float gr = a.y + zm.y, gi = zm.x - a.x;
                const cplx pn = {(fr * gr - fi * gi) * scale, (fr * gi + fi * gr) * scale};
                p[m] = {p[m].x - pn.y, p[m].y + pn.x};  // P0 + i * PN
            }
        }
        fft_group<M, true, L>(p, g, xb, tw);
#pragma unroll
        for (int m = 0; m < 8; m++) rg[S::rslot(g + G * m)] = p[m];
    }
    bar_sync<T, NAMED>(bar);

    // ---- 4. row-pair pass + per-lane peak scoring ----
    uint64_t best = 0ull;
    uint32_t best_ij = 0u;
    float minf = 3.402823466e38f;
    float *regf = reinterpret_cast<float *>(reg);
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int pr = S::task_pair(grp, r);
        const int ra_ = 2 * pr, rb_ = 2 * pr + 1;
        cplx y[8];
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const int k2 = g + G * m;
            if (k2 == 0 || k2 == N) {
                const cplx qa = reg[S::rslot(ra_)], qb = reg[S::rslot(rb_)];
                y[m] = (k2 == 0) ? cplx{qa.x, qb.x} : cplx{qa.y, qb.y};
            } else if (k2 < N) {
                const cplx qa = reg[k2 * RP + S::rslot(ra_)], qb = reg[k2 * RP + S::rslot(rb_)];
                y[m] = {qa.x - qb.y, qa.y + qb.x};
            } else {
                const int cc = M - k2;
                const cplx qa = reg[cc * RP + S::rslot(ra_)], qb = reg[cc * RP + S::rslot(rb_)];
                y[m] = {qa.x + qb.y, qb.x - qa.y};
            }
        }
        fft_group<M, true, L>(y, g, xb, tw);
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const int n2 = g + G * m;
            // keep the plane in the row slots this pair has consumed
            regf[2 * ((n2 >> 1) * RP + S::rslot(ra_)) + (n2 & 1)] = y[m].x;
            regf[2 * ((n2 >> 1) * RP + S::rslot(rb_)) + (n2 & 1)] = y[m].y;
            if (multi > 0) {
                // FindMaximumMultiPeaks visits every cell of the (2N-1)^2 plane
                if (n2 <= M - 2) {
                    minf = fminf(minf, y[m].x);
                    if (rb_ <= M - 2) minf = fminf(minf, y[m].y);
                }
            } else if (n2 >= 1 && n2 <= M - 2) {
                if (ra_ >= 1) {
                    minf = fminf(minf, y[m].x);
                    const uint64_t k = peak_key(y[m].x, ra_, n2, N);
                    if (k > best) { best = k; best_ij = ((uint32_t)ra_ << 16) | (uint32_t)n2; }
                }
                if (rb_ <= M - 2) {
                    minf = fminf(minf, y[m].y);
                    const uint64_t k = peak_key(y[m].y, rb_, n2, N);
                    if (k > best) { best = k; best_ij = ((uint32_t)rb_ << 16) | (uint32_t)n2; }
                }
            }
            if (job.planes != nullptr && n2 < D) {
                float *pl = job.planes + ia * (long)(D * D);
                pl[ra_ * D + n2] = y[m].x;
                if (rb_ < D) pl[rb_ * D + n2] = y[m].y;
            }
        }
    }

    // ---- 5. CTA reduction; the fit is queued and run 32 IAs at a time ----
    auto P = [&](int i, int j) -> float { return regf[2 * ((j >> 1) * RP + S::rslot(i)) + (j & 1)]; };
    if (multi == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t ok = __shfl_xor_sync(0xffffffffu, best, o);
            const uint32_t oij = __shfl_xor_sync(0xffffffffu, best_ij, o);
            if (ok > best) { best = ok; best_ij = oij; }
            minf = fminf(minf, __shfl_xor_sync(0xffffffffu, minf, o));
        }
        bar_sync<T, NAMED>(bar);  // red[] reuse after the max reduction
        if (lane == 0) {
            red[warp] = best;
            red[32 + warp] = ((uint64_t)best_ij << 32) | (uint64_t)__float_as_uint(minf);
        }
        bar_sync<T, NAMED>(bar);
        if (warp == 0) {
            uint64_t bk = 0ull;
            uint32_t bij = 0u;
            float mn = 3.402823466e38f;
            if (lane < NWARPS) {
                bk = red[lane];
                bij = (uint32_t)(red[32 + lane] >> 32);
                mn = __uint_as_float((uint32_t)red[32 + lane]);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const uint64_t ok = __shfl_xor_sync(0xffffffffu, bk, o);
                const uint32_t oij = __shfl_xor_sync(0xffffffffu, bij, o);
                // ties on the full key cannot occur between distinct cells (the rank is unique)
                if (ok > bk) { bk = ok; bij = oij; }
                mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            }
            if (lane == 0) {
                FitRec r;
                r.ia = ia;
                r.mn = mn;
                r.pi = 0;
                r.pj = 0;
                r.pv = 0.0f;
                if (bk != 0ull) {
                    r.pi = (int)(bij >> 16);
                    r.pj = (int)(bij & 0xffffu);
                    r.pv = __uint_as_float((uint32_t)(bk >> 32));
                }
                r.slot = 0;
                r.npk = 1;
                fit_stencil<D>(r, job, P, fitv + qn * 2 * job.subpix_pixels);
                fitq[qn] = r;
            }
        }
    } else if (mpb == nullptr) {
        multipeak_select<N>(job, ia, minf, regf, scr, red, fitq, fitv, qn, mp_lv, mp_li, mp_lj);
    } else {
        multipeak_stage<D, T>(job, ia, minf, P, scr, red, mpb, nb);
        if (++nb == kMpBatch) {
            if (warp == 0) mp_batch_run<D, PP>(mpb, nb, lane, job, fitq, fitv);
            nb = 0;
        }
    }
    if (mpb == nullptr) {
        qn += KQ;
        if (qn + KQ > 32) {
            if (warp == 0) fit_flush<D, PP>(fitq, fitv, qn, lane, job);
            qn = 0;
        }
    }
    bar_sync<T, NAMED>(bar);  // regions are rewritten by the next IA
}

template <int N, typename Pix, bool PP>
__global__ void __launch_bounds__(XcorrShape<N>::T, XcorrShape<N>::MIN_BLOCKS)
xcorr_kernel(IaJob job) {
    using S = XcorrShape<N>;
    constexpr int T = S::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const CtaSmem<N> sm = cta_smem<N>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int D = S::D;
    FitRec *const fitq = sm.fitq;
    float *const fitv = sm.fitv;
    int qn = 0;  // uniform across the CTA
    const int multi = job.num_peaks;

    for (int e = tid; e < S::M; e += T) sm.tw[e] = job.twiddles[e];
    __syncthreads();

    // batched multi-peak replay: a batch claimed for this CTA (filled and replayed by warp 0) and
    // its fill (CTA-uniform)
    __shared__ int s_slot;
    MpBatch *mpb = nullptr;
    if (multi > 0 && mp_batched(job)) {
        if (tid == 0) s_slot = mp_claim(job.mp_slots, job.mp_batch_units, (int)(blockIdx.x % 1024u));
        __syncthreads();
        if (s_slot >= 0) mpb = job.mp_batch + s_slot;
    }
    int nb = 0;
    const long count = job.ia_list != nullptr ? (long)job.ia_list[0] : job.count;
    for (long k = blockIdx.x; k < count; k += gridDim.x) {
        const long ia = job.ia_list != nullptr ? (long)job.ia_list[1 + k] : k;
        xcorr_cta_ia<N, Pix, PP, false>(job, ia, sm, tid, 0, qn, mpb, nb);
    }
    if (qn > 0 && warp == 0) fit_flush<D, PP>(fitq, fitv, qn, lane, job);
    if (mpb != nullptr) {
        if (nb > 0 && warp == 0) mp_batch_run<D, PP>(mpb, nb, lane, job, fitq, fitv);
        __syncthreads();
        if (tid == 0) mp_release(job.mp_slots, s_slot);
    }
}

}  // namespace qlpiv
