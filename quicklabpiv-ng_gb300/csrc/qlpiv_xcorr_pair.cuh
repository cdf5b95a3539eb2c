// K1 for IA side 128: one thread-block cluster of two CTAs per interrogation area.
//
// The 256 x 256 spectrum of an IA pair needs 128 column-pair regions of 289 complex (296 KB),
// more than one SM's shared memory, so the two CTAs of a cluster share the IA, split by the
// parity of the column frequency (region c pairs columns c and 256 - c, which have the same
// parity; region 0 pairs columns 0 and 128).  CTA q owns the regions of parity q, and every
// phase but the last runs on its own shared memory:
//
//   1. tile maxima: both CTAs read both whole tiles (no exchange);
//   2. row pass: the odd / even frequencies of a 256-point transform whose upper half is zero
//      are the 128-point transform of z[n] (q = 0) or of z[n] w256^n (q = 1), so CTA q
//      transforms all 128 rows for its parity and writes them into its own regions;
//   3. column tasks on its own 64 regions (as in K1: forward columns c and 256 - c, product,
//      inverse column transform);
//   4. row pairs: the packed inverse row transform of a row pair splits the same way,
//      y[n] = E[n mod 128] + w256^-n O[n mod 128] with E / O the 128-point inverse transforms of
//      the even / odd frequencies: CTA q computes its partial (E or O) for all 128 row pairs,
//      in place in the slots the pair consumed;
//   5. after one cluster barrier CTA q combines the partials of row pairs [64q, 64q + 64),
//      reading the peer's through distributed shared memory (64 KB per CTA per IA), and scores
//      the peak; rank 1 hands its candidate to rank 0, which recomputes the stencil values from
//      the partials and queues the fit.
//
// Reference semantics are K1's (qlpiv_xcorr.cuh): normalisation, Hermitian split and product,
// FindMaximumFromCenter order and the sub-pixel interpolators.  FindMaximumMultiPeaks needs the
// whole plane: in that mode the combine writes the plane to a per-cluster scratch in global memory
// (L2-resident, 254 KB) and rank 0 runs K1's multi-peak search over it (pair_multipeak).
#pragma once
#include <cooperative_groups.h>

#include "qlpiv_xcorr.cuh"

namespace qlpiv {

struct PairShape {
    static constexpr int N = 128, M = 256, D = 255;
    static constexpr int NR = 64;                // regions per CTA
    static constexpr int RP = M + M / 8 + 1;     // region pitch (complex), odd
    static constexpr int T = 768;                // 24 warps: 32 groups do not divide the phases
    static constexpr int G1 = 16, NG1 = T / G1;  // 128-point transforms: 16 lanes, 32 groups
    static constexpr int G2 = 32, NG2 = T / G2;  // 256-point column transforms: a warp each
    static constexpr int RP1 = 128 + 16 + 1;     // scratch pitch of a 128-point transform
    static constexpr size_t SMEM = sizeof(cplx) * (size_t)(M + M / 2 + NR * RP + NG1 * RP1) +
                                   64 * sizeof(uint64_t) + 32 * sizeof(FitRec) + 256 /* multi-peak list */;
    // the FFT exchanges use layout 1 (qlpiv_fft.cuh): the 256-point column transforms exchange in
    // their region, the 128-point row transforms in their scratch
    static_assert(xbuf_size<M, 1>() <= RP && xbuf_size<M / 2, 1>() <= RP1, "exchange buffers too small");
};

__device__ __forceinline__ uint32_t cluster_addr(const void *p, unsigned rank) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}

__device__ __forceinline__ cplx cluster_ld(uint32_t addr) {
    cplx v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

__device__ __forceinline__ void cluster_st_u64(uint32_t addr, uint64_t v) {
    asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}

// y[n] and y[n + 128] of a row pair from the even-frequency partial E, the odd one O and
// w = w256^-n (n < 128): E + w O and E - w O, with rounded single operations (the peak search
// and the fit stencil evaluate the same expression and must agree bit for bit).
__device__ __forceinline__ void pair_combine(cplx e, cplx o, cplx w, cplx &lo, cplx &hi) {
    const float tx = __fsub_rn(__fmul_rn(w.x, o.x), __fmul_rn(w.y, o.y));
    const float ty = __fadd_rn(__fmul_rn(w.x, o.y), __fmul_rn(w.y, o.x));
    lo = {__fadd_rn(e.x, tx), __fadd_rn(e.y, ty)};
    hi = {__fsub_rn(e.x, tx), __fsub_rn(e.y, ty)};
}

// Slot of partial element n' of row pair p: region n' / 2, slot 2p + n' % 2.
__device__ __forceinline__ int pair_slot(int p, int np) {
    return (np >> 1) * PairShape::RP + pad8(2 * p + (np & 1));
}

// Multi-peak mode of step 5 (out of line; inlined it measured the same on single-peak passes).
// Both CTAs have written their row pairs of the plane to the cluster's global scratch `mp`; rank 1
// hands its min floor to rank 0, and rank 0 runs FindMaximumMultiPeaks over the plane (L2 reads),
// staging the cell records in its regions (the partials are no longer needed) and queueing one fit
// per peak.  Called by every thread of both CTAs.
static __device__ __noinline__ void pair_multipeak(const IaJob &job, long ia, float minf, const float *mp, cplx *reg,
                                                   uint64_t *red, FitRec *fitq, float *fitv, int qn, float *mp_lv,
                                                   int *mp_li, int *mp_lj, int q, uint32_t xch0) {
    constexpr int D = PairShape::D, T = PairShape::T, NWARPS = T / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) minf = fminf(minf, __shfl_xor_sync(0xffffffffu, minf, o));
    float *redf = reinterpret_cast<float *>(red);
    __syncthreads();
    if (lane == 0) redf[warp] = minf;
    __syncthreads();
    if (q == 1 && tid == 0) {
        float m = redf[0];
        for (int k = 1; k < NWARPS; k++) m = fminf(m, redf[k]);
        cluster_st_u64(xch0 + 16u, (uint64_t)__float_as_uint(m));
    }
    __threadfence();  // the plane rows written to global memory, before the barrier
    cooperative_groups::this_cluster().sync();
    if (q == 0) {
        if (tid == 0) minf = fminf(minf, __uint_as_float((uint32_t)red[62]));
        auto P = [&](int i, int j) -> float { return __ldcg(mp + i * D + j); };
        multipeak_core<D, T>(job, ia, minf, P, reg, red, fitq, fitv, qn, mp_lv, mp_li, mp_lj);
    }
}

template <typename Pix, bool PP>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(PairShape::T, 1) xcorr_pair_kernel(IaJob job) {
    using S = PairShape;
    constexpr int N = S::N, M = S::M, D = S::D, RP = S::RP, T = S::T, G1 = S::G1, NG1 = S::NG1, G2 = S::G2,
                  NG2 = S::NG2, RP1 = S::RP1;
    constexpr int NWARPS = T / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx *tw = reinterpret_cast<cplx *>(smem_raw);  // w256^e, e < 256
    cplx *tw1 = tw + M;                              // w128^e = w256^2e, e < 128
    cplx *reg = tw1 + M / 2;                         // 64 regions of this CTA's parity
    cplx *scr = reg + S::NR * RP;                    // 32 scratch buffers of the 128-point transforms
    uint64_t *red = reinterpret_cast<uint64_t *>(scr + NG1 * RP1);  // 64 words
    FitRec *fitq = reinterpret_cast<FitRec *>(red + 64);           // 32 queued fits
    float *mp_lv = reinterpret_cast<float *>(fitq + 32);           // multi-peak list (ascending)
    int *mp_li = reinterpret_cast<int *>(mp_lv + QLPIV_MAX_PEAKS + 1);
    int *mp_lj = mp_li + QLPIV_MAX_PEAKS + 1;
    float *fitv = reinterpret_cast<float *>(mp_lj + QLPIV_MAX_PEAKS + 1);  // P-point stencils
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    const int q = (int)cl.block_rank();
    const uint32_t peer_reg = cluster_addr(reg, (unsigned)(q ^ 1));
    const uint32_t xch0 = cluster_addr(red + 60, 0u);  // rank 0's exchange words red[60..62]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g1 = tid % G1, grp1 = tid / G1;
    const int g2 = lane, grp2 = warp;
    int qn = 0;
    const int multi = job.num_peaks;  // 0: FindMaximumFromCenter; k: FindMaximumMultiPeaks
    const int KQ = multi > 0 ? multi : 1;

    for (int e = tid; e < M; e += T) tw[e] = job.twiddles[e];
    for (int e = tid; e < M / 2; e += T) tw1[e] = job.twiddles[2 * e];
    __syncthreads();
    cl.sync();  // both CTAs are running before any distributed shared memory access

    const long count = job.ia_list != nullptr ? (long)job.ia_list[0] : job.count;
    for (long k = blockIdx.x / 2; k < count; k += gridDim.x / 2) {
        const long ia = job.ia_list != nullptr ? (long)job.ia_list[1 + k] : k;
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
        } else {
            at = bt = (int)(ia * N);
            al = bl = 0;
        }

        // ---- 1. tile maxima (each CTA reads both whole tiles) ----
        float maxA, maxB;
        if (job.max_mode == QLPIV_MAX_COMPUTE || job.max_mode == QLPIV_MAX_FIXED_A ||
            job.max_mode == QLPIV_MAX_FIXED_B) {
            float mxa = 0.0f, mxb = 0.0f;
            for (int k = tid; k < N * N; k += T) {
                const int y = k / N, x = k % N;
                mxa = fmaxf(mxa, load_pix(imgA, pitch_a, img_h, img_w, at + y, al + x));
                mxb = fmaxf(mxb, load_pix(imgB, pitch_b, img_h, img_w, bt + y, bl + x));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                mxa = fmaxf(mxa, __shfl_xor_sync(0xffffffffu, mxa, o));
                mxb = fmaxf(mxb, __shfl_xor_sync(0xffffffffu, mxb, o));
            }
            float *redf = reinterpret_cast<float *>(red);
            if (lane == 0) { redf[warp] = mxa; redf[32 + warp] = mxb; }
            __syncthreads();
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

        // ---- 2. row pass: frequencies of parity q of every row ----
#pragma unroll 1
        for (int r = 0; r < (N + NG1 - 1) / NG1; r++) {
            const int n1 = grp1 + NG1 * r;
            if (n1 >= N) break;  // whole warps (N - NG1 * r is even)
            cplx v[8];
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int n2 = g1 + G1 * m;
                float a = load_pix(imgA, pitch_a, img_h, img_w, at + (N - 1 - n1), al + (N - 1 - n2));
                float b = load_pix(imgB, pitch_b, img_h, img_w, bt + n1, bl + n2);
                if (normalize) {
                    // (v / max) * 16 + 1 with IEEE single operations, as in Java
                    a = __fadd_rn(__fmul_rn(__fdiv_rn(a, maxA), 16.0f), 1.0f);
                    b = __fadd_rn(__fmul_rn(__fdiv_rn(b, maxB), 16.0f), 1.0f);
                }
                v[m] = q ? cmul(cplx{a, b}, tw[n2]) : cplx{a, b};
            }
            fft_group<M / 2, false, 1>(v, g1, scr + grp1 * RP1, tw1);
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int k2 = 2 * (g1 + G1 * m) + q;
                int c, slot;
                if (k2 == 0) { c = 0; slot = n1; }
                else if (k2 == N) { c = 0; slot = N + n1; }
                else if (k2 < N) { c = k2; slot = n1; }
                else { c = M - k2; slot = N + n1; }
                reg[(c >> 1) * RP + pad8(slot)] = v[m];
            }
        }
        __syncthreads();

        // ---- 3. column tasks on this CTA's regions (as in K1) ----
#pragma unroll 1
        for (int r = 0; r < (S::NR + NG2 - 1) / NG2; r++) {
            const int lc = grp2 + NG2 * r;
            if (lc >= S::NR) break;  // one warp per region
            const int c = 2 * lc + q;
            cplx *rg = reg + lc * RP;
            cplx z1[8], z2[8];
#pragma unroll
            for (int m = 0; m < 4; m++) {
                z1[m] = rg[pad8(g2 + G2 * m)];
                z2[m] = rg[pad8(N + g2 + G2 * m)];
                z1[m + 4] = {0.0f, 0.0f};
                z2[m + 4] = {0.0f, 0.0f};
            }
            __syncwarp();
            fft_group<M, false, 1>(z1, g2, rg, tw);
            fft_group<M, false, 1>(z2, g2, rg, tw);
            const int src = (G2 - g2) & (G2 - 1);
            const float scale = 0.5f * 0.5f / (float)(M * M);
            cplx p[8];
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const cplx s2 = (g2 == 0) ? z2[(8 - m) & 7] : z2[7 - m];
                const cplx s1 = (g2 == 0) ? z1[(8 - m) & 7] : z1[7 - m];
                const cplx snd = (c == 0) ? s1 : s2;
                cplx zm;
                zm.x = __shfl_sync(0xffffffffu, snd.x, src);
                zm.y = __shfl_sync(0xffffffffu, snd.y, src);
                const cplx a = z1[m];
                const float fr = a.x + zm.x, fi = a.y - zm.y;
                const float gr = a.y + zm.y, gi = zm.x - a.x;
                p[m] = {(fr * gr - fi * gi) * scale, (fr * gi + fi * gr) * scale};
            }
            if (c == 0) {
#pragma unroll
                for (int m = 0; m < 8; m++) {
                    const cplx snd = (g2 == 0) ? z2[(8 - m) & 7] : z2[7 - m];
                    cplx zm;
                    zm.x = __shfl_sync(0xffffffffu, snd.x, src);
                    zm.y = __shfl_sync(0xffffffffu, snd.y, src);
                    const cplx a = z2[m];
                    const float fr = a.x + zm.x, fi = a.y - zm.y;
                    const float gr = a.y + zm.y, gi = zm.x - a.x;
                    const cplx pn = {(fr * gr - fi * gi) * scale, (fr * gi + fi * gr) * scale};
                    p[m] = {p[m].x - pn.y, p[m].y + pn.x};
                }
            }
            fft_group<M, true, 1>(p, g2, rg, tw);
            __syncwarp();
#pragma unroll
            for (int m = 0; m < 8; m++) rg[pad8(g2 + G2 * m)] = p[m];
        }
        __syncthreads();

        // ---- 4. partial inverse row-pair transforms (frequencies of parity q), in place ----
#pragma unroll 1
        for (int r = 0; r < (M / 2 + NG1 - 1) / NG1; r++) {
            const int pr = grp1 + NG1 * r;
            if (pr >= M / 2) break;
            const int ra_ = 2 * pr, rb_ = 2 * pr + 1;
            cplx y[8];
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int k2 = 2 * (g1 + G1 * m) + q;
                if (k2 == 0 || k2 == N) {
                    const cplx qa = reg[pad8(ra_)], qb = reg[pad8(rb_)];
                    y[m] = (k2 == 0) ? cplx{qa.x, qb.x} : cplx{qa.y, qb.y};
                } else if (k2 < N) {
                    const cplx *rk = reg + (k2 >> 1) * RP;
                    const cplx qa = rk[pad8(ra_)], qb = rk[pad8(rb_)];
                    y[m] = {qa.x - qb.y, qa.y + qb.x};
                } else {
                    const cplx *rk = reg + ((M - k2) >> 1) * RP;
                    const cplx qa = rk[pad8(ra_)], qb = rk[pad8(rb_)];
                    y[m] = {qa.x + qb.y, qb.x - qa.y};
                }
            }
            fft_group<M / 2, true, 1>(y, g1, scr + grp1 * RP1, tw1);
            __syncwarp();
#pragma unroll
            for (int m = 0; m < 8; m++) reg[pair_slot(pr, g1 + G1 * m)] = y[m];
        }
        cl.sync();  // both parities' partials are complete

        // ---- 5. combine row pairs [64q, 64q + 64) and score the peak ----
        // (multi-peak mode: write the plane to this cluster's global scratch instead)
        float *mp = multi > 0 ? job.mp_planes + (long)(blockIdx.x / 2) * (D * D) : nullptr;
        uint64_t best = 0ull;
        uint32_t best_ij = 0u;
        float minf = 3.402823466e38f;
        {
            const int np = tid & (M / 2 - 1);
            const cplx w = {tw[np].x, -tw[np].y};  // w256^-n'
#pragma unroll 4
            for (int k = 0; k < (M / 4 + T / (M / 2) - 1) / (T / (M / 2)); k++) {
                const int pl = (tid >> 7) + (T / (M / 2)) * k;  // this CTA's row pair index
                if (pl >= M / 4) break;
                const int pr = (M / 4) * q + pl;
                const int off = pair_slot(pr, np);
                const cplx own = reg[off], other = cluster_ld(peer_reg + 8u * (uint32_t)off);
                cplx ylo, yhi;
                pair_combine(q == 0 ? own : other, q == 0 ? other : own, w, ylo, yhi);
                const int ra_ = 2 * pr, rb_ = 2 * pr + 1;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int n2 = np + h * (M / 2);
                    const cplx yv = h ? yhi : ylo;
                    if (multi > 0) {
                        // FindMaximumMultiPeaks visits every cell of the (2N-1)^2 plane
                        if (n2 <= M - 2) {
                            minf = fminf(minf, yv.x);
                            if (rb_ <= M - 2) minf = fminf(minf, yv.y);
                        }
                        if (n2 < D) {
                            mp[ra_ * D + n2] = yv.x;
                            if (rb_ < D) mp[rb_ * D + n2] = yv.y;
                        }
                    } else if (n2 >= 1 && n2 <= M - 2) {
                        if (ra_ >= 1) {
                            minf = fminf(minf, yv.x);
                            const uint64_t kk = peak_key(yv.x, ra_, n2, N);
                            if (kk > best) { best = kk; best_ij = ((uint32_t)ra_ << 16) | (uint32_t)n2; }
                        }
                        if (rb_ <= M - 2) {
                            minf = fminf(minf, yv.y);
                            const uint64_t kk = peak_key(yv.y, rb_, n2, N);
                            if (kk > best) { best = kk; best_ij = ((uint32_t)rb_ << 16) | (uint32_t)n2; }
                        }
                    }
                    if (job.planes != nullptr && n2 < D) {
                        float *pl = job.planes + ia * (long)(D * D);
                        pl[ra_ * D + n2] = yv.x;
                        if (rb_ < D) pl[rb_ * D + n2] = yv.y;
                    }
                }
            }
        }
        if (multi > 0) {
            pair_multipeak(job, ia, minf, mp, reg, red, fitq, fitv, qn, mp_lv, mp_li, mp_lj, q, xch0);
        } else {
    #pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const uint64_t ok = __shfl_xor_sync(0xffffffffu, best, o);
                const uint32_t oij = __shfl_xor_sync(0xffffffffu, best_ij, o);
                if (ok > best) { best = ok; best_ij = oij; }
                minf = fminf(minf, __shfl_xor_sync(0xffffffffu, minf, o));
            }
            __syncthreads();  // red[] reuse after the max reduction
            if (lane == 0) {
                red[warp] = best;
                red[32 + warp] = ((uint64_t)best_ij << 32) | (uint64_t)__float_as_uint(minf);
            }
            __syncthreads();
            uint64_t bk = 0ull;
            uint32_t bij = 0u;
            float mn = 3.402823466e38f;
            if (warp == 0) {
                if (lane < NWARPS) {
                    bk = red[lane];
                    bij = (uint32_t)(red[32 + lane] >> 32);
                    mn = __uint_as_float((uint32_t)red[32 + lane]);
                }
    #pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const uint64_t ok = __shfl_xor_sync(0xffffffffu, bk, o);
                    const uint32_t oij = __shfl_xor_sync(0xffffffffu, bij, o);
                    if (ok > bk) { bk = ok; bij = oij; }
                    mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
                }
            }
            if (q == 1 && tid == 0) {
                cluster_st_u64(xch0, bk);
                cluster_st_u64(xch0 + 8u, ((uint64_t)bij << 32) | (uint64_t)__float_as_uint(mn));
            }
            cl.sync();  // rank 1's candidate has arrived
            if (q == 0 && tid == 0) {
                const uint64_t ok = red[60];
                const uint32_t oij = (uint32_t)(red[61] >> 32);
                if (ok > bk) { bk = ok; bij = oij; }
                mn = fminf(mn, __uint_as_float((uint32_t)red[61]));
                // plane value (i, j) recomputed from the partials: E here, O in rank 1
                auto P = [&](int i, int j) -> float {
                    const int np = j & (M / 2 - 1);
                    const int off = pair_slot(i >> 1, np);
                    const cplx w = {tw[np].x, -tw[np].y};
                    cplx ylo, yhi;
                    pair_combine(reg[off], cluster_ld(peer_reg + 8u * (uint32_t)off), w, ylo, yhi);
                    const cplx yv = (j >> 7) ? yhi : ylo;
                    return (i & 1) ? yv.y : yv.x;
                };
                FitRec rec;
                rec.ia = ia;
                rec.mn = mn;
                rec.pi = 0;
                rec.pj = 0;
                rec.pv = 0.0f;
                if (bk != 0ull) {
                    rec.pi = (int)(bij >> 16);
                    rec.pj = (int)(bij & 0xffffu);
                    rec.pv = __uint_as_float((uint32_t)(bk >> 32));
                }
                rec.slot = 0;
                rec.npk = 1;
                fit_stencil<D>(rec, job, P, fitv + qn * 2 * job.subpix_pixels);
                fitq[qn] = rec;
            }
        }
        qn += KQ;
        if (qn + KQ > 32) {
            if (warp == 0 && q == 0) fit_flush<D, PP>(fitq, fitv, qn, lane, job);
            qn = 0;
        }
        cl.sync();  // the partials are rewritten by the next IA
    }
    if (qn > 0 && warp == 0 && q == 0) fit_flush<D, PP>(fitq, fitv, qn, lane, job);
}

}  // namespace qlpiv
