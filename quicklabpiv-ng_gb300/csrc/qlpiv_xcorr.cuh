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
#pragma once
#include "qlpiv_fft.cuh"
#include "qlpiv.h"

namespace qlpiv {

template <int N>
struct XcorrShape {
    static constexpr int M = 2 * N;
    static constexpr int D = M - 1;
    static constexpr int G = N / 4;                    // lanes per transform
    static constexpr int T = N == 16 ? 64 : (N == 32 ? 256 : 512);  // threads per CTA
    static constexpr int NG = T / G;                   // concurrent transforms
    static constexpr int ROUNDS = N / NG;              // tasks per group per phase
    static constexpr int RP = M + M / 8 + 1;           // region pitch (complex), odd
    static constexpr int MIN_BLOCKS = N == 16 ? 16 : (N == 32 ? 4 : 2);
    static constexpr size_t SMEM =
        sizeof(cplx) * (size_t)(M + N * RP + NG * RP) + 64 * sizeof(uint64_t) + 32 * 48;  // + fit queue
};

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
    const int *a_top, *a_left, *b_top, *b_left;  // per IA origins
    const float *max_a, *max_b;  // per IA maxima (max_mode == QLPIV_MAX_GIVEN)
    long count;
    int norm_mode, max_mode, subpix;
    float fixed_max_a, fixed_max_b;
    qlpiv_vector *out;           // optional per-IA vectors
    float *planes;               // optional (2N-1)^2 planes per IA
    float *acc_u, *acc_v;        // optional: tile displacements += (u, v)  (Tile.accumulateDisplacement)
};

// Integer peak and 3-point stencil of one IA, queued for the sub-pixel fit.
struct FitRec {
    long ia;
    int pi, pj, kind;   // kind: 0 fit, 1 no peak, 2 stencil off the plane, 3 no sub-pixel
    float pv, mn, c0, yu, yd, xl, xr;
};

// Gaussian1DPolynomialInterpolator.interpolate (S/interpolators/Gaussian1DPolynomialInterpolator.java:25-106)
// for q[0..n): lane k handles record k, so the double logarithms of 32 IAs share one
// warp instruction.  Called by one full warp.
template <int D>
__device__ void fit_flush(const FitRec *q, int n, int lane, const IaJob &job) {
    __syncwarp();
    if (lane < n) {
        const FitRec r = q[lane];
        float si = (float)r.pi, sj = (float)r.pj;
        uint32_t flags = 0;
        if (r.kind == 1) {
            flags |= QLPIV_F_NO_PEAK;
        } else if (r.kind == 2) {
            flags |= QLPIV_F_EDGE;
        } else if (r.kind == 0) {
            const bool neg = r.c0 < 0.0f || r.yu < 0.0f || r.yd < 0.0f || r.xl < 0.0f || r.xr < 0.0f;
            const float y0 = r.yu + 1e-8f, y1 = r.c0 + 1e-8f, y2 = r.yd + 1e-8f;
            const float x0 = r.xl + 1e-8f, x1 = r.c0 + 1e-8f, x2 = r.xr + 1e-8f;
            float ti, tj;
            if (!neg) {
                const double ly0 = log((double)y0), ly1 = log((double)y1), ly2 = log((double)y2);
                const double lx0 = log((double)x0), lx1 = log((double)x1), lx2 = log((double)x2);
                const double di = __dadd_rn(__dadd_rn(__dmul_rn(2.0, ly0), -__dmul_rn(4.0, ly1)), __dmul_rn(2.0, ly2));
                const double dj = __dadd_rn(__dadd_rn(__dmul_rn(2.0, lx0), -__dmul_rn(4.0, lx1)), __dmul_rn(2.0, lx2));
                ti = __fadd_rn((float)r.pi, __fdiv_rn((float)(ly0 - ly2), (float)di));
                tj = __fadd_rn((float)r.pj, __fdiv_rn((float)(lx0 - lx2), (float)dj));
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
        o.peak_value = r.pv;
        o.min_floor = r.mn;
        o.peak_i = (int16_t)r.pi;
        o.peak_j = (int16_t)r.pj;
        o.flags = flags;
        if (job.out != nullptr) job.out[r.ia] = o;
        if (job.acc_u != nullptr) {
            job.acc_u[r.ia] += o.u;
            job.acc_v[r.ia] += o.v;
        }
    }
    __syncwarp();
}

template <int N, typename Pix>
__global__ void __launch_bounds__(XcorrShape<N>::T, XcorrShape<N>::MIN_BLOCKS)
xcorr_kernel(IaJob job) {
    using S = XcorrShape<N>;
    constexpr int M = S::M, D = S::D, G = S::G, NG = S::NG, ROUNDS = S::ROUNDS, RP = S::RP, T = S::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx *tw = reinterpret_cast<cplx *>(smem_raw);
    cplx *reg = tw + M;           // N regions of RP complex
    cplx *scr = reg + N * RP;     // NG scratch buffers of RP complex
    uint64_t *red = reinterpret_cast<uint64_t *>(scr + NG * RP);  // 64 words
    FitRec *fitq = reinterpret_cast<FitRec *>(red + 64);           // 32 queued fits
    int qn = 0;                                                    // uniform across the CTA

    const int tid = threadIdx.x;
    const int g = tid % G;
    const int grp = tid / G;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    constexpr int NWARPS = T / 32;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
    const int gbase = lane & ~(G - 1);

    for (int e = tid; e < M; e += T) {
        double s, c;
        sincospi(-2.0 * (double)e / (double)M, &s, &c);
        tw[e] = {(float)c, (float)s};
    }
    __syncthreads();

    for (long ia = blockIdx.x; ia < job.count; ia += gridDim.x) {
        const Pix *imgA, *imgB;
        long pitch_a, pitch_b;
        int img_h, img_w;
        if (job.frames != nullptr) {
            const qlpiv_frame fr = job.frames[job.frame_idx[ia]];
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
            const int n1 = grp + NG * r;
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
        if (job.max_mode == QLPIV_MAX_COMPUTE) {
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
            maxA = fmaxf(mxa, 16.0f);
            maxB = fmaxf(mxb, 16.0f);
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
            const int n1 = grp + NG * r;
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
            fft_group<M, false>(v, g, scr + grp * RP, tw);
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int k2 = g + G * m;
                int region, slot;
                if (k2 == 0) { region = 0; slot = n1; }
                else if (k2 == N) { region = 0; slot = N + n1; }
                else if (k2 < N) { region = k2; slot = n1; }
                else { region = M - k2; slot = N + n1; }
                reg[region * RP + pad8(slot)] = v[m];
            }
        }
        __syncthreads();

        // ---- 3. column tasks ----
#pragma unroll
        for (int r = 0; r < ROUNDS; r++) {
            const int c = grp + NG * r;
            cplx *rg = reg + c * RP;
            cplx z1[8], z2[8];
#pragma unroll
            for (int m = 0; m < 4; m++) {
                z1[m] = rg[pad8(g + G * m)];
                z2[m] = rg[pad8(N + g + G * m)];
                z1[m + 4] = {0.0f, 0.0f};
                z2[m + 4] = {0.0f, 0.0f};
            }
            __syncwarp();
            fft_group<M, false>(z1, g, rg, tw);
            fft_group<M, false>(z2, g, rg, tw);
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
            fft_group<M, true>(p, g, rg, tw);
            __syncwarp();
#pragma unroll
            for (int m = 0; m < 8; m++) rg[pad8(g + G * m)] = p[m];
        }
        __syncthreads();

        // ---- 4. row-pair pass + per-lane peak scoring ----
        uint64_t best = 0ull;
        uint32_t best_ij = 0u;
        float minf = 3.402823466e38f;
        float *regf = reinterpret_cast<float *>(reg);
#pragma unroll
        for (int r = 0; r < ROUNDS; r++) {
            const int pr = grp + NG * r;
            const int ra_ = 2 * pr, rb_ = 2 * pr + 1;
            cplx y[8];
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int k2 = g + G * m;
                if (k2 == 0 || k2 == N) {
                    const cplx qa = reg[pad8(ra_)], qb = reg[pad8(rb_)];
                    y[m] = (k2 == 0) ? cplx{qa.x, qb.x} : cplx{qa.y, qb.y};
                } else if (k2 < N) {
                    const cplx qa = reg[k2 * RP + pad8(ra_)], qb = reg[k2 * RP + pad8(rb_)];
                    y[m] = {qa.x - qb.y, qa.y + qb.x};
                } else {
                    const int cc = M - k2;
                    const cplx qa = reg[cc * RP + pad8(ra_)], qb = reg[cc * RP + pad8(rb_)];
                    y[m] = {qa.x + qb.y, qb.x - qa.y};
                }
            }
            fft_group<M, true>(y, g, scr + grp * RP, tw);
            __syncwarp();
#pragma unroll
            for (int m = 0; m < 8; m++) {
                const int n2 = g + G * m;
                // keep the plane in the row slots this pair has consumed
                regf[2 * ((n2 >> 1) * RP + pad8(ra_)) + (n2 & 1)] = y[m].x;
                regf[2 * ((n2 >> 1) * RP + pad8(rb_)) + (n2 & 1)] = y[m].y;
                if (n2 >= 1 && n2 <= M - 2) {
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
                auto P = [&](int i, int j) -> float { return regf[2 * ((j >> 1) * RP + pad8(i)) + (j & 1)]; };
                r.kind = 0;
                if (!job.subpix) r.kind = 3;
                else if (r.pi == 0 && r.pj == 0) r.kind = 1;
                else if (r.pi - 1 < 0 || r.pi + 1 >= D || r.pj - 1 < 0 || r.pj + 1 >= D) r.kind = 2;
                if (r.kind == 0) {
                    r.c0 = P(r.pi, r.pj);
                    r.yu = P(r.pi - 1, r.pj);
                    r.yd = P(r.pi + 1, r.pj);
                    r.xl = P(r.pi, r.pj - 1);
                    r.xr = P(r.pi, r.pj + 1);
                }
                fitq[qn] = r;
            }
        }
        qn++;
        if (qn == 32) {
            if (warp == 0) fit_flush<D>(fitq, qn, lane, job);
            qn = 0;
        }
        __syncthreads();  // regions are rewritten by the next IA
    }
    if (qn > 0 && warp == 0) fit_flush<D>(fitq, qn, lane, job);
}

}  // namespace qlpiv
