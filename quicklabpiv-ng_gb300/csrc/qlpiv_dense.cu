// Dense optical flow after PIV (device code and C ABI).
//
//   C-filter  GaussianFilter2D (S/images/filters/GaussianFilter2D.java:31-46,
//             S/images/filters/GaussianFilter2DInternal.java:49-97, DirectConvolution.java:14-53):
//             rows, then columns of the row result; a line of n values is padded on the
//             left with its first h values mirrored (edge repeated) and on the right with its
//             last h values in order; out[j] accumulates in[j + h - q] * k[q], q = 0..2h.
//             ImageFloat.normalize (S/images/ImageFloat.java:571-596).
//   C-LK      DenseLucasKanadeGpuKernel (S/jobs/interpolators/DenseLucasKanadeGpuKernel.java:203-751):
//             a 16 x 16 pixel tile per CTA.  The CTA stages the image-A region its windows
//             span (clamped; 2x2 averages for the half-pixel offset) and the derivatives
//             (3, 10, 3) / 32 of every window point once in shared memory; each pixel then
//             sums its W x W A matrix and, per iteration, its b vector from bilinear samples
//             of image B.  Where the window's sample positions are exact (or round uniformly
//             past one power of two) the samples come from horizontal interpolations of B
//             rows computed once per row; elsewhere every sample is read as the reference
//             reads it.  Window 27 runs two vertically adjacent pixels per thread with those
//             rows in registers; other windows one pixel per thread.
//   C-LS      DenseLiuShenGpuKernel (S/jobs/interpolators/DenseLiuShenGpuKernel.java:66-588):
//             fixed-image terms once per pixel, then one Jacobi pass per launch; the pass
//             reads the previous pass's total error on the device and becomes a copy once
//             the mean error is below 1e-8.
// Sums run in window row-major order with IEEE single operations and no contraction
// (--fmad=false), the order of the CPU oracle's restatement: every stage is bit-identical
// to it.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "qlpiv_adaptive.h"
#include "qlpiv_dense.h"
#include "qlpiv_handle.h"
#include "qlpiv_internal.h"

namespace qlpiv {

namespace {

int blocks_of(long n, int b) { return (int)((n + b - 1) / b); }

// ---------------- Gaussian prefilter ----------------

__device__ __forceinline__ int filter_index(int x, int n, int h) {
    if (x < 0) return -1 - x;          // mirrored, edge repeated
    if (x >= n) return n - h + (x - n);  // the last h values, in order
    return x;
}

template <typename Pix>
__global__ void gauss_rows_kernel(const Pix *in, long pitch, int h, int w, const float *k, int K, float *out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= h || j >= w) return;
    const int hk = K / 2;
    const Pix *row = in + (long)i * pitch;
    float acc = 0.0f;
    for (int q = 0; q < K; q++) acc = __fadd_rn(acc, __fmul_rn((float)row[filter_index(j + hk - q, w, hk)], k[q]));
    out[(long)i * w + j] = acc;
}

__global__ void gauss_cols_kernel(const float *in, int h, int w, const float *k, int K, float *out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
    if (i >= h || j >= w) return;
    const int hk = K / 2;
    float acc = 0.0f;
    for (int q = 0; q < K; q++)
        acc = __fadd_rn(acc, __fmul_rn(in[(long)filter_index(i + hk - q, h, hk) * w + j], k[q]));
    out[(long)i * w + j] = acc;
}

// max of the non-negative values (the reference's running max starts at 0)
__global__ void max_kernel(const float *in, long n, unsigned *mx) {
    float m = 0.0f;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        m = fmaxf(m, in[q] > 0.0f ? in[q] : 0.0f);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, __float_as_uint(m));
}

__global__ void divide_kernel(const float *in, long n, const unsigned *mx, float *out) {
    const float m = __uint_as_float(*mx);
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        out[q] = __fdiv_rn(in[q], m);
}

// ---------------- dense Lucas-Kanade ----------------

constexpr int kLkTile = 16;

__device__ __forceinline__ float clamp_read(const float *img, int h, int w, int i, int j) {
    i = i < 0 ? 0 : (i > h - 1 ? h - 1 : i);
    j = j < 0 ? 0 : (j > w - 1 ? w - 1 : j);
    return img[(long)i * w + j];
}

// readPixelWithWarp: anchor at the floor, bilinear weights, clamped reads
__device__ __forceinline__ float warp_read(const float *img, int h, int w, float li, float lj) {
    int i = (int)li, j = (int)lj;
    float di = __fsub_rn(li, (float)i), dj = __fsub_rn(lj, (float)j);
    const int si = di < 0.0f ? 1 : 0;
    i -= si;
    di = __fadd_rn(di, (float)si);
    const int sj = dj < 0.0f ? 1 : 0;
    j -= sj;
    dj = __fadd_rn(dj, (float)sj);
    const float omj = __fsub_rn(1.0f, dj), omi = __fsub_rn(1.0f, di);
    const float top = __fadd_rn(__fmul_rn(omj, clamp_read(img, h, w, i, j)), __fmul_rn(dj, clamp_read(img, h, w, i, j + 1)));
    const float bot =
        __fadd_rn(__fmul_rn(omj, clamp_read(img, h, w, i + 1, j)), __fmul_rn(dj, clamp_read(img, h, w, i + 1, j + 1)));
    return __fadd_rn(__fmul_rn(omi, top), __fmul_rn(di, bot));
}

// One axis of a Lucas-Kanade window: sample k (0 <= k < W) sits at fl(o + k) and reads the
// pixels floor(fl(o + k)) and the next one with the fraction as weight.  For o >= 1 the samples
// of one binade are exact (o + k needs no rounding); past the next power of two they round to the
// coarser spacing, by the same amount for every k (k is a multiple of twice that spacing).  So
// when the window spans at most one boundary and the anchors stay contiguous, anchor(k) = base + k
// and the fraction is f1 below `split`, f2 from `split` on: exactly the per-sample arithmetic.
struct LkAxis {
    int base, split;
    float f1, f2;
};

__device__ __forceinline__ bool lk_axis(float o, int W, LkAxis &ax) {
    if (!(o >= 1.0f) || !(o < 1048576.0f)) return false;
    const unsigned eo = __float_as_uint(o) >> 23;
    const unsigned el = __float_as_uint(__fadd_rn(o, (float)(W - 1))) >> 23;
    ax.base = (int)o;
    ax.f1 = __fsub_rn(o, (float)ax.base);
    if (el == eo) {
        ax.split = W;
        ax.f2 = ax.f1;
        return true;
    }
    if (el != eo + 1) return false;
    const float t = __uint_as_float((eo + 1) << 23);   // the boundary 2^(e+1); t - o is exact
    const int split = (int)ceilf(__fsub_rn(t, o));     // first k with o + k >= t
    const float ls = __fadd_rn(o, (float)split);
    const int as = (int)ls;
    if (as != ax.base + split) return false;           // the rounding moved the anchor
    ax.split = split;
    ax.f2 = __fsub_rn(ls, (float)as);
    return true;
}

// The window points of a CTA's pixel tile: image A and its derivatives dj, di, GS x GS each,
// rows `ws` floats apart.  A warp reads one window point per thread from two groups of 16
// lanes (two thread rows); the row stride is padded so that the groups land 16 banks apart:
// ws = 8 (mod 16) when the groups are two rows of pixel pairs (2 ws apart), ws = 16 (mod 32)
// when they are two pixel rows.  GS = 42 (window 27) read at stride 42 put the groups 20 banks
// apart and half of the kernel's shared wavefronts were conflict replays.
__host__ __device__ constexpr int lk_pair_stride(int GS) { return GS + (24 - GS % 16) % 16; }
__host__ __device__ constexpr int lk_row_stride(int GS) { return GS + (48 - GS % 32) % 32; }

struct LkWin {
    const float *a, *dj, *di;
};

// Stages the A region (clamped; 2x2 averages for the half-pixel offset) of a tile with origin
// (ti0, tj0) in reg (RS x RS) and computes the window points' values and derivatives.
__device__ __forceinline__ void lk_stage(const float *A, int h, int w, int W, int half_pixel, int ti0, int tj0,
                                         int tid, int nthr, int tile, int ws, float *reg, float *wa, float *wj,
                                         float *wi) {
    const int hw = W / 2;
    const int RS = tile + W + 1, GS = tile + W - 1;
    for (int q = tid; q < RS * RS; q += nthr) {
        const int r = q / RS, c = q - r * RS;
        const int y = ti0 - hw - 1 + r, x = tj0 - hw - 1 + c;
        if (half_pixel) {
            const float s = __fadd_rn(__fadd_rn(__fadd_rn(clamp_read(A, h, w, y, x), clamp_read(A, h, w, y, x + 1)),
                                                clamp_read(A, h, w, y + 1, x)),
                                      clamp_read(A, h, w, y + 1, x + 1));
            reg[q] = __fdiv_rn(s, 4.0f);
        } else {
            reg[q] = clamp_read(A, h, w, y, x);
        }
    }
    __syncthreads();
    const float c3 = 3.0f / 32.0f;
    for (int q = tid; q < GS * GS; q += nthr) {
        const int gy = q / GS, gx = q - gy * GS;
        const float *r0 = reg + gy * RS + gx, *r1 = r0 + RS, *r2 = r1 + RS;
        const float TL = r0[0], T = r0[1], TR = r0[2], L = r1[0], C = r1[1], R = r1[2], BL = r2[0], Bt = r2[1],
                    BR = r2[2];
        const int o = gy * ws + gx;
        wj[o] = __fadd_rn(__fmul_rn(__fsub_rn(__fsub_rn(__fadd_rn(TL, BL), TR), BR), c3),
                          __fdiv_rn(__fmul_rn(__fsub_rn(L, R), 10.0f), 32.0f));
        wi[o] = __fadd_rn(__fmul_rn(__fsub_rn(__fsub_rn(__fadd_rn(TR, TL), BR), BL), c3),
                          __fdiv_rn(__fmul_rn(__fsub_rn(T, Bt), 10.0f), 32.0f));
        wa[o] = C;
    }
    __syncthreads();
}

// Per-pixel state of the iterations.
struct LkPix {
    long p;
    int pi, pj;
    bool active;
    float locI, locJ, i00, i01, i11;
};

// The A matrix of the pixel whose first window point is g (offset into the window arrays),
// its inverse and the start location; sets `active`.
__device__ __forceinline__ void lk_begin(const LkWin &win, int g, int GS, int W, const float *us, const float *vs,
                                         int half_pixel, LkPix &px) {
    float a00 = 0.0f, a01 = 0.0f, a11 = 0.0f;
    for (int a = 0; a < W; a++) {
        const float *wj = win.dj + g + a * GS, *wi = win.di + g + a * GS;
        for (int b = 0; b < W; b++) {
            const float dj = wj[b], di = wi[b];
            a00 = __fadd_rn(__fmul_rn(dj, dj), a00);
            a01 = __fadd_rn(__fmul_rn(dj, di), a01);
            a11 = __fadd_rn(__fmul_rn(di, di), a11);
        }
    }
    const float det = __fadd_rn(__fmul_rn(a00, a11), -__fmul_rn(a01, a01));
    px.active = !(det < 1.192092896e-7f);
    px.i00 = __fdiv_rn(a11, det);
    px.i01 = __fdiv_rn(-a01, det);
    px.i11 = __fdiv_rn(a00, det);
    px.locI = __fadd_rn((float)px.pi, vs[px.p]);
    px.locJ = __fadd_rn((float)px.pj, us[px.p]);
    if (half_pixel) {
        px.locI = __fadd_rn(px.locI, 0.5f);
        px.locJ = __fadd_rn(px.locJ, 0.5f);
    }
}

// Applies one iteration's window sums; returns false when the pixel stops.
__device__ __forceinline__ bool lk_update(LkPix &px, float b0, float b1) {
    const float incU = __fadd_rn(__fmul_rn(b0, px.i00), __fmul_rn(b1, px.i01));
    const float incV = __fadd_rn(__fmul_rn(b0, px.i01), __fmul_rn(b1, px.i11));
    if (fabsf(incU) < 1e-3f && fabsf(incV) < 1e-3f) return false;
    px.locI = __fadd_rn(px.locI, incV);
    px.locJ = __fadd_rn(px.locJ, incU);
    return true;
}

__device__ __forceinline__ void lk_end(const LkPix &px, int half_pixel, float *us, float *vs) {
    float v = __fsub_rn(px.locI, (float)px.pi), u = __fsub_rn(px.locJ, (float)px.pj);
    if (half_pixel) {
        v = __fsub_rn(v, 0.5f);
        u = __fsub_rn(u, 0.5f);
    }
    vs[px.p] = v;
    us[px.p] = u;
}

// Window sums from per-sample bilinear reads (any location, clamped).
__device__ __forceinline__ void lk_sums_slow(const float *B, int h, int w, int W, float oi, float oj,
                                             const LkWin &win, int g, int GS, float &b0, float &b1) {
    for (int a = 0; a < W; a++) {
        const int r = g + a * GS;
        const float li = __fadd_rn(oi, (float)a);
        for (int b = 0; b < W; b++) {
            const float dT = __fsub_rn(warp_read(B, h, w, li, __fadd_rn(oj, (float)b)), win.a[r + b]);
            b0 = __fadd_rn(__fmul_rn(dT, win.dj[r + b]), b0);
            b1 = __fadd_rn(__fmul_rn(dT, win.di[r + b]), b1);
        }
    }
}

// The register fast path of one pixel (window side WT): window row a reads B rows base + a (top)
// and base + a + 1 (bottom); the horizontal interpolation of a B row is the bottom of window row
// a and the top of window row a + 1, so each is computed once and kept in hb.  SPLIT: the column
// fraction changes at ax.split (selected per column from a bit mask), else it is ax.f1.
template <int WT, bool SPLIT>
struct LkRows {
    float hb[WT];
    const float *br;
    unsigned upper;
    float f1, f2, om1, om2;
    LkAxis ay;
    float b0, b1;

    __device__ __forceinline__ float wj(int b) const { return SPLIT && ((upper >> b) & 1u) ? f2 : f1; }
    __device__ __forceinline__ float womj(int b) const { return SPLIT && ((upper >> b) & 1u) ? om2 : om1; }

    __device__ __forceinline__ void init(const float *B, int w, const LkAxis &ay_, const LkAxis &ax) {
        ay = ay_;
        upper = SPLIT ? ~((1u << ax.split) - 1u) : 0u;
        f1 = ax.f1;
        f2 = ax.f2;
        om1 = __fsub_rn(1.0f, f1);
        om2 = __fsub_rn(1.0f, f2);
        br = B + (long)ay.base * w + ax.base;
        b0 = 0.0f;
        b1 = 0.0f;
        float x0 = br[0];
#pragma unroll
        for (int b = 0; b < WT; b++) {
            const float x1 = br[b + 1];
            hb[b] = __fadd_rn(__fmul_rn(womj(b), x0), __fmul_rn(wj(b), x1));
            x0 = x1;
        }
    }
    // window row a against the window points va/vj/vi of that row
    __device__ __forceinline__ void row(int a, int w, const float *va, const float *vj, const float *vi) {
        const float di = a < ay.split ? ay.f1 : ay.f2, omi = __fsub_rn(1.0f, di);
        br += w;
        float x0 = br[0];
#pragma unroll
        for (int b = 0; b < WT; b++) {
            const float x1 = br[b + 1];
            const float bot = __fadd_rn(__fmul_rn(womj(b), x0), __fmul_rn(wj(b), x1));
            x0 = x1;
            const float smp = __fadd_rn(__fmul_rn(omi, hb[b]), __fmul_rn(di, bot));
            hb[b] = bot;
            const float dT = __fsub_rn(smp, va[b]);
            b0 = __fadd_rn(__fmul_rn(dT, vj[b]), b0);
            b1 = __fadd_rn(__fmul_rn(dT, vi[b]), b1);
        }
    }
};

// Two vertically adjacent pixels (rows pi, pi + 1) share all but one window row: window row r of
// the upper pixel is row r - 1 of the lower one, so both consume each loaded window point.
template <int WT, bool S0, bool S1>
__device__ __forceinline__ void lk_pair_sums(const float *B, int w, const LkAxis &ay0, const LkAxis &ax0,
                                             const LkAxis &ay1, const LkAxis &ax1, const LkWin &win, int g, int GS,
                                             float &s00, float &s01, float &s10, float &s11) {
    LkRows<WT, S0> r0;
    LkRows<WT, S1> r1;
    r0.init(B, w, ay0, ax0);
    r1.init(B, w, ay1, ax1);
    r0.row(0, w, win.a + g, win.dj + g, win.di + g);
#pragma unroll 1
    for (int r = 1; r < WT; r++) {
        const int o = g + r * GS;
        const float *va = win.a + o, *vj = win.dj + o, *vi = win.di + o;
        const float di0 = r < ay0.split ? ay0.f1 : ay0.f2, omi0 = __fsub_rn(1.0f, di0);
        const float di1 = r - 1 < ay1.split ? ay1.f1 : ay1.f2, omi1 = __fsub_rn(1.0f, di1);
        r0.br += w;
        r1.br += w;
        float x00 = r0.br[0], x10 = r1.br[0];
#pragma unroll
        for (int b = 0; b < WT; b++) {
            const float a_ = va[b], j_ = vj[b], i_ = vi[b];
            const float x01 = r0.br[b + 1], x11 = r1.br[b + 1];
            const float bot0 = __fadd_rn(__fmul_rn(r0.womj(b), x00), __fmul_rn(r0.wj(b), x01));
            const float bot1 = __fadd_rn(__fmul_rn(r1.womj(b), x10), __fmul_rn(r1.wj(b), x11));
            x00 = x01;
            x10 = x11;
            const float smp0 = __fadd_rn(__fmul_rn(omi0, r0.hb[b]), __fmul_rn(di0, bot0));
            const float smp1 = __fadd_rn(__fmul_rn(omi1, r1.hb[b]), __fmul_rn(di1, bot1));
            r0.hb[b] = bot0;
            r1.hb[b] = bot1;
            const float dT0 = __fsub_rn(smp0, a_), dT1 = __fsub_rn(smp1, a_);
            r0.b0 = __fadd_rn(__fmul_rn(dT0, j_), r0.b0);
            r0.b1 = __fadd_rn(__fmul_rn(dT0, i_), r0.b1);
            r1.b0 = __fadd_rn(__fmul_rn(dT1, j_), r1.b0);
            r1.b1 = __fadd_rn(__fmul_rn(dT1, i_), r1.b1);
        }
    }
    const int o = g + WT * GS;
    r1.row(WT - 1, w, win.a + o, win.dj + o, win.di + o);
    s00 = r0.b0;
    s01 = r0.b1;
    s10 = r1.b0;
    s11 = r1.b1;
}

template <int WT, bool S>
__device__ __forceinline__ void lk_one_sums(const float *B, int w, const LkAxis &ay, const LkAxis &ax,
                                            const LkWin &win, int g, int GS, float &b0, float &b1) {
    LkRows<WT, S> r;
    r.init(B, w, ay, ax);
#pragma unroll 1
    for (int a = 0; a < WT; a++) {
        const int o = g + a * GS;
        r.row(a, w, win.a + o, win.dj + o, win.di + o);
    }
    b0 = r.b0;
    b1 = r.b1;
}

// Whether one iteration of pixel px may take the register fast path; fills the axes.
__device__ __forceinline__ bool lk_fast(const LkPix &px, int h, int w, int W, float oi, float oj, LkAxis &ay,
                                        LkAxis &ax) {
    return lk_axis(oi, W, ay) && lk_axis(oj, W, ax) && ay.base + W <= h - 1 && ax.base + W <= w - 1;
}

// Window side WT, two vertically adjacent pixels per thread: a CTA of 16 x 8 threads covers
// 16 x 16 pixels.  Shared memory: the window arrays (3 x GS rows of SS floats), then the staged
// region.
template <int WT, int MB>
__global__ void __launch_bounds__(128, MB) dense_lk_pair_kernel(const float *A, const float *B, int h, int w,
                                                                float *us, float *vs, int iterations, int half_pixel) {
    extern __shared__ float smf[];
    constexpr int W = WT, hw = WT / 2, GS = kLkTile + WT - 1, SS = lk_pair_stride(GS);
    float *wa = smf, *wj = wa + GS * SS, *wi = wj + GS * SS, *reg = wi + GS * SS;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int ti0 = blockIdx.y * kLkTile, tj0 = blockIdx.x * kLkTile;
    lk_stage(A, h, w, W, half_pixel, ti0, tj0, tid, blockDim.x * blockDim.y, kLkTile, SS, reg, wa, wj, wi);
    const LkWin win{wa, wj, wi};
    const int pj = tj0 + threadIdx.x, pi0 = ti0 + 2 * threadIdx.y;
    if (pj >= w || pi0 >= h) return;
    const bool two = pi0 + 1 < h;
    const int g0 = 2 * threadIdx.y * SS + threadIdx.x, g1 = g0 + SS;
    LkPix px[2];
    px[0].pi = pi0;
    px[0].pj = pj;
    px[0].p = (long)pi0 * w + pj;
    lk_begin(win, g0, SS, W, us, vs, half_pixel, px[0]);
    px[1].pi = pi0 + 1;
    px[1].pj = pj;
    px[1].p = px[0].p + w;
    if (two) lk_begin(win, g1, SS, W, us, vs, half_pixel, px[1]);
    else px[1].active = false;
    for (int it = 0; it < iterations && (px[0].active || px[1].active); it++) {
        bool run[2], fast[2];
        LkAxis ay[2], ax[2];
        float oi[2], oj[2];
#pragma unroll
        for (int k = 0; k < 2; k++) {
            run[k] = px[k].active;
            if (run[k] && (px[k].locI < 0.0f || px[k].locI >= (float)(h + hw) || px[k].locJ < 0.0f ||
                           px[k].locJ >= (float)(w + hw))) {
                px[k].active = false;
                run[k] = false;
            }
            oi[k] = __fsub_rn(px[k].locI, (float)hw);
            oj[k] = __fsub_rn(px[k].locJ, (float)hw);
            fast[k] = run[k] && lk_fast(px[k], h, w, W, oi[k], oj[k], ay[k], ax[k]);
        }
        float s[2][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
        if (fast[0] && fast[1]) {
            const bool sp0 = ax[0].split != W, sp1 = ax[1].split != W;
            if (!sp0 && !sp1)
                lk_pair_sums<WT, false, false>(B, w, ay[0], ax[0], ay[1], ax[1], win, g0, SS, s[0][0], s[0][1],
                                               s[1][0], s[1][1]);
            else if (sp0 && !sp1)
                lk_pair_sums<WT, true, false>(B, w, ay[0], ax[0], ay[1], ax[1], win, g0, SS, s[0][0], s[0][1],
                                              s[1][0], s[1][1]);
            else if (!sp0 && sp1)
                lk_pair_sums<WT, false, true>(B, w, ay[0], ax[0], ay[1], ax[1], win, g0, SS, s[0][0], s[0][1],
                                              s[1][0], s[1][1]);
            else
                lk_pair_sums<WT, true, true>(B, w, ay[0], ax[0], ay[1], ax[1], win, g0, SS, s[0][0], s[0][1],
                                             s[1][0], s[1][1]);
        } else {
#pragma unroll
            for (int k = 0; k < 2; k++) {
                if (!run[k]) continue;
                const int g = k ? g1 : g0;
                if (fast[k]) {
                    if (ax[k].split == W) lk_one_sums<WT, false>(B, w, ay[k], ax[k], win, g, SS, s[k][0], s[k][1]);
                    else lk_one_sums<WT, true>(B, w, ay[k], ax[k], win, g, SS, s[k][0], s[k][1]);
                } else {
                    lk_sums_slow(B, h, w, W, oi[k], oj[k], win, g, SS, s[k][0], s[k][1]);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 2; k++)
            if (run[k] && !lk_update(px[k], s[k][0], s[k][1])) px[k].active = false;
    }
    lk_end(px[0], half_pixel, us, vs);
    if (two) lk_end(px[1], half_pixel, us, vs);
}

// Any window side, one pixel per thread (16 x 16 threads per tile); the uniform fast path keeps
// each thread's row of horizontal samples in shared memory (stride = threads, bank = lane).
__global__ void __launch_bounds__(kLkTile *kLkTile, 2) dense_lk_kernel(const float *A, const float *B, int h, int w,
                                                                        float *us, float *vs, int W, int iterations,
                                                                        int half_pixel) {
    extern __shared__ float smf[];
    constexpr int kThreads = kLkTile * kLkTile;
    const int hw = W / 2, GS = kLkTile + W - 1, SS = lk_row_stride(GS);
    float *wa = smf, *wj = wa + GS * SS, *wi = wj + GS * SS, *reg = wi + GS * SS;
    const int tid = threadIdx.y * kLkTile + threadIdx.x;
    const int ti0 = blockIdx.y * kLkTile, tj0 = blockIdx.x * kLkTile;
    lk_stage(A, h, w, W, half_pixel, ti0, tj0, tid, kThreads, kLkTile, SS, reg, wa, wj, wi);
    const LkWin win{wa, wj, wi};
    const int pi = ti0 + threadIdx.y, pj = tj0 + threadIdx.x;
    if (pi >= h || pj >= w) return;
    const int g = threadIdx.y * SS + threadIdx.x;
    LkPix px;
    px.pi = pi;
    px.pj = pj;
    px.p = (long)pi * w + pj;
    lk_begin(win, g, SS, W, us, vs, half_pixel, px);
    float *hb = reg + tid;  // the staged region is dead: per-thread rows, stride kThreads
    for (int it = 0; it < iterations && px.active; it++) {
        if (px.locI < 0.0f || px.locI >= (float)(h + hw) || px.locJ < 0.0f || px.locJ >= (float)(w + hw)) break;
        float b0 = 0.0f, b1 = 0.0f;
        const float oi = __fsub_rn(px.locI, (float)hw), oj = __fsub_rn(px.locJ, (float)hw);
        LkAxis ay, ax;
        if (lk_fast(px, h, w, W, oi, oj, ay, ax) && ay.split == W && ax.split == W) {
            const float dj = ax.f1, omj = __fsub_rn(1.0f, dj);
            const float di = ay.f1, omi = __fsub_rn(1.0f, di);
            const float *br = B + (long)ay.base * w + ax.base;
            float x0 = br[0];
            for (int b = 0; b < W; b++) {
                const float x1 = br[b + 1];
                hb[b * kThreads] = __fadd_rn(__fmul_rn(omj, x0), __fmul_rn(dj, x1));
                x0 = x1;
            }
            for (int a = 0; a < W; a++) {
                const int r = g + a * SS;
                br += w;
                x0 = br[0];
                for (int b = 0; b < W; b++) {
                    const float x1 = br[b + 1];
                    const float bot = __fadd_rn(__fmul_rn(omj, x0), __fmul_rn(dj, x1));
                    x0 = x1;
                    const float top = hb[b * kThreads];
                    hb[b * kThreads] = bot;
                    const float smp = __fadd_rn(__fmul_rn(omi, top), __fmul_rn(di, bot));
                    const float dT = __fsub_rn(smp, wa[r + b]);
                    b0 = __fadd_rn(__fmul_rn(dT, wj[r + b]), b0);
                    b1 = __fadd_rn(__fmul_rn(dT, wi[r + b]), b1);
                }
            }
        } else {
            lk_sums_slow(B, h, w, W, oi, oj, win, g, SS, b0, b1);
        }
        if (!lk_update(px, b0, b1)) break;
    }
    lk_end(px, half_pixel, us, vs);
}

// Shared memory: 3 window arrays plus the staged region (which later holds the per-thread rows of
// the generic kernel).
size_t lk_smem(int W, bool rows_in_smem) {
    const size_t RS = kLkTile + W + 1, GS = kLkTile + W - 1;
    const size_t SS = rows_in_smem ? lk_row_stride((int)GS) : lk_pair_stride((int)GS);
    const size_t rows = rows_in_smem ? (size_t)W * kLkTile * kLkTile : 0;
    return sizeof(float) * (3 * GS * SS + (RS * RS > rows ? RS * RS : rows));
}

template <int WT, int MB>
static cudaError_t launch_lk_pair(cudaStream_t s, const float *a, const float *b, int h, int w, float *us, float *vs,
                                  int iterations, int half_pixel) {
    const size_t sm = lk_smem(WT, false);
    cudaError_t e =
        cudaFuncSetAttribute(dense_lk_pair_kernel<WT, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dim3 blk(kLkTile, kLkTile / 2), grd(blocks_of(w, kLkTile), blocks_of(h, kLkTile));
    dense_lk_pair_kernel<WT, MB><<<grd, blk, sm, s>>>(a, b, h, w, us, vs, iterations, half_pixel);
    return cudaGetLastError();
}

static cudaError_t launch_lk_generic(cudaStream_t s, const float *a, const float *b, int h, int w, float *us,
                                     float *vs, int W, int iterations, int half_pixel) {
    const size_t sm = lk_smem(W, true);
    cudaError_t e = cudaFuncSetAttribute(dense_lk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dim3 blk(kLkTile, kLkTile), grd(blocks_of(w, kLkTile), blocks_of(h, kLkTile));
    dense_lk_kernel<<<grd, blk, sm, s>>>(a, b, h, w, us, vs, W, iterations, half_pixel);
    return cudaGetLastError();
}

// ---------------- Liu-Shen ----------------

enum { kTL = 0, kT = 1, kTR = 2, kL = 3, kC = 4, kR = 5, kBL = 6, kB = 7, kBR = 8 };

__device__ __forceinline__ void ls_load(const float *img, int h, int w, int pi, int pj, int half_pixel, float *n9) {
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            const int y = pi - 1 + a, x = pj - 1 + b;
            float v;
            if (half_pixel) {
                v = 0.0f;
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++) v = __fadd_rn(__fmul_rn(clamp_read(img, h, w, y + i, x + j), 0.25f), v);
            } else {
                v = clamp_read(img, h, w, y, x);
            }
            n9[a * 3 + b] = v;
        }
}

__device__ __forceinline__ void ls_weights(int pi, int pj, int h, int w, float *wq) {
    wq[kTL] = (pi - 1) >= 0 && (pj - 1) >= 0 && (pi - 1) < h && (pj - 1) < w ? 1.0f : 0.0f;
    wq[kT] = (pi - 1) >= 0 && (pi - 1) < h && pj < w ? 1.0f : 0.0f;
    wq[kTR] = (pi - 1) >= 0 && (pj + 1) >= 0 && (pi - 1) < h && (pj + 1) < w ? 1.0f : 0.0f;
    wq[kL] = (pj - 1) >= 0 && pi < h && (pj - 1) < w ? 1.0f : 0.0f;
    wq[kC] = 0.0f;
    wq[kR] = pi < h && (pj + 1) < w ? 1.0f : 0.0f;
    wq[kBL] = (pj - 1) >= 0 && (pi + 1) < h && (pj - 1) < w ? 1.0f : 0.0f;
    wq[kB] = (pi + 1) < h && pj < w ? 1.0f : 0.0f;
    wq[kBR] = (pi + 1) < h && (pj + 1) < w ? 1.0f : 0.0f;
}

// Fixed terms, 8 planes of h x w: IIx, IIy, II, Ixt, Iyt, B11, B12, B22.
__global__ void ls_fixed_kernel(const float *la, const float *lb, int h, int w, float lambda, int half_pixel,
                                float *fx) {
    const int pj = blockIdx.x * blockDim.x + threadIdx.x, pi = blockIdx.y * blockDim.y + threadIdx.y;
    if (pi >= h || pj >= w) return;
    float a9[9], b9[9], wq[9];
    ls_load(la, h, w, pi, pj, half_pixel, a9);
    ls_load(lb, h, w, pi, pj, half_pixel, b9);
    ls_weights(pi, pj, h, w, wq);
    const int ring[8] = {kTL, kT, kTR, kL, kR, kBL, kB, kBR};
    float ws = 0.0f;
#pragma unroll
    for (int t = 0; t < 8; t++) ws = __fadd_rn(ws, wq[ring[t]]);
    const float c = a9[kC], c2 = __fmul_rn(2.0f, c);
    const float IIx = __fdiv_rn(__fmul_rn(c, __fsub_rn(a9[kB], a9[kT])), 2.0f);
    const float IIy = __fdiv_rn(__fmul_rn(c, __fsub_rn(a9[kR], a9[kL])), 2.0f);
    const float II = __fmul_rn(c, c);
    const float Ixt =
        __fdiv_rn(__fmul_rn(c, __fsub_rn(__fsub_rn(b9[kB], a9[kB]), __fsub_rn(b9[kT], a9[kT]))), 2.0f);
    const float Iyt =
        __fdiv_rn(__fmul_rn(c, __fsub_rn(__fsub_rn(b9[kR], a9[kR]), __fsub_rn(b9[kL], a9[kL]))), 2.0f);
    const float lw = -__fmul_rn(lambda, ws);
    const float A11 = __fadd_rn(__fmul_rn(c, __fsub_rn(__fsub_rn(__fadd_rn(a9[kB], a9[kT]), c2), c2)), lw);
    const float A22 = __fadd_rn(__fmul_rn(c, __fsub_rn(__fsub_rn(__fadd_rn(a9[kR], a9[kL]), c2), c2)), lw);
    const float A12 =
        __fdiv_rn(__fmul_rn(c, __fadd_rn(__fsub_rn(__fsub_rn(a9[kTL], a9[kTR]), a9[kBL]), a9[kBR])), 4.0f);
    const float det = __fadd_rn(__fmul_rn(A11, A22), -__fmul_rn(A12, A12));
    const long n = (long)h * w, p = (long)pi * w + pj;
    fx[0 * n + p] = IIx;
    fx[1 * n + p] = IIy;
    fx[2 * n + p] = II;
    fx[3 * n + p] = Ixt;
    fx[4 * n + p] = Iyt;
    fx[5 * n + p] = __fdiv_rn(A22, det);
    fx[6 * n + p] = __fdiv_rn(-A12, det);
    fx[7 * n + p] = __fdiv_rn(A11, det);
}

// The Liu-Shen update of one pixel from its 3 x 3 neighbourhoods U (columns field) and V (rows
// field) and its fixed terms.  INTERIOR: every neighbour exists, all weights are 1 and the
// weighted sums are plain sums (x * 1.0f == x exactly).
template <bool INTERIOR>
__device__ __forceinline__ void ls_update(const float *U, const float *V, const float *wq, const float *fx, long n,
                                          long p, float lambda, float &unew, float &vnew) {
    const float IIx = fx[0 * n + p], IIy = fx[1 * n + p], II = fx[2 * n + p];
    const float Ixt = fx[3 * n + p], Iyt = fx[4 * n + p];
    const float B11 = fx[5 * n + p], B12 = fx[6 * n + p], B22 = fx[7 * n + p];
    const int ring[7] = {kT, kTR, kL, kR, kBL, kB, kBR};
    float sV, sU;
    if (INTERIOR) {
        sV = V[kTL];
        sU = U[kTL];
    } else {
        sV = __fmul_rn(V[kTL], wq[kTL]);
        sU = __fmul_rn(U[kTL], wq[kTL]);
    }
#pragma unroll
    for (int t = 0; t < 7; t++) {
        const int q = ring[t];
        sV = __fadd_rn(sV, INTERIOR ? V[q] : __fmul_rn(V[q], wq[q]));
        sU = __fadd_rn(sU, INTERIOR ? U[q] : __fmul_rn(U[q], wq[q]));
    }
    const float hu = __fadd_rn(__fmul_rn(lambda, sV), Ixt);
    const float hv = __fadd_rn(__fmul_rn(lambda, sU), Iyt);
    const float u_xy = __fdiv_rn(__fadd_rn(__fsub_rn(__fsub_rn(U[kTL], U[kTR]), U[kBL]), U[kBR]), 4.0f);
    const float v_xy = __fdiv_rn(__fadd_rn(__fsub_rn(__fsub_rn(V[kTL], V[kTR]), V[kBL]), V[kBR]), 4.0f);
    const float bu = __fadd_rn(
        __fmul_rn(__fmul_rn(2.0f, IIx), __fdiv_rn(__fsub_rn(V[kB], V[kT]), 2.0f)),
        __fadd_rn(__fmul_rn(IIx, __fdiv_rn(__fsub_rn(U[kR], U[kL]), 2.0f)),
                  __fadd_rn(__fmul_rn(IIy, __fdiv_rn(__fsub_rn(U[kB], U[kT]), 2.0f)),
                            __fadd_rn(__fmul_rn(II, __fadd_rn(V[kT], V[kB])), __fadd_rn(__fmul_rn(II, u_xy), hu)))));
    const float bv = __fadd_rn(
        __fmul_rn(__fmul_rn(2.0f, IIy), __fdiv_rn(__fsub_rn(U[kR], U[kL]), 2.0f)),
        __fadd_rn(__fmul_rn(IIx, __fdiv_rn(__fsub_rn(V[kR], V[kL]), 2.0f)),
                  __fadd_rn(__fmul_rn(IIy, __fdiv_rn(__fsub_rn(V[kB], V[kT]), 2.0f)),
                            __fadd_rn(__fmul_rn(II, __fadd_rn(U[kL], U[kR])), __fadd_rn(__fmul_rn(II, v_xy), hv)))));
    unew = -__fadd_rn(__fmul_rn(B11, bu), __fmul_rn(B12, bv));
    vnew = -__fadd_rn(__fmul_rn(B12, bu), __fmul_rn(B22, bv));
}

// One Jacobi pass: (us_in, vs_in) -> (us_out, vs_out).  A pass's total error (the sum of the
// pixels' update lengths, in double) is spread over kLsSlots accumulators err[pass][slot] so
// that the CTAs' atomics do not queue on one address; once the previous pass's mean error is
// below 1e-8 the pass copies.  A CTA of 32 x 8 threads covers 32 x (8 kLsRows) pixels.
constexpr int kLsRows = 4;
constexpr int kLsSlots = 32;

// s + c += x exactly (TwoSum), so a thread's few errors need one conversion to double.
__device__ __forceinline__ void two_sum_acc(float &s, float &c, float x) {
    const float t = __fadd_rn(s, x);
    const float bp = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    s = t;
    c = __fadd_rn(c, e);
}

__global__ void __launch_bounds__(256) ls_pass_kernel(const float *fx, int h, int w, float lambda,
                                                      const float *us_in, const float *vs_in, float *us_out,
                                                      float *vs_out, double *err, int pass) {
    const int pj = blockIdx.x * blockDim.x + threadIdx.x;
    const long n = (long)h * w;
    const int t = threadIdx.y * blockDim.x + threadIdx.x;
    __shared__ double wsum[8];
    __shared__ bool stop_s;
    if (t < 32) {  // the previous pass's total from its slots
        double prev = pass > 0 ? err[(pass - 1) * kLsSlots + t] : 0.0;
        for (int o = 16; o > 0; o >>= 1) prev += __shfl_xor_sync(0xffffffffu, prev, o);
        if (t == 0) stop_s = pass > 0 && prev / (double)n < 1e-8;
    }
    __syncthreads();
    const bool stop = stop_s;
    float es = 0.0f, ec = 0.0f;
#pragma unroll
    for (int r = 0; r < kLsRows; r++) {
        const int pi = (blockIdx.y * kLsRows + r) * blockDim.y + threadIdx.y;
        if (pi >= h || pj >= w) continue;
        const long p = (long)pi * w + pj;
        if (stop) {
            us_out[p] = us_in[p];
            vs_out[p] = vs_in[p];
            continue;
        }
        float U[9], V[9], unew, vnew;
        if (pi >= 1 && pi <= h - 2 && pj >= 1 && pj <= w - 2) {
            const float *u0 = us_in + p - w - 1, *v0 = vs_in + p - w - 1;
#pragma unroll
            for (int a = 0; a < 3; a++)
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    U[a * 3 + b] = u0[(long)a * w + b];
                    V[a * 3 + b] = v0[(long)a * w + b];
                }
            ls_update<true>(U, V, nullptr, fx, n, p, lambda, unew, vnew);
        } else {
            float wq[9];
            ls_load(us_in, h, w, pi, pj, 0, U);
            ls_load(vs_in, h, w, pi, pj, 0, V);
            ls_weights(pi, pj, h, w, wq);
            ls_update<false>(U, V, wq, fx, n, p, lambda, unew, vnew);
        }
        const float du = __fsub_rn(unew, V[kC]), dv = __fsub_rn(vnew, U[kC]);
        two_sum_acc(es, ec, __fsqrt_rn(__fadd_rn(__fmul_rn(du, du), __fmul_rn(dv, dv))));
        us_out[p] = vnew;  // columns <- vnew, rows <- unew (copyVectors)
        vs_out[p] = unew;
    }
    const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
    if (stop) {  // carry the previous total forward
        if (bid == 0 && t < kLsSlots) err[pass * kLsSlots + t] = err[(pass - 1) * kLsSlots + t];
        return;
    }
    double e = (double)es + (double)ec;
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if ((t & 31) == 0) wsum[t >> 5] = e;
    __syncthreads();
    if (t == 0) {
        double sum = 0.0;
        for (int k = 0; k < (int)(blockDim.x * blockDim.y) / 32; k++) sum += wsum[k];
        if (sum != 0.0) atomicAdd(&err[pass * kLsSlots + (bid % kLsSlots)], sum);
    }
}

// Tile displacements from the dense field (rows vs, columns us) at top + n/2 - 1, left + n/2 - 1,
// or the 2x2 average there with dense export (Tile.replaceDisplacement(v, u)); with clip
// (NoOutOfBoundClipping, image h x w) a value that moves the tile out of the image is refused and
// the tile keeps its displacement.
__global__ void tiles_from_dense_kernel(const float *us, const float *vs, int h, int w, int n, int ni, int nj,
                                        const int *tops, const int *lefts, int dense, int clip, float *tile_u,
                                        float *tile_v) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ni * nj) return;
    const int ti = t / nj, tj = t - ti * nj;
    const int i = tops[ti] + n / 2 - 1, j = lefts[tj] + n / 2 - 1;
    const long idx = (long)i * w + j, idx2 = (long)(i + 1) * w + j;
    float u, v;
    if (!dense) {
        u = us[idx];
        v = vs[idx];
    } else {
        u = __fdiv_rn(__fadd_rn(__fadd_rn(__fadd_rn(us[idx], us[idx + 1]), us[idx2]), us[idx2 + 1]), 4.0f);
        v = __fdiv_rn(__fadd_rn(__fadd_rn(__fadd_rn(vs[idx], vs[idx + 1]), vs[idx2]), vs[idx2 + 1]), 4.0f);
    }
    if (clip && !tile_inside(n, h, w, tops[ti], lefts[tj], v, u)) return;
    tile_u[t] = v;
    tile_v[t] = u;
}

// ignorePIVBaseDisplacements on the per-pixel PIV field fu (rows) / fv (columns)
// (DenseLucasKanadeAparapiJobInterpolator.java:233-277).
__global__ void ignore_piv_kernel(float *fu, float *fv, long n, int mode, float fill) {
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float u = fu[p], v = fv[p];
    if (mode == QLPIV_IGNORE_PIV_AUTO || mode == QLPIV_IGNORE_PIV_AUTO_SMALL) {
        const float lim = mode == QLPIV_IGNORE_PIV_AUTO ? 3.0f : 0.9f;
        if (fabsf(u) < lim) u = 0.0f;
        if (fabsf(v) < lim) v = 0.0f;
    }
    if (mode == QLPIV_IGNORE_PIV_V || mode == QLPIV_IGNORE_PIV_UV) u = fill;
    if (mode == QLPIV_IGNORE_PIV_U || mode == QLPIV_IGNORE_PIV_UV) v = fill;
    fu[p] = u;
    fv[p] = v;
}

}  // namespace


const char *check_flow_desc(const qlpiv_flow_desc *d, int h, int w) {
    if (!d) return "flow descriptor is NULL";
    if (d->pyramid_levels < 0 || d->pyramid_levels > 4) return "Lucas-Kanade pyramid: 0..4 levels";
    if (d->pyramid_levels > 1 && ((h >> (d->pyramid_levels - 1)) < 8 || (w >> (d->pyramid_levels - 1)) < 8))
        return "Lucas-Kanade pyramid: the coarsest level must keep at least 8 x 8 pixels";
    if (d->mode != QLPIV_FLOW_LUCAS_KANADE && d->mode != QLPIV_FLOW_LIU_SHEN) return "unknown optical-flow mode";
    if (d->window_lk < 3 || d->window_lk > 31 || d->window_lk % 2 == 0)
        return "dense Lucas-Kanade: window size must be odd, 3..31";
    if (d->iterations_lk <= 0) return "dense Lucas-Kanade: Number of iterations must greater or equal to 1";
    if (d->ignore_piv < QLPIV_IGNORE_PIV_NONE || d->ignore_piv > QLPIV_IGNORE_PIV_AUTO_SMALL)
        return "unknown ignore-PIV mode";
    if (d->clipping_mode < QLPIV_CLIP_ALLOWED || d->clipping_mode > QLPIV_CLIP_NO_OUT_OF_BOUND)
        return "unknown clipping mode";
    if (d->filter_px_lk < 1 || d->filter_px_lk % 2 == 0 || d->filter_px_lk > 63) return "Lucas-Kanade filter width";
    if (d->mode == QLPIV_FLOW_LIU_SHEN) {
        if (d->iterations_ls <= 0) return "dense Liu-Shen: Number of iterations must greater or equal to 1";
        if (d->filter_px_ls < 1 || d->filter_px_ls % 2 == 0 || d->filter_px_ls > 63) return "Liu-Shen filter width";
    }
    return nullptr;
}

void gauss_weights(float sigma, int px, float *k) {
    std::vector<double> kd(px);
    const int half = px / 2;
    double sum = 0.0;
    for (int i = 0; i < px; i++) {
        const double x = i - half, s = (double)sigma;
        kd[i] = 1.0 / std::sqrt(2.0 * M_PI * s * s) * std::exp(-x * x / (2.0 * s * s));
        sum += kd[i];
    }
    for (int i = 0; i < px; i++) k[i] = (float)(kd[i] / sum);
}

cudaError_t launch_gauss(cudaStream_t s, int pixel_type, const void *in, long pitch, int h, int w, const float *k,
                         int K, float *tmp, float *out) {
    dim3 blk(32, 8), grd(blocks_of(w, 32), blocks_of(h, 8));
    switch (pixel_type) {
        case QLPIV_PIX_U8:
            gauss_rows_kernel<uint8_t><<<grd, blk, 0, s>>>((const uint8_t *)in, pitch, h, w, k, K, tmp);
            break;
        case QLPIV_PIX_U16:
            gauss_rows_kernel<uint16_t><<<grd, blk, 0, s>>>((const uint16_t *)in, pitch, h, w, k, K, tmp);
            break;
        default:
            gauss_rows_kernel<float><<<grd, blk, 0, s>>>((const float *)in, pitch, h, w, k, K, tmp);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    gauss_cols_kernel<<<grd, blk, 0, s>>>(tmp, h, w, k, K, out);
    return cudaGetLastError();
}

cudaError_t launch_normalize(cudaStream_t s, const float *in, long n, unsigned *mx, float *out) {
    cudaError_t e = cudaMemsetAsync(mx, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    const int blocks = blocks_of(n, 256) < 1024 ? blocks_of(n, 256) : 1024;
    max_kernel<<<blocks, 256, 0, s>>>(in, n, mx);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    divide_kernel<<<blocks, 256, 0, s>>>(in, n, mx, out);
    return cudaGetLastError();
}

cudaError_t launch_dense_lk(cudaStream_t s, const float *a, const float *b, int h, int w, float *us, float *vs, int W,
                            int iterations, int half_pixel) {
    // the reference's example window (27) runs with its sample rows in registers
    if (W == 27) return launch_lk_pair<27, 2>(s, a, b, h, w, us, vs, iterations, half_pixel);
    return launch_lk_generic(s, a, b, h, w, us, vs, W, iterations, half_pixel);
}

// Liu-Shen passes on (us, vs) in place; fx: 8 planes, tmp: 2 planes, err: ls_err_bytes.
size_t ls_err_bytes(int h, int w, int iterations) {
    (void)h;
    (void)w;
    return sizeof(double) * kLsSlots * (size_t)(iterations > 0 ? iterations : 1);
}

cudaError_t launch_liu_shen(cudaStream_t s, const float *la, const float *lb, int h, int w, float *us, float *vs,
                            float lambda, int iterations, int half_pixel, float *fx, float *tmp, double *err) {
    dim3 blk(32, 8), grd(blocks_of(w, 32), blocks_of(h, 8));
    const long n = (long)h * w;
    const dim3 pgrd(blocks_of(w, 32), blocks_of(h, 8 * kLsRows));
    cudaError_t e = cudaMemsetAsync(err, 0, ls_err_bytes(h, w, iterations), s);
    if (e != cudaSuccess) return e;
    ls_fixed_kernel<<<grd, blk, 0, s>>>(la, lb, h, w, lambda, half_pixel, fx);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    float *cu = us, *cv = vs, *nu = tmp, *nv = tmp + n;
    for (int it = 0; it < iterations; it++) {
        ls_pass_kernel<<<pgrd, blk, 0, s>>>(fx, h, w, lambda, cu, cv, nu, nv, err, it);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        float *t = cu; cu = nu; nu = t;
        t = cv; cv = nv; nv = t;
    }
    if (cu != us) {  // odd pass count: the result sits in tmp
        if ((e = cudaMemcpyAsync(us, cu, sizeof(float) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess ||
            (e = cudaMemcpyAsync(vs, cv, sizeof(float) * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}


// ---------------- Lucas-Kanade pyramid (coarse to fine) ----------------
// This library's own design (the reference's dense LK runs at full resolution only): 2 x 2 box
// down-sampling, ((a + b) + (c + d)) * 0.25 * scale with rounded single operations (scale 0.5 for
// the displacement field), and nearest up-sampling of a level's result, doubled.

__global__ void pyr_down_kernel(const float *s, int h, int w, float *d, float scale) {
    const int h2 = h / 2, w2 = w / 2;
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (long)h2 * w2) return;
    const int i = (int)(k / w2), j = (int)(k - (long)i * w2);
    const float *r0 = s + (long)(2 * i) * w + 2 * j, *r1 = r0 + w;
    const float t = __fadd_rn(__fadd_rn(r0[0], r0[1]), __fadd_rn(r1[0], r1[1]));
    d[k] = __fmul_rn(__fmul_rn(t, 0.25f), scale);
}

__global__ void pyr_up_kernel(const float *s, int hs, int ws, float *d, int h, int w) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (long)h * w) return;
    const int i = (int)(k / w), j = (int)(k - (long)i * w);
    const int si = min(i >> 1, hs - 1), sj = min(j >> 1, ws - 1);
    d[k] = __fmul_rn(2.0f, s[(long)si * ws + sj]);
}

// Dense LK over `levels` pyramid levels on the prefiltered frames a, b (h x w) and the start field
// us / vs (columns, rows), which receives the finest level's result.  pyr: scratch of at least
// 4 x h x w / 3 floats plus alignment (FlowBufs::pyr).
static cudaError_t lk_pyramid(cudaStream_t s, const float *a, const float *b, int h, int w, float *us, float *vs,
                              int window, int iterations, int half, int levels, float *pyr, long *launches) {
    if (levels <= 1) {
        *launches += 1;
        return launch_dense_lk(s, a, b, h, w, us, vs, window, iterations, half);
    }
    const float *la[4] = {a}, *lb[4] = {b};
    float *lu[4] = {us}, *lv[4] = {vs};
    int lh[4] = {h}, lw[4] = {w};
    float *c = pyr;
    cudaError_t e;
    for (int l = 1; l < levels; l++) {
        lh[l] = lh[l - 1] / 2;
        lw[l] = lw[l - 1] / 2;
        const long n = (long)lh[l] * lw[l], step = (n + 63) & ~63L;
        float *na = c, *nb = c + step, *nu = c + 2 * step, *nv = c + 3 * step;
        c += 4 * step;
        const unsigned g = (unsigned)((n + 255) / 256);
        pyr_down_kernel<<<g, 256, 0, s>>>(la[l - 1], lh[l - 1], lw[l - 1], na, 1.0f);
        pyr_down_kernel<<<g, 256, 0, s>>>(lb[l - 1], lh[l - 1], lw[l - 1], nb, 1.0f);
        pyr_down_kernel<<<g, 256, 0, s>>>(lu[l - 1], lh[l - 1], lw[l - 1], nu, 0.5f);
        pyr_down_kernel<<<g, 256, 0, s>>>(lv[l - 1], lh[l - 1], lw[l - 1], nv, 0.5f);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        *launches += 4;
        la[l] = na;
        lb[l] = nb;
        lu[l] = nu;
        lv[l] = nv;
    }
    for (int l = levels - 1; l >= 0; l--) {
        if (l < levels - 1) {  // start from the coarser level's result
            const long n = (long)lh[l] * lw[l];
            const unsigned g = (unsigned)((n + 255) / 256);
            pyr_up_kernel<<<g, 256, 0, s>>>(lu[l + 1], lh[l + 1], lw[l + 1], lu[l], lh[l], lw[l]);
            pyr_up_kernel<<<g, 256, 0, s>>>(lv[l + 1], lh[l + 1], lw[l + 1], lv[l], lh[l], lw[l]);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            *launches += 2;
        }
        if ((e = launch_dense_lk(s, la[l], lb[l], lh[l], lw[l], lu[l], lv[l], window, iterations, half)) !=
            cudaSuccess)
            return e;
        *launches += 1;
    }
    return cudaSuccess;
}

// prefilter of a frame; sigma < 1e-5 keeps the frame (converted to float)
static cudaError_t filter_or_copy(cudaStream_t s, int pixel_type, const void *img, long pitch, int h, int w, float sigma,
                                  const float *k, int K, float *tmp, float *out, long *launches) {
    *launches += 2;
    // sigma < 1e-5: the weights hold a one-point unit kernel, which converts and copies exactly
    return launch_gauss(s, pixel_type, img, pitch, h, w, k, sigma < 1e-5f ? 1 : K, tmp, out);
}

cudaError_t run_flow(cudaStream_t s, const qlpiv_flow_desc &d, int pixel_type, const void *img_a, const void *img_b,
                     long pitch, int h, int w, int n, int ni, int nj, const float2 *kfy, const float2 *kfx,
                     const float *cyf, const float *cxf, const int *tops, const int *lefts, float *tile_u,
                     float *tile_v, float *dense_u, float *dense_v, const FlowBufs &b, long *launches,
                     const FlowMarks *marks, const SplineCoef *given) {
    cudaError_t e;
    const long np = (long)h * w;
    auto mark = [&](const char *stage, bool begin) {
        if (marks) marks->fn(marks->ctx, stage, begin);
    };
    mark("flow:prefilter", true);
    if ((e = filter_or_copy(s, pixel_type, img_a, pitch, h, w, d.filter_sigma_lk, b.k_lk, d.filter_px_lk, b.tmp, b.lka,
                            launches)) != cudaSuccess ||
        (e = filter_or_copy(s, pixel_type, img_b, pitch, h, w, d.filter_sigma_lk, b.k_lk, d.filter_px_lk, b.tmp, b.lkb,
                            launches)) != cudaSuccess)
        return e;
    if (d.mode == QLPIV_FLOW_LIU_SHEN) {
        if ((e = filter_or_copy(s, pixel_type, img_a, pitch, h, w, d.filter_sigma_ls, b.k_ls, d.filter_px_ls, b.tmp,
                                b.fu, launches)) != cudaSuccess ||
            (e = launch_normalize(s, b.fu, np, b.mx, b.lsa)) != cudaSuccess ||
            (e = filter_or_copy(s, pixel_type, img_b, pitch, h, w, d.filter_sigma_ls, b.k_ls, d.filter_px_ls, b.tmp,
                                b.fu, launches)) != cudaSuccess ||
            (e = launch_normalize(s, b.fu, np, b.mx, b.lsb)) != cudaSuccess)
            return e;
        *launches += 4;
    }
    mark("flow:prefilter", false);
    mark("flow:field", true);
    // per-pixel field from the tiles (knots at the tile centres), offset 0.5 unless dense export
    SplineCoef coef;
    if (given) {  // solved by the caller (all pairs at once)
        coef = *given;
    } else {
        coef = spline_coef_at(b.coef, (long)ni * nj);
        if ((e = launch_spline(s, 1, kfy, ni, kfx, nj, tile_u, tile_v, coef)) != cudaSuccess) return e;
        *launches += 1;
    }
    const float off = d.dense_export ? 0.0f : 0.5f;
    if ((e = launch_field(s, h, w, cyf, ni, cxf, nj, coef, b.fu, b.fv, off, off)) != cudaSuccess) return e;
    *launches += 1;
    if (d.ignore_piv != QLPIV_IGNORE_PIV_NONE) {
        ignore_piv_kernel<<<blocks_of(np, 256), 256, 0, s>>>(b.fu, b.fv, np, d.ignore_piv,
                                                             d.dense_export ? 0.0f : 0.5f);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        *launches += 1;
    }
    mark("flow:field", false);
    float *us = b.fv, *vs = b.fu;  // the flow jobs take columns (us) and rows (vs)
    const int half = d.dense_export ? 0 : 1;
    mark("flow:lucas_kanade", true);
    if ((e = lk_pyramid(s, b.lka, b.lkb, h, w, us, vs, d.window_lk, d.iterations_lk, half, d.pyramid_levels, b.pyr,
                        launches)) != cudaSuccess)
        return e;
    mark("flow:lucas_kanade", false);
    if (d.mode == QLPIV_FLOW_LIU_SHEN) {
        mark("flow:liu_shen", true);
        if ((e = launch_liu_shen(s, b.lsa, b.lsb, h, w, us, vs, d.lambda_ls, d.iterations_ls, half, b.fx, b.fx + 8 * np,
                                 b.err)) != cudaSuccess)
            return e;
        *launches += 1 + d.iterations_ls;
        mark("flow:liu_shen", false);
    }
    tiles_from_dense_kernel<<<blocks_of((long)ni * nj, 128), 128, 0, s>>>(
        us, vs, h, w, n, ni, nj, tops, lefts, d.dense_export, d.clipping_mode == QLPIV_CLIP_NO_OUT_OF_BOUND, tile_u,
        tile_v);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    *launches += 1;
    if (dense_u && (e = cudaMemcpyAsync(dense_u, vs, sizeof(float) * np, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return e;
    if (dense_v && (e = cudaMemcpyAsync(dense_v, us, sizeof(float) * np, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return e;
    return cudaSuccess;
}

// Carves FlowBufs for an h x w frame and ni x nj tiles out of one device buffer.
cudaError_t flow_buffers(DevBuf &buf, int h, int w, int ni, int nj, int iterations_ls, FlowBufs *b) {
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t pl = al(sizeof(float) * (size_t)h * w);
    const size_t total = 7 * pl + 10 * pl + 2 * pl + al(ls_err_bytes(h, w, iterations_ls)) + 256 +
                         2 * al(sizeof(float) * 64) + al(spline_coef_bytes((long)ni * nj));
    cudaError_t e = buf.ensure(total);
    if (e != cudaSuccess) return e;
    char *c = buf.as<char>();
    float **planes[7] = {&b->lka, &b->lkb, &b->lsa, &b->lsb, &b->tmp, &b->fu, &b->fv};
    for (float **p : planes) { *p = (float *)c; c += pl; }
    b->fx = (float *)c; c += 10 * pl;
    b->pyr = (float *)c; c += 2 * pl;
    b->err = (double *)c; c += al(ls_err_bytes(h, w, iterations_ls));
    b->mx = (unsigned *)c; c += 256;
    b->k_lk = (float *)c; c += al(sizeof(float) * 64);
    b->k_ls = (float *)c; c += al(sizeof(float) * 64);
    b->coef = c;
    return cudaSuccess;
}

// Uploads both filters' weights (a one-point unit kernel when sigma < 1e-5).
cudaError_t upload_flow_weights(cudaStream_t s, const qlpiv_flow_desc &d, const FlowBufs &b, std::vector<float> &host) {
    host.assign(128, 0.0f);
    if (d.filter_sigma_lk < 1e-5f) host[0] = 1.0f; else gauss_weights(d.filter_sigma_lk, d.filter_px_lk, host.data());
    if (d.mode == QLPIV_FLOW_LIU_SHEN) {
        if (d.filter_sigma_ls < 1e-5f) host[64] = 1.0f;
        else gauss_weights(d.filter_sigma_ls, d.filter_px_ls, host.data() + 64);
    }
    cudaError_t e = cudaMemcpyAsync(b.k_lk, host.data(), sizeof(float) * 64, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(b.k_ls, host.data() + 64, sizeof(float) * 64, cudaMemcpyHostToDevice, s);
}

}  // namespace qlpiv

using namespace qlpiv;

namespace {

qlpiv_status check_image(int pixel_type, int height, int width) {
    if (pixel_type != QLPIV_PIX_U8 && pixel_type != QLPIV_PIX_U16 && pixel_type != QLPIV_PIX_F32)
        return fail(QLPIV_E_ARG, "unknown pixel type %d", pixel_type);
    if (height < 1 || width < 1) return fail(QLPIV_E_SHAPE, "image size %d x %d", height, width);
    return QLPIV_OK;
}

}  // namespace

extern "C" {

qlpiv_status qlpiv_gaussian_filter(qlpiv_handle *h, int pixel_type, const void *img, int height, int width,
                                   float sigma, int kernel_px, float *out) {
    if (!h || !img || !out) return fail(QLPIV_E_ARG, "NULL argument");
    qlpiv_status st = check_image(pixel_type, height, width);
    if (st != QLPIV_OK) return st;
    if (kernel_px < 1 || kernel_px % 2 == 0 || kernel_px > 63)
        return fail(QLPIV_E_ARG, "kernel width %d must be odd, 1..63", kernel_px);
    if (kernel_px / 2 > height || kernel_px / 2 > width)
        return fail(QLPIV_E_SHAPE, "image %d x %d smaller than half the kernel", height, width);
    const long n = (long)height * width;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaStream_t s = h->stream;
    if (sigma < 1e-5f) {  // GaussianFilter2D.applyFilter returns the input unchanged
        std::vector<float> f(n);
        for (long q = 0; q < n; q++)
            f[q] = pixel_type == QLPIV_PIX_U8 ? (float)((const uint8_t *)img)[q]
                   : pixel_type == QLPIV_PIX_U16 ? (float)((const uint16_t *)img)[q]
                                                 : ((const float *)img)[q];
        std::copy(f.begin(), f.end(), out);
        return QLPIV_OK;
    }
    std::vector<float> k(kernel_px);
    gauss_weights(sigma, kernel_px, k.data());
    DevBuf *b = h->scratch;
    const size_t ib = (size_t)n * pixel_bytes(pixel_type);
    cudaError_t e;
    if ((e = b[0].ensure(ib)) != cudaSuccess || (e = b[1].ensure(sizeof(float) * n)) != cudaSuccess ||
        (e = b[2].ensure(sizeof(float) * n)) != cudaSuccess || (e = b[3].ensure(sizeof(float) * 64)) != cudaSuccess)
        return cuda_fail(e, "filter buffers");
    if ((e = cudaMemcpyAsync(b[0].p, img, ib, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b[3].p, k.data(), sizeof(float) * kernel_px, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "filter upload");
    if ((e = launch_gauss(s, pixel_type, b[0].p, width, height, width, b[3].as<float>(), kernel_px, b[1].as<float>(),
                          b[2].as<float>())) != cudaSuccess)
        return cuda_fail(e, "filter");
    h->launches += 2;
    if ((e = cudaMemcpyAsync(out, b[2].p, sizeof(float) * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "filter download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_normalize(qlpiv_handle *h, const float *img, int height, int width, float *out) {
    if (!h || !img || !out) return fail(QLPIV_E_ARG, "NULL argument");
    if (height < 1 || width < 1) return fail(QLPIV_E_SHAPE, "image size %d x %d", height, width);
    const long n = (long)height * width;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaStream_t s = h->stream;
    DevBuf *b = h->scratch;
    cudaError_t e;
    if ((e = b[0].ensure(sizeof(float) * n)) != cudaSuccess || (e = b[1].ensure(sizeof(float) * n)) != cudaSuccess ||
        (e = b[3].ensure(256)) != cudaSuccess)
        return cuda_fail(e, "normalize buffers");
    if ((e = cudaMemcpyAsync(b[0].p, img, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "normalize upload");
    if ((e = launch_normalize(s, b[0].as<float>(), n, b[3].as<unsigned>(), b[1].as<float>())) != cudaSuccess)
        return cuda_fail(e, "normalize");
    h->launches += 2;
    if ((e = cudaMemcpyAsync(out, b[1].p, sizeof(float) * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "normalize download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_dense_lk(qlpiv_handle *h, const float *img_a, const float *img_b, int height, int width, float *us,
                            float *vs, int window, int iterations, int half_pixel) {
    if (!h || !img_a || !img_b || !us || !vs) return fail(QLPIV_E_ARG, "NULL argument");
    if (height < 1 || width < 1) return fail(QLPIV_E_SHAPE, "image size %d x %d", height, width);
    // DenseLucasKanadeAparapiJob.analyze limits
    if (window < 3) return fail(QLPIV_E_ARG, "dense Lucas-Kanade: Window size too small");
    if (window > 31) return fail(QLPIV_E_ARG, "dense Lucas-Kanade: Window size too large");
    if (window % 2 == 0) return fail(QLPIV_E_ARG, "dense Lucas-Kanade: window size must be odd");
    if (iterations <= 0) return fail(QLPIV_E_ARG, "dense Lucas-Kanade: Number of iterations must greater or equal to 1");
    const long n = (long)height * width;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaStream_t s = h->stream;
    DevBuf *b = h->scratch;
    cudaError_t e;
    for (int q = 0; q < 4; q++)
        if ((e = b[q].ensure(sizeof(float) * n)) != cudaSuccess) return cuda_fail(e, "dense LK buffers");
    if ((e = cudaMemcpyAsync(b[0].p, img_a, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b[1].p, img_b, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b[2].p, us, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b[3].p, vs, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "dense LK upload");
    if ((e = launch_dense_lk(s, b[0].as<float>(), b[1].as<float>(), height, width, b[2].as<float>(), b[3].as<float>(),
                             window, iterations, half_pixel)) != cudaSuccess)
        return cuda_fail(e, "dense LK");
    h->launches++;
    if ((e = cudaMemcpyAsync(us, b[2].p, sizeof(float) * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(vs, b[3].p, sizeof(float) * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "dense LK download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_liu_shen(qlpiv_handle *h, const float *lk_a, const float *lk_b, const float *ls_a,
                            const float *ls_b, int height, int width, float *us, float *vs, int window,
                            int iterations_lk, float lambda, int iterations_ls, int half_pixel) {
    if (!h || !ls_a || !ls_b || !us || !vs) return fail(QLPIV_E_ARG, "NULL argument");
    if (height < 1 || width < 1) return fail(QLPIV_E_SHAPE, "image size %d x %d", height, width);
    if (iterations_ls <= 0) return fail(QLPIV_E_ARG, "dense Liu-Shen: Number of iterations must greater or equal to 1");
    if (iterations_lk > 0) {
        if (!lk_a || !lk_b) return fail(QLPIV_E_ARG, "NULL Lucas-Kanade image");
        if (window < 3 || window > 31 || window % 2 == 0)
            return fail(QLPIV_E_ARG, "dense Lucas-Kanade: window size %d must be odd, 3..31", window);
    }
    const long n = (long)height * width;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaStream_t s = h->stream;
    DevBuf *b = h->scratch;
    cudaError_t e;
    for (int q = 0; q < 6; q++)
        if ((e = b[q].ensure(sizeof(float) * n)) != cudaSuccess) return cuda_fail(e, "Liu-Shen buffers");
    if ((e = b[6].ensure(sizeof(float) * 10 * n)) != cudaSuccess ||
        (e = b[7].ensure(ls_err_bytes(height, width, iterations_ls))) != cudaSuccess)
        return cuda_fail(e, "Liu-Shen buffers");
    if ((iterations_lk > 0 &&
         ((e = cudaMemcpyAsync(b[0].p, lk_a, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
          (e = cudaMemcpyAsync(b[1].p, lk_b, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess)) ||
        (e = cudaMemcpyAsync(b[2].p, ls_a, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b[3].p, ls_b, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b[4].p, us, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b[5].p, vs, sizeof(float) * n, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "Liu-Shen upload");
    if (iterations_lk > 0) {  // pass 0 of DenseLiuShenGpuKernel: Lucas-Kanade
        if ((e = launch_dense_lk(s, b[0].as<float>(), b[1].as<float>(), height, width, b[4].as<float>(),
                                 b[5].as<float>(), window, iterations_lk, half_pixel)) != cudaSuccess)
            return cuda_fail(e, "dense LK");
        h->launches++;
    }
    float *fx = b[6].as<float>();
    if ((e = launch_liu_shen(s, b[2].as<float>(), b[3].as<float>(), height, width, b[4].as<float>(), b[5].as<float>(),
                             lambda, iterations_ls, half_pixel, fx, fx + 8 * n, b[7].as<double>())) != cudaSuccess)
        return cuda_fail(e, "Liu-Shen");
    h->launches += 1 + iterations_ls;
    if ((e = cudaMemcpyAsync(us, b[4].p, sizeof(float) * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(vs, b[5].p, sizeof(float) * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "Liu-Shen download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_flow_after_piv(qlpiv_handle *h, const qlpiv_flow_desc *desc, int pixel_type, const void *img_a,
                                  const void *img_b, int height, int width, int n, int ni, int nj,
                                  const int32_t *tops, const int32_t *lefts, float *tile_u, float *tile_v,
                                  float *dense_u, float *dense_v) {
    if (!h || !img_a || !img_b || !tops || !lefts || !tile_u || !tile_v) return fail(QLPIV_E_ARG, "NULL argument");
    if (const char *m = check_flow_desc(desc, height, width)) return fail(QLPIV_E_ARG, "%s", m);
    qlpiv_status st = check_image(pixel_type, height, width);
    if (st != QLPIV_OK) return st;
    if (ni < 3 || nj < 3) return fail(QLPIV_E_SHAPE, "the spline needs at least 3 tiles per axis");
    for (int i = 0; i < ni; i++)
        if (tops[i] + n / 2 < 1 || tops[i] + n / 2 >= height) return fail(QLPIV_E_SHAPE, "tile row %d outside the image", i);
    for (int j = 0; j < nj; j++)
        if (lefts[j] + n / 2 < 1 || lefts[j] + n / 2 >= width) return fail(QLPIV_E_SHAPE, "tile column %d outside the image", j);
    const long np = (long)height * width, nt = (long)ni * nj;
    std::vector<double> knots(ni + nj);
    std::vector<float2> kf((size_t)KF_ARRAYS * (ni + nj));
    std::vector<float> fknots(ni + nj);
    for (int i = 0; i < ni; i++) {
        fknots[i] = (float)tops[i] + (float)n / 2.0f - 0.5f;
        knots[i] = fknots[i];
    }
    for (int j = 0; j < nj; j++) {
        fknots[ni + j] = (float)lefts[j] + (float)n / 2.0f - 0.5f;
        knots[ni + j] = fknots[ni + j];
    }
    knot_factors_dw(knots.data(), ni, kf.data());
    knot_factors_dw(knots.data() + ni, nj, kf.data() + (size_t)KF_ARRAYS * ni);
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaStream_t s = h->stream;
    DevBuf *sb = h->scratch;
    const size_t ib = (size_t)np * pixel_bytes(pixel_type);
    cudaError_t e;
    FlowBufs fb;
    if ((e = flow_buffers(sb[9], height, width, ni, nj, desc->iterations_ls, &fb)) != cudaSuccess ||
        (e = sb[0].ensure(2 * ((ib + 255) & ~(size_t)255))) != cudaSuccess ||
        (e = sb[1].ensure(sizeof(float2) * kf.size() + sizeof(float) * (ni + nj) + sizeof(int32_t) * (ni + nj) +
                          sizeof(float) * 2 * nt + 1024)) != cudaSuccess ||
        (e = sb[2].ensure(sizeof(float) * 2 * np)) != cudaSuccess)
        return cuda_fail(e, "flow buffers");
    char *im = sb[0].as<char>();
    char *ib2 = im + ((ib + 255) & ~(size_t)255);
    float2 *dk = sb[1].as<float2>();
    float *dfk = (float *)(dk + kf.size());
    int32_t *dtl = (int32_t *)(dfk + ni + nj);
    float *dtu = (float *)(dtl + ni + nj);
    float *dtv = dtu + nt;
    std::vector<int32_t> tl(tops, tops + ni);
    tl.insert(tl.end(), lefts, lefts + nj);
    std::vector<float> wts;
    if ((e = cudaMemcpyAsync(im, img_a, ib, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(ib2, img_b, ib, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dk, kf.data(), sizeof(float2) * kf.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dfk, fknots.data(), sizeof(float) * (ni + nj), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dtl, tl.data(), sizeof(int32_t) * (ni + nj), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dtu, tile_u, sizeof(float) * nt, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dtv, tile_v, sizeof(float) * nt, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = upload_flow_weights(s, *desc, fb, wts)) != cudaSuccess)
        return cuda_fail(e, "flow upload");
    float *du = sb[2].as<float>(), *dv = du + np;
    long launches = 0;
    if ((e = run_flow(s, *desc, pixel_type, im, ib2, width, height, width, n, ni, nj, dk,
                      dk + (size_t)KF_ARRAYS * ni, dfk, dfk + ni, dtl,
                      dtl + ni, dtu, dtv, du, dv, fb, &launches, nullptr)) != cudaSuccess)
        return cuda_fail(e, "optical flow after PIV");
    h->launches += launches;
    if ((e = cudaMemcpyAsync(tile_u, dtu, sizeof(float) * nt, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(tile_v, dtv, sizeof(float) * nt, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (dense_u && (e = cudaMemcpyAsync(dense_u, du, sizeof(float) * np, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
        (dense_v && (e = cudaMemcpyAsync(dense_v, dv, sizeof(float) * np, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "flow download");
    return QLPIV_OK;
}

}  // extern "C"

