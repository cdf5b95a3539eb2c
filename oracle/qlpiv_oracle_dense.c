/*
 * qlpiv oracle, dense optical flow stages -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, in Java float semantics (no contraction; the kernels' mad(a, b, c) is
 * a * b + c as in the reference's Java execution), the dense stages that follow PIV:
 *
 *  C-filter  GaussianFilter2D.createKernel (S/images/filters/GaussianFilter2D.java:31-46),
 *            GaussianFilter2DInternal.applyFilter (S/images/filters/GaussianFilter2DInternal.java:49-97),
 *            DirectConvolution.convolve1D (S/images/filters/DirectConvolution.java:14-53):
 *            rows then columns, padding = the first halfSize values mirrored on the
 *            left (edge repeated) and the last halfSize values copied in order on the
 *            right; accumulation from the +h neighbour down to the -h neighbour.
 *            ImageFloat.normalize (S/images/ImageFloat.java:571-596): divide by the max.
 *  C-LK      DenseLucasKanadeGpuKernel (S/jobs/interpolators/DenseLucasKanadeGpuKernel.java:203-751):
 *            per pixel, image A (optionally 2x2-averaged: half-pixel offset) over a W x W
 *            window, derivatives (3, 10, 3)/32, A matrix, inverse with det < FLT_EPSILON
 *            rejected, iterations of the b vector from bilinear samples of image B,
 *            stop on |increment| < 1e-3 (update skipped) or out of bounds.
 *  C-LS      DenseLiuShenGpuKernel (S/jobs/interpolators/DenseLiuShenGpuKernel.java:66-588):
 *            fixed-image terms from the 3x3 neighbourhoods of the Liu-Shen images,
 *            Jacobi passes of the 2x2 update, total-error stop at 1e-8.
 * Sums run in window row-major order.
 */
#define _GNU_SOURCE
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_types.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* GaussianFilter2D.createKernel: double weights, normalised, rounded to float. */
void orc_gauss_kernel(float sigma, int px, float *k) {
    double *kd = (double *)malloc(sizeof(double) * px);
    const int half = px / 2;
    double sum = 0.0;
    for (int i = 0; i < px; i++) {
        const double x = i - half;
        const double s = (double)sigma;
        kd[i] = 1.0 / sqrt(2.0 * M_PI * s * s) * exp(-x * x / (2.0 * s * s));
        sum += kd[i];
    }
    for (int i = 0; i < px; i++) k[i] = (float)(kd[i] / sum);
    free(kd);
}

/* one padded line through DirectConvolution (line of n values, stride `st`) */
static void filter_line(const float *in, long st, int n, const float *k, int K, float *buf, float *out, long ost) {
    const int h = K / 2;
    for (int j = 0; j < n; j++) buf[j + h] = in[(long)j * st];
    for (int j = 0; j < h; j++) {
        buf[h - 1 - j] = in[(long)j * st];
        buf[n + 2 * h - 1 - j] = in[(long)(n - 1 - j) * st];
    }
    for (int j = 0; j < n; j++) {
        float acc = 0.0f;
        for (int q = 0; q < K; q++) acc = acc + buf[j + 2 * h - q] * k[q];
        out[(long)j * ost] = acc;
    }
}

/* GaussianFilter2DInternal.applyFilter: rows, then columns of the row result. */
void orc_gauss_filter(const float *in, int h, int w, const float *k, int K, float *out) {
    const int n = h > w ? h : w;
    float *buf = (float *)malloc(sizeof(float) * (n + K));
    float *tmp = (float *)malloc(sizeof(float) * n);
    for (int i = 0; i < h; i++) filter_line(in + (long)i * w, 1, w, k, K, buf, out + (long)i * w, 1);
    for (int j = 0; j < w; j++) {
        filter_line(out + j, w, h, k, K, buf, tmp, 1);
        for (int i = 0; i < h; i++) out[(long)i * w + j] = tmp[i];
    }
    free(buf);
    free(tmp);
}

/* ImageFloat.normalize: value / max (max starts at 0). */
void orc_normalize(const float *in, long n, float *out) {
    float mx = 0.0f;
    for (long q = 0; q < n; q++)
        if (in[q] > mx) mx = in[q];
    for (long q = 0; q < n; q++) out[q] = in[q] / mx;
}

static float clamp_read(const float *img, int h, int w, int i, int j) {
    i = i < 0 ? 0 : (i > h - 1 ? h - 1 : i);
    j = j < 0 ? 0 : (j > w - 1 ? w - 1 : j);
    return img[(long)i * w + j];
}

/* readPixelWithWarp: floor anchor, bilinear, clamped reads. */
static float warp_read(const float *img, int h, int w, float li, float lj) {
    int i = (int)li, j = (int)lj;
    float di = li - (float)i, dj = lj - (float)j;
    const int si = di < 0.0f ? 1 : 0;
    i -= si;
    di += (float)si;
    const int sj = dj < 0.0f ? 1 : 0;
    j -= sj;
    dj += (float)sj;
    const float top = (1.0f - dj) * clamp_read(img, h, w, i, j) + dj * clamp_read(img, h, w, i, j + 1);
    const float bot = (1.0f - dj) * clamp_read(img, h, w, i + 1, j) + dj * clamp_read(img, h, w, i + 1, j + 1);
    return (1.0f - di) * top + di * bot;
}

/* Dense Lucas-Kanade of every pixel, in place on us (columns) / vs (rows). */
void orc_dense_lk(const float *A, const float *B, int h, int w, float *us, float *vs, int win, int iterations,
                  int half_pixel) {
    const int W = win, hw = win / 2;
    const int R = W + 2;  /* window plus the derivative margin */
    float *reg = (float *)malloc(sizeof(float) * R * R);
    float *val = (float *)malloc(sizeof(float) * W * W);
    float *dJ = (float *)malloc(sizeof(float) * W * W);
    float *dI = (float *)malloc(sizeof(float) * W * W);
    const float c3 = 3.0f / 32.0f;
    for (int pi = 0; pi < h; pi++) {
        for (int pj = 0; pj < w; pj++) {
            /* image A around the pixel: rows pi - hw - 1 ... , clamped */
            for (int a = 0; a < R; a++)
                for (int b = 0; b < R; b++) {
                    const int y = pi + a - hw - 1, x = pj + b - hw - 1;
                    if (half_pixel)
                        reg[a * R + b] = (clamp_read(A, h, w, y, x) + clamp_read(A, h, w, y, x + 1) +
                                          clamp_read(A, h, w, y + 1, x) + clamp_read(A, h, w, y + 1, x + 1)) / 4.0f;
                    else
                        reg[a * R + b] = clamp_read(A, h, w, y, x);
                }
            float a00 = 0.0f, a01 = 0.0f, a11 = 0.0f;
            for (int a = 0; a < W; a++)
                for (int b = 0; b < W; b++) {
                    const float *r0 = reg + a * R + b, *r1 = r0 + R, *r2 = r1 + R;
                    const float TL = r0[0], T = r0[1], TR = r0[2], L = r1[0], C = r1[1], Rt = r1[2];
                    const float BL = r2[0], Bt = r2[1], BR = r2[2];
                    const float dj = (((TL + BL) - TR) - BR) * c3 + (L - Rt) * 10.0f / 32.0f;
                    const float di = (((TR + TL) - BR) - BL) * c3 + (T - Bt) * 10.0f / 32.0f;
                    val[a * W + b] = C;
                    dJ[a * W + b] = dj;
                    dI[a * W + b] = di;
                    a00 = dj * dj + a00;
                    a01 = dj * di + a01;
                    a11 = di * di + a11;
                }
            const long p = (long)pi * w + pj;
            int status = 1;
            const float det = a00 * a11 + -(a01 * a01);
            if (det < 1.192092896e-7f) status = 0;
            const float i00 = a11 / det, i01 = -a01 / det, i11 = a00 / det;
            float locI = (float)pi + vs[p], locJ = (float)pj + us[p];
            if (half_pixel) {
                locI += 0.5f;
                locJ += 0.5f;
            }
            for (int it = 0; it < iterations && status; it++) {
                if (locI < 0.0f || locI >= (float)(h + hw)) { status = 0; break; }
                if (locJ < 0.0f || locJ >= (float)(w + hw)) { status = 0; break; }
                float b0 = 0.0f, b1 = 0.0f;
                for (int a = 0; a < W; a++)
                    for (int b = 0; b < W; b++) {
                        const float dT = warp_read(B, h, w, locI - (float)hw + (float)a, locJ - (float)hw + (float)b) -
                                         val[a * W + b];
                        b0 = dT * dJ[a * W + b] + b0;
                        b1 = dT * dI[a * W + b] + b1;
                    }
                const float incU = b0 * i00 + b1 * i01;
                const float incV = b0 * i01 + b1 * i11;
                if (fabsf(incU) < 1e-3f && fabsf(incV) < 1e-3f) { status = 0; break; }
                locI += incV;
                locJ += incU;
            }
            /* the integer pixel comes off first, then the half pixel */
            vs[p] = half_pixel ? (locI - (float)pi) - 0.5f : locI - (float)pi;
            us[p] = half_pixel ? (locJ - (float)pj) - 0.5f : locJ - (float)pj;
        }
    }
    free(reg);
    free(val);
    free(dJ);
    free(dI);
}

/* Liu-Shen 3x3 neighbourhood (row-major TL..BR) of img around (pi, pj), clamped; with the
 * half-pixel offset every value is the 2x2 average accumulated as v = P * 0.25 + v. */
static void ls_load(const float *img, int h, int w, int pi, int pj, int half_pixel, float *n9) {
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            const int y = pi - 1 + a, x = pj - 1 + b;
            if (half_pixel) {
                float v = 0.0f;
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++) v = clamp_read(img, h, w, y + i, x + j) * 0.25f + v;
                n9[a * 3 + b] = v;
            } else {
                n9[a * 3 + b] = clamp_read(img, h, w, y, x);
            }
        }
}

enum { TLi = 0, Ti = 1, TRi = 2, Li = 3, Ci = 4, Ri = 5, BLi = 6, Bi = 7, BRi = 8 };

/* Fixed-image terms of one pixel: out[0..11] = w, IIx, IIy, II, Ixt, Iyt, A11, A12, A22,
 * B11, B12, B22 (B = inverse of A). */
static void ls_fixed(const float *la, const float *lb, int h, int w, int pi, int pj, float lambda, int half_pixel,
                     float *o, float *wts) {
    float a9[9], b9[9];
    ls_load(la, h, w, pi, pj, half_pixel, a9);
    ls_load(lb, h, w, pi, pj, half_pixel, b9);
    const float wTL = (pi - 1) >= 0 && (pj - 1) >= 0 && (pi - 1) < h && (pj - 1) < w ? 1.0f : 0.0f;
    const float wT = (pi - 1) >= 0 && (pi - 1) < h && pj < w ? 1.0f : 0.0f;
    const float wTR = (pi - 1) >= 0 && (pj + 1) >= 0 && (pi - 1) < h && (pj + 1) < w ? 1.0f : 0.0f;
    const float wL = (pj - 1) >= 0 && pi < h && (pj - 1) < w ? 1.0f : 0.0f;
    const float wR = pi < h && (pj + 1) < w ? 1.0f : 0.0f;
    const float wBL = (pj - 1) >= 0 && (pi + 1) < h && (pj - 1) < w ? 1.0f : 0.0f;
    const float wB = (pi + 1) < h && pj < w ? 1.0f : 0.0f;
    const float wBR = (pi + 1) < h && (pj + 1) < w ? 1.0f : 0.0f;
    const float wsum = ((((((wTL + wT) + wTR) + wL) + wR) + wBL) + wB) + wBR;
    const float c = a9[Ci];
    const float IIx = c * (a9[Bi] - a9[Ti]) / 2.0f;
    const float IIy = c * (a9[Ri] - a9[Li]) / 2.0f;
    const float II = c * c;
    const float Ixt = c * ((b9[Bi] - a9[Bi]) - (b9[Ti] - a9[Ti])) / 2.0f;
    const float Iyt = c * ((b9[Ri] - a9[Ri]) - (b9[Li] - a9[Li])) / 2.0f;
    const float A11 = c * (((a9[Bi] + a9[Ti]) - 2.0f * c) - 2.0f * c) + -(lambda * wsum);
    const float A22 = c * (((a9[Ri] + a9[Li]) - 2.0f * c) - 2.0f * c) + -(lambda * wsum);
    const float A12 = c * (((a9[TLi] - a9[TRi]) - a9[BLi]) + a9[BRi]) / 4.0f;
    const float det = A11 * A22 + -(A12 * A12);
    o[0] = wsum; o[1] = IIx; o[2] = IIy; o[3] = II; o[4] = Ixt; o[5] = Iyt;
    o[6] = A11; o[7] = A12; o[8] = A22;
    o[9] = A22 / det; o[10] = -A12 / det; o[11] = A11 / det;
    if (wts) {
        wts[0] = wTL; wts[1] = wT; wts[2] = wTR; wts[3] = wL; wts[4] = 0.0f; wts[5] = wR;
        wts[6] = wBL; wts[7] = wB; wts[8] = wBR;
    }
}

/* Liu-Shen refinement passes (after the Lucas-Kanade pass) on us (columns) / vs (rows),
 * Jacobi: every pass reads the previous field.  fixed_out (optional, 12 x h x w) receives
 * the fixed terms; unews/vnews (optional, iterations x h x w) every pass's new rows /
 * columns displacement.  Returns the passes run. */
int orc_liu_shen(const float *la, const float *lb, int h, int w, float *us, float *vs, float lambda, int iterations,
                 int half_pixel, float *fixed_out, float *unews, float *vnews) {
    const long n = (long)h * w;
    float *fx = (float *)malloc(sizeof(float) * 12 * n);
    float *wt = (float *)malloc(sizeof(float) * 9 * n);
    float *un = (float *)malloc(sizeof(float) * n), *vn = (float *)malloc(sizeof(float) * n);
    for (int pi = 0; pi < h; pi++)
        for (int pj = 0; pj < w; pj++) {
            const long p = (long)pi * w + pj;
            float o[12];
            ls_fixed(la, lb, h, w, pi, pj, lambda, half_pixel, o, wt + 9 * p);
            for (int q = 0; q < 12; q++) fx[q * n + p] = o[q];
        }
    if (fixed_out) memcpy(fixed_out, fx, sizeof(float) * 12 * n);
    double total = FLT_MAX;
    int passes = 0;
    for (int it = 0; it < iterations; it++) {
        if (total < 1e-8) break;
        double err = 0.0;
        for (int pi = 0; pi < h; pi++)
            for (int pj = 0; pj < w; pj++) {
                const long p = (long)pi * w + pj;
                float U[9], V[9];
                ls_load(us, h, w, pi, pj, 0, U);
                ls_load(vs, h, w, pi, pj, 0, V);
                const float *wq = wt + 9 * p;
                const float IIx = fx[1 * n + p], IIy = fx[2 * n + p], II = fx[3 * n + p];
                const float Ixt = fx[4 * n + p], Iyt = fx[5 * n + p];
                const float B11 = fx[9 * n + p], B12 = fx[10 * n + p], B22 = fx[11 * n + p];
                const float sV = ((((((V[TLi] * wq[0] + V[Ti] * wq[1]) + V[TRi] * wq[2]) + V[Li] * wq[3]) +
                                    V[Ri] * wq[5]) + V[BLi] * wq[6]) + V[Bi] * wq[7]) + V[BRi] * wq[8];
                const float sU = ((((((U[TLi] * wq[0] + U[Ti] * wq[1]) + U[TRi] * wq[2]) + U[Li] * wq[3]) +
                                    U[Ri] * wq[5]) + U[BLi] * wq[6]) + U[Bi] * wq[7]) + U[BRi] * wq[8];
                const float hu = lambda * sV + Ixt;
                const float hv = lambda * sU + Iyt;
                const float bu = (2.0f * IIx) * ((V[Bi] - V[Ti]) / 2.0f) +
                                 (IIx * ((U[Ri] - U[Li]) / 2.0f) +
                                  (IIy * ((U[Bi] - U[Ti]) / 2.0f) +
                                   (II * (V[Ti] + V[Bi]) +
                                    (II * ((((U[TLi] - U[TRi]) - U[BLi]) + U[BRi]) / 4.0f) + hu))));
                const float bv = (2.0f * IIy) * ((U[Ri] - U[Li]) / 2.0f) +
                                 (IIx * ((V[Ri] - V[Li]) / 2.0f) +
                                  (IIy * ((V[Bi] - V[Ti]) / 2.0f) +
                                   (II * (U[Li] + U[Ri]) +
                                    (II * ((((V[TLi] - V[TRi]) - V[BLi]) + V[BRi]) / 4.0f) + hv))));
                const float unew = -(B11 * bu + B12 * bv);
                const float vnew = -(B12 * bu + B22 * bv);
                const float du = unew - V[Ci], dv = vnew - U[Ci];
                err += (double)sqrtf(du * du + dv * dv);
                un[p] = unew;
                vn[p] = vnew;
            }
        /* copyVectors: columns <- vnew, rows <- unew */
        memcpy(us, vn, sizeof(float) * n);
        memcpy(vs, un, sizeof(float) * n);
        if (unews) memcpy(unews + (long)it * n, un, sizeof(float) * n);
        if (vnews) memcpy(vnews + (long)it * n, vn, sizeof(float) * n);
        total = err / (double)n;
        passes++;
    }
    free(fx);
    free(wt);
    free(un);
    free(vn);
    return passes;
}

/* Lucas-Kanade pyramid (coarse to fine): this library's own design, not the reference's (its
 * DenseLucasKanade runs at full resolution only).  A level halves both sides (floor) by 2 x 2 box
 * averaging, ((a + b) + (c + d)) * 0.25 * scale, scale 0.5 for the displacement field; a coarser
 * level's result starts the next finer level through nearest up-sampling, doubled, with the
 * source index clamped to the coarser level. */
static void pyr_down(const float *s, int h, int w, float *d, float scale) {
    const int h2 = h / 2, w2 = w / 2;
    for (int i = 0; i < h2; i++)
        for (int j = 0; j < w2; j++) {
            const float *r0 = s + (long)(2 * i) * w + 2 * j, *r1 = r0 + w;
            const float t = (r0[0] + r0[1]) + (r1[0] + r1[1]);
            d[(long)i * w2 + j] = (t * 0.25f) * scale;
        }
}

static void pyr_up(const float *s, int hs, int ws, float *d, int h, int w) {
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            const int si = (i >> 1) < hs - 1 ? (i >> 1) : hs - 1, sj = (j >> 1) < ws - 1 ? (j >> 1) : ws - 1;
            d[(long)i * w + j] = 2.0f * s[(long)si * ws + sj];
        }
}

void orc_dense_lk_pyramid(const float *A, const float *B, int h, int w, float *us, float *vs, int win, int iterations,
                          int half_pixel, int levels) {
    if (levels <= 1) {
        orc_dense_lk(A, B, h, w, us, vs, win, iterations, half_pixel);
        return;
    }
    const float *la[4] = {A}, *lb[4] = {B};
    float *lu[4] = {us}, *lv[4] = {vs};
    int lh[4] = {h}, lw[4] = {w};
    for (int l = 1; l < levels; l++) {
        lh[l] = lh[l - 1] / 2;
        lw[l] = lw[l - 1] / 2;
        const long n = (long)lh[l] * lw[l];
        float *na = (float *)malloc(sizeof(float) * n), *nb = (float *)malloc(sizeof(float) * n);
        float *nu = (float *)malloc(sizeof(float) * n), *nv = (float *)malloc(sizeof(float) * n);
        pyr_down(la[l - 1], lh[l - 1], lw[l - 1], na, 1.0f);
        pyr_down(lb[l - 1], lh[l - 1], lw[l - 1], nb, 1.0f);
        pyr_down(lu[l - 1], lh[l - 1], lw[l - 1], nu, 0.5f);
        pyr_down(lv[l - 1], lh[l - 1], lw[l - 1], nv, 0.5f);
        la[l] = na;
        lb[l] = nb;
        lu[l] = nu;
        lv[l] = nv;
    }
    for (int l = levels - 1; l >= 0; l--) {
        if (l < levels - 1) {
            pyr_up(lu[l + 1], lh[l + 1], lw[l + 1], lu[l], lh[l], lw[l]);
            pyr_up(lv[l + 1], lh[l + 1], lw[l + 1], lv[l], lh[l], lw[l]);
        }
        orc_dense_lk(la[l], lb[l], lh[l], lw[l], lu[l], lv[l], win, iterations, half_pixel);
    }
    for (int l = 1; l < levels; l++) {
        free((void *)la[l]);
        free((void *)lb[l]);
        free(lu[l]);
        free(lv[l]);
    }
}

/* IOpticalFlowInterpolator.interpolate(stepTilesA, stepTilesB) of the LucasKanade (mode 1) and
 * LiuShenWithLucasKanade (mode 2) interpolators
 * (S/interpolators/DenseLucasKanadeAparapiJobInterpolator.java:247-334,
 *  S/interpolators/DenseLiuShenAparapiJobInterpolator.java:226-341) for the last adaptive step:
 * images filtered (LK: sigma_lk/px_lk; LS: sigma_ls/px_ls then normalised), the tile field
 * interpolated per pixel (offset 0 with dense export, else 0.5), Lucas-Kanade (+ Liu-Shen) with the
 * half-pixel offset unless dense export, tile displacements replaced from the pixel at
 * top + N/2 - 1 (average of the 2x2 pixels there with dense export).  img: float copies of the
 * frames.  tu/tv: tile displacements (rows, columns), ni x nj, updated in place; dense_u/dense_v
 * (rows, columns) receive the dense field when non-NULL. */
void orc_flow_after_piv(const float *img_a, const float *img_b, int h, int w, int n, int ni, int nj, const int *tops,
                        const int *lefts, float *tu, float *tv, int mode, float sigma_lk, int px_lk, float sigma_ls,
                        int px_ls, int window, int iters_lk, float lambda, int iters_ls, int dense_export,
                        int ignore_piv, int pyramid_levels, float *dense_u, float *dense_v) {
    const long np = (long)h * w;
    float *lka = (float *)malloc(sizeof(float) * np), *lkb = (float *)malloc(sizeof(float) * np);
    float *lsa = NULL, *lsb = NULL;
    float k[64];
    orc_gauss_kernel(sigma_lk, px_lk, k);
    if (sigma_lk < 1e-5f) { memcpy(lka, img_a, sizeof(float) * np); memcpy(lkb, img_b, sizeof(float) * np); }
    else { orc_gauss_filter(img_a, h, w, k, px_lk, lka); orc_gauss_filter(img_b, h, w, k, px_lk, lkb); }
    if (mode == 2) {
        lsa = (float *)malloc(sizeof(float) * np);
        lsb = (float *)malloc(sizeof(float) * np);
        float *t = (float *)malloc(sizeof(float) * np);
        orc_gauss_kernel(sigma_ls, px_ls, k);
        if (sigma_ls < 1e-5f) memcpy(t, img_a, sizeof(float) * np); else orc_gauss_filter(img_a, h, w, k, px_ls, t);
        orc_normalize(t, np, lsa);
        if (sigma_ls < 1e-5f) memcpy(t, img_b, sizeof(float) * np); else orc_gauss_filter(img_b, h, w, k, px_ls, t);
        orc_normalize(t, np, lsb);
        free(t);
    }
    double *ys = (double *)malloc(sizeof(double) * ni), *xs = (double *)malloc(sizeof(double) * nj);
    for (int i = 0; i < ni; i++) ys[i] = (double)((float)tops[i] + (float)n / 2.0f - 0.5f);
    for (int j = 0; j < nj; j++) xs[j] = (double)((float)lefts[j] + (float)n / 2.0f - 0.5f);
    float *fu = (float *)malloc(sizeof(float) * np), *fv = (float *)malloc(sizeof(float) * np);
    const float off = dense_export ? 0.0f : 0.5f;
    orc_displacement_field_off(ys, ni, xs, nj, tu, tv, h, w, 0, off, off, fu, fv);
    /* ignorePIVBaseDisplacements (DenseLucasKanadeAparapiJobInterpolator.java:233-277) */
    if (ignore_piv == 4 || ignore_piv == 5) {
        const float lim = ignore_piv == 4 ? 3.0f : 0.9f;
        for (long p = 0; p < np; p++) {
            if (fabsf(fu[p]) < lim) fu[p] = 0.0f;
            if (fabsf(fv[p]) < lim) fv[p] = 0.0f;
        }
    }
    if (ignore_piv == 2 || ignore_piv == 3)
        for (long p = 0; p < np; p++) fu[p] = dense_export ? 0.0f : 0.5f;
    if (ignore_piv == 1 || ignore_piv == 3)
        for (long p = 0; p < np; p++) fv[p] = dense_export ? 0.0f : 0.5f;
    /* the flow jobs take columns (us) and rows (vs) */
    float *us = fv, *vs = fu;
    const int half = dense_export ? 0 : 1;
    orc_dense_lk_pyramid(lka, lkb, h, w, us, vs, window, iters_lk, half, pyramid_levels);
    if (mode == 2) orc_liu_shen(lsa, lsb, h, w, us, vs, lambda, iters_ls, half, NULL, NULL, NULL);
    for (int ti = 0; ti < ni; ti++)
        for (int tj = 0; tj < nj; tj++) {
            const int i = tops[ti] + n / 2 - 1, j = lefts[tj] + n / 2 - 1;
            const long idx = (long)i * w + j, idx2 = (long)(i + 1) * w + j;
            float u, v;
            if (!dense_export) {
                u = us[idx];
                v = vs[idx];
            } else {
                u = (((us[idx] + us[idx + 1]) + us[idx2]) + us[idx2 + 1]) / 4.0f;
                v = (((vs[idx] + vs[idx + 1]) + vs[idx2]) + vs[idx2 + 1]) / 4.0f;
            }
            tu[ti * nj + tj] = v;   /* Tile.replaceDisplacement(v, u): rows, columns */
            tv[ti * nj + tj] = u;
        }
    if (dense_u) memcpy(dense_u, vs, sizeof(float) * np);
    if (dense_v) memcpy(dense_v, us, sizeof(float) * np);
    free(lka); free(lkb); free(lsa); free(lsb); free(ys); free(xs); free(fu); free(fv);
}

