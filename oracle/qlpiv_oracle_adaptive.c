/*
 * qlpiv oracle, adaptive multi-pass stages -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, from the reference sources and the published mathematics of the
 * third-party routines they call (commons-math3 3.6.1 is not part of the reference
 * tree, so its interpolators are written here from their mathematical definitions):
 *
 *  B-field   BiCubicSplineInterpolatorWithBiLinearBackup.interpolateDisplacements
 *            (S/iareas/BiCubicSplineInterpolatorWithBiLinearBackup.java:57-107, 224-249):
 *            commons-math3 BicubicSplineInterpolator = natural cubic splines along each
 *            grid line give the first derivatives at the knots, central finite
 *            differences (one-sided at the border) give the cross derivative, and each
 *            grid cell is a bicubic Hermite patch; pixel coordinates are clamped to the
 *            tile-centre box.
 *  B-inherit AdaptiveInterVelocityInheritanceStrategyBiCubicSpline
 *            (S/iareas/AdaptiveInterVelocityInheritanceStrategyBiCubicSpline.java:27-136):
 *            commons-math3 PiecewiseBicubicSplineInterpolator = for every evaluation a
 *            5x5 knot window around the point, Akima splines (Akima 1970) along the first
 *            coordinate for each of the 5 second-coordinate knots, then one along the
 *            second coordinate; end derivatives from the parabola through 3 knots.
 *            The Direct / Area / Distance strategies are in qlpiv_oracle_inherit.c.
 *  B-warp    BiLinearImageWarpingStrategy.doBiLinearWarp / warpPixelOnImage
 *            (S/images/BiLinearImageWarpingStrategy.java:143-265), BothImages mode: the
 *            field is halved, image A sampled at (i-u, j-v), image B at (i+u, j+v).
 *  A-accum   Tile.accumulateDisplacement (S/iareas/Tile.java:103-136), clipping mode
 *            AllowedOutOfBoundClipping (the UI converter's default).
 *  A-loop    LocalPIVOpenCLGpuJob (S/jobs/LocalPIVOpenCLGpuJob.java:188-411) with
 *            SimpleStrategy (one correlation per level); optionally the multi-peak
 *            normalised-median validation after every level (qlpiv_oracle_validate.c).
 *
 * The reference evaluates both interpolators in double.  The FP32 pipeline here
 * evaluates them in float (spline knot derivatives solved in double-word arithmetic with
 * precomputed reciprocals of the knot steps, then rounded to float), the formulation of
 * the CUDA kernels, so the GPU stages can be checked bit for bit; the FP64 twin evaluates
 * them in double with the divisions of the mathematical definition.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_dword.h"
#include "oracle_types.h"

/* ---------------- natural cubic spline: first derivative at every knot ---------------- */
static void natural_spline_deriv(const double *x, const double *y, long ys, int n, double *d) {
    /* second derivatives m[0] = m[n-1] = 0, tridiagonal solve (Thomas) */
    double *m = (double *)calloc((size_t)n, sizeof(double));
    double *cp = (double *)calloc((size_t)n, sizeof(double));
    double *dp = (double *)calloc((size_t)n, sizeof(double));
    for (int i = 1; i < n - 1; i++) {
        const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
        const double a = h0, b = 2.0 * (h0 + h1), c = h1;
        const double r = 6.0 * ((y[(i + 1) * ys] - y[i * ys]) / h1 - (y[i * ys] - y[(i - 1) * ys]) / h0);
        const double den = b - a * cp[i - 1];
        cp[i] = c / den;
        dp[i] = (r - a * dp[i - 1]) / den;
    }
    for (int i = n - 2; i >= 1; i--) m[i] = dp[i] - cp[i] * m[i + 1];
    for (int i = 0; i < n - 1; i++) {
        const double h = x[i + 1] - x[i];
        d[i] = (y[(i + 1) * ys] - y[i * ys]) / h - h * (2.0 * m[i] + m[i + 1]) / 6.0;
    }
    {
        const double h = x[n - 1] - x[n - 2];
        d[n - 1] = (y[(n - 1) * ys] - y[(n - 2) * ys]) / h + h * (m[n - 2] + 2.0 * m[n - 1]) / 6.0;
    }
    free(m); free(cp); free(dp);
}

/* The float path's formulation of the same solve (the CUDA kernels'): per-axis factors computed
 * once per grid in double, kf holding 6 arrays of n:
 *   h[i] = x[i+1] - x[i], ih[i] = 1 / h[i], h6[i] = h[i] / 6                        (i < n-1)
 *   den[i] = 2 (h[i-1] + h[i]) - h[i-1] cp[i-1], cp[i] = h[i] / den[i], iden[i] = 1 / den[i]
 *   rc[i] = 1 / (x[min(i+1, n-1)] - x[max(i-1, 0)])                 (cross-derivative steps)
 * rounded to double-words, and line solves that multiply by them in double-word arithmetic
 * (oracle_dword.h, ~44 bits), each derivative rounded to float. */
enum { KF_H = 0, KF_IH, KF_H6, KF_CP, KF_IDEN, KF_RC, KF_ARRAYS };

static void knot_factors(const double *x, int n, double *kf) {
    double *h = kf + KF_H * n, *ih = kf + KF_IH * n, *h6 = kf + KF_H6 * n;
    double *cp = kf + KF_CP * n, *iden = kf + KF_IDEN * n, *rc = kf + KF_RC * n;
    for (int k = 0; k < KF_ARRAYS * n; k++) kf[k] = 0.0;
    for (int i = 0; i + 1 < n; i++) {
        h[i] = x[i + 1] - x[i];
        ih[i] = 1.0 / h[i];
        h6[i] = h[i] / 6.0;
    }
    for (int i = 1; i + 1 < n; i++) {
        const double den = 2.0 * (h[i - 1] + h[i]) - h[i - 1] * cp[i - 1];
        cp[i] = h[i] / den;
        iden[i] = 1.0 / den;
    }
    for (int i = 0; i < n; i++) {
        const int nx = i + 1 < n ? i + 1 : n - 1, pv = i - 1 >= 0 ? i - 1 : 0;
        rc[i] = 1.0 / (x[nx] - x[pv]);
    }
}

static orc_dw *knot_factors_dw(const double *x, int n) {
    double *kf = (double *)malloc(sizeof(double) * KF_ARRAYS * (size_t)n);
    orc_dw *out = (orc_dw *)malloc(sizeof(orc_dw) * KF_ARRAYS * (size_t)n);
    knot_factors(x, n, kf);
    for (int k = 0; k < KF_ARRAYS * n; k++) out[k] = dw_of(kf[k]);
    free(kf);
    return out;
}

/* Values y (float) along one line with stride ys:
 *   s[i]  = (y[i+1] - y[i]) ih[i]          (the float difference is exact as a double-word)
 *   m[i]  = dp[i] = (6 (s[i] - s[i-1]) - h[i-1] dp[i-1]) iden[i],   dp[0] = 0
 *   m[i]  = dp[i] - cp[i] m[i+1],   m[0] = m[n-1] = 0
 *   d[i]  = s[i] - h6[i] (2 m[i] + m[i+1]),   d[n-1] = s[n-2] + h6[n-2] (m[n-2] + 2 m[n-1]) */
static void natural_spline_deriv_dw(const orc_dw *kf, const float *y, long ys, int n, float *d) {
    const orc_dw *h = kf + KF_H * n, *ih = kf + KF_IH * n, *h6 = kf + KF_H6 * n;
    const orc_dw *cp = kf + KF_CP * n, *iden = kf + KF_IDEN * n;
    const orc_dw zero = {0.0f, 0.0f};
    orc_dw *m = (orc_dw *)calloc((size_t)n, sizeof(orc_dw));
    orc_dw *s = (orc_dw *)calloc((size_t)n, sizeof(orc_dw));
    for (int i = 0; i + 1 < n; i++) s[i] = dw_mul(dw_two_sum(y[(i + 1) * ys], -y[i * ys]), ih[i]);
    for (int i = 1; i < n - 1; i++)
        m[i] = dw_mul(dw_sub(dw_mul_f(dw_sub(s[i], s[i - 1]), 6.0f), dw_mul(h[i - 1], m[i - 1])), iden[i]);
    for (int i = n - 2; i >= 1; i--) m[i] = dw_sub(m[i], dw_mul(cp[i], m[i + 1]));
    m[0] = zero;
    m[n - 1] = zero;
    for (int i = 0; i < n - 1; i++) d[i] = dw_float(dw_sub(s[i], dw_mul(h6[i], dw_add(dw_twice(m[i]), m[i + 1]))));
    d[n - 1] = dw_float(dw_add(s[n - 2], dw_mul(h6[n - 2], dw_add(m[n - 2], dw_twice(m[n - 1])))));
    free(m); free(s);
}

/* Float path of bicubic_nodes: f and the node quadruples in float. */
static void bicubic_nodes_dw(const double *ys, int ni, const double *xs, int nj, const float *f, float *c4) {
    const size_t nn = (size_t)ni * nj;
    orc_dw *kfy = knot_factors_dw(ys, ni), *kfx = knot_factors_dw(xs, nj);
    float *tmp = (float *)malloc(sizeof(float) * (ni > nj ? ni : nj));
    for (size_t k = 0; k < nn; k++) c4[4 * k] = f[k];
    for (int j = 0; j < nj; j++) {
        natural_spline_deriv_dw(kfy, f + j, nj, ni, tmp);
        for (int i = 0; i < ni; i++) c4[4 * ((size_t)i * nj + j) + 1] = tmp[i];
    }
    for (int i = 0; i < ni; i++) {
        natural_spline_deriv_dw(kfx, f + (size_t)i * nj, 1, nj, tmp);
        for (int j = 0; j < nj; j++) c4[4 * ((size_t)i * nj + j) + 2] = tmp[j];
    }
    for (int i = 0; i < ni; i++) {
        const int ni_ = i + 1 < ni ? i + 1 : ni - 1, pi = i - 1 >= 0 ? i - 1 : 0;
        for (int j = 0; j < nj; j++) {
            const int nj_ = j + 1 < nj ? j + 1 : nj - 1, pj = j - 1 >= 0 ? j - 1 : 0;
            orc_dw t = dw_two_sum(f[(size_t)ni_ * nj + nj_], -f[(size_t)ni_ * nj + pj]);
            t = dw_add_f(t, -f[(size_t)pi * nj + nj_]);
            t = dw_add_f(t, f[(size_t)pi * nj + pj]);
            c4[4 * ((size_t)i * nj + j) + 3] = dw_float(dw_mul(dw_mul(t, kfy[KF_RC * ni + i]), kfx[KF_RC * nj + j]));
        }
    }
    free(tmp); free(kfy); free(kfx);
}

/* Node quadruples (f, fy, fx, fyx) of the bicubic spline surface through f (ni x nj) at
 * knots ys x xs, in double (the FP64 twin): natural-spline knot derivatives along each grid
 * line and central-difference cross derivatives (one-sided at the border). */
static void bicubic_nodes(const double *ys, int ni, const double *xs, int nj, const double *f, double *c4) {
    const size_t nn = (size_t)ni * nj;
    double *tmp = (double *)malloc(sizeof(double) * (ni > nj ? ni : nj));
    for (size_t k = 0; k < nn; k++) c4[4 * k] = f[k];
    for (int j = 0; j < nj; j++) {            /* along the first coordinate, per column */
        natural_spline_deriv(ys, f + j, nj, ni, tmp);
        for (int i = 0; i < ni; i++) c4[4 * ((size_t)i * nj + j) + 1] = tmp[i];
    }
    for (int i = 0; i < ni; i++) {            /* along the second coordinate, per row */
        natural_spline_deriv(xs, f + (size_t)i * nj, 1, nj, tmp);
        for (int j = 0; j < nj; j++) c4[4 * ((size_t)i * nj + j) + 2] = tmp[j];
    }
    for (int i = 0; i < ni; i++) {
        const int ni_ = i + 1 < ni ? i + 1 : ni - 1, pi = i - 1 >= 0 ? i - 1 : 0;
        for (int j = 0; j < nj; j++) {
            const int nj_ = j + 1 < nj ? j + 1 : nj - 1, pj = j - 1 >= 0 ? j - 1 : 0;
            c4[4 * ((size_t)i * nj + j) + 3] =
                (f[(size_t)ni_ * nj + nj_] - f[(size_t)ni_ * nj + pj] - f[(size_t)pi * nj + nj_] + f[(size_t)pi * nj + pj]) /
                ((ys[ni_] - ys[pi]) * (xs[nj_] - xs[pj]));
        }
    }
    free(tmp);
}

#define REAL float
#define SUFFIX _f32
#include "oracle_interp_impl.h"
#undef REAL
#undef SUFFIX

#define REAL double
#define SUFFIX _f64
#include "oracle_interp_impl.h"
#undef REAL
#undef SUFFIX

/* ---------------- warp ---------------- */
static float read_pix(const void *img, int pix_bytes, int w, int y, int x) {
    return pix_bytes == 1 ? (float)((const uint8_t *)img)[(size_t)y * w + x]
                          : (float)((const uint16_t *)img)[(size_t)y * w + x];
}

static int java_round(float x) { return (int)floorf(x + 0.5f); }

/* warpPixelOnImage (BiLinearImageWarpingStrategy.java:185-265) */
static float warp_pixel(const void *img, int pix_bytes, int h, int w, float u, float v, int i, int j, int first) {
    float sI = first ? (float)i - u : (float)i + u;
    float sJ = first ? (float)j - v : (float)j + v;
    int pI = (int)(short)java_round(sI), pJ = (int)(short)java_round(sJ);
    if (pI < 0) { sI = 0.0f; pI = 0; }
    else if (pI >= h) { sI = (float)(h - 1); pI = h - 1; }
    if (pJ < 0) { sJ = 0.0f; pJ = 0; }
    else if (pJ >= w) { sJ = (float)(w - 1); pJ = w - 1; }
    const float dU = sI - (float)pI, dV = sJ - (float)pJ;
    int oI = dU >= 0.0f ? 1 : -1, oJ = dV >= 0.0f ? 1 : -1;
    if (oI + pI < 0 || oI + pI >= h) oI = 0;
    if (oJ + pJ < 0 || oJ + pJ >= w) oJ = 0;
    const float wU = fabsf(dU), wV = fabsf(dV);
    const float tl = read_pix(img, pix_bytes, w, pI, pJ);
    const float tr = read_pix(img, pix_bytes, w, pI, pJ + oJ);
    const float bl = read_pix(img, pix_bytes, w, pI + oI, pJ);
    const float br = read_pix(img, pix_bytes, w, pI + oI, pJ + oJ);
    const float a = (1.0f - wU) * (1.0f - wV) * tl;
    const float b = (1.0f - wU) * wV * tr;
    const float c = wU * (1.0f - wV) * bl;
    const float d = wU * wV * br;
    const float fv = a + b + c + d;
    return (float)java_round(fv);
}

/* Stores a warped value as MatrixByte/MatrixInt16.setElement(float) would.  The reference's
 * 16-bit matrix narrows through a signed byte (S/MatrixInt16.java:95-101); int16_quirk = 1
 * reproduces that, 0 stores the rounded 16-bit value. */
static void store_pix(void *img, int pix_bytes, int w, int y, int x, float v, int int16_quirk) {
    const int r = java_round(v);
    if (pix_bytes == 1) {
        ((uint8_t *)img)[(size_t)y * w + x] = (uint8_t)(int8_t)r;
    } else if (int16_quirk) {
        ((uint16_t *)img)[(size_t)y * w + x] = (uint16_t)(int16_t)(int8_t)r;
    } else {
        ((uint16_t *)img)[(size_t)y * w + x] = (uint16_t)r;
    }
}

/* Exported pieces (ctypes) ------------------------------------------------------- */

/* Per-pixel field of one level: tile displacements u, v (ni x nj, row-major) at tile
 * centres ys[ni], xs[nj] -> fu, fv (h x w float).  Coordinates clamped to the centre box.
 * precision 0: the surface is evaluated in float (the CUDA formulation); 1: in double. */
/* Pixel (i, j) is evaluated at (off_y + i, off_x + j): interpolateDisplacements(height, width,
 * offsetY, offsetX) (S/iareas/BiCubicSplineInterpolatorWithBiLinearBackup.java:108-160). */
void orc_displacement_field_off(const double *ys, int ni, const double *xs, int nj, const float *u, const float *v,
                                int h, int w, int precision, float off_y, float off_x, float *fu, float *fv) {
    const size_t nn = (size_t)ni * nj;
    double *du = (double *)malloc(nn * sizeof(double)), *dv = (double *)malloc(nn * sizeof(double));
    double *cu = (double *)malloc(4 * nn * sizeof(double)), *cv = (double *)malloc(4 * nn * sizeof(double));
    for (size_t k = 0; k < nn; k++) { du[k] = u[k]; dv[k] = v[k]; }
    const float ymin = (float)ys[0], ymax = (float)ys[ni - 1], xmin = (float)xs[0], xmax = (float)xs[nj - 1];
    float *fcu = (float *)malloc(4 * nn * sizeof(float)), *fcv = (float *)malloc(4 * nn * sizeof(float));
    float *fys = (float *)malloc(ni * sizeof(float)), *fxs = (float *)malloc(nj * sizeof(float));
    if (precision == 0) {
        bicubic_nodes_dw(ys, ni, xs, nj, u, fcu);
        bicubic_nodes_dw(ys, ni, xs, nj, v, fcv);
    } else {
        bicubic_nodes(ys, ni, xs, nj, du, cu);
        bicubic_nodes(ys, ni, xs, nj, dv, cv);
    }
    for (int i = 0; i < ni; i++) fys[i] = (float)ys[i];
    for (int j = 0; j < nj; j++) fxs[j] = (float)xs[j];
    for (int i = 0; i < h; i++) {
        float y = off_y + (float)i;
        if (y < ymin) y = ymin; else if (y > ymax) y = ymax;
        for (int j = 0; j < w; j++) {
            float x = off_x + (float)j;
            if (x < xmin) x = xmin; else if (x > xmax) x = xmax;
            if (precision == 0) {
                fu[(size_t)i * w + j] = bicubic_value_f32(fys, ni, fxs, nj, fcu, y, x);
                fv[(size_t)i * w + j] = bicubic_value_f32(fys, ni, fxs, nj, fcv, y, x);
            } else {
                fu[(size_t)i * w + j] = (float)bicubic_value_f64(ys, ni, xs, nj, cu, (double)y, (double)x);
                fv[(size_t)i * w + j] = (float)bicubic_value_f64(ys, ni, xs, nj, cv, (double)y, (double)x);
            }
        }
    }
    free(du); free(dv); free(cu); free(cv); free(fcu); free(fcv); free(fys); free(fxs);
}

void orc_displacement_field(const double *ys, int ni, const double *xs, int nj, const float *u, const float *v, int h,
                            int w, int precision, float *fu, float *fv) {
    orc_displacement_field_off(ys, ni, xs, nj, u, v, h, w, precision, 0.0f, 0.0f, fu, fv);
}

/* BothImages bilinear warp of a pair with a per-pixel field (halved inside). */
/* image_mode: 3 BothImages (both frames, half the field), 1 FirstImage (frame A, whole field),
 * 2 SecondImage (frame B, whole field) -- BiLinearImageWarpingStrategy.doBiLinearWarp
 * (S/images/BiLinearImageWarpingStrategy.java:143-183).  The frame that is not warped is copied. */
void orc_warp_full(const void *img_a, const void *img_b, int h, int w, int pix_bytes, const float *fu, const float *fv,
                   int int16_quirk, int image_mode, void *out_a, void *out_b) {
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            float u = fu[(size_t)i * w + j], v = fv[(size_t)i * w + j];
            if (image_mode == 3) {
                u /= 2.0f;
                v /= 2.0f;
            }
            const size_t off = ((size_t)i * w + j) * pix_bytes;
            if (image_mode & 1)
                store_pix(out_a, pix_bytes, w, i, j, warp_pixel(img_a, pix_bytes, h, w, u, v, i, j, 1), int16_quirk);
            else
                memcpy((char *)out_a + off, (const char *)img_a + off, pix_bytes);
            if (image_mode & 2)
                store_pix(out_b, pix_bytes, w, i, j, warp_pixel(img_b, pix_bytes, h, w, u, v, i, j, 0), int16_quirk);
            else
                memcpy((char *)out_b + off, (const char *)img_b + off, pix_bytes);
        }
}

void orc_warp_both(const void *img_a, const void *img_b, int h, int w, int pix_bytes, const float *fu, const float *fv,
                   int int16_quirk, void *out_a, void *out_b) {
    orc_warp_full(img_a, img_b, h, w, pix_bytes, fu, fv, int16_quirk, 3, out_a, out_b);
}

/* Micro / mini per-tile warping (BiLinearImageMicroAndMiniWarpingStrategy.warpAndClipImage,
 * S/images/BiLinearImageMicroAndMiniWarpingStrategy.java:39-186, createMicroDisplacements :188-202,
 * createMiniDisplacements :204-290, doBiLinearWarp :292-336, warpPixelOnImage :338-407) of the
 * tiles of one level (grid tops[ni] x lefts[nj], side n, tile displacements cu/cv row-major).
 * image_mode: 1 first image, 2 second image, 3 both; mini: 0 micro (the tile's fractional
 * displacement everywhere), 1 mini (bicubic spline over the tile's up to 7 x 7 neighbours, values
 * relative to floor of the tile's displacement, evaluated over the tile region of the displaced B
 * tile).  Warped tiles keep the full-scale maximum `full_max`; clipped tiles their own maximum
 * (floor 16).  Outputs: count x n x n float tiles and per-tile maxima. */
static void mini_field(const int *tops, const int *lefts, int ni, int nj, int n, const float *cu, const float *cv,
                       int ti, int tj, int eval_top, int eval_left, float *fu, float *fv) {
    const int R = 7, r2 = R / 2;
    const int i0 = ti - r2 < 0 ? 0 : ti - r2, i1 = ti + r2 > ni - 1 ? ni - 1 : ti + r2;
    const int j0 = tj - r2 < 0 ? 0 : tj - r2, j1 = tj + r2 > nj - 1 ? nj - 1 : tj + r2;
    const int di = i1 - i0 + 1, dj = j1 - j0 + 1;
    double ys[7], xs[7];
    float us[49], vs[49];
    const long kc = (long)ti * nj + tj;
    const double fu0 = floor((double)cu[kc]), fv0 = floor((double)cv[kc]);
    for (int i = 0; i < di; i++) ys[i] = (double)((float)tops[i0 + i] + (float)n / 2.0f - 0.5f);
    for (int j = 0; j < dj; j++) xs[j] = (double)((float)lefts[j0 + j] + (float)n / 2.0f - 0.5f);
    for (int i = 0; i < di; i++)
        for (int j = 0; j < dj; j++) {
            const long k = (long)(i0 + i) * nj + (j0 + j);
            us[i * dj + j] = (float)((double)cu[k] - fu0);
            vs[i * dj + j] = (float)((double)cv[k] - fv0);
        }
    orc_displacement_field_off(ys, di, xs, dj, us, vs, n, n, 0, (float)eval_top, (float)eval_left, fu, fv);
}

void orc_tile_warp(const void *img_a, const void *img_b, int h, int w, int pix_bytes, int n, int ni, int nj,
                   const int *tops, const int *lefts, const float *cu, const float *cv, int image_mode, int mini,
                   float full_max, float *tiles_a, float *tiles_b, float *max_a, float *max_b) {
    float *fu = (float *)malloc(sizeof(float) * n * n), *fv = (float *)malloc(sizeof(float) * n * n);
    for (int ti = 0; ti < ni; ti++)
        for (int tj = 0; tj < nj; tj++) {
            const long k = (long)ti * nj + tj;
            float *ta = tiles_a + k * n * n, *tb = tiles_b + k * n * n;
            const int top = tops[ti], left = lefts[tj];
            const float du = cu[k], dv = cv[k];
            const double flu = floor((double)du), flv = floor((double)dv);
            const double flu2 = floor((double)(du / 2.0f)), flv2 = floor((double)(dv / 2.0f));
            const int topRefB = (int)(short)((double)top + flu), leftRefB = (int)(short)((double)left + flv);
            /* the pixel displacements of the tile region */
            if (mini) {
                mini_field(tops, lefts, ni, nj, n, cu, cv, ti, tj, topRefB, leftRefB, fu, fv);
            } else {
                const float mu = du - (float)flu, mv = dv - (float)flv;
                for (int q = 0; q < n * n; q++) { fu[q] = mu; fv[q] = mv; }
            }
            /* image A */
            if (image_mode == 2) {
                max_a[k] = orc_clip_tile(img_a, h, w, pix_bytes, top, left, n, ta);
            } else {
                int topA, leftA;
                float uo = 0.0f, vo = 0.0f;
                if (image_mode == 1) {
                    topA = (int)(short)((double)top - flu);
                    leftA = (int)(short)((double)left - flv);
                } else {
                    topA = (int)(short)((double)top - flu2);
                    leftA = (int)(short)((double)left - flv2);
                    uo = (float)((double)(du / 2.0f) - flu2) - (float)((double)du - flu);
                    vo = (float)((double)(dv / 2.0f) - flv2) - (float)((double)dv - flv);
                }
                for (int i = 0; i < n; i++)
                    for (int j = 0; j < n; j++) {
                        float u = fu[i * n + j], v = fv[i * n + j];
                        if (image_mode == 3) {
                            u = u / 2.0f + uo;
                            v = v / 2.0f + vo;
                        }
                        ta[i * n + j] = warp_pixel(img_a, pix_bytes, h, w, u, v, (int)(short)(i + topA),
                                                   (int)(short)(j + leftA), 1);
                    }
                max_a[k] = full_max;
            }
            /* image B */
            if (image_mode == 1) {
                max_b[k] = orc_clip_tile(img_b, h, w, pix_bytes, top, left, n, tb);
            } else {
                int topB, leftB;
                float uo = 0.0f, vo = 0.0f;
                if (image_mode == 2) {
                    topB = topRefB;
                    leftB = leftRefB;
                } else {
                    topB = (int)(short)((double)top + flu2);
                    leftB = (int)(short)((double)left + flv2);
                    uo = (float)((double)(du / 2.0f) - flu2);
                    vo = (float)((double)(dv / 2.0f) - flv2);
                }
                for (int i = 0; i < n; i++)
                    for (int j = 0; j < n; j++) {
                        float u = fu[i * n + j], v = fv[i * n + j];
                        if (image_mode == 3) {
                            u = u / 2.0f + uo;
                            v = v / 2.0f + vo;
                        }
                        tb[i * n + j] = warp_pixel(img_b, pix_bytes, h, w, u, v, (int)(short)(i + topB),
                                                   (int)(short)(j + leftB), 0);
                    }
                max_b[k] = full_max;
            }
        }
    free(fu);
    free(fv);
}

/* Inherited displacement of child tiles at centres (cy[ci], cx[cj]) from parent tiles
 * (pu, pv at centres py[pi], px[pj]), clamped to the parent box; needs >= 5 parent
 * tiles per axis, otherwise nothing is inherited (the reference computes a bilinear
 * value in that case but does not apply it).  precision 0: Akima splines in float (the
 * CUDA formulation); 1: in double. */
void orc_inherit(const double *py, int pni, const double *px, int pnj, const float *pu, const float *pv, const float *cy,
                 int cni, const float *cx, int cnj, int round_int, int precision, float *cu, float *cv) {
    if (pni < 5 || pnj < 5) {
        memset(cu, 0, sizeof(float) * cni * cnj);
        memset(cv, 0, sizeof(float) * cni * cnj);
        return;
    }
    const size_t nn = (size_t)pni * pnj;
    double *du = (double *)malloc(nn * sizeof(double)), *dv = (double *)malloc(nn * sizeof(double));
    float *fpy = (float *)malloc(pni * sizeof(float)), *fpx = (float *)malloc(pnj * sizeof(float));
    for (size_t k = 0; k < nn; k++) { du[k] = pu[k]; dv[k] = pv[k]; }
    for (int i = 0; i < pni; i++) fpy[i] = (float)py[i];
    for (int j = 0; j < pnj; j++) fpx[j] = (float)px[j];
    const float ymin = (float)py[0], ymax = (float)py[pni - 1], xmin = (float)px[0], xmax = (float)px[pnj - 1];
    for (int i = 0; i < cni; i++) {
        float y = cy[i];
        if (y < ymin) y = ymin; else if (y > ymax) y = ymax;
        for (int j = 0; j < cnj; j++) {
            float x = cx[j];
            if (x < xmin) x = xmin; else if (x > xmax) x = xmax;
            float iu, iv;
            if (precision == 0) {
                iu = akima2d_value_f32(fpy, pni, fpx, pnj, pu, y, x);
                iv = akima2d_value_f32(fpy, pni, fpx, pnj, pv, y, x);
            } else {
                iu = (float)akima2d_value_f64(py, pni, px, pnj, du, (double)y, (double)x);
                iv = (float)akima2d_value_f64(py, pni, px, pnj, dv, (double)y, (double)x);
            }
            /* Tile.accumulateDisplacement on a reset tile: 0 + value, rounded first for
             * non-warping modes (FastMath.round(float)) */
            cu[(size_t)i * cnj + j] = 0.0f + (round_int ? (float)java_round(iu) : iu);
            cv[(size_t)i * cnj + j] = 0.0f + (round_int ? (float)java_round(iv) : iv);
        }
    }
    free(du); free(dv); free(fpy); free(fpx);
}

/* Adaptive multi-pass PIV with BothImages bilinear warping (SimpleStrategy); SuperPosition grids
 * from level sp_start on, NoSuperPosition grids before (0: SuperPosition throughout).
 * Level L uses IA n_start >> L.  warp_mode 1 = BothImages bilinear warping, 0 = no
 * warping (B tiles displaced by the rounded inherited displacement).  Tile maxima are
 * fixed_max when > 0 (full-image-warp tiles: 255 / 65535), else the tile max.
 * Outputs the last level's displacement (u rows, v columns) and, optionally, every
 * level's vectors concatenated (level_vectors, sized by the caller). */
int orc_piv_adaptive_ex(const void *img_a, const void *img_b, int h, int w, int pix_bytes, int n_start, int n_end,
                        float overlap_factor, int warp_mode, int inherit_mode, int clip_mode, int norm_mode,
                        float fixed_max, int int16_quirk, int precision, int nthreads, const orc_valid_cfg *val,
                        float *out_u, float *out_v, int *out_ni, int *out_nj, orc_vector *level_vectors,
                        float *level_uv, unsigned char *level_invalid, int sp_start, int stab_retries,
                        float stab_max) {
    const int validate = val != NULL && val->enabled;
    /* the multi-peak model searches num_peaks peaks (FindMaximumMultiPeaks); the other models keep
     * FindMaximumFromCenter and one validation strategy */
    const int multi = validate && val->model <= 1;
    const int kpk = validate ? (multi ? val->num_peaks : 1) : 0;
    /* ClippingModeEnum: 2 = NoOutOfBoundClipping (Tile.accumulateDisplacement / replaceDisplacement
     * refuse displacements that move a tile out of the image) */
    const int clip = clip_mode == 2;
    if (validate && (kpk < 1 || kpk > 64 || (multi && val->kernel_width < 1))) return -2;
    int levels = 0;
    for (int n = n_start; n >= n_end; n >>= 1) levels++;
    const int cap = 65536;
    int *tops = (int *)malloc(sizeof(int) * cap), *lefts = (int *)malloc(sizeof(int) * cap);
    int *ptops = (int *)malloc(sizeof(int) * cap), *plefts = (int *)malloc(sizeof(int) * cap);
    float *pu = NULL, *pv = NULL;
    int pni = 0, pnj = 0, pn = 0;
    const size_t ib = (size_t)h * w * pix_bytes;
    void *wa = malloc(ib), *wb = malloc(ib);
    float *fu = (float *)malloc(sizeof(float) * h * w), *fv = (float *)malloc(sizeof(float) * h * w);
    long vec_off = 0;
    int rc = 0;
    for (int lv = 0; lv < levels; lv++) {
        /* the mixed division (AdaptiveInterAreaStrategyMixedSuperPosition.java:31-92): NoSuperPosition
         * before sp_start, then SuperPosition restarted with IA n_start >> sp_start */
        orc_grid g;
        const int grc = lv < sp_start
                            ? orc_grid_nosuperposition(h, w, 0, 0, 0, 0, n_start, lv, &g, tops, lefts, cap)
                            : orc_grid_superposition(h, w, 0, 0, 0, 0, n_start >> sp_start, lv - sp_start,
                                                     overlap_factor, &g, tops, lefts, cap);
        if (grc != 0) {
            rc = -1;
            break;
        }
        const int n = g.n, ni = g.tiles_i, nj = g.tiles_j;
        const long cnt = (long)ni * nj;
        float *cu = (float *)calloc((size_t)cnt, sizeof(float)), *cv = (float *)calloc((size_t)cnt, sizeof(float));
        double *cyd = (double *)malloc(sizeof(double) * ni), *cxd = (double *)malloc(sizeof(double) * nj);
        float *cyf = (float *)malloc(sizeof(float) * ni), *cxf = (float *)malloc(sizeof(float) * nj);
        for (int i = 0; i < ni; i++) { cyf[i] = (float)tops[i] + (float)n / 2.0f - 0.5f; cyd[i] = cyf[i]; }
        for (int j = 0; j < nj; j++) { cxf[j] = (float)lefts[j] + (float)n / 2.0f - 0.5f; cxd[j] = cxf[j]; }
        const void *sa = img_a, *sb = img_b;
        /* warp_mode: 0 none, 1 BothImages full-image bilinear, 4/5/6 First/Second/Both micro,
         * 7/8/9 First/Second/Both mini */
        const int per_tile = warp_mode >= 4 && warp_mode <= 9;
        float *wta = NULL, *wtb = NULL, *wma = NULL, *wmb = NULL;
        if (lv > 0) {
            double *pyd = (double *)malloc(sizeof(double) * pni), *pxd = (double *)malloc(sizeof(double) * pnj);
            for (int i = 0; i < pni; i++) pyd[i] = (double)((float)ptops[i] + (float)pn / 2.0f - 0.5f);
            for (int j = 0; j < pnj; j++) pxd[j] = (double)((float)plefts[j] + (float)pn / 2.0f - 0.5f);
            if (inherit_mode == 0) {
                orc_inherit(pyd, pni, pxd, pnj, pu, pv, cyf, ni, cxf, nj, warp_mode == 0, precision, cu, cv);
            } else if (orc_inherit_tiles(inherit_mode, pn, pni, pnj, ptops, plefts, pu, pv, n, ni, nj, tops, lefts,
                                         warp_mode == 0, cu, cv) != 0) {
                free(pyd); free(pxd); free(cu); free(cv); free(cyd); free(cxd); free(cyf); free(cxf);
                rc = -3;
                break;
            }
            free(pyd); free(pxd);
            if (clip)  /* the new tiles take the inherited value through accumulateDisplacement */
                for (int i = 0; i < ni; i++)
                    for (int j = 0; j < nj; j++) {
                        const size_t k = (size_t)i * nj + j;
                        const float nu = 0.0f + cu[k], nv = 0.0f + cv[k];
                        const int ok = orc_clip_ok(n, h, w, tops[i], lefts[j], nu, nv);
                        cu[k] = ok ? nu : 0.0f;
                        cv[k] = ok ? nv : 0.0f;
                    }
            if (per_tile) {
                wta = (float *)malloc(sizeof(float) * cnt * n * n);
                wtb = (float *)malloc(sizeof(float) * cnt * n * n);
                wma = (float *)malloc(sizeof(float) * cnt);
                wmb = (float *)malloc(sizeof(float) * cnt);
                const float full = fixed_max > 0.0f ? fixed_max : (pix_bytes == 1 ? 255.0f : 65535.0f);
                orc_tile_warp(img_a, img_b, h, w, pix_bytes, n, ni, nj, tops, lefts, cu, cv, (warp_mode - 4) % 3 + 1,
                              warp_mode >= 7, full, wta, wtb, wma, wmb);
            }
            if (warp_mode >= 1 && warp_mode <= 3) {
                orc_displacement_field(cyd, ni, cxd, nj, cu, cv, h, w, precision, fu, fv);
                orc_warp_full(img_a, img_b, h, w, pix_bytes, fu, fv, int16_quirk,
                              warp_mode == 1 ? 3 : (warp_mode == 2 ? 1 : 2), wa, wb);
                sa = wa; sb = wb;
            }
        }
        int *at = (int *)malloc(sizeof(int) * cnt), *al = (int *)malloc(sizeof(int) * cnt);
        int *bt = (int *)malloc(sizeof(int) * cnt), *bl = (int *)malloc(sizeof(int) * cnt);
        for (int i = 0; i < ni; i++)
            for (int j = 0; j < nj; j++) {
                const size_t k = (size_t)i * nj + j;
                at[k] = tops[i];
                al[k] = lefts[j];
                /* NoImageWarpingStrategy: B tile at round(top + u), round(left + v) */
                bt[k] = warp_mode == 0 ? java_round((float)tops[i] + cu[k]) : tops[i];
                bl[k] = warp_mode == 0 ? java_round((float)lefts[j] + cv[k]) : lefts[j];
            }
        float fm = fixed_max > 0.0f && !per_tile ? fixed_max : 0.0f, fma = fm, fmb = fm;
        int nm = fixed_max > 0.0f && !per_tile ? 2 : norm_mode;
        if (fm > 0.0f && (warp_mode == 2 || warp_mode == 3)) {
            /* FirstImage / SecondImage: the tiles cut from the warped (level 0: whole) frame keep the
             * fixed maximum, the tiles clipped from the other frame their own (Image.clipImageMatrix) */
            nm = norm_mode | 8;
            fma = warp_mode == 2 ? fm : 0.0f;
            fmb = warp_mode == 3 ? fm : 0.0f;
        }
        orc_vector *vec = (orc_vector *)malloc(sizeof(orc_vector) * cnt);
        orc_vector *mvec = NULL;
        int *npk = NULL;
        if (multi) {
            /* FindMaximumMultiPeaks (the finder the multi-peak validation model selects) */
            mvec = (orc_vector *)malloc(sizeof(orc_vector) * cnt * kpk);
            npk = (int *)malloc(sizeof(int) * cnt);
            if (wta)
                orc_tiles_pass(wta, wtb, wma, wmb, cnt, n, norm_mode, 1, precision, val->kernel_width, kpk, mvec, npk);
            else
                orc_piv_pass_multi(sa, sb, h, w, pix_bytes, n, cnt, at, al, bt, bl, nm, fma, fmb, 1, precision,
                                   val->kernel_width, kpk, mvec, npk, nthreads);
            for (long k = 0; k < cnt; k++) vec[k] = mvec[k * kpk];
        } else if (wta) {
            orc_tiles_pass(wta, wtb, wma, wmb, cnt, n, norm_mode, 1, precision, 0, 0, vec, NULL);
        } else {
            orc_piv_pass(sa, sb, h, w, pix_bytes, n, cnt, at, al, bt, bl, nm, fma, fmb, 1, precision, vec, nthreads);
        }
        free(wta); free(wtb); free(wma); free(wmb);
        if (level_vectors) memcpy(level_vectors + vec_off, vec, sizeof(orc_vector) * cnt);
        for (long k = 0; k < cnt; k++) {
            float nu, nv;
            if (precision == 0) { nu = cu[k] + vec[k].u; nv = cv[k] + vec[k].v; }
            else { nu = (float)((double)cu[k] + vec[k].u64); nv = (float)((double)cv[k] + vec[k].v64); }
            /* Tile.accumulateDisplacement drops an increment that moves the tile out of the image */
            if (!clip || orc_clip_ok(n, h, w, tops[k / nj], lefts[k % nj], nu, nv)) { cu[k] = nu; cv[k] = nv; }
        }
        if (stab_retries > 1) {
            /* InterAreaDisplacementStableStrategy (S/iareas/InterAreaDisplacementStableStrategy.java:19-36)
             * in the loop of S/jobs/LocalPIVOpenCLGpuJob.java:233-405: pass r re-warps with every
             * tile's current displacement (not at the first level), correlates the EVALUATING tiles and
             * accumulates; a tile stays EVALUATING while |increment| > stab_max and r < stab_retries */
            unsigned char *ev = (unsigned char *)malloc((size_t)cnt);
            int *idx = (int *)malloc(sizeof(int) * cnt);
            orc_vector *v2 = (orc_vector *)malloc(sizeof(orc_vector) * cnt);
            long nev = 0;
            for (long k = 0; k < cnt; k++) {
                const double du = precision == 0 ? vec[k].u : (float)vec[k].u64;
                const double dv = precision == 0 ? vec[k].v : (float)vec[k].v64;
                ev[k] = (float)sqrt(du * du + dv * dv) > stab_max && 1 < stab_retries;
                nev += ev[k];
            }
            for (int r = 2; r <= stab_retries && nev > 0; r++) {
                if (lv > 0 && warp_mode >= 1 && warp_mode <= 3) {
                    orc_displacement_field(cyd, ni, cxd, nj, cu, cv, h, w, precision, fu, fv);
                    orc_warp_full(img_a, img_b, h, w, pix_bytes, fu, fv, int16_quirk,
                                  warp_mode == 1 ? 3 : (warp_mode == 2 ? 1 : 2), wa, wb);
                }
                long m = 0;
                for (long k = 0; k < cnt; k++) {
                    if (!ev[k]) continue;
                    const int i = (int)(k / nj), j = (int)(k % nj);
                    idx[m] = (int)k;
                    at[m] = tops[i];
                    al[m] = lefts[j];
                    bt[m] = warp_mode == 0 ? java_round((float)tops[i] + cu[k]) : tops[i];
                    bl[m] = warp_mode == 0 ? java_round((float)lefts[j] + cv[k]) : lefts[j];
                    m++;
                }
                orc_piv_pass(sa, sb, h, w, pix_bytes, n, m, at, al, bt, bl, nm, fma, fmb, 1, precision, v2, nthreads);
                nev = 0;
                for (long q = 0; q < m; q++) {
                    const long k = idx[q];
                    float nu, nv;
                    if (precision == 0) { nu = cu[k] + v2[q].u; nv = cv[k] + v2[q].v; }
                    else { nu = (float)((double)cu[k] + v2[q].u64); nv = (float)((double)cv[k] + v2[q].v64); }
                    if (!clip || orc_clip_ok(n, h, w, tops[k / nj], lefts[k % nj], nu, nv)) { cu[k] = nu; cv[k] = nv; }
                    const double du = precision == 0 ? v2[q].u : (float)v2[q].u64;
                    const double dv = precision == 0 ? v2[q].v : (float)v2[q].v64;
                    ev[k] = (float)sqrt(du * du + dv * dv) > stab_max && r < stab_retries;
                    nev += ev[k];
                }
            }
            free(ev); free(idx); free(v2);
        }
        if (validate) {
            /* VectorValidatorJob after IterationStepTiles.updateDisplacementsFromMaxCrossResults
             * (S/jobs/LocalPIVOpenCLGpuJob.java:384-402) */
            float *pku = (float *)malloc(sizeof(float) * cnt * kpk), *pkv = (float *)malloc(sizeof(float) * cnt * kpk);
            int *npk1 = NULL;
            for (long q = 0; q < cnt * kpk; q++) {
                const orc_vector *src = multi ? &mvec[q] : &vec[q];
                pku[q] = precision == 0 ? src->u : (float)src->u64;
                pkv[q] = precision == 0 ? src->v : (float)src->v64;
            }
            if (!multi) {
                npk1 = (int *)malloc(sizeof(int) * cnt);
                for (long q = 0; q < cnt; q++) npk1[q] = 1;
            }
            orc_valid_cfg vc = *val;
            vc.clip_n = clip ? n : 0;
            vc.clip_h = clip ? h : 0;
            vc.clip_w = clip ? w : 0;
            orc_validate(ni, nj, tops, lefts, cu, cv, pku, pkv, multi ? npk : npk1, kpk, &vc,
                         level_invalid ? level_invalid + vec_off : NULL);
            free(pku); free(pkv); free(npk1);
        }
        if (level_uv) {
            memcpy(level_uv + 2 * vec_off, cu, sizeof(float) * cnt);
            memcpy(level_uv + 2 * vec_off + cnt, cv, sizeof(float) * cnt);
        }
        vec_off += cnt;
        free(mvec); free(npk);
        free(at); free(al); free(bt); free(bl); free(vec); free(cyd); free(cxd); free(cyf); free(cxf);
        free(pu); free(pv);
        pu = cu; pv = cv;
        pni = ni; pnj = nj; pn = n;
        memcpy(ptops, tops, sizeof(int) * ni);
        memcpy(plefts, lefts, sizeof(int) * nj);
    }
    if (rc == 0) {
        memcpy(out_u, pu, sizeof(float) * pni * pnj);
        memcpy(out_v, pv, sizeof(float) * pni * pnj);
        *out_ni = pni;
        *out_nj = pnj;
    }
    free(pu); free(pv); free(tops); free(lefts); free(ptops); free(plefts); free(wa); free(wb); free(fu); free(fv);
    return rc;
}

int orc_piv_adaptive(const void *img_a, const void *img_b, int h, int w, int pix_bytes, int n_start, int n_end,
                     float overlap_factor, int warp_mode, int norm_mode, float fixed_max, int int16_quirk, int precision,
                     int nthreads, float *out_u, float *out_v, int *out_ni, int *out_nj, orc_vector *level_vectors) {
    return orc_piv_adaptive_ex(img_a, img_b, h, w, pix_bytes, n_start, n_end, overlap_factor, warp_mode, 0, 0,
                               norm_mode, fixed_max, int16_quirk, precision, nthreads, NULL, out_u, out_v, out_ni,
                               out_nj, level_vectors, NULL, NULL, 0, 1, 0.0f);
}
