/*
 * qlpiv oracle: CPU restatement of QuickLabPIV-ng's FFT-PIV path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is loaded by tests/, by
 * __graft_entry__.smoke() and by the cpu_baseline / reference legs of bench.py,
 * always as the checker or the timed CPU baseline, never as part of the product.
 * The product (quicklabpiv-ng_gb300/) neither links nor loads it.
 *
 * The reference is Java (QuickLabPIV-ng 0.8.7); no JVM exists on the build or the
 * GPU machines, so the reference cannot be run.  This file restates its CPU path
 * from the sources (citations use S/ = src/main/java/pt/quickLabPIV/):
 *   tile clip + max          S/images/Image.java:386-494, S/MatrixByte.java:16-33,204-226
 *   normalise + pack + FFT   S/jobs/xcorr/FastRealFFTXCorr.java:44-116, S/jobs/xcorr/SimpleFFT.java
 *   peak search              S/maximum/FindMaximumFromCenter.java:33-183
 *   3-point Gaussian fit     S/interpolators/Gaussian1DPolynomialInterpolator.java:25-106
 *   displacement             S/maximum/MaxCrossResult.java:304-326
 *   IA grids                 S/iareas/AdaptiveInterAreaStrategySuperPosition.java:31-197,
 *                            S/iareas/AdaptiveInterAreaStrategyNoSuperPosition.java:32-157
 * Pinned against the reference's golden vectors by tests/test_oracle_golden.py.
 *
 * Build: oracle/Makefile (gcc -O3 -ffp-contract=off, no fast-math).
 */
#define _GNU_SOURCE
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define ORC_F_SUB_I 1u
#define ORC_F_SUB_J 2u
#define ORC_F_PARABOLIC 4u
#define ORC_F_EDGE 8u
#define ORC_F_NO_PEAK 16u

#include "oracle_types.h"

/* perfectShuffleFFTInput (S/jobs/xcorr/SimpleFFT.java:32-69) produces the
 * bit-reversal permutation; tests/test_oracle_golden.py restates the swap loop and
 * checks the equality for every power of two up to 512. */
static void bitrev_perm(int n, int *perm) {
    int bits = 0;
    while ((1 << bits) < n) bits++;
    for (int k = 0; k < n; k++) {
        int r = 0;
        for (int b = 0; b < bits; b++)
            if (k & (1 << b)) r |= 1 << (bits - 1 - b);
        perm[k] = r;
    }
}

#define REAL float
#define SUFFIX _f32
#include "oracle_impl.h"
#undef REAL
#undef SUFFIX

#define REAL double
#define SUFFIX _f64
#include "oracle_impl.h"
#undef REAL
#undef SUFFIX

/* ---------------------------------------------------------------------------
 * Exported single-IA entry points (ctypes)
 * ------------------------------------------------------------------------- */

void orc_xcorr_fft_f32(const float *ta, const float *tb, int n, float maxA, float maxB, int normalize,
                       float *plane) {
    xcorr_fft_f32(ta, tb, n, maxA, maxB, normalize, plane);
}

void orc_xcorr_fft_f64(const float *ta, const float *tb, int n, float maxA, float maxB, int normalize,
                       double *plane) {
    xcorr_fft_f64(ta, tb, n, maxA, maxB, normalize, plane);
}

/* By-definition correlation (T/CrossCorrelationTestHelper.localCrossCorrelation,
 * tests/pt/quickLabPIV/CrossCorrelationTestHelper.java:32-72):
 * R[s1+N-1][s2+N-1] = sum_m a'(m) * b'(m+s), in double. */
void orc_xcorr_direct_f64(const float *ta, const float *tb, int n, float maxA, float maxB, int normalize,
                          double *plane) {
    const int d = 2 * n - 1;
    double *a = (double *)malloc(sizeof(double) * n * n);
    double *b = (double *)malloc(sizeof(double) * n * n);
    for (int k = 0; k < n * n; k++) {
        a[k] = normalize ? (double)ta[k] / (double)maxA * 16.0 + 1.0 : (double)ta[k];
        b[k] = normalize ? (double)tb[k] / (double)maxB * 16.0 + 1.0 : (double)tb[k];
    }
    for (int s1 = -(n - 1); s1 < n; s1++) {
        for (int s2 = -(n - 1); s2 < n; s2++) {
            const int i0 = s1 < 0 ? -s1 : 0, i1 = s1 > 0 ? n - s1 : n;
            const int j0 = s2 < 0 ? -s2 : 0, j1 = s2 > 0 ? n - s2 : n;
            double acc = 0.0;
            for (int i = i0; i < i1; i++)
                for (int j = j0; j < j1; j++) acc += a[i * n + j] * b[(i + s1) * n + (j + s2)];
            plane[(size_t)(s1 + n - 1) * d + (s2 + n - 1)] = acc;
        }
    }
    free(a);
    free(b);
}

void orc_find_max_from_center_f32(const float *p, int di, int dj, int *oi, int *oj, float *ov, float *ominf) {
    find_max_from_center_f32(p, di, dj, oi, oj, ov, ominf);
}

void orc_find_max_from_center_f64(const double *p, int di, int dj, int *oi, int *oj, double *ov,
                                  double *ominf) {
    find_max_from_center_f64(p, di, dj, oi, oj, ov, ominf);
}

void orc_subpixel_gauss3_f32(const float *p, int di, int dj, int mi, int mj, float *pi, float *pj,
                             uint32_t *flags) {
    subpixel_gauss3_f32(p, di, dj, mi, mj, pi, pj, flags);
}

void orc_subpixel_gauss3_f64(const double *p, int di, int dj, int mi, int mj, double *pi, double *pj,
                             uint32_t *flags) {
    subpixel_gauss3_f64(p, di, dj, mi, mj, pi, pj, flags);
}

/* ---------------------------------------------------------------------------
 * Tile clipping (Image.clipImageMatrix, S/images/Image.java:386-494): pixels outside
 * the image are zero (partial clipping), the tile max is the max of the copied
 * pixels floored at 16 (S/MatrixByte.java:30-31, S/MatrixInt16.java:35-36).
 * pix_bytes: 1 = u8, 2 = u16 (little-endian host order).
 * ------------------------------------------------------------------------- */
float orc_clip_tile(const void *img, int h, int w, int pix_bytes, int top, int left, int n, float *tile) {
    int maxv = 0;
    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) {
            const int y = top + i, x = left + j;
            int v = 0;
            if (y >= 0 && y < h && x >= 0 && x < w) {
                v = pix_bytes == 1 ? (int)((const uint8_t *)img)[(size_t)y * w + x]
                                   : (int)((const uint16_t *)img)[(size_t)y * w + x];
            }
            if (v > maxv) maxv = v;
            tile[i * n + j] = (float)v;
        }
    }
    return (float)(maxv < 16 ? 16 : maxv);
}

/* FastMath.round(float) = (int) floor(x + 0.5f) */
static int java_round_f(float x) { return (int)floorf(x + 0.5f); }

/* ---------------------------------------------------------------------------
 * IA grids
 * ------------------------------------------------------------------------- */
/* orc_grid (oracle_types.h): IA side, tiles per axis, margins */
/* AdaptiveInterAreaStrategySuperPosition (S/iareas/AdaptiveInterAreaStrategySuperPosition.java:31-197).
 * level 0: tile origin = margin + round(k * f * N); levels > 0: origins accumulate the
 * float increment (:107-116).  Margins of level L are computed from that level's
 * tile size.  tops/lefts receive tiles_i / tiles_j entries; returns 0 or -1. */
int orc_grid_superposition(int h, int w, int mtop, int mbottom, int mleft, int mright, int n_start, int level,
                           float overlap_factor, orc_grid *g, int *tops, int *lefts, int cap) {
    const int n = n_start >> level;
    const float inc = overlap_factor * (float)n;
    const int nj = (int)(0.01f + ((float)(w - (mleft + mright)) - ((float)n - inc)) / inc);
    const int ni = (int)(0.01f + ((float)(h - (mtop + mbottom)) - ((float)n - inc)) / inc);
    const int remI = h - (int)ceil((double)((float)(ni - 1) * inc + (float)n)) - (mtop + mbottom);
    const int remJ = w - (int)ceil((double)((float)(nj - 1) * inc + (float)n)) - (mleft + mright);
    const int floorDivI = remI >= 0 ? remI / 2 : -((-remI + 1) / 2);
    const int floorDivJ = remJ >= 0 ? remJ / 2 : -((-remJ + 1) / 2);
    g->n = n;
    g->tiles_i = ni;
    g->tiles_j = nj;
    g->margin_top = mtop + floorDivI;
    g->margin_bottom = mbottom + (int)ceil((double)((float)remI / 2.0f));
    g->margin_left = mleft + floorDivJ;
    g->margin_right = mright + (int)ceil((double)((float)remJ / 2.0f));
    if (ni > cap || nj > cap) return -1;
    if (level == 0) {
        for (int k = 0; k < ni; k++) tops[k] = g->margin_top + java_round_f((float)k * inc);
        for (int k = 0; k < nj; k++) lefts[k] = g->margin_left + java_round_f((float)k * inc);
    } else {
        float p = (float)g->margin_top;
        for (int k = 0; k < ni; k++, p += inc) tops[k] = java_round_f(p);
        p = (float)g->margin_left;
        for (int k = 0; k < nj; k++, p += inc) lefts[k] = java_round_f(p);
    }
    return 0;
}

/* AdaptiveInterAreaStrategyNoSuperPosition (S/iareas/AdaptiveInterAreaStrategyNoSuperPosition.java:32-157) */
int orc_grid_nosuperposition(int h, int w, int mtop, int mbottom, int mleft, int mright, int n_start, int level,
                             orc_grid *g, int *tops, int *lefts, int cap) {
    const int n = n_start >> level;
    const int ni = (h - (mtop + mbottom)) / n;
    const int nj = (w - (mleft + mright)) / n;
    const int leftI = h - mtop - mbottom - n * ni;
    const int leftJ = w - mleft - mright - n * nj;
    g->n = n;
    g->tiles_i = ni;
    g->tiles_j = nj;
    g->margin_top = mtop + leftI / 2;
    g->margin_bottom = h - n * ni - g->margin_top;
    g->margin_left = mleft + leftJ / 2;
    g->margin_right = w - n * nj - g->margin_left;
    if (ni > cap || nj > cap) return -1;
    for (int k = 0; k < ni; k++) tops[k] = g->margin_top + k * n;
    for (int k = 0; k < nj; k++) lefts[k] = g->margin_left + k * n;
    return 0;
}

/* ---------------------------------------------------------------------------
 * Batched single pass over an image pair (the timed CPU baseline and the parity
 * checker for the frame API).  IA k has tile A at (a_top[k], a_left[k]) of image A
 * and tile B at (b_top[k], b_left[k]) of image B (integer origins, already rounded).
 * norm_mode: 0 = both tiles by tile A's max (reference CPU path),
 *            1 = each tile by its own max (reference OpenCL path),
 *            2 = fixed maxima fixed_max_a / fixed_max_b (full-image warp tiles),
 *            3 = raw values (no normalisation);
 *            | 8: first replace the tile maxima by fixed_max_a / fixed_max_b where those are > 0
 *            (FirstImage / SecondImage warping: only the warped side keeps a fixed maximum).
 * precision: 0 = FP32 restatement, 1 = FP64 twin.
 * Work is split over nthreads POSIX threads by IA index.
 * ------------------------------------------------------------------------- */
typedef struct {
    const void *img_a, *img_b;
    int h, w, pix_bytes, n, norm_mode, precision, subpix;
    float fixed_max_a, fixed_max_b;
    const int *a_top, *a_left, *b_top, *b_left;
    orc_vector *out;
    long begin, end;
    int kw, k;        /* k > 0: FindMaximumMultiPeaks with kw x kw cells, k peaks per IA */
    int *npeaks;      /* multi-peak mode: peaks found per IA; out holds k vectors per IA */
} orc_job;

static void *orc_worker(void *arg) {
    orc_job *j = (orc_job *)arg;
    const int n = j->n, d = 2 * n - 1;
    float *ta = (float *)malloc(sizeof(float) * n * n);
    float *tb = (float *)malloc(sizeof(float) * n * n);
    void *plane = malloc(sizeof(double) * d * d);
    for (long k = j->begin; k < j->end; k++) {
        float maxA = orc_clip_tile(j->img_a, j->h, j->w, j->pix_bytes, j->a_top[k], j->a_left[k], n, ta);
        float maxB = orc_clip_tile(j->img_b, j->h, j->w, j->pix_bytes, j->b_top[k], j->b_left[k], n, tb);
        int normalize = 1;
        if (j->norm_mode & 8) {
            if (j->fixed_max_a > 0.0f) maxA = j->fixed_max_a;
            if (j->fixed_max_b > 0.0f) maxB = j->fixed_max_b;
        }
        switch (j->norm_mode & 7) {
            case 0: maxB = maxA; break;
            case 1: break;
            case 2: maxA = j->fixed_max_a; maxB = j->fixed_max_b; break;
            default: normalize = 0; break;
        }
        if (j->k > 0) {
            orc_vector *o = &j->out[k * j->k];
            memset(o, 0, sizeof(orc_vector) * j->k);
            j->npeaks[k] = j->precision == 0
                ? ia_vectors_multi_f32(ta, tb, n, maxA, maxB, normalize, j->subpix, j->kw, j->k, o, (float *)plane)
                : ia_vectors_multi_f64(ta, tb, n, maxA, maxB, normalize, j->subpix, j->kw, j->k, o, (double *)plane);
        } else if (j->precision == 0) {
            ia_vector_f32(ta, tb, n, maxA, maxB, normalize, j->subpix, &j->out[k], (float *)plane);
        } else {
            ia_vector_f64(ta, tb, n, maxA, maxB, normalize, j->subpix, &j->out[k], (double *)plane);
        }
    }
    free(ta);
    free(tb);
    free(plane);
    return NULL;
}

static int run_pass(const void *img_a, const void *img_b, int h, int w, int pix_bytes, int n, long count,
                    const int *a_top, const int *a_left, const int *b_top, const int *b_left, int norm_mode,
                    float fixed_max_a, float fixed_max_b, int subpix, int precision, orc_vector *out, int nthreads,
                    int kw, int k, int *npeaks) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if ((long)nthreads > count) nthreads = count > 0 ? (int)count : 1;
    pthread_t th[256];
    orc_job jobs[256];
    for (int t = 0; t < nthreads; t++) {
        orc_job *j = &jobs[t];
        j->img_a = img_a; j->img_b = img_b; j->h = h; j->w = w; j->pix_bytes = pix_bytes; j->n = n;
        j->norm_mode = norm_mode; j->precision = precision; j->subpix = subpix;
        j->fixed_max_a = fixed_max_a; j->fixed_max_b = fixed_max_b;
        j->a_top = a_top; j->a_left = a_left; j->b_top = b_top; j->b_left = b_left; j->out = out;
        j->begin = count * t / nthreads;
        j->end = count * (t + 1) / nthreads;
        j->kw = kw;
        j->k = k;
        j->npeaks = npeaks;
    }
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, orc_worker, &jobs[t]);
    orc_worker(&jobs[0]);
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
    return 0;
}

int orc_piv_pass(const void *img_a, const void *img_b, int h, int w, int pix_bytes, int n, long count,
                 const int *a_top, const int *a_left, const int *b_top, const int *b_left, int norm_mode,
                 float fixed_max_a, float fixed_max_b, int subpix, int precision, orc_vector *out, int nthreads) {
    return run_pass(img_a, img_b, h, w, pix_bytes, n, count, a_top, a_left, b_top, b_left, norm_mode, fixed_max_a,
                    fixed_max_b, subpix, precision, out, nthreads, 0, 0, NULL);
}

/* The same pass with FindMaximumMultiPeaks (kw x kw cells, k <= 64 peaks): out holds k
 * vectors per IA, largest peak first, npeaks[k] the number found. */
int orc_piv_pass_multi(const void *img_a, const void *img_b, int h, int w, int pix_bytes, int n, long count,
                       const int *a_top, const int *a_left, const int *b_top, const int *b_left, int norm_mode,
                       float fixed_max_a, float fixed_max_b, int subpix, int precision, int kw, int k,
                       orc_vector *out, int *npeaks, int nthreads) {
    if (k < 1 || k > 64 || kw < 1) return -1;
    return run_pass(img_a, img_b, h, w, pix_bytes, n, count, a_top, a_left, b_top, b_left, norm_mode, fixed_max_a,
                    fixed_max_b, subpix, precision, out, nthreads, kw, k, npeaks);
}

/* FindMaximumMultiPeaks on one plane (d_i x d_j, row-major). */
int orc_find_max_multipeaks_f32(const float *p, int di, int dj, int kw, int k, int *oi, int *oj, float *ov,
                                float *ominf) {
    if (k < 1 || k > 64 || kw < 1) return -1;
    return find_max_multipeaks_f32(p, di, dj, kw, k, oi, oj, ov, ominf);
}

/* SimpleFixedLengthFloatLinkedList(max_size, kernel_width): a sequence of
 * addInAscendOrder calls; the list is returned in ascending order. */
int orc_mp_list_run(int max_size, int kernel_width, int count, const float *v, const int *i, const int *j,
                    float *ov, int *oi, int *oj) {
    if (max_size < 1 || max_size > 64) return -1;
    mp_entry_f32 lst[65];
    int size = 0;
    const float kd = (float)((kernel_width - 1) * kernel_width);
    for (int q = 0; q < count; q++) mp_add_f32(lst, &size, max_size, kd, v[q], i[q], j[q]);
    for (int r = 0; r < size; r++) { ov[r] = lst[r].v; oi[r] = lst[r].i; oj[r] = lst[r].j; }
    return size;
}

/* One pass over ready tiles (count x n x n floats) with given per-tile maxima: the CPU path from
 * the correlation on.  norm_mode as orc_piv_pass (0: both by A's max, 1: own, 3: raw); k > 0:
 * FindMaximumMultiPeaks with k peaks (out holds k vectors per tile, npeaks the peaks found). */
int orc_tiles_pass(const float *tiles_a, const float *tiles_b, const float *max_a, const float *max_b, long count,
                   int n, int norm_mode, int subpix, int precision, int kw, int k, orc_vector *out, int *npeaks) {
    const int d = 2 * n - 1;
    void *plane = malloc(sizeof(double) * d * d);
    for (long q = 0; q < count; q++) {
        const float *ta = tiles_a + q * n * n, *tb = tiles_b + q * n * n;
        float maxA = max_a[q], maxB = max_b[q];
        int normalize = 1;
        if (norm_mode == 0) maxB = maxA;
        else if (norm_mode != 1) normalize = 0;
        if (k > 0) {
            orc_vector *o = out + q * k;
            const int np = precision == 0
                ? ia_vectors_multi_f32(ta, tb, n, maxA, maxB, normalize, subpix, kw, k, o, (float *)plane)
                : ia_vectors_multi_f64(ta, tb, n, maxA, maxB, normalize, subpix, kw, k, o, (double *)plane);
            if (npeaks) npeaks[q] = np;
        } else if (precision == 0) {
            ia_vector_f32(ta, tb, n, maxA, maxB, normalize, subpix, &out[q], (float *)plane);
        } else {
            ia_vector_f64(ta, tb, n, maxA, maxB, normalize, subpix, &out[q], (double *)plane);
        }
    }
    free(plane);
    return 0;
}

int orc_vector_size(void) { return (int)sizeof(orc_vector); }
