/*
 * Types and cross-file prototypes of the qlpiv CPU oracle -- TEST INFRASTRUCTURE ONLY.
 */
#ifndef QLPIV_ORACLE_TYPES_H
#define QLPIV_ORACLE_TYPES_H

#include <math.h>
#include <stdint.h>

typedef struct {
    float u, v;
    float sub_i, sub_j;
    float peak_value, min_floor;
    int16_t peak_i, peak_j;
    uint32_t flags;
    double u64, v64;
} orc_vector; /* 48 bytes */

typedef struct {
    int n, tiles_i, tiles_j, margin_top, margin_left, margin_bottom, margin_right;
} orc_grid;

/* Vector validation as the converter configures it (PIVConfigurationConverterVisitor.visit of the
 * five VelocityValidationOptions models, ui/.../PIVConfigurationConverterVisitor.java:546-641):
 *   model 0 or 1  multi-peak normalised median: num_peaks k >= 1 strategies, strategy s < k-1
 *                 replaces by peak s+1, the last one by bilinear interpolation (FindMaximumMultiPeaks)
 *   model 2 / 3   DifferenceValidator, no replacement / bilinear (FindMaximumFromCenter)
 *   model 4 / 5   NormalizedMedianValidator, no replacement / bilinear (FindMaximumFromCenter)
 * enabled == 0: no validation, FindMaximumFromCenter.  clip_n / clip_h / clip_w: tile side and
 * image size when replacements follow NoOutOfBoundClipping (clip_n == 0: clipping allowed). */
typedef struct {
    int enabled;
    int num_peaks;        /* k: peaks searched per IA and validation strategies (model 0/1) */
    int kernel_width;     /* FindMaximumMultiPeaks cell width */
    float threshold;      /* distance threshold (pixels for the difference validator) */
    float epsilon0;
    int max_iterations;
    int iterate_until_no_corrections;
    int model;
    int clip_n, clip_h, clip_w;
} orc_valid_cfg;

/* Tile.accumulateDisplacement / replaceDisplacement under NoOutOfBoundClipping
 * (S/iareas/Tile.java:103-136, 156-189): a displacement (u, v) is refused when the tile of side n at
 * (top, left), moved by the rounded displacement (FastMath.round: floor(x + 0.5f)), fails the
 * reference's test top + ru < 0, top + n + ru >= h, left + rv < 0, left + n + rv >= w.  n == 0:
 * clipping allowed (AllowedOutOfBoundClipping, LoggedOutOfBoundClipping), nothing refused. */
static inline int orc_clip_ok(int n, int h, int w, int top, int left, float u, float v) {
    if (n == 0) return 1;
    const float ru = floorf(u + 0.5f), rv = floorf(v + 0.5f);
    return !((float)top + ru < 0.0f || (float)(top + n) + ru >= (float)h || (float)left + rv < 0.0f ||
             (float)(left + n) + rv >= (float)w);
}

/* Sub-pixel interpolators of qlpiv_oracle_subpix.c.  A pass's `subpix` argument packs the mode
 * (bits 0-7: 0 none, 1 Gaussian 3-point, 2 Gaussian least squares, 3 Hongwei Guo), the stencil
 * pixels (bits 8-15) and the Hongwei Guo iterations (bits 16-23). */
int orc_gauss_lm_fit(const double *x, const double *y, int n, double *mean_out);
int orc_hongwei_guo_fit(const float *xs, const float *ys, int n, int iterations, float *mean, float *amplitude);
void orc_subpixel_lm(const float *plane, int d, int mi, int mj, int P, float min_floor, float *si, float *sj,
                     uint32_t *flags);
void orc_subpixel_hg(const float *plane, int d, int mi, int mj, int P, int iterations, float min_floor, float *si,
                     float *sj, float *pv, uint32_t *flags);

int orc_tiles_pass(const float *tiles_a, const float *tiles_b, const float *max_a, const float *max_b, long count,
                   int n, int norm_mode, int subpix, int precision, int kw, int k, orc_vector *out, int *npeaks);
void orc_tile_warp(const void *img_a, const void *img_b, int h, int w, int pix_bytes, int n, int ni, int nj,
                   const int *tops, const int *lefts, const float *cu, const float *cv, int image_mode, int mini,
                   float full_max, float *tiles_a, float *tiles_b, float *max_a, float *max_b);
float orc_clip_tile(const void *img, int h, int w, int pix_bytes, int top, int left, int n, float *tile);

int orc_grid_superposition(int h, int w, int mtop, int mbottom, int mleft, int mright, int n_start, int level,
                           float overlap_factor, orc_grid *g, int *tops, int *lefts, int cap);
int orc_grid_nosuperposition(int h, int w, int mtop, int mbottom, int mleft, int mright, int n_start, int level,
                             orc_grid *g, int *tops, int *lefts, int cap);
int orc_piv_pass(const void *img_a, const void *img_b, int h, int w, int pix_bytes, int n, long count,
                 const int *a_top, const int *a_left, const int *b_top, const int *b_left, int norm_mode,
                 float fixed_max_a, float fixed_max_b, int subpix, int precision, orc_vector *out, int nthreads);
int orc_piv_pass_multi(const void *img_a, const void *img_b, int h, int w, int pix_bytes, int n, long count,
                       const int *a_top, const int *a_left, const int *b_top, const int *b_left, int norm_mode,
                       float fixed_max_a, float fixed_max_b, int subpix, int precision, int kw, int k,
                       orc_vector *out, int *npeaks, int nthreads);
int orc_spiral_order(int ni, int nj, int *order);
float orc_area_overlap(int pt, int pl, int pn, int ct, int cl, int cn, int *flags);
int orc_inherit_tiles(int mode, int pn, int pni, int pnj, const int *ptops, const int *plefts, const float *pu,
                      const float *pv, int cn, int cni, int cnj, const int *ctops, const int *clefts, int round_int,
                      float *cu, float *cv);
int orc_validate(int ni, int nj, const int *tops, const int *lefts, float *u, float *v, const float *pu,
                 const float *pv, const int *npeaks, int k, const orc_valid_cfg *cfg, unsigned char *invalid_out);

void orc_displacement_field_off(const double *ys, int ni, const double *xs, int nj, const float *u, const float *v,
                                int h, int w, int precision, float off_y, float off_x, float *fu, float *fv);
void orc_gauss_kernel(float sigma, int px, float *k);
void orc_gauss_filter(const float *in, int h, int w, const float *k, int K, float *out);
void orc_normalize(const float *in, long n, float *out);
void orc_dense_lk(const float *A, const float *B, int h, int w, float *us, float *vs, int win, int iterations,
                  int half_pixel);
void orc_dense_lk_pyramid(const float *A, const float *B, int h, int w, float *us, float *vs, int win, int iterations,
                          int half_pixel, int levels);
int orc_liu_shen(const float *la, const float *lb, int h, int w, float *us, float *vs, float lambda, int iterations,
                 int half_pixel, float *fixed_out, float *unews, float *vnews);

#endif
