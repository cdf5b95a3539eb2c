// Adaptive multi-pass stage launchers (qlpiv_adaptive.cu) and host-side grids
// (qlpiv_grid.cu).
#pragma once
#include <cuda_runtime.h>

#include "qlpiv.h"

namespace qlpiv {

// The bicubic displacement surfaces of [pairs][ni*nj] tiles: double-word scratch of the line
// solves (column lines, row lines; per component) and the float node quadruples
// (f, fy, fx, fyx) the evaluation reads.
struct SplineCoef {
    float2 *col_u, *row_u, *col_v, *row_v;
    float4 *c4_u, *c4_v;
};
inline size_t spline_coef_bytes(long n) { return (size_t)n * (4 * sizeof(float2) + 2 * sizeof(float4)); }
// base: 16-byte aligned, spline_coef_bytes(n) long.
inline SplineCoef spline_coef_at(void *base, long n) {
    float2 *c = reinterpret_cast<float2 *>(base);
    float4 *q = reinterpret_cast<float4 *>(c + 4 * n);
    return SplineCoef{c, c + n, c + 2 * n, c + 3 * n, q, q + n};
}
inline SplineCoef spline_coef_offset(const SplineCoef &c, long off) {
    return SplineCoef{c.col_u + off, c.row_u + off, c.col_v + off, c.row_v + off, c.c4_u + off, c.c4_v + off};
}

// Factors of the natural-spline line solves along one axis with knots x[n] (n >= 2): KF_ARRAYS
// arrays of n values, computed once per grid in double so that the per-line solves multiply
// instead of divide:
//   h[i] = x[i+1] - x[i], ih[i] = 1 / h[i], h6[i] = h[i] / 6                       (i < n-1)
//   den[i] = 2 (h[i-1] + h[i]) - h[i-1] cp[i-1], cp[i] = h[i] / den[i], iden[i] = 1 / den[i]
//                                                                              (0 < i < n-1)
//   rc[i] = 1 / (x[min(i+1, n-1)] - x[max(i-1, 0)])       (the cross-derivative differences)
// Unused entries are 0.  The solves take them as double-words (knot_factors_dw).
enum { KF_H = 0, KF_IH, KF_H6, KF_CP, KF_IDEN, KF_RC, KF_ARRAYS };
__host__ __device__ void knot_factors(const double *x, int n, double *kf);
// knot_factors rounded to double-words (hi, lo) for the device solves; out: KF_ARRAYS * n.
void knot_factors_dw(const double *x, int n, float2 *out);

// ru/rv: scratch of pairs x cni x pnj floats (stage-1 row values).
cudaError_t launch_inherit(cudaStream_t s, int pairs, const float *py, int pni, const float *px, int pnj,
                           const float *pu, const float *pv, const float *cy, int cni, const float *cx, int cnj,
                           int round_int, float *ru, float *rv, float *cu, float *cv);
// Vertical (or horizontal) overlap in pixels of the child span [c, c + cn) with the parent span
// [p, p + pn), in checkOverlappingFactor's branch form (Area.java:222-299).
__host__ __device__ __forceinline__ int span_overlap(int p, int pn, int c, int cn) {
    if (p <= c) {
        if (p + pn > c) {
            int end = c + cn;
            if (end - 1 >= p + pn) end = p + pn;
            return end - c;
        }
        return 0;
    }
    return c + cn > p ? c + cn - p : 0;
}

// Direct / Area / Distance inheritance (mode: qlpiv_inherit_mode); tables: cni row entries then
// cnj column entries built by inherit_tables (qlpiv_pipeline.cu).
cudaError_t launch_inherit_tiles(cudaStream_t s, int pairs, int mode, int pn, int pni, int pnj, const int *ptops,
                                 const int *plefts, const float *pu, const float *pv, int cn, int cni, int cnj,
                                 const int *ctops, const int *clefts, const int2 *tables, int round_int, float *cu,
                                 float *cv);
// Node quadruples of every pair's u and v surfaces in one launch; kfy / kfx: device knot
// factors (knot_factors_dw) of the ni row knots and the nj column knots.
// gate (optional, device): nothing is done when *gate == 0.
cudaError_t launch_spline(cudaStream_t s, int pairs, const float2 *kfy, int ni, const float2 *kfx, int nj,
                          const float *u, const float *v, SplineCoef coef, const int *gate = nullptr);
cudaError_t launch_warp(cudaStream_t s, int pixel_type, int pairs, int h, int w, const qlpiv_frame *src,
                        const qlpiv_frame *dst, const float *ys, int ni, const float *xs, int nj, SplineCoef coef,
                        int int16_quirk, int image_mode, const int *gate = nullptr);
// Tile states after a stabilisation pass (InterAreaDisplacementStableStrategy): the tiles of
// in_list ([0] count, then tiles; NULL = all `count`) still EVALUATING go to out_list.
cudaError_t launch_stable_update(cudaStream_t s, int pass, int max_retries, float max_disp, const qlpiv_vector *out,
                                 const int *in_list, long count, int *out_list);
// Micro / mini per-tile warping of every pair's tiles (grid tops[ni] x lefts[nj], side n; tile
// displacements cu / cv [pairs][ni*nj]); image_mode 1 first, 2 second, 3 both.  Writes
// [pairs][tiles][n][n] pixels of pixel_type and per-tile maxima.
cudaError_t launch_tile_warp(cudaStream_t s, int pixel_type, int pairs, const qlpiv_frame *frames, int n, int ni,
                             int nj, const int *tops, const int *lefts, const float *cu, const float *cv,
                             int image_mode, int mini, float full_max, void *tiles_a, void *tiles_b, float *max_a,
                             float *max_b);
// Per-pixel field; pixel (i, j) is evaluated at (off_y + i, off_x + j), clamped to the knot box.
cudaError_t launch_field(cudaStream_t s, int h, int w, const float *ys, int ni, const float *xs, int nj,
                         SplineCoef coef, float *fu, float *fv, float off_y = 0.0f, float off_x = 0.0f);
cudaError_t launch_displaced_origins(cudaStream_t s, long count, const int *a_top, const int *a_left, const float *u,
                                     const float *v, int *b_top, int *b_left);
// NoOutOfBoundClipping of inherited displacements: count tiles with origins top/left (side n) in
// an h x w image; a value that moves its tile out of the image is replaced by zero.
cudaError_t launch_clip_inherited(cudaStream_t s, long count, const int *top, const int *left, int n, int h, int w,
                                  float *u, float *v);

int grid_superposition(int h, int w, const int margins[4], int ia_start, int level, float ofac, qlpiv_grid *g,
                       int32_t *tops, int32_t *lefts, int cap);
int grid_nosuperposition(int h, int w, const int margins[4], int ia_start, int level, qlpiv_grid *g, int32_t *tops,
                         int32_t *lefts, int cap);
// The grid of adaptive level `level` with SuperPosition starting at level sp_start (the mixed
// division; 0: SuperPosition throughout).
int grid_level(int h, int w, const int margins[4], int ia_start, int level, float ofac, int sp_start, qlpiv_grid *g,
               int32_t *tops, int32_t *lefts, int cap);

}  // namespace qlpiv
