// Dense optical-flow stage launchers (qlpiv_dense.cu).
#pragma once
#include <cuda_runtime.h>

#include "qlpiv.h"
#include "qlpiv_adaptive.h"

#include <vector>

namespace qlpiv {

// GaussianFilter2D.createKernel weights (double, normalised, rounded to float).
void gauss_weights(float sigma, int px, float *k);
// Separable Gaussian prefilter of an image of `pixel_type` (pitch in elements) -> float out;
// tmp: h x w floats.
cudaError_t launch_gauss(cudaStream_t s, int pixel_type, const void *in, long pitch, int h, int w, const float *k,
                         int K, float *tmp, float *out);
// out = in / max(0, max(in)); mx: one device word.
cudaError_t launch_normalize(cudaStream_t s, const float *in, long n, unsigned *mx, float *out);
// Dense Lucas-Kanade in place on us (columns) / vs (rows).
cudaError_t launch_dense_lk(cudaStream_t s, const float *a, const float *b, int h, int w, float *us, float *vs, int W,
                            int iterations, int half_pixel);
// Liu-Shen passes in place; fx: 10 x h x w floats of scratch, err: ls_err_bytes(h, w, iterations)
// (every pass's error sum, spread over a few accumulators).
size_t ls_err_bytes(int h, int w, int iterations);
cudaError_t launch_liu_shen(cudaStream_t s, const float *la, const float *lb, int h, int w, float *us, float *vs,
                            float lambda, int iterations, int half_pixel, float *fx, float *tmp, double *err);

// Device buffers of one frame pair's optical flow after PIV (h x w floats each unless noted).
struct FlowBufs {
    float *lka, *lkb, *lsa, *lsb, *tmp, *fu, *fv;
    float *fx;        // 10 x h x w (Liu-Shen fixed terms and ping-pong field)
    float *pyr;       // 2 x h x w: the coarser Lucas-Kanade pyramid levels (images and field)
    double *err;      // ls_err_bytes(h, w, iterations_ls)
    unsigned *mx;     // one word
    float *k_lk, *k_ls;  // filter weights (device)
    void *coef;       // spline coefficients of ni x nj tiles (spline_coef_bytes)
};

// Optional sub-stage hook of run_flow: fn(ctx, stage, true) before a sub-stage's launches are
// queued, fn(ctx, stage, false) after them (stage timing).
struct FlowMarks {
    void (*fn)(void *ctx, const char *stage, bool begin);
    void *ctx;
};

// Optical flow after PIV of one frame pair on the device (see qlpiv_flow_after_piv): frames of
// pixel_type with `pitch` elements per row; knot factors kfy/kfx of the tile grid's ni / nj
// centres (knot_factors_dw, device) and the centres cyf/cxf (float); tops/lefts (device int);
// tile_u/tile_v (rows, columns) updated in place; dense_u / dense_v (rows, columns) optional.  *launches counts the kernels queued.  given: the spline
// coefficients of this pair's tiles when the caller solved them already (else solved here).
cudaError_t run_flow(cudaStream_t s, const qlpiv_flow_desc &d, int pixel_type, const void *img_a, const void *img_b,
                     long pitch, int h, int w, int n, int ni, int nj, const float2 *kfy, const float2 *kfx,
                     const float *cyf, const float *cxf, const int *tops, const int *lefts, float *tile_u,
                     float *tile_v, float *dense_u, float *dense_v, const FlowBufs &b, long *launches,
                     const FlowMarks *marks = nullptr, const SplineCoef *given = nullptr);
// Carves the buffers of one frame pair's flow out of `buf` (grown on demand).
cudaError_t flow_buffers(struct DevBuf &buf, int h, int w, int ni, int nj, int iterations_ls, FlowBufs *b);
// Uploads both prefilters' weights (host staging kept by the caller until the stream syncs).
cudaError_t upload_flow_weights(cudaStream_t s, const qlpiv_flow_desc &d, const FlowBufs &b, std::vector<float> &host);
// Checks a flow descriptor; returns a message or nullptr.
const char *check_flow_desc(const qlpiv_flow_desc *d, int h, int w);

}  // namespace qlpiv
