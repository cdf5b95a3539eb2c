// Dense optical-flow stage launchers (qlpiv_dense.cu).
#pragma once
#include <cuda_runtime.h>

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
// Liu-Shen passes in place; fx: 10 x h x w floats of scratch, err: `iterations` doubles.
cudaError_t launch_liu_shen(cudaStream_t s, const float *la, const float *lb, int h, int w, float *us, float *vs,
                            float lambda, int iterations, int half_pixel, float *fx, float *tmp, double *err);

}  // namespace qlpiv
