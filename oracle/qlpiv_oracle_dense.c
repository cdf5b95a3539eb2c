/*
 * qlpiv oracle, dense optical flow stages -- TEST INFRASTRUCTURE ONLY.
 *
 * The stages' bodies live in oracle_dense_impl.h, included twice:
 *   float  (orc_gauss_filter, orc_normalize, orc_dense_lk, orc_liu_shen, orc_dense_lk_pyramid,
 *           orc_flow_after_piv): Java float semantics, bit-faithful to the reference's order;
 *   double (the same names with _f64): the FP64 twin, the error reference of the CUDA dense
 *           stages (filter weights unrounded, the per-pixel field evaluated in double).
 */
#define _GNU_SOURCE
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "oracle_types.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* GaussianFilter2D.createKernel (S/images/filters/GaussianFilter2D.java:31-46): double weights,
 * normalised, rounded to float. */
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

/* The same weights kept in double (the FP64 twin). */
void orc_gauss_kernel_f64(float sigma, int px, double *k) {
    const int half = px / 2;
    double sum = 0.0;
    for (int i = 0; i < px; i++) {
        const double x = i - half;
        const double s = (double)sigma;
        k[i] = 1.0 / sqrt(2.0 * M_PI * s * s) * exp(-x * x / (2.0 * s * s));
        sum += k[i];
    }
    for (int i = 0; i < px; i++) k[i] = k[i] / sum;
}

static void orc_kernel(float sigma, int px, float *k) { orc_gauss_kernel(sigma, px, k); }
static void orc_kernel_f64(float sigma, int px, double *k) { orc_gauss_kernel_f64(sigma, px, k); }

#define REAL float
#define DFN(name) orc_##name
#define RFABS fabsf
#define RSQRT sqrtf
#define FIELD_PRECISION 0
#include "oracle_dense_impl.h"
#undef REAL
#undef DFN
#undef RFABS
#undef RSQRT
#undef FIELD_PRECISION

#define REAL double
#define DFN(name) orc_##name##_f64
#define RFABS fabs
#define RSQRT sqrt
#define FIELD_PRECISION 1
#include "oracle_dense_impl.h"
#undef REAL
#undef DFN
#undef RFABS
#undef RSQRT
#undef FIELD_PRECISION
