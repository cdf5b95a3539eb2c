// Natural logarithm of a positive normal float as an unevaluated pair of floats (hi + lo),
// absolute error below 1e-11, using only FP32 operations.
//
// The 3-point Gaussian sub-pixel fit takes the logarithms of float samples in double
// (Gaussian1DPolynomialInterpolator, FastMath.log) and rounds the combinations to float.  GB300's
// FP64 rate is a small fraction of its FP32 rate, and with K1's fit queue running 32 fits per warp
// the double logarithms kept the FP64 pipe the busiest unit of the IA-16 multi-peak kernel.  This
// is Tang's table-driven method (P. T. P. Tang, "Table-driven implementation of the logarithm
// function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990) carried in float-float:
//
//   x = 2^e m, m in [1, 2);  k = round(64 (m - 1));  c_k = 1 / inv_k with inv_k ~ 1 / (1 + k/64)
//   ln x = e ln 2 - ln(inv_k) + ln(1 + r),  r = m inv_k - 1  (|r| < 1/100)
//
// m inv_k is split exactly into p + pe with one FMA, so r = (p - 1) + pe holds exactly (p - 1 is
// exact by Sterbenz's lemma); ln(1 + r) = r - r^2/2 + r^3/3 - r^4/4 + r^5/5 with the tail beyond
// the first term evaluated in float (its magnitude is below 5e-5, so its rounding stays near
// 3e-12), and the terms are added with error-free two-sums.  The table holds inv_k and -ln(inv_k)
// split into two floats, computed on the host in double.  Tested against CUDA's double log.
#pragma once
#include <cuda_runtime.h>

namespace qlpiv {

struct fpair {
    float hi, lo;
};

// hi + lo = a + b exactly (Knuth's two-sum).
__device__ __forceinline__ fpair two_sum_f(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, err};
}

__device__ __forceinline__ fpair fp_add(fpair a, fpair b) {
    const fpair s = two_sum_f(a.hi, b.hi);
    const float lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return two_sum_f(s.hi, lo);
}

__device__ __forceinline__ fpair fp_scale2(fpair a, float p2) { return {__fmul_rn(a.hi, p2), __fmul_rn(a.lo, p2)}; }

// The pair rounded to the nearest float (what a cast of the double value gives, barring
// values within the pair's error of a rounding boundary).
__device__ __forceinline__ float fp_round(fpair a) { return __fadd_rn(a.hi, a.lo); }

// tab[k] = {inv_k, -ln(inv_k) hi, -ln(inv_k) lo, 0}, k = 0..64.
__device__ __forceinline__ fpair log_fpair(float x, const float4 *tab) {
    const uint32_t b = __float_as_uint(x);
    const int e = (int)(b >> 23) - 127;
    const float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
    const int k = __float2int_rn(__fmul_rn(__fsub_rn(m, 1.0f), 64.0f));
    const float4 t = __ldg(tab + k);
    const float p = __fmul_rn(m, t.x);
    const float pe = __fmaf_rn(m, t.x, -p);  // m inv_k = p + pe exactly
    const float rh = __fsub_rn(p, 1.0f);     // exact
    // ln(1 + r) - rh with r = rh + pe: pe - rh pe - rh^2/2 + rh^3/3 - rh^4/4 + rh^5/5
    float poly = __fmaf_rn(rh, 0.2f, -0.25f);
    poly = __fmaf_rn(rh, poly, 0.333333343f);
    poly = __fmaf_rn(rh, poly, -0.5f);
    const float tail = __fmaf_rn(__fmul_rn(rh, rh), poly, __fsub_rn(pe, __fmul_rn(rh, pe)));
    // e ln2: ln2 = 0.693145751953125 (exact in 15 bits, e ln2_hi exact) + 1.42860677e-6
    const float eh = __fmul_rn((float)e, 0.693145751953125f);
    const float el = __fmul_rn((float)e, 1.42860677e-06f);
    fpair s = two_sum_f(eh, t.y);
    s = fp_add(s, two_sum_f(rh, tail));
    return fp_add(s, two_sum_f(el, t.z));
}

}  // namespace qlpiv
