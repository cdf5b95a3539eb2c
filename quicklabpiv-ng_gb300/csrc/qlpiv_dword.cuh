// Double-word ("float-float") arithmetic: a value is the unevaluated sum hi + lo of two floats
// with |lo| <= ulp(hi) / 2, about 44 significant bits.  Built from the error-free
// transformations TwoSum (Knuth), Fast2Sum (Dekker) and TwoProd (one FMA), and the double-word
// algorithms of Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic building
// blocks of double-word arithmetic" (ACM TOMS 44(2), 2017): AccurateDWPlusDW (relative error
// <= 3u^2), DWPlusFP, DWTimesFP3 (<= 2u^2) and DWTimesDW3 (<= 4u^2), u = 2^-24.
//
// Everything runs on the FP32 pipe, where GB300 has ~64x the FP64 rate.  Each step is one IEEE
// float operation or one fmaf; in translation units compiled without contraction
// (--fmad=false, -ffp-contract=off) host and device produce the same bits.
#pragma once
#include <math.h>

namespace qlpiv {

struct dword {
    float hi, lo;
};

__host__ __device__ __forceinline__ dword two_sum(float a, float b) {
    const float s = a + b;
    const float ap = s - b;
    const float bp = s - ap;
    const float da = a - ap;
    const float db = b - bp;
    return dword{s, da + db};
}

__host__ __device__ __forceinline__ dword fast_two_sum(float a, float b) {
    const float s = a + b;
    const float z = s - a;
    return dword{s, b - z};
}

__host__ __device__ __forceinline__ dword two_prod(float a, float b) {
    const float p = a * b;
    return dword{p, fmaf(a, b, -p)};
}

__host__ __device__ __forceinline__ dword dw_add(dword x, dword y) {
    const dword s = two_sum(x.hi, y.hi);
    const dword t = two_sum(x.lo, y.lo);
    const float c = s.lo + t.hi;
    const dword v = fast_two_sum(s.hi, c);
    const float w = t.lo + v.lo;
    return fast_two_sum(v.hi, w);
}

__host__ __device__ __forceinline__ dword dw_neg(dword x) { return dword{-x.hi, -x.lo}; }
__host__ __device__ __forceinline__ dword dw_sub(dword x, dword y) { return dw_add(x, dw_neg(y)); }
__host__ __device__ __forceinline__ dword dw_twice(dword x) { return dword{2.0f * x.hi, 2.0f * x.lo}; }

__host__ __device__ __forceinline__ dword dw_add_f(dword x, float y) {
    const dword s = two_sum(x.hi, y);
    const float v = x.lo + s.lo;
    return fast_two_sum(s.hi, v);
}

__host__ __device__ __forceinline__ dword dw_mul(dword x, dword y) {
    const dword c = two_prod(x.hi, y.hi);
    const float tl0 = x.lo * y.lo;
    const float tl1 = fmaf(x.hi, y.lo, tl0);
    const float cl2 = fmaf(x.lo, y.hi, tl1);
    const float cl3 = c.lo + cl2;
    return fast_two_sum(c.hi, cl3);
}

__host__ __device__ __forceinline__ dword dw_mul_f(dword x, float y) {
    const dword c = two_prod(x.hi, y);
    const float cl3 = fmaf(x.lo, y, c.lo);
    return fast_two_sum(c.hi, cl3);
}

// Nearest double-word of a double (hi = RN(v); v - hi is exact in double).
__host__ __device__ __forceinline__ dword dw_of(double v) {
    const float hi = (float)v;
    return dword{hi, (float)(v - (double)hi)};
}

// Float nearest hi + lo.
__host__ __device__ __forceinline__ float dw_float(dword x) { return x.hi + x.lo; }

}  // namespace qlpiv
