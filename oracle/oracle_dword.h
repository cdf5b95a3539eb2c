/*
 * qlpiv oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * Double-word ("float-float") arithmetic for the float path's spline solves: a value is the
 * unevaluated sum hi + lo of two floats.  Error-free transformations TwoSum (Knuth), Fast2Sum
 * (Dekker), TwoProd (fmaf), and the double-word algorithms AccurateDWPlusDW, DWPlusFP,
 * DWTimesFP3 and DWTimesDW3 of Joldes, Muller and Popescu (ACM TOMS 44(2), 2017), written here
 * from that paper.  Compiled with -ffp-contract=off: every step is one IEEE float operation or
 * one fmaf, so the results are those of the CUDA kernels bit for bit.
 */
#ifndef QLPIV_ORACLE_DWORD_H
#define QLPIV_ORACLE_DWORD_H
#include <math.h>

typedef struct { float hi, lo; } orc_dw;

static inline orc_dw dw_two_sum(float a, float b) {
    orc_dw r;
    const float s = a + b, ap = s - b, bp = s - ap, da = a - ap, db = b - bp;
    r.hi = s;
    r.lo = da + db;
    return r;
}
static inline orc_dw dw_fast_two_sum(float a, float b) {
    orc_dw r;
    const float s = a + b, z = s - a;
    r.hi = s;
    r.lo = b - z;
    return r;
}
static inline orc_dw dw_two_prod(float a, float b) {
    orc_dw r;
    r.hi = a * b;
    r.lo = fmaf(a, b, -r.hi);
    return r;
}
static inline orc_dw dw_add(orc_dw x, orc_dw y) {
    const orc_dw s = dw_two_sum(x.hi, y.hi), t = dw_two_sum(x.lo, y.lo);
    const float c = s.lo + t.hi;
    const orc_dw v = dw_fast_two_sum(s.hi, c);
    const float w = t.lo + v.lo;
    return dw_fast_two_sum(v.hi, w);
}
static inline orc_dw dw_sub(orc_dw x, orc_dw y) {
    y.hi = -y.hi;
    y.lo = -y.lo;
    return dw_add(x, y);
}
static inline orc_dw dw_twice(orc_dw x) {
    x.hi = 2.0f * x.hi;
    x.lo = 2.0f * x.lo;
    return x;
}
static inline orc_dw dw_add_f(orc_dw x, float y) {
    const orc_dw s = dw_two_sum(x.hi, y);
    const float v = x.lo + s.lo;
    return dw_fast_two_sum(s.hi, v);
}
static inline orc_dw dw_mul(orc_dw x, orc_dw y) {
    const orc_dw c = dw_two_prod(x.hi, y.hi);
    const float tl0 = x.lo * y.lo;
    const float tl1 = fmaf(x.hi, y.lo, tl0);
    const float cl2 = fmaf(x.lo, y.hi, tl1);
    const float cl3 = c.lo + cl2;
    return dw_fast_two_sum(c.hi, cl3);
}
static inline orc_dw dw_mul_f(orc_dw x, float y) {
    const orc_dw c = dw_two_prod(x.hi, y);
    const float cl3 = fmaf(x.lo, y, c.lo);
    return dw_fast_two_sum(c.hi, cl3);
}
static inline orc_dw dw_of(double v) {
    orc_dw r;
    r.hi = (float)v;
    r.lo = (float)(v - (double)r.hi);
    return r;
}
static inline float dw_float(orc_dw x) { return x.hi + x.lo; }

#endif
