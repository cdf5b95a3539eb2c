// Adaptive multi-pass stages between correlation passes (device code).
//
//   B-inherit  AdaptiveInterVelocityInheritanceStrategyBiCubicSpline
//              (S/iareas/AdaptiveInterVelocityInheritanceStrategyBiCubicSpline.java:27-136):
//              child tile displacement = piecewise bicubic (Akima, 5x5 knot window)
//              interpolation of the parent tiles' displacement at the child centre,
//              clamped to the parent centre box; rounded for non-warping modes.
//   B-field    BiCubicSplineInterpolatorWithBiLinearBackup (S/iareas/...:57-107,224-249):
//              bicubic spline surface through the current level's tile displacements
//              (natural-spline knot derivatives, finite-difference cross derivatives,
//              Hermite patches), evaluated per pixel with coordinates clamped to the
//              tile-centre box.  Knot derivatives are solved in double-word (float-float)
//              arithmetic, ~44 bits, and rounded to float; the surface is evaluated in float
//              (the reference works in double: GB300's FP64 rate is ~1/64 of FP32, and this
//              keeps the field within ~1e-6 px of the double one).
//   B-warp     BiLinearImageWarpingStrategy.warpPixelOnImage (S/images/...:143-265),
//              BothImages mode: field halved, A sampled at (i-u, j-v), B at (i+u, j+v),
//              nearest-pixel anchor plus the neighbour on the residual's side, output
//              rounded.
// The commons-math3 interpolators the reference calls are restated from their
// mathematics.  This translation unit is compiled with --fmad=false so every double
// and float expression rounds exactly like the CPU oracle's restatement (same
// operand order, no contraction): the warp stage is bit-identical to the oracle.
#include <cuda_runtime.h>
#include <stdint.h>

#include "qlpiv_adaptive.h"
#include "qlpiv_dword.cuh"
#include "qlpiv_internal.h"

namespace qlpiv {

// ---------------- shared device helpers ----------------

// Interpolators in float, same formulation and operand order as the CPU oracle's
// float path (oracle/oracle_interp_impl.h).
__host__ __device__ __forceinline__ int knot_interval(const float *v, int n, float c) {
    int lo = 0, hi = n - 1;
    if (c >= v[n - 1]) return n - 2;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (v[mid] <= c) lo = mid; else hi = mid;
    }
    return lo;
}

__host__ __device__ __forceinline__ void hermite_basis(float t, float h0[2], float h1[2]) {
    const float t2 = t * t, t3 = t2 * t;
    h0[0] = 2.0f * t3 - 3.0f * t2 + 1.0f;
    h0[1] = -2.0f * t3 + 3.0f * t2;
    h1[0] = t3 - 2.0f * t2 + t;
    h1[1] = t3 - t2;
}

__host__ __device__ __forceinline__ float parabola_deriv(const float *x, const float *y, int at, int i0, int i1, int i2) {
    const float X = x[at];
    const float x0 = x[i0], x1 = x[i1], x2 = x[i2];
    return y[i0] * ((X - x1) + (X - x2)) / ((x0 - x1) * (x0 - x2)) +
           y[i1] * ((X - x0) + (X - x2)) / ((x1 - x0) * (x1 - x2)) +
           y[i2] * ((X - x0) + (X - x1)) / ((x2 - x0) * (x2 - x1));
}

// Akima spline through 5 knots, evaluated at t (knots ascending, t inside).
__host__ __device__ float akima5_value(const float *x, const float *y, float t) {
    float d[4], w[4] = {0.0f, 0.0f, 0.0f, 0.0f}, fd[5];
    for (int k = 0; k < 4; k++) d[k] = (y[k + 1] - y[k]) / (x[k + 1] - x[k]);
    for (int k = 1; k < 4; k++) w[k] = fabsf(d[k] - d[k - 1]);
    {
        const float wp = w[3], wm = w[1];
        if (wp == 0.0f && wm == 0.0f)
            fd[2] = ((x[3] - x[2]) * d[1] + (x[2] - x[1]) * d[2]) / (x[3] - x[1]);
        else
            fd[2] = (wp * d[1] + wm * d[2]) / (wp + wm);
    }
    fd[0] = parabola_deriv(x, y, 0, 0, 1, 2);
    fd[1] = parabola_deriv(x, y, 1, 0, 1, 2);
    fd[3] = parabola_deriv(x, y, 3, 2, 3, 4);
    fd[4] = parabola_deriv(x, y, 4, 2, 3, 4);
    const int k = knot_interval(x, 5, t);
    const float h = x[k + 1] - x[k], s = t - x[k];
    const float c2 = (3.0f * (y[k + 1] - y[k]) / h - 2.0f * fd[k] - fd[k + 1]) / h;
    const float c3 = (2.0f * (y[k] - y[k + 1]) / h + fd[k] + fd[k + 1]) / (h * h);
    return y[k] + s * (fd[k] + s * (c2 + s * c3));
}

__host__ __device__ __forceinline__ int akima_window(const float *v, int n, float c) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (v[mid] <= c) lo = mid + 1; else hi = mid;
    }
    int r;
    if (lo > 0 && v[lo - 1] == c) r = (lo - 1) - 2;
    else r = lo - 2;
    if (r < 0) r = 0;
    if (r + 5 >= n) r = n - 5;
    return r;
}

__host__ __device__ __forceinline__ int java_round(float x) { return (int)floorf(x + 0.5f); }

// ---------------- B-inherit ----------------

// Stage 1, entry gid = (pair, child row i, parent column pj): Akima spline along the
// first coordinate through parent column pj (5-knot window around the clamped child
// centre y), evaluated at y.  These are the row[] values of every child tile of row i.
__host__ __device__ void inherit_rows_one(long gid, const float *py, int pni, int pnj, const float *pu, const float *pv,
                                          const float *cy, int cni, float *ru, float *rv) {
    const long per = (long)cni * pnj;
    const int pair = (int)(gid / per);
    const long k = gid - (long)pair * per;
    const int i = (int)(k / pnj), pj = (int)(k - (long)i * pnj);
    const float ymin = py[0], ymax = py[pni - 1];
    float y = cy[i];
    if (y < ymin) y = ymin; else if (y > ymax) y = ymax;
    const int wi = akima_window(py, pni, y);
    const float *fu = pu + (long)pair * pni * pnj;
    const float *fv = pv + (long)pair * pni * pnj;
    float cu[5], cv[5];
    for (int a = 0; a < 5; a++) {
        cu[a] = fu[(long)(wi + a) * pnj + pj];
        cv[a] = fv[(long)(wi + a) * pnj + pj];
    }
    ru[gid] = akima5_value(py + wi, cu, y);
    rv[gid] = akima5_value(py + wi, cv, y);
}

// Stage 2, child tile gid = (pair, i, j): Akima spline along the second coordinate
// through the 5 stage-1 values of the window around the clamped child centre x.
__host__ __device__ void inherit_cols_one(long gid, const float *px, int pnj, const float *cx, int cni, int cnj,
                                          const float *ru, const float *rv, int round_int, float *cu, float *cv) {
    const long cnt = (long)cni * cnj;
    const int pair = (int)(gid / cnt);
    const long k = gid - (long)pair * cnt;
    const int i = (int)(k / cnj), j = (int)(k - (long)i * cnj);
    const float xmin = px[0], xmax = px[pnj - 1];
    float x = cx[j];
    if (x < xmin) x = xmin; else if (x > xmax) x = xmax;
    const int wj = akima_window(px, pnj, x);
    const long row = ((long)pair * cni + i) * pnj + wj;
    const float iu = akima5_value(px + wj, ru + row, x);
    const float iv = akima5_value(px + wj, rv + row, x);
    if (round_int) {
        cu[gid] = 0.0f + (float)java_round(iu);
        cv[gid] = 0.0f + (float)java_round(iv);
    } else {
        cu[gid] = 0.0f + iu;
        cv[gid] = 0.0f + iv;
    }
}

__global__ void inherit_rows_kernel(int pairs, const float *py, int pni, int pnj, const float *pu, const float *pv,
                                    const float *cy, int cni, float *ru, float *rv) {
    const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long)pairs * cni * pnj) return;
    inherit_rows_one(gid, py, pni, pnj, pu, pv, cy, cni, ru, rv);
}

__global__ void inherit_cols_kernel(int pairs, const float *px, int pnj, const float *cx, int cni, int cnj,
                                    const float *ru, const float *rv, int round_int, float *cu, float *cv) {
    const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long)pairs * cni * cnj) return;
    inherit_cols_one(gid, px, pnj, cx, cni, cnj, ru, rv, round_int, cu, cv);
}

// ---------------- B-inherit: Direct, Area, Distance ----------------
//
// The reference walks the child tiles serially, carrying a parent "reference tile" from tile
// to tile (S/iareas/AdaptiveInterVelocityInheritanceStrategy{Direct,Area,DistanceGeneric}.java).
// On the regular separable grids of the adaptive levels that walk resolves, per child row and
// per child column independently, to a parent index range (Area) or a parent index and a side
// flag (Distance); inherit_tables computes those on the host, rejecting the geometries where
// the walk throws, and inherit_tiles_kernel evaluates every child tile on its own with the
// reference's float operations in the walk's order.

__global__ void inherit_tiles_kernel(int pairs, int mode, int pn, int pni, int pnj, const int *ptops,
                                     const int *plefts, const float *pu, const float *pv, int cn, int cni, int cnj,
                                     const int *ctops, const int *clefts, const int2 *rows, const int2 *cols,
                                     int round_int, float *cu, float *cv) {
    const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long cnt = (long)cni * cnj;
    if (gid >= (long)pairs * cnt) return;
    const int pair = (int)(gid / cnt);
    const long k = gid - (long)pair * cnt;
    const int i = (int)(k / cnj), j = (int)(k - (long)i * cnj);
    const float *fu = pu + (long)pair * pni * pnj, *fv = pv + (long)pair * pni * pnj;
    float du = 0.0f, dv = 0.0f;
    if (mode == QLPIV_INHERIT_DIRECT) {
        const int qi = i >> 1, qj = j >> 1;
        if (qi < pni && qj < pnj) {
            du = fu[(long)qi * pnj + qj];
            dv = fv[(long)qi * pnj + qj];
        }
    } else if (mode == QLPIV_INHERIT_AREA) {
        const int2 R = rows[i], C = cols[j];
        const int ct = ctops[i], cl = clefts[j];
        float acc = 0.0f;
        for (int r = R.x; r <= R.y; r++) {
            const int vo = span_overlap(ptops[r], pn, ct, cn);
            for (int c = C.x; c <= C.y; c++) acc += (float)(vo * span_overlap(plefts[c], pn, cl, cn));
        }
        for (int r = R.x; r <= R.y; r++) {
            const int vo = span_overlap(ptops[r], pn, ct, cn);
            for (int c = C.x; c <= C.y; c++) {
                const float w = (float)(vo * span_overlap(plefts[c], pn, cl, cn)) / acc;
                du += w * fu[(long)r * pnj + c];
                dv += w * fv[(long)r * pnj + c];
            }
        }
    } else {  // Distance: parents (p, q), (p, q + 1), (p + 1, q), (p + 1, q + 1) in that order
        const int2 R = rows[i], C = cols[j];
        const float ccy = (float)ctops[i] + (float)cn / 2.0f, ccx = (float)clefts[j] + (float)cn / 2.0f;
        const bool has_r = C.x + 1 < pnj && !C.y, has_d = R.x + 1 < pni && !R.y;
        int qi[4], qj[4];
        float dist[4];
        bool ok[4] = {true, has_r, has_d, has_r && has_d};
        int zero = -1;
        float total = 0.0f;
        for (int a = 0; a < 4; a++) {
            qi[a] = R.x + (a >> 1);
            qj[a] = C.x + (a & 1);
            if (!ok[a]) continue;
            const float py = (float)ptops[qi[a]] + (float)pn / 2.0f, px = (float)plefts[qj[a]] + (float)pn / 2.0f;
            const double dx = (double)(ccx - px), dy = (double)(ccy - py);
            dist[a] = (float)sqrt(dx * dx + dy * dy);
            if (zero < 0 && dist[a] == 0.0f) zero = a;
        }
        if (zero >= 0) {
            du = fu[(long)qi[zero] * pnj + qj[zero]];
            dv = fv[(long)qi[zero] * pnj + qj[zero]];
        } else {
            for (int a = 0; a < 4; a++)
                if (ok[a]) total += 1.0f / dist[a];
            for (int a = 0; a < 4; a++) {
                if (!ok[a]) continue;
                const float w = (1.0f / dist[a]) / total;
                du += w * fu[(long)qi[a] * pnj + qj[a]];
                dv += w * fv[(long)qi[a] * pnj + qj[a]];
            }
        }
    }
    if (round_int) {
        du = (float)java_round(du);
        dv = (float)java_round(dv);
    }
    cu[gid] = 0.0f + du;
    cv[gid] = 0.0f + dv;
}

// ---------------- B-field spline set-up ----------------

__host__ __device__ void knot_factors(const double *x, int n, double *kf) {
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

void knot_factors_dw(const double *x, int n, float2 *out) {
    double *kf = new double[(size_t)KF_ARRAYS * n];
    knot_factors(x, n, kf);
    for (int k = 0; k < KF_ARRAYS * n; k++) {
        const dword d = dw_of(kf[k]);
        out[k] = make_float2(d.hi, d.lo);
    }
    delete[] kf;
}

__host__ __device__ __forceinline__ dword dw_at(const float2 *p, int i) {
    const float2 v = p[i];
    return dword{v.x, v.y};
}

// Natural-spline first derivatives at the n knots of one grid line, in double-word arithmetic
// with factors kf (knot_factors_dw): values y(i) (float), scratch S(i) (float2), float results
// out(i, d).  A forward elimination, then one backward sweep that forms the second derivatives
// m (m[0] = m[n-1] = 0) and, from m[i] and m[i+1], the derivative at knot i:
//   s[i]  = (y[i+1] - y[i]) ih[i]                   (the difference is exact as a double-word)
//   dp[i] = (6 (s[i] - s[i-1]) - h[i-1] dp[i-1]) iden[i],   dp[0] = 0
//   m[i]  = dp[i] - cp[i] m[i+1]
//   d[i]  = s[i] - h6[i] (2 m[i] + m[i+1]),   d[n-1] = s[n-2] + h6[n-2] (m[n-2] + 2 m[n-1])
// The oracle's float path restates these operations.  The loads of C knots are issued ahead of
// their part of the dependent chain.
template <int C, typename YF, typename SF, typename OF>
__host__ __device__ __forceinline__ void spline_line_dw(const float2 *kf, int n, YF y, SF S, OF out) {
    const float2 *h = kf + KF_H * n, *ih = kf + KF_IH * n, *h6 = kf + KF_H6 * n;
    const float2 *cp = kf + KF_CP * n, *iden = kf + KF_IDEN * n;
    const dword zero{0.0f, 0.0f};
    float ycur = y(1);
    dword sp = dw_mul(two_sum(ycur, -y(0)), dw_at(ih, 0));
    dword dprev = zero;
    for (int i0 = 1; i0 < n - 1; i0 += C) {
        float yv[C];
#pragma unroll
        for (int k = 0; k < C; k++) yv[k] = i0 + k < n - 1 ? y(i0 + k + 1) : 0.0f;
#pragma unroll
        for (int k = 0; k < C; k++) {
            const int i = i0 + k;
            if (i < n - 1) {
                const dword si = dw_mul(two_sum(yv[k], -ycur), dw_at(ih, i));
                const dword r = dw_mul_f(dw_sub(si, sp), 6.0f);
                const dword dp = dw_mul(dw_sub(r, dw_mul(dw_at(h, i - 1), dprev)), dw_at(iden, i));
                S(i) = make_float2(dp.hi, dp.lo);
                dprev = dp;
                sp = si;
                ycur = yv[k];
            }
        }
    }
    dword mnext = zero;  // m[n-1]
    float ynext = y(n - 1);
    for (int i0 = n - 2; i0 >= 1; i0 -= C) {
        float yv[C];
        float2 dv[C];
#pragma unroll
        for (int k = 0; k < C; k++) {
            yv[k] = i0 - k >= 1 ? y(i0 - k) : 0.0f;
            dv[k] = i0 - k >= 1 ? S(i0 - k) : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int k = 0; k < C; k++) {
            const int i = i0 - k;
            if (i >= 1) {
                const dword m = dw_sub(dword{dv[k].x, dv[k].y}, dw_mul(dw_at(cp, i), mnext));
                const dword si = dw_mul(two_sum(ynext, -yv[k]), dw_at(ih, i));
                const dword hh = dw_at(h6, i);
                if (i == n - 2) out(n - 1, dw_float(dw_add(si, dw_mul(hh, dw_add(m, dw_twice(mnext))))));
                out(i, dw_float(dw_sub(si, dw_mul(hh, dw_add(dw_twice(m), mnext)))));
                mnext = m;
                ynext = yv[k];
            }
        }
    }
    const dword s0 = dw_mul(two_sum(ynext, -y(0)), dw_at(ih, 0));
    if (n == 2) out(1, dw_float(dw_add(s0, dw_mul(dw_at(h6, 0), dw_add(zero, dw_twice(zero))))));
    out(0, dw_float(dw_sub(s0, dw_mul(dw_at(h6, 0), dw_add(dw_twice(zero), mnext)))));
}

// Cross derivative of node (i, j) from the node values around it (central differences,
// one-sided at the border), in double-word arithmetic: ((a - b - c + d) rcy[i]) rcx[j].
template <typename FF>
__host__ __device__ __forceinline__ float spline_cross(FF f, int ni, int nj, int i, int j, const float2 *rcy,
                                                       const float2 *rcx) {
    const int in = i + 1 < ni ? i + 1 : ni - 1, ip = i - 1 >= 0 ? i - 1 : 0;
    const int jn = j + 1 < nj ? j + 1 : nj - 1, jp = j - 1 >= 0 ? j - 1 : 0;
    dword t = two_sum(f(in, jn), -f(in, jp));
    t = dw_add_f(t, -f(ip, jn));
    t = dw_add_f(t, f(ip, jp));
    return dw_float(dw_mul(dw_mul(t, dw_at(rcy, i)), dw_at(rcx, j)));
}

// One warp per strip of 32 grid lines of one component of one pair.  Column strips solve the
// lines along the first coordinate and write the node value, fy and the cross derivative of
// their 32 columns; row strips solve the lines along the second coordinate and write fx.
// Lanes walk their own line: per knot the lanes of a column strip touch 32 consecutive nodes;
// the scratch of a row strip is laid out knot-major (knot, lane) so its accesses stay
// coalesced.  The two kinds write disjoint floats of the node quadruples.
__global__ void __launch_bounds__(128) spline_nodes_kernel(int pairs, const float2 *kfy, int ni, const float2 *kfx,
                                                           int nj, const float *u, const float *v, SplineCoef coef,
                                                           const int *gate) {
    if (gate != nullptr && *gate == 0) return;
    const int sj = (nj + 31) / 32, si = (ni + 31) / 32, per = 2 * (sj + si);
    const long wid = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wid >= (long)pairs * per) return;
    const int lane = threadIdx.x & 31;
    const int pair = (int)(wid / per);
    int r = (int)(wid - (long)pair * per);
    const int comp = r / (sj + si);
    r -= comp * (sj + si);
    const long base = (long)pair * ni * nj;
    const float *f = (comp == 0 ? u : v) + base;
    float *c4 = reinterpret_cast<float *>((comp == 0 ? coef.c4_u : coef.c4_v) + base);
    if (r < sj) {
        const int j = r * 32 + lane;
        if (j >= nj) return;
        float2 *S = (comp == 0 ? coef.col_u : coef.col_v) + base;
        const float2 *rcy = kfy + KF_RC * ni, *rcx = kfx + KF_RC * nj;
        auto F = [&](int a, int b) { return __ldg(f + (long)a * nj + b); };
        // node values and cross derivatives first: independent of the line solve
#pragma unroll 4
        for (int i = 0; i < ni; i++) {
            const long k = (long)i * nj + j;
            c4[4 * k] = __ldg(f + k);
            c4[4 * k + 3] = spline_cross(F, ni, nj, i, j, rcy, rcx);
        }
        spline_line_dw<8>(
            kfy, ni, [&](int i) { return __ldg(f + (long)i * nj + j); },
            [&](int i) -> float2 & { return S[(long)i * nj + j]; },
            [&](int i, float d) { c4[4 * ((long)i * nj + j) + 1] = d; });
    } else {
        const int i0 = (r - sj) * 32, rows = ni - i0 < 32 ? ni - i0 : 32;
        if (lane >= rows) return;
        const int i = i0 + lane;
        float2 *S = (comp == 0 ? coef.row_u : coef.row_v) + base + (long)i0 * nj;
        const float *fr = f + (long)i * nj;
        spline_line_dw<8>(
            kfx, nj, [&](int j) { return __ldg(fr + j); }, [&](int j) -> float2 & { return S[(long)j * rows + lane]; },
            [&](int j, float d) { c4[4 * ((long)i * nj + j) + 2] = d; });
    }
}

// ---------------- B-field evaluation + B-warp ----------------

template <typename Pix>
__host__ __device__ __forceinline__ float warp_read(const Pix *img, long pitch, int y, int x) {
    return (float)img[(long)y * pitch + x];
}

// warpPixelOnImage (S/images/BiLinearImageWarpingStrategy.java:185-265) on an h x w image with
// `pitch` elements per row.
template <typename Pix>
__host__ __device__ float warp_pixel(const Pix *img, int h, int w, long pitch, float u, float v, int i, int j,
                                     bool first) {
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
    const float tl = warp_read(img, pitch, pI, pJ);
    const float tr = warp_read(img, pitch, pI, pJ + oJ);
    const float bl = warp_read(img, pitch, pI + oI, pJ);
    const float br = warp_read(img, pitch, pI + oI, pJ + oJ);
    const float a = (1.0f - wU) * (1.0f - wV) * tl;
    const float b = (1.0f - wU) * wV * tr;
    const float c = wU * (1.0f - wV) * bl;
    const float d = wU * wV * br;
    return (float)java_round(a + b + c + d);
}

// warp_pixel split in two so that several samples' reads can be in flight at once: the taps
// (anchor rows p0 / p1, columns pJ / pJ + oJ, weights) and then the same float operations on
// the four values.
template <typename Pix>
struct WarpTap {
    const Pix *p0, *p1;
    int pJ, oJ;
    float wU, wV;
};

template <typename Pix>
__device__ __forceinline__ WarpTap<Pix> warp_tap(const Pix *img, int h, int w, long pitch, float u, float v, int i,
                                                 int j, bool first) {
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
    return WarpTap<Pix>{img + (long)pI * pitch, img + (long)(pI + oI) * pitch, pJ, oJ, fabsf(dU), fabsf(dV)};
}

struct WarpVals {
    float tl, tr, bl, br;
};

template <typename Pix>
__device__ __forceinline__ WarpVals warp_load(const WarpTap<Pix> &t) {
    return WarpVals{(float)__ldg(t.p0 + t.pJ), (float)__ldg(t.p0 + t.pJ + t.oJ), (float)__ldg(t.p1 + t.pJ),
                    (float)__ldg(t.p1 + t.pJ + t.oJ)};
}

template <typename Pix>
__device__ __forceinline__ float warp_value(const WarpTap<Pix> &t, const WarpVals &q) {
    const float wU = t.wU, wV = t.wV;
    const float a = (1.0f - wU) * (1.0f - wV) * q.tl;
    const float b = (1.0f - wU) * wV * q.tr;
    const float c = wU * (1.0f - wV) * q.bl;
    const float d = wU * wV * q.br;
    return (float)java_round(a + b + c + d);
}

template <typename Pix>
__host__ __device__ __forceinline__ Pix warp_store(float value, int int16_quirk) {
    const int r = java_round(value);
    if (sizeof(Pix) == 1) return (Pix)(uint8_t)(int8_t)r;
    if (int16_quirk) return (Pix)(uint16_t)(int16_t)(int8_t)r;  // MatrixInt16.setElement(float) narrows via byte
    return (Pix)(uint16_t)r;
}

// Canonical field evaluation order shared with the oracle's float path: column basis
// X = (h00, h01, dx*h10, dx*h11)(tx), row basis Y likewise; the four column sums w
// first, then ((w0*Y0 + w1*Y1) + w2*Y2) + w3*Y3.
// Knot interval k of coordinate c and its Hermite basis (h00, h01, d*h10, d*h11)(t).
__host__ __device__ __forceinline__ int field_basis(const float *v, int n, float c, float B[4]) {
    const int k = knot_interval(v, n, c);
    const float d = v[k + 1] - v[k];
    const float t = (c - v[k]) / d;
    float a0[2], a1[2];
    hermite_basis(t, a0, a1);
    B[0] = a0[0];
    B[1] = a0[1];
    B[2] = d * a1[0];
    B[3] = d * a1[1];
    return k;
}

// Patch (i, j) of the node quadruples evaluated with row basis Y and column basis X.
__host__ __device__ __forceinline__ float field_combine(const float4 *c4, int nj, int i, int j, const float X[4],
                                                        const float Y[4]) {
    float w[4];
#pragma unroll
    for (int a = 0; a < 2; a++) {
        const long k0 = (long)(i + a) * nj + j;
        const float4 n0 = c4[k0], n1 = c4[k0 + 1];
        w[a] = n0.x * X[0] + n1.x * X[1] + n0.z * X[2] + n1.z * X[3];
        w[2 + a] = n0.y * X[0] + n1.y * X[1] + n0.w * X[2] + n1.w * X[3];
    }
    return w[0] * Y[0] + w[1] * Y[1] + w[2] * Y[2] + w[3] * Y[3];
}

__host__ __device__ __forceinline__ float field_value(const float *ys, int ni, const float *xs, int nj,
                                                      const float4 *c4, float y, float x) {
    float X[4], Y[4];
    const int i = field_basis(ys, ni, y, Y), j = field_basis(xs, nj, x, X);
    return field_combine(c4, nj, i, j, X, Y);
}

// Column weights of patch row i at column basis X: w[a] (values) and w[2 + a] (row
// derivatives) of node rows i + a, the first half of field_combine.
__device__ __forceinline__ void field_column(const float4 *c4, int nj, int i, int j, const float X[4], float w[4]) {
#pragma unroll
    for (int a = 0; a < 2; a++) {
        const long k0 = (long)(i + a) * nj + j;
        const float4 n0 = __ldg(c4 + k0), n1 = __ldg(c4 + k0 + 1);
        w[a] = n0.x * X[0] + n1.x * X[1] + n0.z * X[2] + n1.z * X[3];
        w[2 + a] = n0.y * X[0] + n1.y * X[1] + n0.w * X[2] + n1.w * X[3];
    }
}

// One block per 32 columns x kWarpRows rows of one pair (blockIdx.z = pair): thread (tx, ty)
// walks column j over kWarpRows / 8 consecutive rows.  The knot search and Hermite basis of the
// block's columns and rows are computed once in shared memory; a thread forms its column
// weights once per knot interval of the rows it walks (the weights do not depend on the row
// inside an interval), so a pixel costs the row combination of field_combine and the two
// samples.  Same operations as field_value per pixel: the field is bit-identical.
constexpr int kWarpRows = 64;

template <typename Pix>
__global__ void __launch_bounds__(256) warp_both_kernel(const qlpiv_frame *src, const qlpiv_frame *dst,
                                                        const float *ys, int ni, const float *xs, int nj,
                                                        const float4 *c4u, const float4 *c4v, int int16_quirk,
                                                        int image_mode, const int *gate) {
    if (gate != nullptr && *gate == 0) return;
    constexpr int kPer = kWarpRows / 8;
    __shared__ float sx[32][4];
    __shared__ float4 sy[kWarpRows];
    __shared__ int sj[32], si[kWarpRows];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
    const int j = blockIdx.x * 32 + tx, row0 = blockIdx.y * kWarpRows;
    const int pair = blockIdx.z;
    if (tid < 32) {
        float x = (float)(blockIdx.x * 32 + tid);
        if (x < xs[0]) x = xs[0]; else if (x > xs[nj - 1]) x = xs[nj - 1];
        sj[tid] = field_basis(xs, nj, x, sx[tid]);
    } else if (tid >= 64 && tid < 64 + kWarpRows) {
        const int r = tid - 64;
        float y = (float)(row0 + r);
        if (y < ys[0]) y = ys[0]; else if (y > ys[ni - 1]) y = ys[ni - 1];
        float Y[4];
        si[r] = field_basis(ys, ni, y, Y);
        sy[r] = make_float4(Y[0], Y[1], Y[2], Y[3]);
    }
    __syncthreads();
    const qlpiv_frame fs = src[pair];
    const int h = fs.height, w = fs.width;
    if (j >= w) return;
    const qlpiv_frame fd = dst[pair];
    const long base = (long)pair * ni * nj;
    const float4 *cu = c4u + base, *cv = c4v + base;
    float X[4];
#pragma unroll
    for (int k = 0; k < 4; k++) X[k] = sx[tx][k];
    const int kj = sj[tx];
    const bool both = image_mode == 3;
    const Pix *ia = reinterpret_cast<const Pix *>(fs.img_a);
    const Pix *ib = reinterpret_cast<const Pix *>(fs.img_b);
    Pix *oa = reinterpret_cast<Pix *>(const_cast<void *>(fd.img_a));
    Pix *ob = reinterpret_cast<Pix *>(const_cast<void *>(fd.img_b));
    int cur = -1;
    float wu[4], wv[4];
    for (int q = 0; q < kPer; q++) {
        const int r = ty * kPer + q, i = row0 + r;
        if (i >= h) break;
        const int ki = si[r];
        if (ki != cur) {
            field_column(cu, nj, ki, kj, X, wu);
            field_column(cv, nj, ki, kj, X, wv);
            cur = ki;
        }
        const float4 Y4 = sy[r];
        const float fu = wu[0] * Y4.x + wu[1] * Y4.y + wu[2] * Y4.z + wu[3] * Y4.w;
        const float fv = wv[0] * Y4.x + wv[1] * Y4.y + wv[2] * Y4.z + wv[3] * Y4.w;
        const float hu = both ? fu / 2.0f : fu, hv = both ? fv / 2.0f : fv;
        // both frames' four reads are issued before the arithmetic that consumes them
        const WarpTap<Pix> ta = warp_tap(ia, h, w, fs.pitch, hu, hv, i, j, true);
        const WarpTap<Pix> tb = warp_tap(ib, h, w, fs.pitch, hu, hv, i, j, false);
        WarpVals va, vb;
        if (image_mode & 1) va = warp_load(ta);
        if (image_mode & 2) vb = warp_load(tb);
        oa[(long)i * fd.pitch + j] =
            image_mode & 1 ? warp_store<Pix>(warp_value(ta, va), int16_quirk) : ia[(long)i * fs.pitch + j];
        ob[(long)i * fd.pitch + j] =
            image_mode & 2 ? warp_store<Pix>(warp_value(tb, vb), int16_quirk) : ib[(long)i * fs.pitch + j];
    }
}

// ---------------- micro / mini per-tile warping ----------------
// BiLinearImageMicroAndMiniWarpingStrategy.warpAndClipImage
// (S/images/BiLinearImageMicroAndMiniWarpingStrategy.java:39-186): one CTA per tile of one pair.
// The pixel displacements of the tile region are the tile's fractional displacement (micro) or a
// bicubic spline over its up to 7 x 7 neighbour tiles, relative to floor of its displacement and
// evaluated over the displaced B tile's region (mini, :204-290); the warped side(s) are sampled
// with the full-image rule, the other side is clipped.  Tiles are written pair-major as
// [pairs][tiles][n][n] pixels with their maxima (warped: full scale; clipped: own, floor 16).
constexpr int kMiniR = 7;

template <typename Pix>
__global__ void __launch_bounds__(256) tile_warp_kernel(const qlpiv_frame *frames, int n, int ni, int nj,
                                                        const int *tops, const int *lefts, const float *cu,
                                                        const float *cv, int image_mode, int mini, float full_max,
                                                        Pix *tiles_a, Pix *tiles_b, float *max_a, float *max_b) {
    const long cnt = (long)ni * nj;
    const int pair = blockIdx.y;
    const long k = blockIdx.x;
    const int ti = (int)(k / nj), tj = (int)(k - (long)ti * nj);
    const qlpiv_frame fr = frames[pair];
    const Pix *ia = (const Pix *)fr.img_a, *ib = (const Pix *)fr.img_b;
    const int h = fr.height, w = fr.width;
    const long pitch = fr.pitch;
    const float *pu = cu + (long)pair * cnt, *pv = cv + (long)pair * cnt;
    const float du = pu[k], dv = pv[k];
    const double flu = floor((double)du), flv = floor((double)dv);
    const double flu2 = floor((double)(du / 2.0f)), flv2 = floor((double)(dv / 2.0f));
    const int top = tops[ti], left = lefts[tj];
    const int topRefB = (int)(short)((double)top + flu), leftRefB = (int)(short)((double)left + flv);
    const int tid = threadIdx.x, nt = blockDim.x;

    // mini: the neighbourhood spline in shared memory
    __shared__ double s_ys[kMiniR], s_xs[kMiniR], s_kd[2][KF_ARRAYS * kMiniR];
    __shared__ float2 s_kfy[KF_ARRAYS * kMiniR], s_kfx[KF_ARRAYS * kMiniR];
    __shared__ float s_fys[kMiniR], s_fxs[kMiniR], s_f[2][kMiniR * kMiniR];
    __shared__ float s_fy[2][kMiniR * kMiniR], s_fx[2][kMiniR * kMiniR];
    __shared__ float2 s_scr[2][2][kMiniR * kMiniR];
    __shared__ float4 s_c4[2][kMiniR * kMiniR];
    __shared__ int s_max[2];
    const int r2 = kMiniR / 2;
    const int i0 = ti - r2 < 0 ? 0 : ti - r2, i1 = ti + r2 > ni - 1 ? ni - 1 : ti + r2;
    const int j0 = tj - r2 < 0 ? 0 : tj - r2, j1 = tj + r2 > nj - 1 ? nj - 1 : tj + r2;
    const int di = i1 - i0 + 1, dj = j1 - j0 + 1;
    if (tid < 2) s_max[tid] = 0;
    if (mini) {
        for (int q = tid; q < di * dj; q += nt) {
            const int a = q / dj, b = q - a * dj;
            const long kk = (long)(i0 + a) * nj + (j0 + b);
            s_f[0][q] = (float)((double)pu[kk] - flu);
            s_f[1][q] = (float)((double)pv[kk] - flv);
        }
        if (tid < di) {
            s_fys[tid] = (float)tops[i0 + tid] + (float)n / 2.0f - 0.5f;
            s_ys[tid] = (double)s_fys[tid];
        }
        if (tid >= 32 && tid < 32 + dj) {
            const int j = tid - 32;
            s_fxs[j] = (float)lefts[j0 + j] + (float)n / 2.0f - 0.5f;
            s_xs[j] = (double)s_fxs[j];
        }
        __syncthreads();
        if (tid == 0) knot_factors(s_ys, di, s_kd[0]);
        if (tid == 1) knot_factors(s_xs, dj, s_kd[1]);
        __syncthreads();
        for (int q = tid; q < KF_ARRAYS * (di + dj); q += nt) {
            const bool y = q < KF_ARRAYS * di;
            const int k = y ? q : q - KF_ARRAYS * di;
            const dword d = dw_of(s_kd[y ? 0 : 1][k]);
            (y ? s_kfy : s_kfx)[k] = make_float2(d.hi, d.lo);
        }
        __syncthreads();
        // knot derivatives: column lines (along y) and row lines (along x) of both components
        for (int q = tid; q < 2 * (dj + di); q += nt) {
            const int comp = q / (dj + di), line = q - comp * (dj + di);
            const float *f = s_f[comp];
            if (line < dj) {
                float2 *scr = s_scr[comp][0] + line;
                float *o = s_fy[comp] + line;
                spline_line_dw<1>(
                    s_kfy, di, [&](int i) { return f[i * dj + line]; }, [&](int i) -> float2 & { return scr[i * dj]; },
                    [&](int i, float d) { o[i * dj] = d; });
            } else {
                const int row = line - dj;
                float2 *scr = s_scr[comp][1] + row * dj;
                float *o = s_fx[comp] + row * dj;
                spline_line_dw<1>(
                    s_kfx, dj, [&](int j) { return f[row * dj + j]; }, [&](int j) -> float2 & { return scr[j]; },
                    [&](int j, float d) { o[j] = d; });
            }
        }
        __syncthreads();
        // cross derivatives and float nodes
        for (int q = tid; q < 2 * di * dj; q += nt) {
            const int comp = q / (di * dj), kk = q - comp * di * dj;
            const int i = kk / dj, j = kk - i * dj;
            const float *f = s_f[comp];
            const float fyx = spline_cross([&](int a, int b) { return f[a * dj + b]; }, di, dj, i, j,
                                           s_kfy + KF_RC * di, s_kfx + KF_RC * dj);
            s_c4[comp][kk] = make_float4(f[kk], s_fy[comp][kk], s_fx[comp][kk], fyx);
        }
        __syncthreads();
    }
    // offsets and origins of the warped sides
    int topA = top, leftA = left, topB = top, leftB = left;
    float uoA = 0.0f, voA = 0.0f, uoB = 0.0f, voB = 0.0f;
    if (image_mode == 1) {
        topA = (int)(short)((double)top - flu);
        leftA = (int)(short)((double)left - flv);
    } else if (image_mode == 2) {
        topB = topRefB;
        leftB = leftRefB;
    } else {
        topA = (int)(short)((double)top - flu2);
        leftA = (int)(short)((double)left - flv2);
        uoA = (float)((double)(du / 2.0f) - flu2) - (float)((double)du - flu);
        voA = (float)((double)(dv / 2.0f) - flv2) - (float)((double)dv - flv);
        topB = (int)(short)((double)top + flu2);
        leftB = (int)(short)((double)left + flv2);
        uoB = (float)((double)(du / 2.0f) - flu2);
        voB = (float)((double)(dv / 2.0f) - flv2);
    }
    const float mu = du - (float)flu, mv = dv - (float)flv;
    const long base = ((long)pair * cnt + k) * n * n;
    int lmax[2] = {0, 0};
    for (int q = tid; q < n * n; q += nt) {
        const int i = q / n, j = q - i * n;
        float u = mu, v = mv;
        if (mini) {
            float y = (float)topRefB + (float)i, x = (float)leftRefB + (float)j;
            const float ymin = s_fys[0], ymax = s_fys[di - 1], xmin = s_fxs[0], xmax = s_fxs[dj - 1];
            if (y < ymin) y = ymin; else if (y > ymax) y = ymax;
            if (x < xmin) x = xmin; else if (x > xmax) x = xmax;
            u = field_value(s_fys, di, s_fxs, dj, s_c4[0], y, x);
            v = field_value(s_fys, di, s_fxs, dj, s_c4[1], y, x);
        }
        // image A
        if (image_mode == 2) {
            const int y = top + i, x = left + j;
            const int val = (y >= 0 && y < h && x >= 0 && x < w) ? (int)ia[(long)y * pitch + x] : 0;
            tiles_a[base + q] = (Pix)val;
            lmax[0] = val > lmax[0] ? val : lmax[0];
        } else {
            float ua = u, va = v;
            if (image_mode == 3) {
                ua = u / 2.0f + uoA;
                va = v / 2.0f + voA;
            }
            const float val =
                warp_pixel(ia, h, w, pitch, ua, va, (int)(short)(i + topA), (int)(short)(j + leftA), true);
            tiles_a[base + q] = (Pix)(int)val;
        }
        // image B
        if (image_mode == 1) {
            const int y = top + i, x = left + j;
            const int val = (y >= 0 && y < h && x >= 0 && x < w) ? (int)ib[(long)y * pitch + x] : 0;
            tiles_b[base + q] = (Pix)val;
            lmax[1] = val > lmax[1] ? val : lmax[1];
        } else {
            float ub = u, vb = v;
            if (image_mode == 3) {
                ub = u / 2.0f + uoB;
                vb = v / 2.0f + voB;
            }
            const float val =
                warp_pixel(ib, h, w, pitch, ub, vb, (int)(short)(i + topB), (int)(short)(j + leftB), false);
            tiles_b[base + q] = (Pix)(int)val;
        }
    }
    if (image_mode != 3) {
        atomicMax(&s_max[0], lmax[0]);
        atomicMax(&s_max[1], lmax[1]);
    }
    __syncthreads();
    if (tid == 0) {
        const long o = (long)pair * cnt + k;
        max_a[o] = image_mode == 2 ? (float)(s_max[0] < 16 ? 16 : s_max[0]) : full_max;
        max_b[o] = image_mode == 1 ? (float)(s_max[1] < 16 ? 16 : s_max[1]) : full_max;
    }
}

// Per-pixel field only (test hook for the field stage): pair 0, outputs h x w floats.
// 32 x 8 pixels per block, the column and row bases shared as in warp_both_kernel.
__global__ void __launch_bounds__(256) field_kernel(int h, int w, const float *ys, int ni, const float *xs, int nj,
                                                    const float4 *c4u, const float4 *c4v, float off_y, float off_x,
                                                    float *fu_out, float *fv_out) {
    __shared__ float sx[32][4], sy[8][4];
    __shared__ int sj[32], si[8];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int j = blockIdx.x * 32 + tx, i = blockIdx.y * 8 + ty;
    // pixel i is evaluated at off_y + i (the reference steps a float from the offset by 1.0f)
    if (ty == 0) {
        float x = off_x + (float)j;
        if (x < xs[0]) x = xs[0]; else if (x > xs[nj - 1]) x = xs[nj - 1];
        sj[tx] = field_basis(xs, nj, x, sx[tx]);
    } else if (ty == 1 && tx < 8) {
        float y = off_y + (float)(blockIdx.y * 8 + tx);
        if (y < ys[0]) y = ys[0]; else if (y > ys[ni - 1]) y = ys[ni - 1];
        si[tx] = field_basis(ys, ni, y, sy[tx]);
    }
    __syncthreads();
    if (i >= h || j >= w) return;
    float X[4], Y[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        X[k] = sx[tx][k];
        Y[k] = sy[ty][k];
    }
    fu_out[(long)i * w + j] = field_combine(c4u, nj, si[ty], sj[tx], X, Y);
    fv_out[(long)i * w + j] = field_combine(c4v, nj, si[ty], sj[tx], X, Y);
}

// B tile origins for non-warping modes: round(top + u), round(left + v)
// (NoImageWarpingStrategy.java:80, FastMath.round of Tile.getDisplacedTileTop()).
__global__ void displaced_origins_kernel(long count, const int *a_top, const int *a_left, const float *u,
                                         const float *v, int *b_top, int *b_left) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    b_top[k] = java_round((float)a_top[k] + u[k]);
    b_left[k] = java_round((float)a_left[k] + v[k]);
}

// Inheritance under NoOutOfBoundClipping: a child tile starts at zero and takes its inherited
// value through Tile.accumulateDisplacement (S/iareas/Tile.java:103-136), which drops a value that
// would move the tile out of the image (the tile then keeps zero).
__global__ void clip_inherited_kernel(long count, const int *top, const int *left, int n, int h, int w, float *u,
                                      float *v) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const float nu = __fadd_rn(0.0f, u[k]), nv = __fadd_rn(0.0f, v[k]);
    const bool ok = tile_inside(n, h, w, top[k], left[k], nu, nv);
    u[k] = ok ? nu : 0.0f;
    v[k] = ok ? nv : 0.0f;
}

// ---------------- launchers ----------------

static inline unsigned blocks_for(long n, int t) { return (unsigned)((n + t - 1) / t); }

cudaError_t launch_inherit(cudaStream_t s, int pairs, const float *py, int pni, const float *px, int pnj,
                           const float *pu, const float *pv, const float *cy, int cni, const float *cx, int cnj,
                           int round_int, float *ru, float *rv, float *cu, float *cv) {
    const long n = (long)pairs * cni * cnj;
    if (n == 0) return cudaSuccess;
    if (pni < 5 || pnj < 5) {  // the reference computes a bilinear value here but never applies it
        cudaError_t e = cudaMemsetAsync(cu, 0, sizeof(float) * n, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(cv, 0, sizeof(float) * n, s);
        return e;
    }
    const long nr = (long)pairs * cni * pnj;
    inherit_rows_kernel<<<blocks_for(nr, 128), 128, 0, s>>>(pairs, py, pni, pnj, pu, pv, cy, cni, ru, rv);
    inherit_cols_kernel<<<blocks_for(n, 128), 128, 0, s>>>(pairs, px, pnj, cx, cni, cnj, ru, rv, round_int, cu, cv);
    return cudaGetLastError();
}

cudaError_t launch_inherit_tiles(cudaStream_t s, int pairs, int mode, int pn, int pni, int pnj, const int *ptops,
                                 const int *plefts, const float *pu, const float *pv, int cn, int cni, int cnj,
                                 const int *ctops, const int *clefts, const int2 *tables, int round_int, float *cu,
                                 float *cv) {
    const long n = (long)pairs * cni * cnj;
    if (n == 0) return cudaSuccess;
    inherit_tiles_kernel<<<blocks_for(n, 128), 128, 0, s>>>(pairs, mode, pn, pni, pnj, ptops, plefts, pu, pv, cn, cni,
                                                              cnj, ctops, clefts, tables, tables + cni, round_int, cu,
                                                              cv);
    return cudaGetLastError();
}

cudaError_t launch_spline(cudaStream_t s, int pairs, const float2 *kfy, int ni, const float2 *kfx, int nj,
                          const float *u, const float *v, SplineCoef coef, const int *gate) {
    const long warps = (long)pairs * 2 * ((ni + 31) / 32 + (nj + 31) / 32);
    spline_nodes_kernel<<<blocks_for(warps * 32, 128), 128, 0, s>>>(pairs, kfy, ni, kfx, nj, u, v, coef, gate);
    return cudaGetLastError();
}

cudaError_t launch_warp(cudaStream_t s, int pixel_type, int pairs, int h, int w, const qlpiv_frame *src,
                        const qlpiv_frame *dst, const float *ys, int ni, const float *xs, int nj, SplineCoef coef,
                        int int16_quirk, int image_mode, const int *gate) {
    if (image_mode < 1 || image_mode > 3) return cudaErrorInvalidValue;
    dim3 blk(32, 8), grd(blocks_for(w, 32), blocks_for(h, kWarpRows), pairs);
    if (pixel_type == QLPIV_PIX_U8)
        warp_both_kernel<uint8_t><<<grd, blk, 0, s>>>(src, dst, ys, ni, xs, nj, coef.c4_u, coef.c4_v, int16_quirk,
                                                      image_mode, gate);
    else if (pixel_type == QLPIV_PIX_U16)
        warp_both_kernel<uint16_t><<<grd, blk, 0, s>>>(src, dst, ys, ni, xs, nj, coef.c4_u, coef.c4_v, int16_quirk,
                                                       image_mode, gate);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_tile_warp(cudaStream_t s, int pixel_type, int pairs, const qlpiv_frame *frames, int n, int ni,
                             int nj, const int *tops, const int *lefts, const float *cu, const float *cv,
                             int image_mode, int mini, float full_max, void *tiles_a, void *tiles_b, float *max_a,
                             float *max_b) {
    const dim3 grd((unsigned)((long)ni * nj), pairs);
    if (pixel_type == QLPIV_PIX_U8)
        tile_warp_kernel<uint8_t><<<grd, 256, 0, s>>>(frames, n, ni, nj, tops, lefts, cu, cv, image_mode, mini,
                                                      full_max, (uint8_t *)tiles_a, (uint8_t *)tiles_b, max_a, max_b);
    else if (pixel_type == QLPIV_PIX_U16)
        tile_warp_kernel<uint16_t><<<grd, 256, 0, s>>>(frames, n, ni, nj, tops, lefts, cu, cv, image_mode, mini,
                                                       full_max, (uint16_t *)tiles_a, (uint16_t *)tiles_b, max_a,
                                                       max_b);
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_field(cudaStream_t s, int h, int w, const float *ys, int ni, const float *xs, int nj,
                         SplineCoef coef, float *fu, float *fv, float off_y, float off_x) {
    dim3 blk(32, 8), grd(blocks_for(w, 32), blocks_for(h, 8), 1);
    field_kernel<<<grd, blk, 0, s>>>(h, w, ys, ni, xs, nj, coef.c4_u, coef.c4_v, off_y, off_x, fu, fv);
    return cudaGetLastError();
}

cudaError_t launch_displaced_origins(cudaStream_t s, long count, const int *a_top, const int *a_left, const float *u,
                                     const float *v, int *b_top, int *b_left) {
    if (count == 0) return cudaSuccess;
    displaced_origins_kernel<<<blocks_for(count, 256), 256, 0, s>>>(count, a_top, a_left, u, v, b_top, b_left);
    return cudaGetLastError();
}

// InterAreaDisplacementStableStrategy.computeStableState (S/iareas/InterAreaDisplacementStableStrategy.java:19-36)
// after pass `pass` of a level: the tiles of in_list (all `count` tiles when NULL) whose
// increment out[ia].(u, v) has (float) sqrt(u^2 + v^2) (double) above max_disp stay EVALUATING
// while pass < max_retries and are listed in out_list ([0] count, then tiles; zeroed before).
__global__ void stable_update_kernel(int pass, int max_retries, float max_disp, const qlpiv_vector *out,
                                     const int *in_list, long count, int *out_list) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long n = in_list != nullptr ? (long)in_list[0] : count;
    if (k >= n) return;
    const long ia = in_list != nullptr ? (long)in_list[1 + k] : k;
    const double du = (double)out[ia].u, dv = (double)out[ia].v;
    const float norm = (float)sqrt(du * du + dv * dv);
    if (norm > max_disp && pass < max_retries) out_list[1 + atomicAdd(out_list, 1)] = (int)ia;
}

cudaError_t launch_stable_update(cudaStream_t s, int pass, int max_retries, float max_disp, const qlpiv_vector *out,
                                 const int *in_list, long count, int *out_list) {
    cudaError_t e = cudaMemsetAsync(out_list, 0, sizeof(int), s);
    if (e != cudaSuccess || count == 0) return e;
    stable_update_kernel<<<blocks_for(count, 256), 256, 0, s>>>(pass, max_retries, max_disp, out, in_list, count,
                                                                  out_list);
    return cudaGetLastError();
}

cudaError_t launch_clip_inherited(cudaStream_t s, long count, const int *top, const int *left, int n, int h, int w,
                                  float *u, float *v) {
    if (count == 0) return cudaSuccess;
    clip_inherited_kernel<<<blocks_for(count, 256), 256, 0, s>>>(count, top, left, n, h, w, u, v);
    return cudaGetLastError();
}

}  // namespace qlpiv
