/*
 * Sub-pixel peak interpolators beyond the 3-point Gaussian -- TEST INFRASTRUCTURE ONLY (the CPU
 * oracle; the product never links it).
 *
 *   Gaussian 1D-1D least squares  S/interpolators/Gaussian1DInterpolator.java:36-115: per axis, P
 *       (odd) plane values through the peak fitted by a * exp(-(x - m)^2 / (2 s^2)) in the least
 *       squares sense (the reference calls commons-math3 3.6.1 GaussianCurveFitter, a
 *       Levenberg-Marquardt optimiser; this is a Levenberg-Marquardt restatement from the
 *       mathematics that converges to the same minimiser); the floor is lifted by -minFloor +
 *       1e-8 when negative (error below -3.15); m is kept when |m - peak| < 2.
 *   Hongwei Guo weighted fit      S/interpolators/Gaussian1DHongweiGuoInterpolator.java:47-250:
 *       ln y = c0 + c1 x + c2 x^2 by least squares weighted with y^2, the weights re-estimated
 *       from the fit `iterations` times (the last solve is used); mean -c1 / (2 c2), amplitude
 *       exp(c0 - c1^2 / (4 c2)); the 3x3 normal equations solved by the textbook LU with
 *       partial pivoting, or by the pseudo-inverse when a pivot is below 1e-11 (the reference:
 *       commons-math3 LUDecomposition, SingularValueDecomposition when singular); the floor is lifted when negative (error below -5.15);
 *       a mean farther than P/2 from the peak keeps the integer peak; the peak value becomes the
 *       fitted amplitude of an accepted axis (the larger of the two).
 * Both skip a peak at (0, 0) and a peak whose P-point stencil leaves the plane.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "oracle_types.h"

#define F_SUB_I 1u
#define F_SUB_J 2u
#define F_EDGE 8u
#define F_NO_PEAK 16u
#define F_FLOOR 64u

/* ---------- Levenberg-Marquardt Gaussian fit of one axis ---------- */

static double lm_cost(const double *x, const double *y, int n, const double *p) {
    double c = 0.0;
    for (int k = 0; k < n; k++) {
        const double d = x[k] - p[1];
        const double r = y[k] - p[0] * exp(-d * d / (2.0 * p[2] * p[2]));
        c += r * r;
    }
    return c;
}

/* Solves the 3x3 system a z = b by Gaussian elimination with partial pivoting; 0 if singular. */
static int solve3(double a[3][3], double b[3], double z[3]) {
    int piv[3] = {0, 1, 2};
    for (int c = 0; c < 3; c++) {
        int best = c;
        for (int r = c + 1; r < 3; r++)
            if (fabs(a[r][c]) > fabs(a[best][c])) best = r;
        if (fabs(a[best][c]) < 1e-300) return 0;
        if (best != c) {
            for (int k = 0; k < 3; k++) {
                const double t = a[c][k];
                a[c][k] = a[best][k];
                a[best][k] = t;
            }
            const double t = b[c];
            b[c] = b[best];
            b[best] = t;
            const int ti = piv[c];
            piv[c] = piv[best];
            piv[best] = ti;
        }
        for (int r = c + 1; r < 3; r++) {
            const double f = a[r][c] / a[c][c];
            for (int k = c; k < 3; k++) a[r][k] -= f * a[c][k];
            b[r] -= f * b[c];
        }
    }
    for (int r = 2; r >= 0; r--) {
        double s = b[r];
        for (int k = r + 1; k < 3; k++) s -= a[r][k] * z[k];
        z[r] = s / a[r][r];
    }
    return 1;
}

/* Least-squares Gaussian through (x[k], y[k]); returns 1 and the mean when the fit converged to a
 * finite mean.  Coordinates are taken relative to the sample of the largest value.  Start: the
 * Gaussian through the three samples around the max (exact for Gaussian data and the least-squares
 * solution for three samples); else amplitude = max y, mean = its x, width 1.
 * Levenberg-Marquardt with Nielsen's damping update; stops when a step no longer lowers the cost
 * or the step is below 1e-13 relative. */
int orc_gauss_lm_fit(const double *x_in, const double *y, int n, double *mean_out) {
    if (n < 3 || n > 64) return 0;
    int im = 0;
    for (int k = 1; k < n; k++)
        if (y[k] > y[im]) im = k;
    const double x0 = x_in[im];
    double x[64];
    for (int k = 0; k < n; k++) x[k] = x_in[k] - x0;
    double p[3] = {y[im], 0.0, 1.0};
    if (!(p[0] > 0.0)) return 0;
    if (im > 0 && im < n - 1 && y[im - 1] > 0.0 && y[im + 1] > 0.0) {
        /* the Gaussian through the three samples around the max (exact for Gaussian data) */
        const double l0 = log(y[im - 1]), l1 = log(y[im]), l2 = log(y[im + 1]);
        const double c2 = 0.5 * (l0 + l2) - l1, c1 = 0.5 * (l2 - l0);
        if (c2 < 0.0) {
            const double m = -c1 / (2.0 * c2), s = sqrt(-1.0 / (2.0 * c2));
            const double amp = exp(l1 - c1 * c1 / (4.0 * c2));
            if (isfinite(m) && isfinite(s) && isfinite(amp) && fabs(m) < 1.0) {
                p[0] = amp;
                p[1] = m;
                p[2] = s;
            }
        }
    }
    double cost = lm_cost(x, y, n, p);
    double mu = -1.0, nu = 2.0;
    for (int it = 0; it < 500 && cost > 0.0; it++) {
        double jtj[3][3] = {{0}}, jtr[3] = {0};
        for (int k = 0; k < n; k++) {
            const double d = x[k] - p[1], s2 = p[2] * p[2];
            const double e = exp(-d * d / (2.0 * s2));
            const double r = y[k] - p[0] * e;
            const double g[3] = {e, p[0] * e * d / s2, p[0] * e * d * d / (s2 * p[2])};
            for (int a = 0; a < 3; a++) {
                jtr[a] += g[a] * r;
                for (int b = 0; b < 3; b++) jtj[a][b] += g[a] * g[b];
            }
        }
        if (mu < 0.0) {
            double dmax = jtj[0][0];
            if (jtj[1][1] > dmax) dmax = jtj[1][1];
            if (jtj[2][2] > dmax) dmax = jtj[2][2];
            mu = 1e-6 * dmax;
        }
        int accepted = 0;
        for (int tries = 0; tries < 60 && !accepted; tries++) {
            double a[3][3], b[3], z[3];
            for (int i = 0; i < 3; i++) {
                for (int j = 0; j < 3; j++) a[i][j] = jtj[i][j];
                a[i][i] += mu;
                b[i] = jtr[i];
            }
            if (!solve3(a, b, z)) {
                mu *= nu;
                nu *= 2.0;
                continue;
            }
            const double q[3] = {p[0] + z[0], p[1] + z[1], p[2] + z[2]};
            const double c2 = q[2] != 0.0 ? lm_cost(x, y, n, q) : INFINITY;
            /* gain ratio: actual / predicted decrease (predicted = z . (mu z + J^T r)) */
            const double pred = z[0] * (mu * z[0] + jtr[0]) + z[1] * (mu * z[1] + jtr[1]) + z[2] * (mu * z[2] + jtr[2]);
            const double rho = pred > 0.0 ? (cost - c2) / pred : -1.0;
            if (isfinite(c2) && c2 <= cost && rho > 0.0) {
                const double step = fabs(z[1]) + fabs(z[2]) / fabs(q[2]);
                p[0] = q[0];
                p[1] = q[1];
                p[2] = q[2];
                const double t = 2.0 * rho - 1.0;
                const double f = 1.0 - t * t * t;
                mu *= f > 1.0 / 3.0 ? f : 1.0 / 3.0;
                nu = 2.0;
                accepted = 1;
                if (step < 1e-13 || c2 == cost) it = 1 << 20;  /* converged */
                cost = c2;
            } else {
                mu *= nu;
                nu *= 2.0;
            }
        }
        if (!accepted) break;  /* no descent step left: at the minimum within rounding */
    }
    if (!isfinite(p[1])) return 0;
    *mean_out = x0 + p[1];
    return 1;
}

/* ---------- Hongwei Guo iteratively weighted log fit of one axis ---------- */

static void hg_accumulate(const float *xs, const float *ys, int n, const double *coefs, double a[3][3],
                          double b[3]) {
    memset(a, 0, sizeof(double) * 9);
    memset(b, 0, sizeof(double) * 3);
    for (int i = 0; i < n; i++) {
        double ySquare;
        if (!coefs) {
            ySquare = (double)(ys[i] * ys[i]);   /* float product, as the reference's float arrays */
        } else {
            const double yk = exp(coefs[0] + coefs[1] * xs[i] + coefs[2] * xs[i] * xs[i]);
            ySquare = yk * yk;
        }
        const double xSquare = (double)(xs[i] * xs[i]);
        const double xCubic = xSquare * xs[i];
        const double xFourth = xCubic * xs[i];
        const double logyEst = log((double)ys[i]);
        a[0][0] += ySquare;
        a[0][1] += xs[i] * ySquare;
        a[0][2] += xSquare * ySquare;
        b[0] += ySquare * logyEst;
        a[1][0] += xs[i] * ySquare;
        a[1][1] += xSquare * ySquare;
        a[1][2] += xCubic * ySquare;
        b[1] += xs[i] * ySquare * logyEst;
        a[2][0] += xSquare * ySquare;
        a[2][1] += xCubic * ySquare;
        a[2][2] += xFourth * ySquare;
        b[2] += xSquare * ySquare * logyEst;
    }
}

/* LU decomposition with partial pivoting in the textbook column order (for each column: the upper
 * entries, then the lower ones with the first largest magnitude as pivot, rows swapped, the lower
 * entries divided by the pivot), then column-oriented forward and back substitution.  0 when a
 * pivot's magnitude is below 1e-11 (singular). */
static int lu_solve3(const double a_in[3][3], const double b_in[3], double x[3]) {
    double lu[3][3];
    memcpy(lu, a_in, sizeof(lu));
    int perm[3] = {0, 1, 2};
    for (int col = 0; col < 3; col++) {
        for (int row = 0; row < col; row++) {
            double sum = lu[row][col];
            for (int i = 0; i < row; i++) sum -= lu[row][i] * lu[i][col];
            lu[row][col] = sum;
        }
        int max = col;
        double largest = -INFINITY;
        for (int row = col; row < 3; row++) {
            double sum = lu[row][col];
            for (int i = 0; i < col; i++) sum -= lu[row][i] * lu[i][col];
            lu[row][col] = sum;
            if (fabs(sum) > largest) {
                largest = fabs(sum);
                max = row;
            }
        }
        if (fabs(lu[max][col]) < 1e-11) return 0;
        if (max != col) {
            for (int i = 0; i < 3; i++) {
                const double t = lu[max][i];
                lu[max][i] = lu[col][i];
                lu[col][i] = t;
            }
            const int t = perm[max];
            perm[max] = perm[col];
            perm[col] = t;
        }
        const double d = lu[col][col];
        for (int row = col + 1; row < 3; row++) lu[row][col] /= d;
    }
    double bp[3] = {b_in[perm[0]], b_in[perm[1]], b_in[perm[2]]};
    for (int col = 0; col < 3; col++)
        for (int i = col + 1; i < 3; i++) bp[i] -= bp[col] * lu[i][col];
    for (int col = 2; col >= 0; col--) {
        bp[col] /= lu[col][col];
        for (int i = 0; i < col; i++) bp[i] -= bp[col] * lu[i][col];
    }
    x[0] = bp[0];
    x[1] = bp[1];
    x[2] = bp[2];
    return 1;
}

/* Least-squares (minimum norm) solution of the symmetric 3x3 system a x = b through the
 * eigendecomposition of a (cyclic Jacobi rotations): for a symmetric matrix the singular values
 * are the eigenvalue magnitudes, and components below 3 * sigma_max * 2^-52 are dropped (the
 * pseudo-inverse a singular-value decomposition solver applies). */
static void svd_solve3_sym(const double a_in[3][3], const double b[3], double x[3]) {
    double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    memcpy(a, a_in, sizeof(a));
    for (int sweep = 0; sweep < 64; sweep++) {
        const double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
        if (off == 0.0) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                if (a[p][q] == 0.0) continue;
                const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 3; k++) {  /* a <- a J */
                    const double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - sn * akq;
                    a[k][q] = sn * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {  /* a <- J^T a */
                    const double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - sn * aqk;
                    a[q][k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {  /* v <- v J */
                    const double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - sn * vkq;
                    v[k][q] = sn * vkp + c * vkq;
                }
            }
    }
    double smax = 0.0;
    for (int k = 0; k < 3; k++)
        if (fabs(a[k][k]) > smax) smax = fabs(a[k][k]);
    double tol = 3.0 * smax * 2.220446049250313e-16;
    if (tol < 1.4916681462400413e-154) tol = 1.4916681462400413e-154;
    x[0] = x[1] = x[2] = 0.0;
    for (int k = 0; k < 3; k++) {
        const double lam = a[k][k];
        if (fabs(lam) <= tol) continue;
        const double proj = (v[0][k] * b[0] + v[1][k] * b[1] + v[2][k] * b[2]) / lam;
        for (int i = 0; i < 3; i++) x[i] += proj * v[i][k];
    }
}

/* Returns 1 with mean and amplitude. */
int orc_hongwei_guo_fit(const float *xs, const float *ys, int n, int iterations, float *mean, float *amplitude) {
    double a[3][3], b[3], coefs[3] = {0.0, 0.0, 0.0};
    hg_accumulate(xs, ys, n, NULL, a, b);
    for (int it = 0; it < iterations; it++) {
        if (!lu_solve3(a, b, coefs)) svd_solve3_sym(a, b, coefs);   /* singular: least squares */
        hg_accumulate(xs, ys, n, coefs, a, b);
    }
    *mean = (float)(-coefs[1] / (2 * coefs[2]));
    *amplitude = (float)exp(coefs[0] - coefs[1] * coefs[1] / (4 * coefs[2]));
    return 1;
}

/* ---------- the two interpolators on a correlation plane ---------- */

static int stencil_fits(int d, int mi, int mj, int P) {
    if (P < 3 || P > 63) return 0;
    return !(mi - P / 2 < 0 || mi + P / 2 >= d || mj - P / 2 < 0 || mj + P / 2 >= d);
}

void orc_subpixel_lm(const float *plane, int d, int mi, int mj, int P, float min_floor, float *si, float *sj,
                     uint32_t *flags) {
    *si = (float)mi;
    *sj = (float)mj;
    *flags = 0;
    if (mi == 0 && mj == 0) { *flags = F_NO_PEAK; return; }
    if (!stencil_fits(d, mi, mj, P)) { *flags = F_EDGE; return; }
    if (min_floor < -3.15f) { *flags = F_FLOOR; return; }
    const float add = min_floor < 0.0f ? -min_floor + 1e-8f : 0.0f;
    double x[64] = {0}, y[64] = {0};
    for (int k = 0; k < P; k++) {
        x[k] = mi - P / 2 + k;
        y[k] = (double)(plane[(size_t)(mi - P / 2 + k) * d + mj] + add);
    }
    double m;
    if (orc_gauss_lm_fit(x, y, P, &m) && fabs(m - (double)(float)mi) < 2.0f) { *si = (float)m; *flags |= F_SUB_I; }
    for (int k = 0; k < P; k++) {
        x[k] = mj - P / 2 + k;
        y[k] = (double)(plane[(size_t)mi * d + mj - P / 2 + k] + add);
    }
    if (orc_gauss_lm_fit(x, y, P, &m) && fabs(m - (double)(float)mj) < 2.0f) { *sj = (float)m; *flags |= F_SUB_J; }
}

void orc_subpixel_hg(const float *plane, int d, int mi, int mj, int P, int iterations, float min_floor, float *si,
                     float *sj, float *pv, uint32_t *flags) {
    *si = (float)mi;
    *sj = (float)mj;
    *flags = 0;
    if (mi == 0 && mj == 0) { *flags = F_NO_PEAK; return; }
    if (!stencil_fits(d, mi, mj, P)) { *flags = F_EDGE; return; }
    if (min_floor < -5.15f) { *flags = F_FLOOR; return; }
    const float add = min_floor < 0.0f ? -min_floor + 1e-8f : 0.0f;
    float xs[64] = {0}, ys[64] = {0};
    for (int k = 0; k < P; k++) {
        xs[k] = (float)(mi - P / 2 + k);
        ys[k] = plane[(size_t)(mi - P / 2 + k) * d + mj] + add;
    }
    float ym = 0.0f, ya = 0.0f, xm = 0.0f, xa = 0.0f;
    const int yok = orc_hongwei_guo_fit(xs, ys, P, iterations, &ym, &ya);
    for (int k = 0; k < P; k++) {
        xs[k] = (float)(mj - P / 2 + k);
        ys[k] = plane[(size_t)mi * d + mj - P / 2 + k] + add;
    }
    const int xok = orc_hongwei_guo_fit(xs, ys, P, iterations, &xm, &xa);
    const int yValid = yok && !(fabsf(ym - (float)mi) > (float)P / 2.0f);
    const int xValid = xok && !(fabsf(xm - (float)mj) > (float)P / 2.0f);
    if (yValid) { *si = ym; *flags |= F_SUB_I; }
    if (xValid) { *sj = xm; *flags |= F_SUB_J; }
    if (yValid) {
        *pv = ya;
        if (xValid && xa > *pv) *pv = xa;
    } else if (xValid) {
        *pv = xa;
    }
}
