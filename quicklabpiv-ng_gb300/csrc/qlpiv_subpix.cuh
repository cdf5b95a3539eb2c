// Sub-pixel interpolators with P-point stencils, per fit-queue lane (double precision):
//   Gaussian 1D-1D least squares  S/interpolators/Gaussian1DInterpolator.java:36-115 (the reference
//       fits a * exp(-(x - m)^2 / (2 s^2)) with commons-math3's GaussianCurveFitter; here
//       Levenberg-Marquardt from the Gaussian through the three samples around the maximum, with
//       Nielsen's damping update, converging to the same least-squares minimiser);
//   Hongwei Guo weighted fit      S/interpolators/Gaussian1DHongweiGuoInterpolator.java:47-250
//       (ln y = c0 + c1 x + c2 x^2 weighted by y^2, re-weighted `iterations` times; the 3x3 normal
//       equations by LU with partial pivoting, the pseudo-inverse when a pivot is below 1e-11).
// The stencil values are the plane's floats; coordinates are plane indices.
#pragma once
#include <cuda_runtime.h>

namespace qlpiv {

constexpr int kMaxSubpixPixels = 15;

__device__ __forceinline__ bool sp_solve3(double a[3][3], double b[3], double z[3]) {
    for (int c = 0; c < 3; c++) {
        int best = c;
        for (int r = c + 1; r < 3; r++)
            if (fabs(a[r][c]) > fabs(a[best][c])) best = r;
        if (fabs(a[best][c]) < 1e-300) return false;
        if (best != c) {
            for (int k = 0; k < 3; k++) {
                const double t = a[c][k];
                a[c][k] = a[best][k];
                a[best][k] = t;
            }
            const double t = b[c];
            b[c] = b[best];
            b[best] = t;
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
    return true;
}

__device__ __forceinline__ double sp_lm_cost(const double *x, const float *y, int n, const double *p) {
    double c = 0.0;
    for (int k = 0; k < n; k++) {
        const double d = x[k] - p[1];
        const double r = (double)y[k] - p[0] * exp(-d * d / (2.0 * p[2] * p[2]));
        c += r * r;
    }
    return c;
}

// Least-squares Gaussian mean of samples y[k] at x0 - n/2 + k (y already floor-lifted); false when
// the fit has no finite mean.
static __device__ __noinline__ bool sp_gauss_lm(const float *y, int n, double x0c, double *mean) {
    int im = 0;
    for (int k = 1; k < n; k++)
        if (y[k] > y[im]) im = k;
    double x[kMaxSubpixPixels];
    for (int k = 0; k < n; k++) x[k] = (double)(k - im);
    const double xm = x0c - (double)(n / 2) + (double)im;  // absolute coordinate of the max
    double p[3] = {(double)y[im], 0.0, 1.0};
    if (!(p[0] > 0.0)) return false;
    if (im > 0 && im < n - 1 && y[im - 1] > 0.0f && y[im + 1] > 0.0f) {
        const double l0 = log((double)y[im - 1]), l1 = log((double)y[im]), l2 = log((double)y[im + 1]);
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
    double cost = sp_lm_cost(x, y, n, p);
    double mu = -1.0, nu = 2.0;
    for (int it = 0; it < 500 && cost > 0.0; it++) {
        double jtj[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, jtr[3] = {0, 0, 0};
        for (int k = 0; k < n; k++) {
            const double d = x[k] - p[1], s2 = p[2] * p[2];
            const double e = exp(-d * d / (2.0 * s2));
            const double r = (double)y[k] - p[0] * e;
            const double g[3] = {e, p[0] * e * d / s2, p[0] * e * d * d / (s2 * p[2])};
            for (int a = 0; a < 3; a++) {
                jtr[a] += g[a] * r;
                for (int b = 0; b < 3; b++) jtj[a][b] += g[a] * g[b];
            }
        }
        if (mu < 0.0) mu = 1e-6 * fmax(jtj[0][0], fmax(jtj[1][1], jtj[2][2]));
        bool accepted = false;
        for (int tries = 0; tries < 60 && !accepted; tries++) {
            double a[3][3], b[3], z[3];
            for (int i = 0; i < 3; i++) {
                for (int j = 0; j < 3; j++) a[i][j] = jtj[i][j];
                a[i][i] += mu;
                b[i] = jtr[i];
            }
            if (!sp_solve3(a, b, z)) {
                mu *= nu;
                nu *= 2.0;
                continue;
            }
            const double q[3] = {p[0] + z[0], p[1] + z[1], p[2] + z[2]};
            const double c2 = q[2] != 0.0 ? sp_lm_cost(x, y, n, q) : INFINITY;
            const double pred = z[0] * (mu * z[0] + jtr[0]) + z[1] * (mu * z[1] + jtr[1]) + z[2] * (mu * z[2] + jtr[2]);
            const double rho = pred > 0.0 ? (cost - c2) / pred : -1.0;
            if (isfinite(c2) && c2 <= cost && rho > 0.0) {
                const double step = fabs(z[1]) + fabs(z[2]) / fabs(q[2]);
                p[0] = q[0];
                p[1] = q[1];
                p[2] = q[2];
                const double t = 2.0 * rho - 1.0, f = 1.0 - t * t * t;
                mu *= f > 1.0 / 3.0 ? f : 1.0 / 3.0;
                nu = 2.0;
                accepted = true;
                if (step < 1e-13 || c2 == cost) it = 1 << 20;
                cost = c2;
            } else {
                mu *= nu;
                nu *= 2.0;
            }
        }
        if (!accepted) break;
    }
    if (!isfinite(p[1])) return false;
    *mean = xm + p[1];
    return true;
}

__device__ inline bool sp_lu_solve3(const double a_in[3][3], const double b_in[3], double x[3]) {
    double lu[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) lu[i][j] = a_in[i][j];
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
        if (fabs(lu[max][col]) < 1e-11) return false;
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
    return true;
}

// Minimum-norm least-squares solution of a symmetric 3x3 system (cyclic Jacobi eigendecomposition).
__device__ inline void sp_svd_solve3(const double a_in[3][3], const double b[3], double x[3]) {
    double a[3][3], v[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) a[i][j] = a_in[i][j];
    for (int sweep = 0; sweep < 64; sweep++) {
        if (fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]) == 0.0) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                if (a[p][q] == 0.0) continue;
                const double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < 3; k++) {
                    const double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - sn * akq;
                    a[k][q] = sn * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {
                    const double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - sn * aqk;
                    a[q][k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {
                    const double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - sn * vkq;
                    v[k][q] = sn * vkp + c * vkq;
                }
            }
    }
    const double smax = fmax(fabs(a[0][0]), fmax(fabs(a[1][1]), fabs(a[2][2])));
    const double tol = fmax(3.0 * smax * 2.220446049250313e-16, 1.4916681462400413e-154);
    x[0] = x[1] = x[2] = 0.0;
    for (int k = 0; k < 3; k++) {
        const double lam = a[k][k];
        if (fabs(lam) <= tol) continue;
        const double proj = (v[0][k] * b[0] + v[1][k] * b[1] + v[2][k] * b[2]) / lam;
        for (int i = 0; i < 3; i++) x[i] += proj * v[i][k];
    }
}

__device__ inline void sp_hg_accumulate(const float *xs, const float *ys, int n, const double *coefs, bool first,
                                        double a[3][3], double b[3]) {
    for (int i = 0; i < 3; i++) {
        b[i] = 0.0;
        for (int j = 0; j < 3; j++) a[i][j] = 0.0;
    }
    for (int i = 0; i < n; i++) {
        double ySquare;
        if (first) {
            ySquare = (double)__fmul_rn(ys[i], ys[i]);
        } else {
            const double yk = exp(coefs[0] + coefs[1] * xs[i] + coefs[2] * xs[i] * xs[i]);
            ySquare = yk * yk;
        }
        const double xSquare = (double)__fmul_rn(xs[i], xs[i]);
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

// Hongwei Guo fit of samples ys at xs; mean and amplitude (floats, like the reference's result).
static __device__ __noinline__ void sp_hongwei_guo(const float *xs, const float *ys, int n, int iterations, float *mean,
                                      float *amplitude) {
    double a[3][3], b[3], coefs[3] = {0.0, 0.0, 0.0};
    sp_hg_accumulate(xs, ys, n, coefs, true, a, b);
    for (int it = 0; it < iterations; it++) {
        if (!sp_lu_solve3(a, b, coefs)) sp_svd_solve3(a, b, coefs);
        sp_hg_accumulate(xs, ys, n, coefs, false, a, b);
    }
    *mean = (float)(-coefs[1] / (2 * coefs[2]));
    *amplitude = (float)exp(coefs[0] - coefs[1] * coefs[1] / (4 * coefs[2]));
}

}  // namespace qlpiv
