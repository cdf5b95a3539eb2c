/*
 * qlpiv oracle -- REAL-typed interpolators of the adaptive stages, included twice by
 * qlpiv_oracle_adaptive.c (float: the formulation the CUDA kernels evaluate, bit for
 * bit; double: the FP64 twin).  TEST INFRASTRUCTURE ONLY.
 *
 * Spline knot derivatives are always solved in double (natural_spline_deriv); the
 * evaluation below runs in REAL.
 */
#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUFFIX)

/* Index of the knot interval holding c (c inside [v0, v_{n-1}]); the last knot maps to
 * the last interval. */
static int FN(knot_interval)(const REAL *v, int n, REAL c) {
    int lo = 0, hi = n - 1;
    if (c >= v[n - 1]) return n - 2;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (v[mid] <= c) lo = mid; else hi = mid;
    }
    return lo;
}

static void FN(hermite_basis)(REAL t, REAL h0[2], REAL h1[2]) {
    const REAL t2 = t * t, t3 = t2 * t;
    h0[0] = (REAL)2.0 * t3 - (REAL)3.0 * t2 + (REAL)1.0;
    h0[1] = (REAL)-2.0 * t3 + (REAL)3.0 * t2;
    h1[0] = t3 - (REAL)2.0 * t2 + t;
    h1[1] = t3 - t2;
}

/* Bicubic Hermite surface: knots ys[ni] x xs[nj]; node values c4[k] = (f, fy, fx, fyx)
 * in REAL.  Canonical order: column basis X = (h00, h01, dx*h10, dx*h11)(tx), row basis Y
 * likewise in ty; the four column sums w first, then ((w0*Y0 + w1*Y1) + w2*Y2) + w3*Y3. */
static REAL FN(bicubic_value)(const REAL *ys, int ni, const REAL *xs, int nj, const REAL *c4, REAL y, REAL x) {
    const int i = FN(knot_interval)(ys, ni, y), j = FN(knot_interval)(xs, nj, x);
    const REAL dy = ys[i + 1] - ys[i], dx = xs[j + 1] - xs[j];
    const REAL ty = (y - ys[i]) / dy, tx = (x - xs[j]) / dx;
    REAL ay0[2], ay1[2], ax0[2], ax1[2];
    FN(hermite_basis)(ty, ay0, ay1);
    FN(hermite_basis)(tx, ax0, ax1);
    const REAL X0 = ax0[0], X1 = ax0[1], X2 = dx * ax1[0], X3 = dx * ax1[1];
    const REAL Y0 = ay0[0], Y1 = ay0[1], Y2 = dy * ay1[0], Y3 = dy * ay1[1];
    REAL w[4];
    for (int a = 0; a < 2; a++) {
        const REAL *n0 = c4 + 4 * ((size_t)(i + a) * nj + j), *n1 = n0 + 4;
        w[a] = n0[0] * X0 + n1[0] * X1 + n0[2] * X2 + n1[2] * X3;
        w[2 + a] = n0[1] * X0 + n1[1] * X1 + n0[3] * X2 + n1[3] * X3;
    }
    return w[0] * Y0 + w[1] * Y1 + w[2] * Y2 + w[3] * Y3;
}

/* derivative at x[at] of the parabola through 3 knots */
static REAL FN(parabola_deriv)(const REAL *x, const REAL *y, int at, int i0, int i1, int i2) {
    const REAL X = x[at];
    const REAL x0 = x[i0], x1 = x[i1], x2 = x[i2];
    return y[i0] * ((X - x1) + (X - x2)) / ((x0 - x1) * (x0 - x2)) +
           y[i1] * ((X - x0) + (X - x2)) / ((x1 - x0) * (x1 - x2)) +
           y[i2] * ((X - x0) + (X - x1)) / ((x2 - x0) * (x2 - x1));
}

/* Akima spline through 5 knots evaluated at t */
static REAL FN(akima5_value)(const REAL *x, const REAL *y, REAL t) {
    REAL d[4], w[4] = {0, 0, 0, 0}, fd[5];
    for (int k = 0; k < 4; k++) d[k] = (y[k + 1] - y[k]) / (x[k + 1] - x[k]);
    for (int k = 1; k < 4; k++) w[k] = (REAL)fabs((double)(d[k] - d[k - 1]));
    {
        const REAL wp = w[3], wm = w[1];
        if (wp == (REAL)0 && wm == (REAL)0)
            fd[2] = ((x[3] - x[2]) * d[1] + (x[2] - x[1]) * d[2]) / (x[3] - x[1]);
        else
            fd[2] = (wp * d[1] + wm * d[2]) / (wp + wm);
    }
    fd[0] = FN(parabola_deriv)(x, y, 0, 0, 1, 2);
    fd[1] = FN(parabola_deriv)(x, y, 1, 0, 1, 2);
    fd[3] = FN(parabola_deriv)(x, y, 3, 2, 3, 4);
    fd[4] = FN(parabola_deriv)(x, y, 4, 2, 3, 4);
    const int k = FN(knot_interval)(x, 5, t);
    const REAL h = x[k + 1] - x[k], s = t - x[k];
    const REAL c2 = ((REAL)3.0 * (y[k + 1] - y[k]) / h - (REAL)2.0 * fd[k] - fd[k + 1]) / h;
    const REAL c3 = ((REAL)2.0 * (y[k] - y[k + 1]) / h + fd[k] + fd[k + 1]) / (h * h);
    return y[k] + s * (fd[k] + s * (c2 + s * c3));
}

/* start of the 5-knot window for c (binary search, centred on the hit or the interval,
 * clamped to the knot range) */
static int FN(akima_window)(const REAL *v, int n, REAL c) {
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

/* Piecewise bicubic (Akima) value: for each of the 5 second-coordinate knots of the
 * window an Akima spline along the first coordinate, then one along the second. */
static REAL FN(akima2d_value)(const REAL *ys, int ni, const REAL *xs, int nj, const REAL *f, REAL y, REAL x) {
    const int i = FN(akima_window)(ys, ni, y), j = FN(akima_window)(xs, nj, x);
    REAL col[5], row[5];
    for (int b = 0; b < 5; b++) {
        for (int a = 0; a < 5; a++) col[a] = f[(size_t)(i + a) * nj + (j + b)];
        row[b] = FN(akima5_value)(ys + i, col, y);
    }
    return FN(akima5_value)(xs + j, row, x);
}

#undef FN
#undef CAT
#undef CAT_
