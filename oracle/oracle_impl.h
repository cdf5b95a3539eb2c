/*
 * qlpiv oracle -- REAL-typed body, included twice by qlpiv_oracle.c:
 *   REAL=float  (suffix _f32): bit-faithful restatement of the reference CPU path
 *                (Java float semantics: IEEE single, no FMA contraction,
 *                 FastMath.sin/log evaluated in double and rounded);
 *   REAL=double (suffix _f64): the same algorithm in double, used as the error
 *                reference for the CUDA path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links this code.
 *
 * Reference citations are paths inside the QuickLabPIV-ng project, with
 *   S/ = src/main/java/pt/quickLabPIV/
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SUFFIX)

/* Sine table of SimpleFFT.initEulerTable (S/jobs/xcorr/SimpleFFT.java:323-330):
 * w[n] = sin(2*pi*n/N), evaluated in double, rounded to REAL. */
static void FN(euler_table)(int n, REAL *w) {
    for (int k = 0; k < n; k++) {
        w[k] = (REAL)sin(2.0 * M_PI * (double)k / (double)n);
    }
}

/* One radix-2 pass sequence of SimpleFFT.computeFFTSerial / computeIFFTSerial
 * (S/jobs/xcorr/SimpleFFT.java:97-221 forward, 229-320 inverse).  The input must
 * already be in bit-reversed order (perfectShuffleFFTInput).  Butterfly operand
 * order is kept exactly: ((a + wr*b) - wi*c) etc. */
static void FN(fft1d_inplace)(REAL *xr, REAL *xi, int n, const REAL *w, int inverse) {
    if (inverse) {
        /* divideArray(xr, N); divideArray(xi, N) (SimpleFFT.java:230-231) */
        for (int k = 0; k < n; k++) { xr[k] /= (REAL)n; xi[k] /= (REAL)n; }
    }
    int step = n;
    for (int level = 1; level < n; level <<= 1) {
        const int level2 = level << 1;
        step >>= 1;
        for (int t = 0; t < n / 2; t++) {
            const int k = step * (t % level);
            const int i = (t / level) * level2 + (t % level);
            const int j = i + level;
            REAL wr, wi;
            if (!inverse) {
                wr = w[k + n / 4];
                wi = -w[k];
            } else {
                const int idx = n / 4 - k;
                wr = idx >= 0 ? w[idx] : w[n + idx];
                wi = w[k];
            }
            const REAL xri = xr[i], xii = xi[i], xrj = xr[j], xij = xi[j];
            const REAL lowR = xri + wr * xrj - wi * xij;
            const REAL lowI = xii + wr * xij + wi * xrj;
            const REAL upR = xri - wr * xrj + wi * xij;
            const REAL upI = xii - wr * xij - wi * xrj;
            xr[i] = lowR; xi[i] = lowI;
            xr[j] = upR;  xi[j] = upI;
        }
    }
}

/* SimpleFFT.computeFFT2DSerial (S/jobs/xcorr/SimpleFFT.java:379-432), Full range:
 * shuffle+FFT every row, transpose, shuffle+FFT every row of the transpose
 * (i.e. every column), transpose back.  Transposes are pure data movement, so the
 * column pass is done through a gather/scatter buffer. */
static void FN(fft2d)(REAL *re, REAL *im, int m, int inverse, const int *perm, const REAL *w,
                      REAL *bufr, REAL *bufi) {
    for (int r = 0; r < m; r++) {
        REAL *rr = re + (size_t)r * m, *ri = im + (size_t)r * m;
        for (int k = 0; k < m; k++) { bufr[k] = rr[perm[k]]; bufi[k] = ri[perm[k]]; }
        FN(fft1d_inplace)(bufr, bufi, m, w, inverse);
        for (int k = 0; k < m; k++) { rr[k] = bufr[k]; ri[k] = bufi[k]; }
    }
    for (int c = 0; c < m; c++) {
        for (int k = 0; k < m; k++) {
            bufr[k] = re[(size_t)perm[k] * m + c];
            bufi[k] = im[(size_t)perm[k] * m + c];
        }
        FN(fft1d_inplace)(bufr, bufi, m, w, inverse);
        for (int k = 0; k < m; k++) {
            re[(size_t)k * m + c] = bufr[k];
            im[(size_t)k * m + c] = bufi[k];
        }
    }
}

/* FastRealFFTXCorr.computeXCorr(Matrix, Matrix) (S/jobs/xcorr/FastRealFFTXCorr.java:44-68)
 * plus commonRealFFTXCorr (:70-116).
 *   re[i][j] = A[N-1-i][N-1-j] / maxA * 16 + 1,  im[i][j] = B[i][j] / maxB * 16 + 1
 * for i, j < N (zero elsewhere).  The CPU reference passes maxB == maxA; the
 * GPU reference (Matrix.copyMirroredMatrixToArrayNormalizeAndOffset / copyMatrixToArray
 * AndNormalizeAndOffset, S/Matrix.java:175-181,282-288) uses each tile's own max.
 * norm_offset == 0 disables the v/max*16+1 map (raw values).
 * Output: the (2N-1)x(2N-1) top-left crop of the real part, row-major. */
static void FN(xcorr_fft)(const float *ta, const float *tb, int n, float maxA, float maxB,
                          int normalize, REAL *plane) {
    const int m = 2 * n;
    REAL *tr = (REAL *)calloc((size_t)m * m, sizeof(REAL));
    REAL *ti = (REAL *)calloc((size_t)m * m, sizeof(REAL));
    REAL *w = (REAL *)malloc(sizeof(REAL) * m);
    REAL *bufr = (REAL *)malloc(sizeof(REAL) * m);
    REAL *bufi = (REAL *)malloc(sizeof(REAL) * m);
    int *perm = (int *)malloc(sizeof(int) * m);
    bitrev_perm(m, perm);
    FN(euler_table)(m, w);

    for (int i = 0; i < n; i++) {
        for (int j = 0; j < n; j++) {
            const REAL a = (REAL)ta[(size_t)(n - 1 - i) * n + (n - 1 - j)];
            const REAL b = (REAL)tb[(size_t)i * n + j];
            if (normalize) {
                tr[(size_t)i * m + j] = a / (REAL)maxA * (REAL)16.0 + (REAL)1.0;
                ti[(size_t)i * m + j] = b / (REAL)maxB * (REAL)16.0 + (REAL)1.0;
            } else {
                tr[(size_t)i * m + j] = a;
                ti[(size_t)i * m + j] = b;
            }
        }
    }

    FN(fft2d)(tr, ti, m, 0, perm, w, bufr, bufi);

    /* Hermitian split of the packed spectrum Z = FFT(a + i b) and product F*G,
     * written at k and as the conjugate at -k (FastRealFFTXCorr.java:73-112). */
#define TR(a, b) tr[(size_t)(a) * m + (b)]
#define TI(a, b) ti[(size_t)(a) * m + (b)]
    for (int i = 0; i <= m / 2; i++) {
        for (int j = 0; j <= m / 2; j++) {
            int k1 = i, nk1 = (m - k1) % m;
            const int k2 = j, nk2 = (m - k2) % m;
            {
                const REAL Gr = (REAL)0.5 * (TI(k1, k2) + TI(nk1, nk2));
                const REAL Gi = (REAL)-0.5 * (TR(k1, k2) - TR(nk1, nk2));
                const REAL Fr = (REAL)0.5 * (TR(k1, k2) + TR(nk1, nk2));
                const REAL Fi = (REAL)0.5 * (TI(k1, k2) - TI(nk1, nk2));
                TR(k1, k2) = Fr * Gr - Fi * Gi;
                TI(k1, k2) = Fr * Gi + Fi * Gr;
                TR(nk1, nk2) = TR(k1, k2);
                TI(nk1, nk2) = -TI(k1, k2);
            }
            if (k1 != 0 && k2 != 0 && k1 < m / 2 && k2 < m / 2) {
                k1 = i + m / 2;
                nk1 = (m - k1) % m;
                const REAL Gr = (REAL)0.5 * (TI(k1, k2) + TI(nk1, nk2));
                const REAL Gi = (REAL)-0.5 * (TR(k1, k2) - TR(nk1, nk2));
                const REAL Fr = (REAL)0.5 * (TR(k1, k2) + TR(nk1, nk2));
                const REAL Fi = (REAL)0.5 * (TI(k1, k2) - TI(nk1, nk2));
                TR(k1, k2) = Fr * Gr - Fi * Gi;
                TI(k1, k2) = Fr * Gi + Fi * Gr;
                TR(nk1, nk2) = TR(k1, k2);
                TI(nk1, nk2) = -TI(k1, k2);
            }
        }
    }
#undef TR
#undef TI

    FN(fft2d)(tr, ti, m, 1, perm, w, bufr, bufi);

    const int d = m - 1;
    for (int i = 0; i < d; i++)
        for (int j = 0; j < d; j++) plane[(size_t)i * d + j] = tr[(size_t)i * m + j];

    free(tr); free(ti); free(w); free(bufr); free(bufi); free(perm);
}

/* FindMaximumFromCenter.findMaximum (S/maximum/FindMaximumFromCenter.java:47-183)
 * with updateMaxResults (:33-44) and MaxCrossResult.computeDistance
 * (S/maximum/MaxCrossResult.java:48-51).  The running maximum starts at 0 at
 * cell (0,0) (MaxCrossResult.reset, :455-461).  Visit order: centre (D/2+1, D/2+1),
 * the centre column outwards, the centre row outwards, then the four quadrants;
 * row/column 0 are never visited.  min_floor is the minimum over visited cells. */
typedef struct {
    int i, j;
    REAL value;
} FN(peak_state);

static void FN(peak_visit)(FN(peak_state) *st, int i, int j, REAL v, int ci, int cj) {
    if (!(v >= st->value)) return;          /* scan loops only call update when v >= max */
    if (v > st->value) {
        st->i = i; st->j = j; st->value = v;
    } else { /* v == max */
        const float dmax = (float)sqrt((double)((float)((st->i - ci) * (st->i - ci) + (st->j - cj) * (st->j - cj))));
        const float dnew = (float)sqrt((double)((float)((i - ci) * (i - ci) + (j - cj) * (j - cj))));
        if (dnew < dmax) { st->i = i; st->j = j; st->value = v; }
    }
}

static void FN(find_max_from_center)(const REAL *p, int di, int dj, int *oi, int *oj, REAL *ov,
                                     REAL *ominf) {
    FN(peak_state) st = {0, 0, (REAL)0};
    const int ci = di / 2 + 1, cj = dj / 2 + 1;
#define P(a, b) p[(size_t)(a) * dj + (b)]
    /* centre cell goes through updateMaxResults unconditionally */
    {
        const REAL v = P(ci, cj);
        if (v > st.value) { st.i = ci; st.j = cj; st.value = v; }
        else if (v == st.value) {
            const float dmax = (float)sqrt((double)((st.i - ci) * (st.i - ci) + (st.j - cj) * (st.j - cj)));
            if (0.0f < dmax) { st.i = ci; st.j = cj; st.value = v; }
        }
    }
    REAL minv = (REAL)FLT_MAX;
    for (int k = 0; k < di / 2; k++) {
        const int r1 = di / 2 - k, r2 = di / 2 + 1 + k;
        const REAL v1 = P(r1, cj), v2 = P(r2, cj);
        if (v1 < minv) minv = v1;
        if (v2 < minv) minv = v2;
        FN(peak_visit)(&st, r1, cj, v1, ci, cj);
        FN(peak_visit)(&st, r2, cj, v2, ci, cj);
    }
    for (int k = 0; k < dj / 2; k++) {
        const int c1 = dj / 2 - k, c2 = dj / 2 + 1 + k;
        const REAL v1 = P(ci, c1), v2 = P(ci, c2);
        if (v1 < minv) minv = v1;
        if (v2 < minv) minv = v2;
        FN(peak_visit)(&st, ci, c1, v1, ci, cj);
        FN(peak_visit)(&st, ci, c2, v2, ci, cj);
    }
    for (int a = 0; a < di / 2; a++) {
        for (int b = 0; b < dj / 2; b++) {
            const int rt = di / 2 - a, rb = di / 2 + 1 + a;
            const int cl = dj / 2 - b, cr = dj / 2 + 1 + b;
            const REAL v1 = P(rt, cl), v2 = P(rb, cl), v3 = P(rt, cr), v4 = P(rb, cr);
            if (v1 < minv) minv = v1;
            if (v2 < minv) minv = v2;
            if (v3 < minv) minv = v3;
            if (v4 < minv) minv = v4;
            FN(peak_visit)(&st, rt, cl, v1, ci, cj);
            FN(peak_visit)(&st, rb, cl, v2, ci, cj);
            FN(peak_visit)(&st, rt, cr, v3, ci, cj);
            FN(peak_visit)(&st, rb, cr, v4, ci, cj);
        }
    }
#undef P
    *oi = st.i; *oj = st.j; *ov = st.value; *ominf = minv;
}

/* Gaussian1DPolynomialInterpolator.interpolate (S/interpolators/Gaussian1DPolynomialInterpolator.java:25-106)
 * for the main peak, then MaxCrossResult.setNthRelativeDisplacementFromPeak
 * (S/maximum/MaxCrossResult.java:304-326): u = peakI - D/2, v = peakJ - D/2.
 * 3-point Gaussian with +1e-8, parabolic fallback when a stencil value is
 * negative; a fit is kept only when finite and within 1 px of the integer peak. */
static void FN(subpixel_gauss3)(const REAL *p, int di, int dj, int mi, int mj, REAL *pi, REAL *pj,
                                uint32_t *flags) {
    REAL peakI = (REAL)mi, peakJ = (REAL)mj;
    uint32_t f = 0;
    if (mi == 0 && mj == 0) {
        f |= ORC_F_NO_PEAK;
    } else if (mi - 1 < 0 || mi + 1 >= di || mj - 1 < 0 || mj + 1 >= dj) {
        f |= ORC_F_EDGE;
    } else {
#define P(a, b) p[(size_t)(a) * dj + (b)]
        int neg = 0;
        REAL y[3], x[3];
        for (int k = -1; k <= 1; k++) {
            if (P(mi + k, mj) < (REAL)0) neg = 1;
            if (P(mi, mj + k) < (REAL)0) neg = 1;
            y[k + 1] = P(mi + k, mj) + (REAL)1e-8f;
            x[k + 1] = P(mi, mj + k) + (REAL)1e-8f;
        }
#undef P
        REAL ti, tj;
        if (!neg) {
            ti = (REAL)mi + (REAL)(log((double)y[0]) - log((double)y[2])) /
                                (REAL)(2.0 * log((double)y[0]) - 4.0 * log((double)y[1]) + 2.0 * log((double)y[2]));
            tj = (REAL)mj + (REAL)(log((double)x[0]) - log((double)x[2])) /
                                (REAL)(2.0 * log((double)x[0]) - 4.0 * log((double)x[1]) + 2.0 * log((double)x[2]));
        } else {
            f |= ORC_F_PARABOLIC;
            ti = (REAL)mi + (REAL)(y[0] - y[2]) / (REAL)((REAL)2.0 * y[0] - (REAL)4.0 * y[1] + (REAL)2.0 * y[2]);
            tj = (REAL)mj + (REAL)(x[0] - x[2]) / (REAL)((REAL)2.0 * x[0] - (REAL)4.0 * x[1] + (REAL)2.0 * x[2]);
        }
        if (isfinite((double)ti) && fabs((double)(ti - (REAL)mi)) <= 1.0) { peakI = ti; f |= ORC_F_SUB_I; }
        if (isfinite((double)tj) && fabs((double)(tj - (REAL)mj)) <= 1.0) { peakJ = tj; f |= ORC_F_SUB_J; }
    }
    *pi = peakI; *pj = peakJ; *flags = f;
}

/* The pass's sub-pixel mode (packed: mode | pixels << 8 | iterations << 16) on peak (mi, mj);
 * the P-point interpolators fit the plane values as floats, like the reference's MatrixFloat. */
static void FN(subpixel_any)(const REAL *p, int d, int mi, int mj, int subpix, REAL minf, REAL *pi, REAL *pj,
                             REAL *pv, uint32_t *flags) {
    const int mode = subpix & 0xff, P = (subpix >> 8) & 0xff, iters = (subpix >> 16) & 0xff;
    *pi = (REAL)mi;
    *pj = (REAL)mj;
    *flags = 0;
    if (mode == 1) {
        FN(subpixel_gauss3)(p, d, d, mi, mj, pi, pj, flags);
    } else if (mode == 2 || mode == 3) {
        float *pf = (float *)malloc(sizeof(float) * (size_t)d * d);
        for (size_t k = 0; k < (size_t)d * d; k++) pf[k] = (float)p[k];
        float si, sj, v = (float)*pv;
        if (mode == 2) orc_subpixel_lm(pf, d, mi, mj, P, (float)minf, &si, &sj, flags);
        else orc_subpixel_hg(pf, d, mi, mj, P, iters, (float)minf, &si, &sj, &v, flags);
        *pi = (REAL)si;
        *pj = (REAL)sj;
        *pv = (REAL)v;
        free(pf);
    }
}

/* One IA through the whole CPU path: xcorr plane -> FindMaximumFromCenter ->
 * Gaussian 1D-1D sub-pixel -> displacement (u rows, v columns). */
static void FN(ia_vector)(const float *ta, const float *tb, int n, float maxA, float maxB, int normalize,
                          int subpix, orc_vector *out, REAL *plane_scratch) {
    const int d = 2 * n - 1;
    FN(xcorr_fft)(ta, tb, n, maxA, maxB, normalize, plane_scratch);
    int mi, mj;
    REAL mv, minf;
    FN(find_max_from_center)(plane_scratch, d, d, &mi, &mj, &mv, &minf);
    REAL pi = (REAL)mi, pj = (REAL)mj;
    uint32_t flags = 0;
    FN(subpixel_any)(plane_scratch, d, mi, mj, subpix, minf, &pi, &pj, &mv, &flags);
    const REAL half = (REAL)(d / 2);
    out->u = (float)(pi - half);
    out->v = (float)(pj - half);
    out->sub_i = (float)pi;
    out->sub_j = (float)pj;
    out->peak_value = (float)mv;
    out->min_floor = (float)minf;
    out->peak_i = (int16_t)mi;
    out->peak_j = (int16_t)mj;
    out->flags = flags;
    /* double-precision twin keeps its own copies of the exact values */
    out->u64 = (double)(pi - half);
    out->v64 = (double)(pj - half);
}


/* FindMaximumMultiPeaks.findMaximum (S/maximum/FindMaximumMultiPeaks.java:42-162) with the
 * sorted, adjacency-suppressing list of SimpleFixedLengthFloatLinkedList.addInAscendOrder
 * (S/util/SimpleFixedLengthFloatLinkedList.java).  The plane is cut into kw x kw cells in four
 * interleaved quadrant groups; each cell's maximum (strict >, starting from 0, position kept
 * from the previous slice when nothing beats 0) is inserted in slice order.  The list holds
 * at most k entries in ascending order; an insertion deletes smaller entries within squared
 * distance (kw-1)*kw and is refused next to an equal or larger one.  Output peaks are sorted
 * largest first.  Returns the number of peaks; *ominf = minimum over every visited cell. */
typedef struct { REAL v; int i, j; } FN(mp_entry);

static int FN(mp_adjacent)(const FN(mp_entry) *e, int i, int j, float kd) {
    const float d = (float)((double)(i - e->i) * (double)(i - e->i) + (double)(j - e->j) * (double)(j - e->j));
    return d < kd;
}

static void FN(mp_add)(FN(mp_entry) *lst, int *size, int maxsize, float kd, REAL v, int i, int j) {
    if (*size == 0) {
        lst[0].v = v; lst[0].i = i; lst[0].j = j;
        *size = 1;
        return;
    }
    int del[64], ndel = 0;
    int pos = 0;
    while (pos < *size && lst[pos].v < v) {
        if (FN(mp_adjacent)(&lst[pos], i, j, kd) && v > lst[pos].v) del[ndel++] = pos;
        pos++;
    }
    if (*size == maxsize && pos == 0) return;
    for (int q = pos; q < *size; q++)
        if (FN(mp_adjacent)(&lst[q], i, j, kd) && v <= lst[q].v) return;
    /* perform the scheduled deletions (all before pos) */
    if (ndel > 0) {
        int w = 0, d = 0;
        for (int r = 0; r < *size; r++) {
            if (d < ndel && del[d] == r) { d++; continue; }
            lst[w++] = lst[r];
        }
        *size -= ndel;
        pos -= ndel;
    }
    if (pos > 0) {  /* insert after the last smaller survivor */
        for (int r = *size; r > pos; r--) lst[r] = lst[r - 1];
        lst[pos].v = v; lst[pos].i = i; lst[pos].j = j;
        (*size)++;
        if (*size > maxsize) {  /* drop the smallest */
            for (int r = 0; r < *size - 1; r++) lst[r] = lst[r + 1];
            (*size)--;
        }
    } else {
        if (*size == maxsize) return;
        for (int r = *size; r > 0; r--) lst[r] = lst[r - 1];
        lst[0].v = v; lst[0].i = i; lst[0].j = j;
        (*size)++;
    }
}

static int FN(find_max_multipeaks)(const REAL *p, int di, int dj, int kw, int k, int *oi, int *oj, REAL *ov,
                                   REAL *ominf) {
    int iS = di / kw; if (iS * kw != di) iS += 1;
    const int iBottom = iS / 2, iTop = iS - iBottom;
    int jS = dj / kw; if (jS * kw != dj) jS += 1;
    const int jRight = jS / 2, jLeft = jS - jRight;
    const float kd = (float)((kw - 1) * kw);
    FN(mp_entry) lst[65];
    int size = 0;
    REAL maxs[4];
    int mi[4] = {0, 0, 0, 0}, mj[4] = {0, 0, 0, 0};
    REAL minv = (REAL)FLT_MAX;
#define P(a, b) p[(size_t)(a) * dj + (b)]
    for (int sI = 0; sI < iTop; sI++) {
        for (int sJ = 0; sJ < jLeft; sJ++) {
            const int top = sI * kw, left = sJ * kw, bottom = sI * kw + iTop * kw, right = sJ * kw + jLeft * kw;
            for (int q = 0; q < 4; q++) maxs[q] = (REAL)0;
            for (int a = 0; a < kw; a++) {
                for (int b = 0; b < kw; b++) {
                    const int i1 = top + a, j1 = left + b;
                    { const REAL v = P(i1, j1);
                      if (v > maxs[0]) { maxs[0] = v; mi[0] = i1; mj[0] = j1; }
                      if (v < minv) minv = v; }
                    const int j2 = right + b;
                    if (j2 < dj) { const REAL v = P(i1, j2);
                      if (v > maxs[1]) { maxs[1] = v; mi[1] = i1; mj[1] = j2; }
                      if (v < minv) minv = v; }
                    const int i3 = bottom + a;
                    if (i3 < di) { const REAL v = P(i3, j1);
                      if (v > maxs[2]) { maxs[2] = v; mi[2] = i3; mj[2] = j1; }
                      if (v < minv) minv = v; }
                    if (i3 < di && j2 < dj) { const REAL v = P(i3, j2);
                      if (v > maxs[3]) { maxs[3] = v; mi[3] = i3; mj[3] = j2; }
                      if (v < minv) minv = v; }
                }
            }
            for (int q = 0; q < 4; q++) FN(mp_add)(lst, &size, k, kd, maxs[q], mi[q], mj[q]);
        }
    }
#undef P
    for (int r = 0; r < size; r++) {  /* largest first */
        oi[r] = lst[size - 1 - r].i;
        oj[r] = lst[size - 1 - r].j;
        ov[r] = lst[size - 1 - r].v;
    }
    *ominf = minv;
    return size;
}

/* One IA through the CPU path with FindMaximumMultiPeaks: up to k vectors, peak 0 the
 * largest, each with the Gaussian 1D-1D sub-pixel fit (the interpolator visits every
 * peak, Gaussian1DPolynomialInterpolator.java:25-106). */
static int FN(ia_vectors_multi)(const float *ta, const float *tb, int n, float maxA, float maxB, int normalize,
                                int subpix, int kw, int k, orc_vector *out, REAL *plane_scratch) {
    const int d = 2 * n - 1;
    FN(xcorr_fft)(ta, tb, n, maxA, maxB, normalize, plane_scratch);
    int pi[64], pj[64];
    REAL pv[64], minf;
    const int np = FN(find_max_multipeaks)(plane_scratch, d, d, kw, k, pi, pj, pv, &minf);
    for (int r = 0; r < np; r++) {
        REAL si = (REAL)pi[r], sj = (REAL)pj[r];
        uint32_t flags = 0;
        FN(subpixel_any)(plane_scratch, d, pi[r], pj[r], subpix, minf, &si, &sj, &pv[r], &flags);
        const REAL half = (REAL)(d / 2);
        orc_vector *o = &out[r];
        o->u = (float)(si - half);
        o->v = (float)(sj - half);
        o->sub_i = (float)si;
        o->sub_j = (float)sj;
        o->peak_value = (float)pv[r];
        o->min_floor = (float)minf;
        o->peak_i = (int16_t)pi[r];
        o->peak_j = (int16_t)pj[r];
        o->flags = flags;
        o->u64 = (double)(si - half);
        o->v64 = (double)(sj - half);
    }
    return np;
}

#undef FN
#undef CAT
#undef CAT_
