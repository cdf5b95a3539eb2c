/*
 * qlpiv oracle, dense optical flow stages -- REAL-typed body, included twice by
 * qlpiv_oracle_dense.c.  TEST INFRASTRUCTURE ONLY.
 *
 *   REAL=float  (names orc_<stage>): Java float semantics, the reference's operation order
 *               (no contraction: the kernels' mad(a, b, c) is a * b + c as Java runs it);
 *   REAL=double (names orc_<stage>_f64): the same algorithm in double with the filter weights
 *               unrounded; the error reference ("FP64 twin") of the CUDA dense stages.
 *
 * Stages (S/ = src/main/java/pt/quickLabPIV/):
 *  C-filter  GaussianFilter2DInternal.applyFilter (S/images/filters/GaussianFilter2DInternal.java:49-97),
 *            DirectConvolution.convolve1D (S/images/filters/DirectConvolution.java:14-53):
 *            rows then columns, padding = the first halfSize values mirrored on the left (edge
 *            repeated) and the last halfSize values copied in order on the right; accumulation
 *            from the +h neighbour down to the -h neighbour.
 *            ImageFloat.normalize (S/images/ImageFloat.java:571-596): divide by the max.
 *  C-LK      DenseLucasKanadeGpuKernel (S/jobs/interpolators/DenseLucasKanadeGpuKernel.java:203-751):
 *            per pixel, image A (optionally 2x2-averaged: half-pixel offset) over a W x W
 *            window, derivatives (3, 10, 3)/32, A matrix, inverse with det < FLT_EPSILON
 *            rejected, iterations of the b vector from bilinear samples of image B, stop on
 *            |increment| < 1e-3 (update skipped) or out of bounds.  Pixels are independent:
 *            rows are split over host threads, which changes no result.
 *  C-LS      DenseLiuShenGpuKernel (S/jobs/interpolators/DenseLiuShenGpuKernel.java:66-588):
 *            fixed-image terms from the 3x3 neighbourhoods of the Liu-Shen images, Jacobi
 *            passes of the 2x2 update, total-error stop at 1e-8.
 * Sums run in window row-major order.  Expects DFN(name), RFABS, RSQRT defined by the includer.
 */

#define RC(x) ((REAL)(x))

/* one padded line through DirectConvolution (line of n values, stride `st`) */
static void DFN(filter_line)(const REAL *in, long st, int n, const REAL *k, int K, REAL *buf, REAL *out, long ost) {
    const int h = K / 2;
    for (int j = 0; j < n; j++) buf[j + h] = in[(long)j * st];
    for (int j = 0; j < h; j++) {
        buf[h - 1 - j] = in[(long)j * st];
        buf[n + 2 * h - 1 - j] = in[(long)(n - 1 - j) * st];
    }
    for (int j = 0; j < n; j++) {
        REAL acc = RC(0.0);
        for (int q = 0; q < K; q++) acc = acc + buf[j + 2 * h - q] * k[q];
        out[(long)j * ost] = acc;
    }
}

/* GaussianFilter2DInternal.applyFilter: rows, then columns of the row result. */
void DFN(gauss_filter)(const REAL *in, int h, int w, const REAL *k, int K, REAL *out) {
    const int n = h > w ? h : w;
    REAL *buf = (REAL *)malloc(sizeof(REAL) * (n + K));
    REAL *tmp = (REAL *)malloc(sizeof(REAL) * n);
    for (int i = 0; i < h; i++) DFN(filter_line)(in + (long)i * w, 1, w, k, K, buf, out + (long)i * w, 1);
    for (int j = 0; j < w; j++) {
        DFN(filter_line)(out + j, w, h, k, K, buf, tmp, 1);
        for (int i = 0; i < h; i++) out[(long)i * w + j] = tmp[i];
    }
    free(buf);
    free(tmp);
}

/* ImageFloat.normalize: value / max (max starts at 0). */
void DFN(normalize)(const REAL *in, long n, REAL *out) {
    REAL mx = RC(0.0);
    for (long q = 0; q < n; q++)
        if (in[q] > mx) mx = in[q];
    for (long q = 0; q < n; q++) out[q] = in[q] / mx;
}

static REAL DFN(clamp_read)(const REAL *img, int h, int w, int i, int j) {
    i = i < 0 ? 0 : (i > h - 1 ? h - 1 : i);
    j = j < 0 ? 0 : (j > w - 1 ? w - 1 : j);
    return img[(long)i * w + j];
}

/* readPixelWithWarp: floor anchor, bilinear, clamped reads. */
static REAL DFN(warp_read)(const REAL *img, int h, int w, REAL li, REAL lj) {
    int i = (int)li, j = (int)lj;
    REAL di = li - (REAL)i, dj = lj - (REAL)j;
    const int si = di < RC(0.0) ? 1 : 0;
    i -= si;
    di += (REAL)si;
    const int sj = dj < RC(0.0) ? 1 : 0;
    j -= sj;
    dj += (REAL)sj;
    const REAL top = (RC(1.0) - dj) * DFN(clamp_read)(img, h, w, i, j) + dj * DFN(clamp_read)(img, h, w, i, j + 1);
    const REAL bot =
        (RC(1.0) - dj) * DFN(clamp_read)(img, h, w, i + 1, j) + dj * DFN(clamp_read)(img, h, w, i + 1, j + 1);
    return (RC(1.0) - di) * top + di * bot;
}

typedef struct {
    const REAL *A, *B;
    int h, w;
    REAL *us, *vs;
    int win, iterations, half_pixel;
    int row0, row1;
} DFN(lk_rows_job);

/* Dense Lucas-Kanade of rows [row0, row1), in place on us (columns) / vs (rows). */
static void *DFN(lk_rows)(void *arg) {
    const DFN(lk_rows_job) *jb = (const DFN(lk_rows_job) *)arg;
    const REAL *A = jb->A, *B = jb->B;
    const int h = jb->h, w = jb->w, W = jb->win, hw = jb->win / 2, iterations = jb->iterations;
    const int half_pixel = jb->half_pixel;
    REAL *us = jb->us, *vs = jb->vs;
    const int R = W + 2;  /* window plus the derivative margin */
    REAL *reg = (REAL *)malloc(sizeof(REAL) * R * R);
    REAL *val = (REAL *)malloc(sizeof(REAL) * W * W);
    REAL *dJ = (REAL *)malloc(sizeof(REAL) * W * W);
    REAL *dI = (REAL *)malloc(sizeof(REAL) * W * W);
    const REAL c3 = RC(3.0) / RC(32.0);
    for (int pi = jb->row0; pi < jb->row1; pi++) {
        for (int pj = 0; pj < w; pj++) {
            /* image A around the pixel: rows pi - hw - 1 ... , clamped */
            for (int a = 0; a < R; a++)
                for (int b = 0; b < R; b++) {
                    const int y = pi + a - hw - 1, x = pj + b - hw - 1;
                    if (half_pixel)
                        reg[a * R + b] = (DFN(clamp_read)(A, h, w, y, x) + DFN(clamp_read)(A, h, w, y, x + 1) +
                                          DFN(clamp_read)(A, h, w, y + 1, x) +
                                          DFN(clamp_read)(A, h, w, y + 1, x + 1)) /
                                         RC(4.0);
                    else
                        reg[a * R + b] = DFN(clamp_read)(A, h, w, y, x);
                }
            REAL a00 = RC(0.0), a01 = RC(0.0), a11 = RC(0.0);
            for (int a = 0; a < W; a++)
                for (int b = 0; b < W; b++) {
                    const REAL *r0 = reg + a * R + b, *r1 = r0 + R, *r2 = r1 + R;
                    const REAL TL = r0[0], T = r0[1], TR = r0[2], L = r1[0], C = r1[1], Rt = r1[2];
                    const REAL BL = r2[0], Bt = r2[1], BR = r2[2];
                    const REAL dj = (((TL + BL) - TR) - BR) * c3 + (L - Rt) * RC(10.0) / RC(32.0);
                    const REAL di = (((TR + TL) - BR) - BL) * c3 + (T - Bt) * RC(10.0) / RC(32.0);
                    val[a * W + b] = C;
                    dJ[a * W + b] = dj;
                    dI[a * W + b] = di;
                    a00 = dj * dj + a00;
                    a01 = dj * di + a01;
                    a11 = di * di + a11;
                }
            const long p = (long)pi * w + pj;
            int status = 1;
            const REAL det = a00 * a11 + -(a01 * a01);
            if (det < RC(1.192092896e-7)) status = 0;
            const REAL i00 = a11 / det, i01 = -a01 / det, i11 = a00 / det;
            REAL locI = (REAL)pi + vs[p], locJ = (REAL)pj + us[p];
            if (half_pixel) {
                locI += RC(0.5);
                locJ += RC(0.5);
            }
            for (int it = 0; it < iterations && status; it++) {
                if (locI < RC(0.0) || locI >= (REAL)(h + hw)) { status = 0; break; }
                if (locJ < RC(0.0) || locJ >= (REAL)(w + hw)) { status = 0; break; }
                REAL b0 = RC(0.0), b1 = RC(0.0);
                for (int a = 0; a < W; a++)
                    for (int b = 0; b < W; b++) {
                        const REAL dT = DFN(warp_read)(B, h, w, locI - (REAL)hw + (REAL)a, locJ - (REAL)hw + (REAL)b) -
                                        val[a * W + b];
                        b0 = dT * dJ[a * W + b] + b0;
                        b1 = dT * dI[a * W + b] + b1;
                    }
                const REAL incU = b0 * i00 + b1 * i01;
                const REAL incV = b0 * i01 + b1 * i11;
                if (RFABS(incU) < RC(1e-3) && RFABS(incV) < RC(1e-3)) { status = 0; break; }
                locI += incV;
                locJ += incU;
            }
            /* the integer pixel comes off first, then the half pixel */
            vs[p] = half_pixel ? (locI - (REAL)pi) - RC(0.5) : locI - (REAL)pi;
            us[p] = half_pixel ? (locJ - (REAL)pj) - RC(0.5) : locJ - (REAL)pj;
        }
    }
    free(reg);
    free(val);
    free(dJ);
    free(dI);
    return NULL;
}

/* Dense Lucas-Kanade of every pixel, in place on us (columns) / vs (rows). */
void DFN(dense_lk)(const REAL *A, const REAL *B, int h, int w, REAL *us, REAL *vs, int win, int iterations,
                   int half_pixel) {
    enum { MAXT = 64 };
    long nt = sysconf(_SC_NPROCESSORS_ONLN);
    if (nt < 1) nt = 1;
    if (nt > MAXT) nt = MAXT;
    if (nt > h) nt = h;
    DFN(lk_rows_job) jobs[MAXT];
    pthread_t th[MAXT];
    for (int t = 0; t < nt; t++) {
        jobs[t] = (DFN(lk_rows_job)){A, B, h, w, us, vs, win, iterations, half_pixel, (int)((long)h * t / nt),
                                     (int)((long)h * (t + 1) / nt)};
        if (t > 0 && pthread_create(&th[t], NULL, DFN(lk_rows), &jobs[t]) != 0) DFN(lk_rows)(&jobs[t]), th[t] = 0;
    }
    DFN(lk_rows)(&jobs[0]);
    for (int t = 1; t < nt; t++)
        if (th[t]) pthread_join(th[t], NULL);
}

/* Liu-Shen 3x3 neighbourhood (row-major TL..BR) of img around (pi, pj), clamped; with the
 * half-pixel offset every value is the 2x2 average accumulated as v = P * 0.25 + v. */
static void DFN(ls_load)(const REAL *img, int h, int w, int pi, int pj, int half_pixel, REAL *n9) {
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            const int y = pi - 1 + a, x = pj - 1 + b;
            if (half_pixel) {
                REAL v = RC(0.0);
                for (int i = 0; i < 2; i++)
                    for (int j = 0; j < 2; j++) v = DFN(clamp_read)(img, h, w, y + i, x + j) * RC(0.25) + v;
                n9[a * 3 + b] = v;
            } else {
                n9[a * 3 + b] = DFN(clamp_read)(img, h, w, y, x);
            }
        }
}

/* Fixed-image terms of one pixel: out[0..11] = w, IIx, IIy, II, Ixt, Iyt, A11, A12, A22,
 * B11, B12, B22 (B = inverse of A). */
static void DFN(ls_fixed)(const REAL *la, const REAL *lb, int h, int w, int pi, int pj, REAL lambda, int half_pixel,
                          REAL *o, REAL *wts) {
    enum { TLi = 0, Ti = 1, TRi = 2, Li = 3, Ci = 4, Ri = 5, BLi = 6, Bi = 7, BRi = 8 };
    REAL a9[9], b9[9];
    DFN(ls_load)(la, h, w, pi, pj, half_pixel, a9);
    DFN(ls_load)(lb, h, w, pi, pj, half_pixel, b9);
    const REAL one = RC(1.0), zero = RC(0.0);
    const REAL wTL = (pi - 1) >= 0 && (pj - 1) >= 0 && (pi - 1) < h && (pj - 1) < w ? one : zero;
    const REAL wT = (pi - 1) >= 0 && (pi - 1) < h && pj < w ? one : zero;
    const REAL wTR = (pi - 1) >= 0 && (pj + 1) >= 0 && (pi - 1) < h && (pj + 1) < w ? one : zero;
    const REAL wL = (pj - 1) >= 0 && pi < h && (pj - 1) < w ? one : zero;
    const REAL wR = pi < h && (pj + 1) < w ? one : zero;
    const REAL wBL = (pj - 1) >= 0 && (pi + 1) < h && (pj - 1) < w ? one : zero;
    const REAL wB = (pi + 1) < h && pj < w ? one : zero;
    const REAL wBR = (pi + 1) < h && (pj + 1) < w ? one : zero;
    const REAL wsum = ((((((wTL + wT) + wTR) + wL) + wR) + wBL) + wB) + wBR;
    const REAL c = a9[Ci];
    const REAL IIx = c * (a9[Bi] - a9[Ti]) / RC(2.0);
    const REAL IIy = c * (a9[Ri] - a9[Li]) / RC(2.0);
    const REAL II = c * c;
    const REAL Ixt = c * ((b9[Bi] - a9[Bi]) - (b9[Ti] - a9[Ti])) / RC(2.0);
    const REAL Iyt = c * ((b9[Ri] - a9[Ri]) - (b9[Li] - a9[Li])) / RC(2.0);
    const REAL A11 = c * (((a9[Bi] + a9[Ti]) - RC(2.0) * c) - RC(2.0) * c) + -(lambda * wsum);
    const REAL A22 = c * (((a9[Ri] + a9[Li]) - RC(2.0) * c) - RC(2.0) * c) + -(lambda * wsum);
    const REAL A12 = c * (((a9[TLi] - a9[TRi]) - a9[BLi]) + a9[BRi]) / RC(4.0);
    const REAL det = A11 * A22 + -(A12 * A12);
    o[0] = wsum; o[1] = IIx; o[2] = IIy; o[3] = II; o[4] = Ixt; o[5] = Iyt;
    o[6] = A11; o[7] = A12; o[8] = A22;
    o[9] = A22 / det; o[10] = -A12 / det; o[11] = A11 / det;
    if (wts) {
        wts[0] = wTL; wts[1] = wT; wts[2] = wTR; wts[3] = wL; wts[4] = zero; wts[5] = wR;
        wts[6] = wBL; wts[7] = wB; wts[8] = wBR;
    }
}

/* Liu-Shen refinement passes (after the Lucas-Kanade pass) on us (columns) / vs (rows),
 * Jacobi: every pass reads the previous field.  fixed_out (optional, 12 x h x w) receives
 * the fixed terms; unews/vnews (optional, iterations x h x w) every pass's new rows /
 * columns displacement.  Returns the passes run. */
int DFN(liu_shen)(const REAL *la, const REAL *lb, int h, int w, REAL *us, REAL *vs, REAL lambda, int iterations,
                  int half_pixel, REAL *fixed_out, REAL *unews, REAL *vnews) {
    enum { TLi = 0, Ti = 1, TRi = 2, Li = 3, Ci = 4, Ri = 5, BLi = 6, Bi = 7, BRi = 8 };
    const long n = (long)h * w;
    REAL *fx = (REAL *)malloc(sizeof(REAL) * 12 * n);
    REAL *wt = (REAL *)malloc(sizeof(REAL) * 9 * n);
    REAL *un = (REAL *)malloc(sizeof(REAL) * n), *vn = (REAL *)malloc(sizeof(REAL) * n);
    for (int pi = 0; pi < h; pi++)
        for (int pj = 0; pj < w; pj++) {
            const long p = (long)pi * w + pj;
            REAL o[12];
            DFN(ls_fixed)(la, lb, h, w, pi, pj, lambda, half_pixel, o, wt + 9 * p);
            for (int q = 0; q < 12; q++) fx[q * n + p] = o[q];
        }
    if (fixed_out) memcpy(fixed_out, fx, sizeof(REAL) * 12 * n);
    double total = FLT_MAX;
    int passes = 0;
    for (int it = 0; it < iterations; it++) {
        if (total < 1e-8) break;
        double err = 0.0;
        for (int pi = 0; pi < h; pi++)
            for (int pj = 0; pj < w; pj++) {
                const long p = (long)pi * w + pj;
                REAL U[9], V[9];
                DFN(ls_load)(us, h, w, pi, pj, 0, U);
                DFN(ls_load)(vs, h, w, pi, pj, 0, V);
                const REAL *wq = wt + 9 * p;
                const REAL IIx = fx[1 * n + p], IIy = fx[2 * n + p], II = fx[3 * n + p];
                const REAL Ixt = fx[4 * n + p], Iyt = fx[5 * n + p];
                const REAL B11 = fx[9 * n + p], B12 = fx[10 * n + p], B22 = fx[11 * n + p];
                const REAL sV = ((((((V[TLi] * wq[0] + V[Ti] * wq[1]) + V[TRi] * wq[2]) + V[Li] * wq[3]) +
                                   V[Ri] * wq[5]) + V[BLi] * wq[6]) + V[Bi] * wq[7]) + V[BRi] * wq[8];
                const REAL sU = ((((((U[TLi] * wq[0] + U[Ti] * wq[1]) + U[TRi] * wq[2]) + U[Li] * wq[3]) +
                                   U[Ri] * wq[5]) + U[BLi] * wq[6]) + U[Bi] * wq[7]) + U[BRi] * wq[8];
                const REAL hu = lambda * sV + Ixt;
                const REAL hv = lambda * sU + Iyt;
                const REAL bu = (RC(2.0) * IIx) * ((V[Bi] - V[Ti]) / RC(2.0)) +
                                (IIx * ((U[Ri] - U[Li]) / RC(2.0)) +
                                 (IIy * ((U[Bi] - U[Ti]) / RC(2.0)) +
                                  (II * (V[Ti] + V[Bi]) +
                                   (II * ((((U[TLi] - U[TRi]) - U[BLi]) + U[BRi]) / RC(4.0)) + hu))));
                const REAL bv = (RC(2.0) * IIy) * ((U[Ri] - U[Li]) / RC(2.0)) +
                                (IIx * ((V[Ri] - V[Li]) / RC(2.0)) +
                                 (IIy * ((V[Bi] - V[Ti]) / RC(2.0)) +
                                  (II * (U[Li] + U[Ri]) +
                                   (II * ((((V[TLi] - V[TRi]) - V[BLi]) + V[BRi]) / RC(4.0)) + hv))));
                const REAL unew = -(B11 * bu + B12 * bv);
                const REAL vnew = -(B12 * bu + B22 * bv);
                const REAL du = unew - V[Ci], dv = vnew - U[Ci];
                err += (double)RSQRT(du * du + dv * dv);
                un[p] = unew;
                vn[p] = vnew;
            }
        /* copyVectors: columns <- vnew, rows <- unew */
        memcpy(us, vn, sizeof(REAL) * n);
        memcpy(vs, un, sizeof(REAL) * n);
        if (unews) memcpy(unews + (long)it * n, un, sizeof(REAL) * n);
        if (vnews) memcpy(vnews + (long)it * n, vn, sizeof(REAL) * n);
        total = err / (double)n;
        passes++;
    }
    free(fx);
    free(wt);
    free(un);
    free(vn);
    return passes;
}

/* Lucas-Kanade pyramid (coarse to fine): this library's own design, not the reference's (its
 * DenseLucasKanade runs at full resolution only).  A level halves both sides (floor) by 2 x 2 box
 * averaging, ((a + b) + (c + d)) * 0.25 * scale, scale 0.5 for the displacement field; a coarser
 * level's result starts the next finer level through nearest up-sampling, doubled, with the
 * source index clamped to the coarser level. */
static void DFN(pyr_down)(const REAL *s, int h, int w, REAL *d, REAL scale) {
    const int h2 = h / 2, w2 = w / 2;
    for (int i = 0; i < h2; i++)
        for (int j = 0; j < w2; j++) {
            const REAL *r0 = s + (long)(2 * i) * w + 2 * j, *r1 = r0 + w;
            const REAL t = (r0[0] + r0[1]) + (r1[0] + r1[1]);
            d[(long)i * w2 + j] = (t * RC(0.25)) * scale;
        }
}

static void DFN(pyr_up)(const REAL *s, int hs, int ws, REAL *d, int h, int w) {
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            const int si = (i >> 1) < hs - 1 ? (i >> 1) : hs - 1, sj = (j >> 1) < ws - 1 ? (j >> 1) : ws - 1;
            d[(long)i * w + j] = RC(2.0) * s[(long)si * ws + sj];
        }
}

void DFN(dense_lk_pyramid)(const REAL *A, const REAL *B, int h, int w, REAL *us, REAL *vs, int win, int iterations,
                           int half_pixel, int levels) {
    if (levels <= 1) {
        DFN(dense_lk)(A, B, h, w, us, vs, win, iterations, half_pixel);
        return;
    }
    const REAL *la[4] = {A}, *lb[4] = {B};
    REAL *lu[4] = {us}, *lv[4] = {vs};
    int lh[4] = {h}, lw[4] = {w};
    for (int l = 1; l < levels; l++) {
        lh[l] = lh[l - 1] / 2;
        lw[l] = lw[l - 1] / 2;
        const long n = (long)lh[l] * lw[l];
        REAL *na = (REAL *)malloc(sizeof(REAL) * n), *nb = (REAL *)malloc(sizeof(REAL) * n);
        REAL *nu = (REAL *)malloc(sizeof(REAL) * n), *nv = (REAL *)malloc(sizeof(REAL) * n);
        DFN(pyr_down)(la[l - 1], lh[l - 1], lw[l - 1], na, RC(1.0));
        DFN(pyr_down)(lb[l - 1], lh[l - 1], lw[l - 1], nb, RC(1.0));
        DFN(pyr_down)(lu[l - 1], lh[l - 1], lw[l - 1], nu, RC(0.5));
        DFN(pyr_down)(lv[l - 1], lh[l - 1], lw[l - 1], nv, RC(0.5));
        la[l] = na;
        lb[l] = nb;
        lu[l] = nu;
        lv[l] = nv;
    }
    for (int l = levels - 1; l >= 0; l--) {
        if (l < levels - 1) {
            DFN(pyr_up)(lu[l + 1], lh[l + 1], lw[l + 1], lu[l], lh[l], lw[l]);
            DFN(pyr_up)(lv[l + 1], lh[l + 1], lw[l + 1], lv[l], lh[l], lw[l]);
        }
        DFN(dense_lk)(la[l], lb[l], lh[l], lw[l], lu[l], lv[l], win, iterations, half_pixel);
    }
    for (int l = 1; l < levels; l++) {
        free((void *)la[l]);
        free((void *)lb[l]);
        free(lu[l]);
        free(lv[l]);
    }
}

/* IOpticalFlowInterpolator.interpolate(stepTilesA, stepTilesB) of the LucasKanade (mode 1) and
 * LiuShenWithLucasKanade (mode 2) interpolators
 * (S/interpolators/DenseLucasKanadeAparapiJobInterpolator.java:247-334,
 *  S/interpolators/DenseLiuShenAparapiJobInterpolator.java:226-341) for the last adaptive step:
 * images filtered (LK: sigma_lk/px_lk; LS: sigma_ls/px_ls then normalised), the tile field
 * interpolated per pixel (offset 0 with dense export, else 0.5), Lucas-Kanade (+ Liu-Shen) with the
 * half-pixel offset unless dense export, tile displacements replaced from the pixel at
 * top + N/2 - 1 (average of the 2x2 pixels there with dense export).  img: float copies of the
 * frames.  tu/tv: tile displacements (rows, columns), ni x nj, updated in place (rounded to float
 * in the FP64 twin); dense_u/dense_v (rows, columns) receive the dense field when non-NULL.  The
 * FP64 twin takes the filter weights unrounded and the per-pixel field in double.  clip_mode 2:
 * NoOutOfBoundClipping of the tile replacement (S/iareas/Tile.java:156-189). */
void DFN(flow_after_piv)(const float *img_a, const float *img_b, int h, int w, int n, int ni, int nj,
                         const int *tops, const int *lefts, float *tu, float *tv, int mode, float sigma_lk, int px_lk,
                         float sigma_ls, int px_ls, int window, int iters_lk, float lambda, int iters_ls,
                         int dense_export, int ignore_piv, int pyramid_levels, int clip_mode, REAL *dense_u,
                         REAL *dense_v) {
    const long np = (long)h * w;
    REAL *ia = (REAL *)malloc(sizeof(REAL) * np), *ib = (REAL *)malloc(sizeof(REAL) * np);
    for (long p = 0; p < np; p++) { ia[p] = (REAL)img_a[p]; ib[p] = (REAL)img_b[p]; }
    REAL *lka = (REAL *)malloc(sizeof(REAL) * np), *lkb = (REAL *)malloc(sizeof(REAL) * np);
    REAL *lsa = NULL, *lsb = NULL;
    REAL k[64];
    DFN(kernel)(sigma_lk, px_lk, k);
    if (sigma_lk < 1e-5f) { memcpy(lka, ia, sizeof(REAL) * np); memcpy(lkb, ib, sizeof(REAL) * np); }
    else { DFN(gauss_filter)(ia, h, w, k, px_lk, lka); DFN(gauss_filter)(ib, h, w, k, px_lk, lkb); }
    if (mode == 2) {
        lsa = (REAL *)malloc(sizeof(REAL) * np);
        lsb = (REAL *)malloc(sizeof(REAL) * np);
        REAL *t = (REAL *)malloc(sizeof(REAL) * np);
        DFN(kernel)(sigma_ls, px_ls, k);
        if (sigma_ls < 1e-5f) memcpy(t, ia, sizeof(REAL) * np); else DFN(gauss_filter)(ia, h, w, k, px_ls, t);
        DFN(normalize)(t, np, lsa);
        if (sigma_ls < 1e-5f) memcpy(t, ib, sizeof(REAL) * np); else DFN(gauss_filter)(ib, h, w, k, px_ls, t);
        DFN(normalize)(t, np, lsb);
        free(t);
    }
    double *ys = (double *)malloc(sizeof(double) * ni), *xs = (double *)malloc(sizeof(double) * nj);
    for (int i = 0; i < ni; i++) ys[i] = (double)((float)tops[i] + (float)n / 2.0f - 0.5f);
    for (int j = 0; j < nj; j++) xs[j] = (double)((float)lefts[j] + (float)n / 2.0f - 0.5f);
    float *ffu = (float *)malloc(sizeof(float) * np), *ffv = (float *)malloc(sizeof(float) * np);
    const float off = dense_export ? 0.0f : 0.5f;
    orc_displacement_field_off(ys, ni, xs, nj, tu, tv, h, w, FIELD_PRECISION, off, off, ffu, ffv);
    REAL *fu = (REAL *)malloc(sizeof(REAL) * np), *fv = (REAL *)malloc(sizeof(REAL) * np);
    for (long p = 0; p < np; p++) { fu[p] = (REAL)ffu[p]; fv[p] = (REAL)ffv[p]; }
    free(ffu);
    free(ffv);
    /* ignorePIVBaseDisplacements (DenseLucasKanadeAparapiJobInterpolator.java:233-277) */
    if (ignore_piv == 4 || ignore_piv == 5) {
        const REAL lim = ignore_piv == 4 ? RC(3.0) : RC(0.9);
        for (long p = 0; p < np; p++) {
            if (RFABS(fu[p]) < lim) fu[p] = RC(0.0);
            if (RFABS(fv[p]) < lim) fv[p] = RC(0.0);
        }
    }
    if (ignore_piv == 2 || ignore_piv == 3)
        for (long p = 0; p < np; p++) fu[p] = dense_export ? RC(0.0) : RC(0.5);
    if (ignore_piv == 1 || ignore_piv == 3)
        for (long p = 0; p < np; p++) fv[p] = dense_export ? RC(0.0) : RC(0.5);
    /* the flow jobs take columns (us) and rows (vs) */
    REAL *us = fv, *vs = fu;
    const int half = dense_export ? 0 : 1;
    DFN(dense_lk_pyramid)(lka, lkb, h, w, us, vs, window, iters_lk, half, pyramid_levels);
    if (mode == 2) DFN(liu_shen)(lsa, lsb, h, w, us, vs, (REAL)lambda, iters_ls, half, NULL, NULL, NULL);
    for (int ti = 0; ti < ni; ti++)
        for (int tj = 0; tj < nj; tj++) {
            const int i = tops[ti] + n / 2 - 1, j = lefts[tj] + n / 2 - 1;
            const long idx = (long)i * w + j, idx2 = (long)(i + 1) * w + j;
            REAL u, v;
            if (!dense_export) {
                u = us[idx];
                v = vs[idx];
            } else {
                u = (((us[idx] + us[idx + 1]) + us[idx2]) + us[idx2 + 1]) / RC(4.0);
                v = (((vs[idx] + vs[idx + 1]) + vs[idx2]) + vs[idx2 + 1]) / RC(4.0);
            }
            /* Tile.replaceDisplacement(v, u): rows, columns; under NoOutOfBoundClipping (clip_mode 2)
             * refused when it moves the tile out of the image */
            if (clip_mode == 2 && !orc_clip_ok(n, h, w, tops[ti], lefts[tj], (float)v, (float)u)) continue;
            tu[ti * nj + tj] = (float)v;
            tv[ti * nj + tj] = (float)u;
        }
    if (dense_u) memcpy(dense_u, vs, sizeof(REAL) * np);
    if (dense_v) memcpy(dense_v, us, sizeof(REAL) * np);
    free(ia); free(ib); free(lka); free(lkb); free(lsa); free(lsb); free(ys); free(xs); free(fu); free(fv);
}

#undef RC
