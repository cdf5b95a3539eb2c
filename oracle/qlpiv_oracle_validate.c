/*
 * qlpiv oracle, vector validation -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates the reference's validation stage in Java float semantics:
 *   VectorValidatorJob.compute / circularVisitor   S/jobs/validator/VectorValidatorJob.java:105-411
 *   NormalizedMedianValidator.validateVector       S/iareas/validation/NormalizedMedianValidator.java:63-136
 *   SecondaryPeakReplacement.replaceVector         S/iareas/replacement/SecondaryPeakReplacement.java:41-76
 *   BilinearReplacement.replaceVector              S/iareas/replacement/BilinearReplacement.java
 *   Tile lock / backup / restore                   S/iareas/Tile.java:140-215
 *   DifferenceValidator.validateVector             S/iareas/validation/DifferenceValidator.java:30-60
 * as the converter configures the five validation models
 * (PIVConfigurationConverterVisitor.visit, ui/.../PIVConfigurationConverterVisitor.java:546-641):
 * multi-peak normalised median (strategies 0..k-2 = median validation + replacement by peak
 * 1..k-1, strategy k-1 = median validation + bilinear replacement), and one strategy of
 * difference or normalised-median validation with no replacement or bilinear replacement.
 * Every tile starts invalid (the Tile constructors, S/iareas/Tile.java:51-67).  No masks.
 * Replacements follow the clipping mode (Tile.replaceDisplacement, S/iareas/Tile.java:156-189).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* VectorValidatorJob.circularVisitor: centre-out rings (right, down, left, up).  Writes
 * the visit order (tile index i*nj + j) and returns its length (ni*nj). */
int orc_spiral_order(int ni, int nj, int *order) {
    int startI = ni / 2, startJ = nj / 2;
    int sideI = 2, sideJ = 2;
    if (ni != startI * 2) sideI = 1; else startI--;
    if (nj != startJ * 2) sideJ = 1; else startJ--;
    const int total = ni * nj;
    unsigned char *seen = (unsigned char *)calloc((size_t)total, 1);
    int visited = 0;
#define VISIT(a, b)                                                       \
    do {                                                                  \
        const int ii = (a), jj = (b);                                     \
        if (ii >= 0 && ii < ni && jj >= 0 && jj < nj && !seen[ii * nj + jj]) { \
            seen[ii * nj + jj] = 1;                                       \
            order[visited++] = ii * nj + jj;                              \
        }                                                                 \
    } while (0)
    while (visited < total) {
        const int m0 = sideJ > 1 ? sideJ - 1 : 0;
        const int m1 = sideI > 1 ? sideI - 1 : 0;
        const int m2 = sideJ > 1 ? sideJ - 1 : 0;
        const int m3 = sideI > 2 ? sideI - 2 : 0;
        int j = startJ, i = startI;
        VISIT(i, j);
        for (int o = 0; o < m0; o++) { ++j; VISIT(i, j); }
        for (int o = 0; o < m1; o++) { ++i; VISIT(i, j); }
        if (m1 > 0) {
            for (int o = 0; o < m2; o++) { --j; VISIT(i, j); }
            for (int o = 0; o < m3; o++) { --i; VISIT(i, j); }
        }
        sideI += 2;
        sideJ += 2;
        startJ--;
        startI--;
    }
#undef VISIT
    free(seen);
    return visited;
}

#include "oracle_types.h"

/* iterate-until-no-corrections bound shared with the CUDA path */
#define ORC_MAX_SWEEPS 1000

typedef struct {
    int ni, nj;
    const int *tops, *lefts;
    float *u, *v, *bu, *bv;
    unsigned char *invalid, *locked;
    int clip_n, clip_h, clip_w;
} vstate;

/* Tile.replaceDisplacement: refused under NoOutOfBoundClipping when the rounded displacement
 * moves the tile out of the image */
static int replace_ok(const vstate *s, int k, float u, float v) {
    return orc_clip_ok(s->clip_n, s->clip_h, s->clip_w, s->tops[k / s->nj], s->lefts[k % s->nj], u, v);
}

static int java_round_v(float x) { return (int)floorf(x + 0.5f); }

static void set_invalid(vstate *s, int k, int state) {
    if (s->locked[k]) return;
    s->invalid[k] = (unsigned char)state;
}

/* NormalizedMedianValidator.validateVector */
static void validate_median(vstate *s, int k, float threshold, float eps0) {
    const int ti = k / s->nj, tj = k % s->nj;
    int nb[8], n = 0;
    for (int a = -1; a <= 1; a++)
        for (int b = -1; b <= 1; b++) {
            if (a == 0 && b == 0) continue;
            const int i = ti + a, j = tj + b;
            if (i < 0 || i >= s->ni || j < 0 || j >= s->nj) continue;
            nb[n++] = i * s->nj + j;
        }
    /* Collections.sort by u^2 + v^2 (stable) */
    float norm[8];
    for (int q = 0; q < n; q++) norm[q] = s->u[nb[q]] * s->u[nb[q]] + s->v[nb[q]] * s->v[nb[q]];
    for (int q = 1; q < n; q++) {
        const int t = nb[q];
        const float nt = norm[q];
        int r = q - 1;
        while (r >= 0 && norm[r] > nt) { nb[r + 1] = nb[r]; norm[r + 1] = norm[r]; r--; }
        nb[r + 1] = t;
        norm[r + 1] = nt;
    }
    float mu = 0.0f, mv = 0.0f;
    if (n > 0) {
        if (n % 2 == 0) {
            mu = (s->u[nb[n / 2 - 1]] + s->u[nb[n / 2]]) / 2.0f;
            mv = (s->v[nb[n / 2 - 1]] + s->v[nb[n / 2]]) / 2.0f;
        } else {
            mu = s->u[nb[n / 2]];
            mv = s->v[nb[n / 2]];
        }
    }
    float r8[8];
    for (int q = 0; q < 8; q++) r8[q] = FLT_MAX;
    for (int q = 0; q < n; q++) {
        const float du = mu - s->u[nb[q]], dv = mv - s->v[nb[q]];
        r8[q] = du * du + dv * dv;
    }
    for (int q = 1; q < 8; q++) {   /* Arrays.sort(float[]) */
        const float t = r8[q];
        int r = q - 1;
        while (r >= 0 && r8[r] > t) { r8[r + 1] = r8[r]; r--; }
        r8[r + 1] = t;
    }
    float rmed;
    const int ri = n;
    if (ri - 1 == 0) rmed = 1.0f;
    else if ((ri - 1) % 2 == 0) rmed = (float)sqrt((double)((r8[(ri - 1) / 2] + r8[(ri - 1) / 2 + 1]) / 2.0f));
    else rmed = (float)sqrt((double)r8[(ri - 1) / 2 + 1]);
    const float du = mu - s->u[k], dv = mv - s->v[k];
    const float dist = (float)sqrt((double)(du * du + dv * dv)) / (rmed + eps0);
    set_invalid(s, k, !(dist < threshold));
}

/* DifferenceValidator.validateVector: adjacents[i][j] for i, j in {0, 1} except (1, 1) -- the
 * top-left, top and left neighbours -- each valid one overwriting the tile's flag with the test
 * |d|^2 < threshold^2; with no valid one among them the flag is left as it is. */
static void validate_difference(vstate *s, int k, float threshold) {
    const float t2 = threshold * threshold;
    const int ti = k / s->nj, tj = k % s->nj;
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) {
            if (a == 1 && b == 1) continue;
            const int i = ti + a - 1, j = tj + b - 1;
            if (i < 0 || i >= s->ni || j < 0 || j >= s->nj) continue;
            const int q = i * s->nj + j;
            if (s->invalid[q]) continue;
            const float du = s->u[q] - s->u[k], dv = s->v[q] - s->v[k];
            const float dist = du * du + dv * dv;
            set_invalid(s, k, !(dist < t2));
        }
}

/* BilinearReplacement.interpV / interpU: linear interpolation between two tiles along
 * the column (left pixel) or row (top pixel) coordinate.  Returns 0 on the reference's
 * "unexpected corner case" (not reachable on a regular grid). */
static int interp_1d(float p1, float p2, float pi, float a1, float a2, float *out) {
    float w1 = 0.0f, w2 = 0.0f;
    if ((p2 - pi) > 1e-6f && (pi - p1) > 1e-6f && (p2 - p1) > 1e-6f) {
        const float wt1 = (p2 - pi) / (p2 - p1);
        w1 = wt1 * a1;
        const float wt2 = (pi - p1) / (p2 - p1);
        w2 = wt2 * a2;
    } else {
        int count = 0;
        if (fabsf(pi - p2) < 1e-6f) { w2 = a2; count++; }
        if (fabsf(pi - p1) < 1e-6f) { w1 = a1; count++; }
        if (count == 0) return 0;
        if (count > 1) { w1 /= (float)count; w2 /= (float)count; }
    }
    *out = w1 + w2;
    return 1;
}

static void replace_bilinear(vstate *s, int k) {
    if (!s->invalid[k]) return;
    const int ti = k / s->nj, tj = k % s->nj;
    int adj[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            const int i = ti + a - 1, j = tj + b - 1;
            adj[a][b] = (i < 0 || i >= s->ni || j < 0 || j >= s->nj) ? -1 : i * s->nj + j;
        }
    const int L = adj[1][0], R = adj[1][2], T = adj[0][1], B = adj[2][1];
    const int TL = adj[0][0], BR = adj[2][2], BL = adj[2][0], TR = adj[0][2];
#define OK(x) ((x) >= 0 && !s->invalid[(x)])
#define TOP(x) ((float)s->tops[(x) / s->nj])
#define LEFT(x) ((float)s->lefts[(x) % s->nj])
    float uV[4] = {0, 0, 0, 0}, uU[4] = {0, 0, 0, 0};
    int cV[4] = {0, 0, 0, 0}, cU[4] = {0, 0, 0, 0};
    int count = 0;
    if (OK(L) && OK(R)) {
        interp_1d(LEFT(L), LEFT(R), LEFT(k), s->v[L], s->v[R], &uV[0]);
        interp_1d(TOP(L), TOP(R), TOP(k), s->u[L], s->u[R], &uU[0]);
        cV[0] = 2; cU[0] = 1; count++;
    }
    if (OK(B) && OK(T)) {
        interp_1d(LEFT(T), LEFT(B), LEFT(k), s->v[T], s->v[B], &uV[1]);
        interp_1d(TOP(T), TOP(B), TOP(k), s->u[T], s->u[B], &uU[1]);
        cV[1] = 1; cU[1] = 2; count++;
    }
    if (OK(TL) && OK(BR) && OK(BL) && OK(TR)) {
        const float wTR = (LEFT(k) - LEFT(TL)) / (LEFT(TR) - LEFT(TL));
        const float wTL = (LEFT(TR) - LEFT(k)) / (LEFT(TR) - LEFT(TL));
        const float wBR = (LEFT(k) - LEFT(BL)) / (LEFT(BR) - LEFT(BL));
        const float wBL = (LEFT(BR) - LEFT(k)) / (LEFT(BR) - LEFT(BL));
        const float wT = (TOP(BL) - TOP(k)) / (TOP(BL) - TOP(TL));
        const float wB = (TOP(k) - TOP(TL)) / (TOP(BL) - TOP(TL));
        uV[2] = wT * (wTR * s->v[TR] + wTL * s->v[TL]) + wB * (wBR * s->v[BR] + wBL * s->v[BL]);
        uU[2] = wT * (wTR * s->u[TR] + wTL * s->u[TL]) + wB * (wBR * s->u[BR] + wBL * s->u[BL]);
        cV[2] = 3; cU[2] = 3; count++;
    } else {
        if (OK(TL) && OK(BR)) {
            interp_1d(LEFT(TL), LEFT(BR), LEFT(k), s->v[TL], s->v[BR], &uV[2]);
            interp_1d(TOP(TL), TOP(BR), TOP(k), s->u[TL], s->u[BR], &uU[2]);
            cV[2] = 1; cU[2] = 1; count++;
        }
        if (OK(BL) && OK(TR)) {
            interp_1d(LEFT(BL), LEFT(TR), LEFT(k), s->v[BL], s->v[TR], &uV[3]);
            interp_1d(TOP(TR), TOP(BL), TOP(k), s->u[TR], s->u[BL], &uU[3]);
            cV[3] = 1; cU[3] = 1; count++;
        }
    }
    if (count == 0) {
        /* The reference's break leaves only the inner loop: every row overwrites the
         * estimate with its first valid neighbour, so the last such row wins. */
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                if (a == 1 && b == 1) continue;
                if (OK(adj[a][b])) {
                    uV[0] = s->v[adj[a][b]];
                    uU[0] = s->u[adj[a][b]];
                    count = 1;
                    break;
                }
            }
        if (count == 0) {
            set_invalid(s, k, 1);
        } else if (replace_ok(s, k, uU[0], uV[0])) {
            s->u[k] = uU[0];
            s->v[k] = uV[0];
            set_invalid(s, k, 0);
        }
    } else {
        float aV = 0.0f, aU = 0.0f;
        int wV = 0, wU = 0;
        for (int q = 0; q < 4; q++) {
            aV += (float)cV[q] * uV[q];
            wV += cV[q];
            aU += (float)cU[q] * uU[q];
            wU += cU[q];
        }
        aV /= (float)wV;
        aU /= (float)wU;
        if (replace_ok(s, k, aU, aV)) {
            s->u[k] = aU;
            s->v[k] = aV;
        }
        set_invalid(s, k, 0);  /* the reference clears the flag whether or not the value was taken */
    }
#undef OK
#undef TOP
#undef LEFT
}

/* VectorValidatorJob.compute for one frame's tiles (in place on u, v).
 * pu/pv: [ni*nj][k] displacement increments of peaks 0..k-1 (0 = main peak, already
 * accumulated into u, v); npeaks: peaks found per tile (multi-peak model only; may be NULL
 * otherwise).  invalid_out: final flags.  Returns the number of correction sweeps made. */
int orc_validate(int ni, int nj, const int *tops, const int *lefts, float *u, float *v, const float *pu,
                 const float *pv, const int *npeaks, int k, const orc_valid_cfg *cfg, unsigned char *invalid_out) {
    const int total = ni * nj;
    const int model = cfg->model <= 1 ? 1 : cfg->model;
    const int difference = model == 2 || model == 3;
    /* strategies: multi-peak k (secondary peaks then bilinear); otherwise one */
    const int nstrat = model == 1 ? cfg->num_peaks : 1;
    const int last_bilinear = model == 1 || model == 3 || model == 5;
    vstate s;
    s.ni = ni; s.nj = nj; s.tops = tops; s.lefts = lefts; s.u = u; s.v = v;
    s.clip_n = cfg->clip_n; s.clip_h = cfg->clip_h; s.clip_w = cfg->clip_w;
    s.bu = (float *)malloc(sizeof(float) * total);
    s.bv = (float *)malloc(sizeof(float) * total);
    s.invalid = (unsigned char *)malloc((size_t)total);
    memset(s.invalid, 1, (size_t)total);   /* new tiles are invalid until validated */
    s.locked = (unsigned char *)calloc((size_t)total, 1);
    int *order = (int *)malloc(sizeof(int) * total);
    orc_spiral_order(ni, nj, order);
    for (int t = 0; t < total; t++) { s.bu[t] = u[t]; s.bv[t] = v[t]; }
#define VALIDATE(t) (difference ? validate_difference(&s, (t), cfg->threshold) \
                                : validate_median(&s, (t), cfg->threshold, cfg->epsilon0))
    for (int q = 0; q < total; q++) {
        const int t = order[q];
        VALIDATE(t);
        if (!s.invalid[t]) s.locked[t] = 1;
    }
    int attempt = 0;
    for (;;) {
        int corrected = 0;
        for (int q = 0; q < total; q++) {
            const int t = order[q];
            VALIDATE(t);
            for (int idx = 0; idx < nstrat && s.invalid[t]; idx++) {
                const int bilinear = idx == nstrat - 1 && last_bilinear;
                const int secondary = model == 1 && idx < nstrat - 1;
                if (bilinear || secondary) {
                    /* restore the main-peak displacement, then replace */
                    s.u[t] = s.bu[t];
                    s.v[t] = s.bv[t];
                }
                if (secondary) {
                    const int peak = idx + 1;
                    if (npeaks[t] > peak && s.invalid[t]) {
                        float nu = s.u[t], nv = s.v[t];
                        nu -= pu[(size_t)t * k];
                        nv -= pv[(size_t)t * k];
                        nu += pu[(size_t)t * k + peak];
                        nv += pv[(size_t)t * k + peak];
                        if (replace_ok(&s, t, nu, nv)) {
                            s.u[t] = nu;
                            s.v[t] = nv;
                            set_invalid(&s, t, 0);
                        }
                    }
                } else if (bilinear) {
                    replace_bilinear(&s, t);
                }
                VALIDATE(t);
                if (!s.invalid[t]) { corrected++; break; }
            }
        }
        attempt++;
        if (corrected == 0) break;
        if (!cfg->iterate_until_no_corrections && attempt >= cfg->max_iterations) break;
        if (attempt >= ORC_MAX_SWEEPS) break;  /* same bound as the CUDA path */
    }
#undef VALIDATE
    for (int t = 0; t < total; t++) {
        /* still-invalid vectors are set to 0 (Tile.replaceDisplacement(0, 0)) */
        if (s.invalid[t] && replace_ok(&s, t, 0.0f, 0.0f)) { s.u[t] = 0.0f; s.v[t] = 0.0f; }
        if (invalid_out) invalid_out[t] = s.invalid[t];
    }
    free(s.bu); free(s.bv); free(s.invalid); free(s.locked); free(order);
    (void)java_round_v;
    return attempt;
}
