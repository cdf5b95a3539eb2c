/* CPU oracle (test infrastructure only): the Direct, Area and Distance velocity inheritance
 * strategies, restated as the reference runs them -- one serial walk over the child tiles with
 * the parent reference tile carried from tile to tile -- in IEEE single arithmetic without
 * contraction (Java float semantics).
 *
 *   Direct    S/iareas/AdaptiveInterVelocityInheritanceStrategyDirect.java:38-92
 *   Area      S/iareas/AdaptiveInterVelocityInheritanceStrategyArea.java:45-210 (walk),
 *             :222-299 (checkOverlappingFactor)
 *   Distance  S/iareas/AdaptiveInterVelocityInheritanceStrategyDistanceGeneric.java:41-231 (walk),
 *             :233-268 (checkDistance)
 *
 * Grids are separable: parent tile (i, j) covers rows ptops[i] .. ptops[i] + pn - 1 and
 * columns plefts[j] .. plefts[j] + pn - 1; child tiles likewise with cn.  Displacements are
 * row-major (tiles_i x tiles_j).  Every function returns 0, or a negative code where the
 * reference throws (IllegalStateException / InvalidStateException / an array index out of
 * range); the child displacements are then undefined.
 *
 * Third-party arithmetic: FastMath.round(float) (commons-math3 3.6.1) is floor(x + 0.5f);
 * FastMath.sqrt is the correctly rounded square root; FastMath.pow(d, 2) of the integer-valued
 * centre differences is their exact square (any of FastMath's pow paths returns the exact
 * value when it is representable, and these squares are below 2^40).
 */
#include <math.h>
#include <string.h>

#include "oracle_types.h"

static int jround(float x) { return (int)floorf(x + 0.5f); }

static float rounded_or_not(float x, int round_int) { return round_int ? (float)jround(x) : x; }

/* ---------------- Direct ---------------- */

int orc_inherit_direct(int pni, int pnj, const float *pu, const float *pv, int cni, int cnj, int round_int,
                       float *cu, float *cv) {
    memset(cu, 0, sizeof(float) * (size_t)cni * cnj); /* resetDisplacements */
    memset(cv, 0, sizeof(float) * (size_t)cni * cnj);
    if (cni < 2 * pni || cnj < 2 * pnj) return -1;    /* currentTiles[2i + 1][2j + 1] out of range */
    for (int i = 0; i < pni; i++)
        for (int j = 0; j < pnj; j++) {
            const float u = rounded_or_not(pu[(size_t)i * pnj + j], round_int);
            const float v = rounded_or_not(pv[(size_t)i * pnj + j], round_int);
            for (int di = 0; di < 2; di++)
                for (int dj = 0; dj < 2; dj++) {
                    const size_t k = (size_t)(2 * i + di) * cnj + (2 * j + dj);
                    cu[k] = 0.0f + u;
                    cv[k] = 0.0f + v;
                }
        }
    return 0;
}

/* ---------------- Area ---------------- */

typedef struct {
    float factor, area;
    int up, down, left, right;
} overlap_t;

/* checkOverlappingFactor: overlap of the child tile (ct, cl, cn) with the parent (pt, pl, pn). */
static overlap_t overlap_of(int pt, int pl, int pn, int ct, int cl, int cn) {
    overlap_t r;
    memset(&r, 0, sizeof(r));
    int vert = 0, horiz = 0;
    if (pt <= ct) {
        if (pt + pn > ct) {
            int end = ct + cn;
            if (end - 1 >= pt + pn) end = pt + pn;
            vert = end - ct;
        } else {
            r.down = 1;
        }
    } else if (ct + cn > pt) {
        vert = ct + cn - pt;
    } else {
        r.up = 1;
    }
    if (pl <= cl) {
        if (pl + pn > cl) {
            int end = cl + cn;
            if (end - 1 >= pl + pn) end = pl + pn;
            horiz = end - cl;
        } else {
            r.right = 1;
        }
    } else if (cl + cn > pl) {
        horiz = cl + cn - pl;
    } else {
        r.left = 1;
    }
    r.area = (float)(vert * horiz);
    r.factor = r.area / (float)(cn * cn);
    return r;
}

/* checkOverlappingFactor alone: the factor and the move flags (bit 0 up, 1 down, 2 left, 3 right). */
float orc_area_overlap(int pt, int pl, int pn, int ct, int cl, int cn, int *flags) {
    overlap_t r = overlap_of(pt, pl, pn, ct, cl, cn);
    *flags = r.up | r.down << 1 | r.left << 2 | r.right << 3;
    return r.factor;
}

int orc_inherit_area(int pn, int pni, int pnj, const int *ptops, const int *plefts, const float *pu, const float *pv,
                     int cn, int cni, int cnj, const int *ctops, const int *clefts, int round_int, float *cu,
                     float *cv) {
    enum { MAXC = 4096 };
    static _Thread_local int ci_of[MAXC], cj_of[MAXC];
    static _Thread_local float area_of[MAXC];
    int pi = 0, pj = 0;
    for (int i = 0; i < cni; i++) {
        pj = 0;
        int ri = pi, rj = pj; /* reference tile */
        for (int j = 0; j < cnj; j++) {
            const int ct = ctops[i], cl = clefts[j];
            overlap_t ref = overlap_of(ptops[ri], plefts[rj], pn, ct, cl, cn);
            if (ref.up || ref.left) return -2;
            if (ref.right) {
                if (ref.down) return -3;
                if (pj + 1 == pnj) return -4;
                pj++;
                ri = pi;
                rj = pj;
            }
            if (ref.down) {
                if (pi + 1 == pni) return -5;
                pi++;
                ri = pi;
                rj = pj;
            }
            float acc = 0.0f;
            int oi = 0, oj = 0, max_j = 0, end = 0, count = 0;
            do {
                const int qi = pi + oi, qj = pj + oj;
                overlap_t c = overlap_of(ptops[qi], plefts[qj], pn, ct, cl, cn);
                if (c.factor == 0.0f) {
                    if (c.right) return -6;
                    if (c.down) return -7;
                    if (c.left) {
                        max_j = oj;
                        oj = 0;
                        oi++;
                        if (pi + oi == pni) end = 1;
                    } else if (c.up) {
                        if (oj != 0) return -8;
                        end = 1;
                    }
                } else {
                    if (count == MAXC) return -9;
                    acc += c.area;
                    ci_of[count] = qi;
                    cj_of[count] = qj;
                    area_of[count] = c.area;
                    count++;
                    oj++;
                    int next_row = pj + oj == pnj || (max_j > 0 && oj == max_j);
                    if (next_row) {
                        oi++;
                        oj = 0;
                        if (pi + oi == pni) end = 1;
                    }
                }
            } while (!end);
            float du = 0.0f, dv = 0.0f;
            for (int k = 0; k < count; k++) {
                const float wgt = area_of[k] / acc;
                const size_t p = (size_t)ci_of[k] * pnj + cj_of[k];
                du += wgt * pu[p];
                dv += wgt * pv[p];
            }
            const size_t q = (size_t)i * cnj + j;
            cu[q] = 0.0f + rounded_or_not(du, round_int);
            cv[q] = 0.0f + rounded_or_not(dv, round_int);
        }
    }
    return 0;
}

/* ---------------- Distance ---------------- */

typedef struct {
    int valid;   /* parentTile != null */
    int pi, pj;
    float dist;
    int is_down, is_right;
} dist_t;

static void distance_of(int pt, int pl, int pn, int ct, int cl, int cn, dist_t *r) {
    const float cy = (float)pt + (float)pn / 2.0f, cx = (float)pl + (float)pn / 2.0f;
    const float ccy = (float)ct + (float)cn / 2.0f, ccx = (float)cl + (float)cn / 2.0f;
    r->is_down = !(cy <= ccy);
    r->is_right = !(cx <= ccx);
    const double dx = (double)(ccx - cx), dy = (double)(ccy - cy);
    r->dist = (float)sqrt(dx * dx + dy * dy);
}

int orc_inherit_distance(int pn, int pni, int pnj, const int *ptops, const int *plefts, const float *pu,
                         const float *pv, int cn, int cni, int cnj, const int *ctops, const int *clefts, int round_int,
                         float *cu, float *cv) {
    int pi = 0, pj = 0;
    dist_t a[4];
    memset(a, 0, sizeof(a));
    for (int i = 0; i < cni; i++) {
        pj = 0;
        for (int j = 0; j < cnj; j++) {
            const int ct = ctops[i], cl = clefts[j];
            int more = 1, guard = 0;
            while (more) {
                if (++guard > 4 * (pni + pnj) + 8) return -1;
                int adjusted = 0;
                distance_of(ptops[pi], plefts[pj], pn, ct, cl, cn, &a[0]);
                a[0].valid = 1;
                a[0].pi = pi;
                a[0].pj = pj;
                if (pi + 1 < pni && pj + 1 < pnj) {
                    distance_of(ptops[pi + 1], plefts[pj + 1], pn, ct, cl, cn, &a[3]);
                    a[3].valid = 1;
                    a[3].pi = pi + 1;
                    a[3].pj = pj + 1;
                    if (!a[3].is_right) {
                        pj++;
                        adjusted = 1;
                    }
                    if (!a[3].is_down) {
                        pi++;
                        adjusted = 1;
                    }
                    if (a[3].is_down && a[3].is_right) more = 0;
                    else continue;
                } else {
                    a[3].valid = 0;
                }
                if (pj + 1 < pnj) {
                    distance_of(ptops[pi], plefts[pj + 1], pn, ct, cl, cn, &a[1]);
                    a[1].valid = 1;
                    a[1].pi = pi;
                    a[1].pj = pj + 1;
                    if (!a[1].is_right) {
                        if (!more) return -2;
                        pj++;
                        adjusted = 1;
                        continue;
                    }
                    more = 0;
                } else {
                    a[1].valid = 0;
                }
                if (pi + 1 < pni) {
                    distance_of(ptops[pi + 1], plefts[pj], pn, ct, cl, cn, &a[2]);
                    a[2].valid = 1;
                    a[2].pi = pi + 1;
                    a[2].pj = pj;
                    if (!a[2].is_down) {
                        if (!more) return -3;
                        adjusted = 1;
                        pi++;
                        continue;
                    }
                    more = 0;
                } else {
                    a[2].valid = 0;
                }
                if (more && !adjusted) more = 0;
            }
            if (a[0].is_right) a[1].valid = a[3].valid = 0;
            if (a[0].is_down) a[2].valid = a[3].valid = 0;
            float total = 0.0f;
            int zero = -1;
            for (int k = 0; k < 4; k++) {
                if (!a[k].valid) continue;
                if (a[k].dist == 0.0f) {
                    zero = k;
                    break;
                }
                total += 1.0f / a[k].dist;
            }
            float du = 0.0f, dv = 0.0f;
            if (zero < 0) {
                for (int k = 0; k < 4; k++) {
                    if (!a[k].valid) continue;
                    const float wgt = (1.0f / a[k].dist) / total;
                    const size_t p = (size_t)a[k].pi * pnj + a[k].pj;
                    du += wgt * pu[p];
                    dv += wgt * pv[p];
                }
            } else {
                const size_t p = (size_t)a[zero].pi * pnj + a[zero].pj;
                du = pu[p];
                dv = pv[p];
            }
            const size_t q = (size_t)i * cnj + j;
            cu[q] = 0.0f + rounded_or_not(du, round_int);
            cv[q] = 0.0f + rounded_or_not(dv, round_int);
        }
    }
    return 0;
}

/* mode: 1 Direct, 2 Area, 3 Distance (the qlpiv_inherit_mode values). */
int orc_inherit_tiles(int mode, int pn, int pni, int pnj, const int *ptops, const int *plefts, const float *pu,
                      const float *pv, int cn, int cni, int cnj, const int *ctops, const int *clefts, int round_int,
                      float *cu, float *cv) {
    switch (mode) {
        case 1: return orc_inherit_direct(pni, pnj, pu, pv, cni, cnj, round_int, cu, cv);
        case 2: return orc_inherit_area(pn, pni, pnj, ptops, plefts, pu, pv, cn, cni, cnj, ctops, clefts, round_int,
                                        cu, cv);
        case 3: return orc_inherit_distance(pn, pni, pnj, ptops, plefts, pu, pv, cn, cni, cnj, ctops, clefts,
                                            round_int, cu, cv);
        default: return -100;
    }
}
