// IA grids of the adaptive levels (host code).
//   SuperPosition    S/iareas/AdaptiveInterAreaStrategySuperPosition.java:31-197
//   NoSuperPosition  S/iareas/AdaptiveInterAreaStrategyNoSuperPosition.java:32-157
// Java float semantics: every float expression below is evaluated in IEEE single
// precision in the reference's operand order (this file is compiled without FMA
// contraction: -Xcompiler -ffp-contract=off).
#include <cmath>

#include "qlpiv_internal.h"

namespace qlpiv {

static int java_round_f(float x) { return (int)std::floor(x + 0.5f); }

static int floor_div(int a, int b) {
    int q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
    return q;
}

int grid_superposition(int h, int w, const int margins[4], int ia_start, int level, float ofac, qlpiv_grid *g,
                       int32_t *tops, int32_t *lefts, int cap) {
    const int mt = margins[0], mb = margins[1], ml = margins[2], mr = margins[3];
    if (ofac < 1.0f / 10.0f || ofac > 1.0f - 1.0f / 10.0f) return -2;
    const int n = ia_start >> level;
    if (n < 1) return -3;
    const float inc = ofac * (float)n;
    const int nj = (int)(0.01f + ((float)(w - (ml + mr)) - ((float)n - inc)) / inc);
    const int ni = (int)(0.01f + ((float)(h - (mt + mb)) - ((float)n - inc)) / inc);
    if (ni < 1 || nj < 1) return -3;
    const int remI = h - (int)std::ceil((double)((float)(ni - 1) * inc + (float)n)) - (mt + mb);
    const int remJ = w - (int)std::ceil((double)((float)(nj - 1) * inc + (float)n)) - (ml + mr);
    g->n = n;
    g->tiles_i = ni;
    g->tiles_j = nj;
    g->margin_top = mt + floor_div(remI, 2);
    g->margin_bottom = mb + (int)std::ceil((double)((float)remI / 2.0f));
    g->margin_left = ml + floor_div(remJ, 2);
    g->margin_right = mr + (int)std::ceil((double)((float)remJ / 2.0f));
    if (ni > cap || nj > cap) return -1;
    if (tops && lefts) {
        if (level == 0) {
            for (int k = 0; k < ni; k++) tops[k] = g->margin_top + java_round_f((float)k * inc);
            for (int k = 0; k < nj; k++) lefts[k] = g->margin_left + java_round_f((float)k * inc);
        } else {
            float p = (float)g->margin_top;
            for (int k = 0; k < ni; k++, p += inc) tops[k] = java_round_f(p);
            p = (float)g->margin_left;
            for (int k = 0; k < nj; k++, p += inc) lefts[k] = java_round_f(p);
        }
    }
    return 0;
}

int grid_nosuperposition(int h, int w, const int margins[4], int ia_start, int level, qlpiv_grid *g, int32_t *tops,
                         int32_t *lefts, int cap) {
    const int mt = margins[0], mb = margins[1], ml = margins[2], mr = margins[3];
    const int n = ia_start >> level;
    if (n < 1) return -3;
    const int ni = floor_div(h - (mt + mb), n), nj = floor_div(w - (ml + mr), n);
    if (ni < 1 || nj < 1) return -3;
    g->n = n;
    g->tiles_i = ni;
    g->tiles_j = nj;
    g->margin_top = mt + (h - mt - mb - n * ni) / 2;
    g->margin_bottom = h - n * ni - g->margin_top;
    g->margin_left = ml + (w - ml - mr - n * nj) / 2;
    g->margin_right = w - n * nj - g->margin_left;
    if (ni > cap || nj > cap) return -1;
    if (tops && lefts) {
        for (int k = 0; k < ni; k++) tops[k] = g->margin_top + k * n;
        for (int k = 0; k < nj; k++) lefts[k] = g->margin_left + k * n;
    }
    return 0;
}

// AdaptiveInterAreaStrategyMixedSuperPosition.createIterationStepTilesParameters
// (S/iareas/AdaptiveInterAreaStrategyMixedSuperPosition.java:31-92): levels before sp_start use
// the NoSuperPosition division; at sp_start the SuperPosition division starts as at its first step
// with IA ia_start >> sp_start (createIterationStepTilesParametersInternal with the step offset,
// S/iareas/AdaptiveInterAreaStrategySuperPosition.java:31-190) and halves from there.
// sp_start == 0 is the plain SuperPosition division, sp_start >= the level count NoSuperPosition.
int grid_level(int h, int w, const int margins[4], int ia_start, int level, float ofac, int sp_start, qlpiv_grid *g,
               int32_t *tops, int32_t *lefts, int cap) {
    if (level < sp_start) return grid_nosuperposition(h, w, margins, ia_start, level, g, tops, lefts, cap);
    return grid_superposition(h, w, margins, ia_start >> sp_start, level - sp_start, ofac, g, tops, lefts, cap);
}

}  // namespace qlpiv
