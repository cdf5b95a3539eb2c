// Vector validation and replacement after a correlation level (device code).
//
// VectorValidatorJob.compute (S/jobs/validator/VectorValidatorJob.java:242-405) with the five
// models the converter builds (PIVConfigurationConverterVisitor.visit,
// ui/src/main/java/pt/quickLabPIV/business/transfer/PIVConfigurationConverterVisitor.java:546-641):
// the multi-peak normalised-median model (k strategies, strategy s < k-1 =
// NormalizedMedianValidator + SecondaryPeakReplacement(peak s+1), strategy k-1 =
// NormalizedMedianValidator + BilinearReplacement), and one strategy of DifferenceValidator or
// NormalizedMedianValidator without or with BilinearReplacement.
//   NormalizedMedianValidator.validateVector  S/iareas/validation/NormalizedMedianValidator.java:63-136
//   DifferenceValidator.validateVector        S/iareas/validation/DifferenceValidator.java:30-60
//   SecondaryPeakReplacement.replaceVector    S/iareas/replacement/SecondaryPeakReplacement.java:41-76
//   BilinearReplacement.replaceVector         S/iareas/replacement/BilinearReplacement.java:23-420
//   Tile backup / restore / lock              S/iareas/Tile.java:138-217
//   circularVisitor visit order               S/jobs/validator/VectorValidatorJob.java:105-204
//
// The reference validates tile by tile in a centre-out spiral, in place, so a tile
// sees the already-updated values of the tiles visited before it.  Two kernels keep
// that result exactly:
//   validate_init_kernel  one thread per tile.  The initial pass only reads the
//                         neighbours' displacements (never changed in that pass) and
//                         writes the tile's own flags, so it is order-free: median test,
//                         lock the valid tiles, back up the displacement.
//   validate_sweep_kernel one CTA per frame pair for the correction sweeps.  Locked tiles
//                         never change, so only the initially invalid ("open") tiles
//                         matter.  An open tile reads only its 8 neighbours; it is
//                         processed in a round once every open neighbour earlier in the
//                         spiral has been processed in an earlier round of the same
//                         sweep, and open neighbours later in the spiral wait for it.
//                         Tiles of one round therefore never touch each other's data and
//                         every tile sees exactly the state of the sequential visit.
//                         When a round makes almost no progress (a long chain of adjacent
//                         open tiles), thread 0 finishes the sweep in spiral order.
// Float arithmetic rounds like Java's (IEEE single, no contraction: this translation
// unit is compiled with --fmad=false; sqrt through double in the reference equals the
// correctly rounded float sqrt).
#include <cuda_runtime.h>
#include <stdint.h>

#include "qlpiv.h"
#include "qlpiv_internal.h"
#include "qlpiv_validate.h"

namespace qlpiv {

namespace {

constexpr uint8_t kInvalid = 1u, kLocked = 2u;
constexpr float kFltMax = 3.402823466e38f;

struct PairView {
    int ni, nj;
    float *u, *v;
    const float *bu, *bv;
    const float2 *puv;
    const uint8_t *npk;
    uint8_t *state;
    const int *tops, *lefts;
    int k;
    int model;
    int clip_n, clip_h, clip_w;
};

// Tile.replaceDisplacement: refused under NoOutOfBoundClipping when the rounded displacement
// moves tile t out of the image.
__device__ __forceinline__ bool replace_ok(const PairView &p, int t, float u, float v) {
    return tile_inside(p.clip_n, p.clip_h, p.clip_w, p.tops[t / p.nj], p.lefts[t % p.nj], u, v);
}

__device__ __forceinline__ bool difference_model(const PairView &p) {
    return p.model == QLPIV_VALIDATE_DIFFERENCE_ONLY || p.model == QLPIV_VALIDATE_DIFFERENCE;
}

__device__ __forceinline__ void set_invalid(const PairView &p, int t, bool inv) {
    const uint8_t st = p.state[t];
    if (st & kLocked) return;  // Tile.setInvalidDisplacement ignores locked tiles
    p.state[t] = inv ? (uint8_t)(st | kInvalid) : (uint8_t)(st & ~kInvalid);
}

__device__ __forceinline__ bool is_invalid(const PairView &p, int t) { return (p.state[t] & kInvalid) != 0; }

// NormalizedMedianValidator.validateVector for tile t.
__device__ void median_validate(const PairView &p, int t, float threshold, float eps0) {
    const int ti = t / p.nj, tj = t - ti * p.nj;
    int nb[8];
    float nrm[8];
    int n = 0;
    for (int a = -1; a <= 1; a++)
        for (int b = -1; b <= 1; b++) {
            if (a == 0 && b == 0) continue;
            const int i = ti + a, j = tj + b;
            if (i < 0 || i >= p.ni || j < 0 || j >= p.nj) continue;
            const int q = i * p.nj + j;
            const float uq = p.u[q], vq = p.v[q];
            const float norm = __fadd_rn(__fmul_rn(uq, uq), __fmul_rn(vq, vq));
            // stable insertion by norm (Collections.sort keeps equal norms in visit order)
            int r = n - 1;
            while (r >= 0 && nrm[r] > norm) {
                nb[r + 1] = nb[r];
                nrm[r + 1] = nrm[r];
                r--;
            }
            nb[r + 1] = q;
            nrm[r + 1] = norm;
            n++;
        }
    float mu = 0.0f, mv = 0.0f;
    if (n > 0) {
        if (n % 2 == 0) {
            mu = __fdiv_rn(__fadd_rn(p.u[nb[n / 2 - 1]], p.u[nb[n / 2]]), 2.0f);
            mv = __fdiv_rn(__fadd_rn(p.v[nb[n / 2 - 1]], p.v[nb[n / 2]]), 2.0f);
        } else {
            mu = p.u[nb[n / 2]];
            mv = p.v[nb[n / 2]];
        }
    }
    float r8[8];
    for (int q = 0; q < 8; q++) r8[q] = kFltMax;
    for (int q = 0; q < n; q++) {
        const float du = __fsub_rn(mu, p.u[nb[q]]), dv = __fsub_rn(mv, p.v[nb[q]]);
        const float ri = __fadd_rn(__fmul_rn(du, du), __fmul_rn(dv, dv));
        int r = q - 1;  // ascending insertion (Arrays.sort)
        while (r >= 0 && r8[r] > ri) {
            r8[r + 1] = r8[r];
            r--;
        }
        r8[r + 1] = ri;
    }
    float rmed;
    if (n - 1 == 0) {
        rmed = 1.0f;
    } else if ((n - 1) % 2 == 0) {
        rmed = __fsqrt_rn(__fdiv_rn(__fadd_rn(r8[(n - 1) / 2], r8[(n - 1) / 2 + 1]), 2.0f));
    } else {
        rmed = __fsqrt_rn(r8[(n - 1) / 2 + 1]);
    }
    const float du = __fsub_rn(mu, p.u[t]), dv = __fsub_rn(mv, p.v[t]);
    const float dist = __fdiv_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(du, du), __fmul_rn(dv, dv))), __fadd_rn(rmed, eps0));
    set_invalid(p, t, !(dist < threshold));
}

// DifferenceValidator.validateVector for tile t: adjacents[i][j] for i, j in {0, 1} except
// (1, 1) -- the top-left, top and left neighbours -- each valid one overwriting the flag with
// |d|^2 < threshold^2; with no valid one among them the flag is left as it is.
__device__ void difference_validate(const PairView &p, int t, float threshold) {
    const float t2 = __fmul_rn(threshold, threshold);
    const int ti = t / p.nj, tj = t - ti * p.nj;
    for (int a = -1; a <= 0; a++)
        for (int b = -1; b <= 0; b++) {
            if (a == 0 && b == 0) continue;
            const int i = ti + a, j = tj + b;
            if (i < 0 || j < 0) continue;
            const int q = i * p.nj + j;
            if (p.state[q] & kInvalid) continue;
            const float du = __fsub_rn(p.u[q], p.u[t]), dv = __fsub_rn(p.v[q], p.v[t]);
            const float dist = __fadd_rn(__fmul_rn(du, du), __fmul_rn(dv, dv));
            set_invalid(p, t, !(dist < t2));
        }
}

__device__ __forceinline__ void validate_vector(const PairView &p, int t, float threshold, float eps0) {
    if (difference_model(p))
        difference_validate(p, t, threshold);
    else
        median_validate(p, t, threshold, eps0);
}

// BilinearReplacement.interpV / interpU: weights along one coordinate of two tiles.
__device__ float interp_1d(float p1, float p2, float pi, float a1, float a2) {
    float w1 = 0.0f, w2 = 0.0f;
    if (__fsub_rn(p2, pi) > 1e-6f && __fsub_rn(pi, p1) > 1e-6f && __fsub_rn(p2, p1) > 1e-6f) {
        w1 = __fmul_rn(__fdiv_rn(__fsub_rn(p2, pi), __fsub_rn(p2, p1)), a1);
        w2 = __fmul_rn(__fdiv_rn(__fsub_rn(pi, p1), __fsub_rn(p2, p1)), a2);
    } else {
        int count = 0;
        if (fabsf(__fsub_rn(pi, p2)) < 1e-6f) { w2 = a2; count++; }
        if (fabsf(__fsub_rn(pi, p1)) < 1e-6f) { w1 = a1; count++; }
        // count == 0 is the reference's "unexpected corner case"; a regular grid never has it
        if (count > 1) {
            w1 = __fdiv_rn(w1, (float)count);
            w2 = __fdiv_rn(w2, (float)count);
        }
    }
    return __fadd_rn(w1, w2);
}

// BilinearReplacement.replaceVector for tile t (invalid on entry).
__device__ void bilinear_replace(const PairView &p, int t) {
    if (!is_invalid(p, t)) return;
    const int ti = t / p.nj, tj = t - ti * p.nj;
    int adj[3][3];
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
            const int i = ti + a - 1, j = tj + b - 1;
            adj[a][b] = (i < 0 || i >= p.ni || j < 0 || j >= p.nj) ? -1 : i * p.nj + j;
        }
    auto ok = [&](int q) { return q >= 0 && !is_invalid(p, q); };
    auto top = [&](int q) { return (float)p.tops[q / p.nj]; };
    auto left = [&](int q) { return (float)p.lefts[q % p.nj]; };
    const int L = adj[1][0], R = adj[1][2], T = adj[0][1], B = adj[2][1];
    const int TL = adj[0][0], BR = adj[2][2], BL = adj[2][0], TR = adj[0][2];
    float uV[4] = {0.0f, 0.0f, 0.0f, 0.0f}, uU[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    int cV[4] = {0, 0, 0, 0}, cU[4] = {0, 0, 0, 0};
    int count = 0;
    if (ok(L) && ok(R)) {
        uV[0] = interp_1d(left(L), left(R), left(t), p.v[L], p.v[R]);
        uU[0] = interp_1d(top(L), top(R), top(t), p.u[L], p.u[R]);
        cV[0] = 2;
        cU[0] = 1;
        count++;
    }
    if (ok(B) && ok(T)) {
        uV[1] = interp_1d(left(T), left(B), left(t), p.v[T], p.v[B]);
        uU[1] = interp_1d(top(T), top(B), top(t), p.u[T], p.u[B]);
        cV[1] = 1;
        cU[1] = 2;
        count++;
    }
    if (ok(TL) && ok(BR) && ok(BL) && ok(TR)) {
        const float wTR = __fdiv_rn(__fsub_rn(left(t), left(TL)), __fsub_rn(left(TR), left(TL)));
        const float wTL = __fdiv_rn(__fsub_rn(left(TR), left(t)), __fsub_rn(left(TR), left(TL)));
        const float wBR = __fdiv_rn(__fsub_rn(left(t), left(BL)), __fsub_rn(left(BR), left(BL)));
        const float wBL = __fdiv_rn(__fsub_rn(left(BR), left(t)), __fsub_rn(left(BR), left(BL)));
        const float wT = __fdiv_rn(__fsub_rn(top(BL), top(t)), __fsub_rn(top(BL), top(TL)));
        const float wB = __fdiv_rn(__fsub_rn(top(t), top(TL)), __fsub_rn(top(BL), top(TL)));
        uV[2] = __fadd_rn(__fmul_rn(wT, __fadd_rn(__fmul_rn(wTR, p.v[TR]), __fmul_rn(wTL, p.v[TL]))),
                          __fmul_rn(wB, __fadd_rn(__fmul_rn(wBR, p.v[BR]), __fmul_rn(wBL, p.v[BL]))));
        uU[2] = __fadd_rn(__fmul_rn(wT, __fadd_rn(__fmul_rn(wTR, p.u[TR]), __fmul_rn(wTL, p.u[TL]))),
                          __fmul_rn(wB, __fadd_rn(__fmul_rn(wBR, p.u[BR]), __fmul_rn(wBL, p.u[BL]))));
        cV[2] = 3;
        cU[2] = 3;
        count++;
    } else {
        if (ok(TL) && ok(BR)) {
            uV[2] = interp_1d(left(TL), left(BR), left(t), p.v[TL], p.v[BR]);
            uU[2] = interp_1d(top(TL), top(BR), top(t), p.u[TL], p.u[BR]);
            cV[2] = 1;
            cU[2] = 1;
            count++;
        }
        if (ok(BL) && ok(TR)) {
            uV[3] = interp_1d(left(BL), left(TR), left(t), p.v[BL], p.v[TR]);
            uU[3] = interp_1d(top(TR), top(BL), top(t), p.u[TR], p.u[BL]);
            cV[3] = 1;
            cU[3] = 1;
            count++;
        }
    }
    if (count == 0) {
        // the reference's break leaves only the inner loop: each row overwrites the
        // estimate with its first valid neighbour, the last such row wins
        int pick = -1;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                if (a == 1 && b == 1) continue;
                if (ok(adj[a][b])) {
                    pick = adj[a][b];
                    break;
                }
            }
        if (pick < 0) {
            set_invalid(p, t, true);
        } else if (replace_ok(p, t, p.u[pick], p.v[pick])) {
            p.u[t] = p.u[pick];
            p.v[t] = p.v[pick];
            set_invalid(p, t, false);
        }
        return;
    }
    float aV = 0.0f, aU = 0.0f;
    int wV = 0, wU = 0;
    for (int q = 0; q < 4; q++) {
        aV = __fadd_rn(aV, __fmul_rn((float)cV[q], uV[q]));
        wV += cV[q];
        aU = __fadd_rn(aU, __fmul_rn((float)cU[q], uU[q]));
        wU += cU[q];
    }
    const float nu = __fdiv_rn(aU, (float)wU), nv = __fdiv_rn(aV, (float)wV);
    if (replace_ok(p, t, nu, nv)) {
        p.u[t] = nu;
        p.v[t] = nv;
    }
    set_invalid(p, t, false);  // cleared whether or not the value was taken, as the reference does
}

// The validator visit of one open tile in a correction sweep; true if it was corrected.
// Strategies: multi-peak model k (secondary peaks 1..k-1, then bilinear), otherwise one
// (bilinear or no replacement).  Only a strategy with a replacement restores the backup first.
__device__ bool visit_open_tile(const PairView &p, int t, float threshold, float eps0) {
    const bool multi = p.model == QLPIV_VALIDATE_MULTIPEAK_MEDIAN;
    const int nstrat = multi ? p.k : 1;
    const bool last_bilinear = multi || p.model == QLPIV_VALIDATE_DIFFERENCE || p.model == QLPIV_VALIDATE_MEDIAN;
    validate_vector(p, t, threshold, eps0);
    for (int s = 0; s < nstrat && is_invalid(p, t); s++) {
        const bool secondary = multi && s < nstrat - 1;
        const bool bilinear = !secondary && last_bilinear;
        if (secondary || bilinear) {
            p.u[t] = p.bu[t];  // Tile.restoreDisplacement
            p.v[t] = p.bv[t];
        }
        if (secondary) {
            const int peak = s + 1;
            if ((int)p.npk[t] > peak) {
                const float2 main = p.puv[(long)t * p.k], sec = p.puv[(long)t * p.k + peak];
                const float nu = __fadd_rn(__fsub_rn(p.u[t], main.x), sec.x);
                const float nv = __fadd_rn(__fsub_rn(p.v[t], main.y), sec.y);
                if (replace_ok(p, t, nu, nv)) {
                    p.u[t] = nu;
                    p.v[t] = nv;
                    set_invalid(p, t, false);
                }
            }
        } else if (bilinear) {
            bilinear_replace(p, t);
        }
        validate_vector(p, t, threshold, eps0);
        if (!is_invalid(p, t)) return true;
    }
    return false;
}

__device__ PairView pair_view(const ValidateBufs &b, const ValidateParams &vp, int pair) {
    const long cnt = (long)vp.ni * vp.nj, base = (long)pair * cnt;
    PairView p;
    p.ni = vp.ni;
    p.nj = vp.nj;
    p.k = vp.num_peaks;
    p.u = b.u + base;
    p.v = b.v + base;
    p.bu = b.bu + base;
    p.bv = b.bv + base;
    p.puv = b.peak_uv + base * vp.num_peaks;
    p.npk = b.npeaks + base;
    p.state = b.state + base;
    p.tops = b.tops;
    p.lefts = b.lefts;
    p.model = vp.model;
    p.clip_n = vp.clip_n;
    p.clip_h = vp.clip_h;
    p.clip_w = vp.clip_w;
    return p;
}

__global__ void validate_init_kernel(ValidateParams vp, ValidateBufs b, int pairs) {
    const long cnt = (long)vp.ni * vp.nj;
    const long total = cnt * pairs;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
        const int pair = (int)(idx / cnt), t = (int)(idx - pair * cnt);
        PairView p = pair_view(b, vp, pair);
        if (difference_model(p)) {
            // Every tile starts invalid (the Tile constructors) and the difference validator only
            // writes a flag when a top-left, top or left neighbour is valid; by induction over the
            // centre-out visit no tile becomes valid in this pass, whatever the order.
            p.state[t] = kInvalid;
        } else {
            p.state[t] = 0;
            median_validate(p, t, vp.threshold, vp.epsilon0);  // writes the flag from any state
            if (!is_invalid(p, t)) p.state[t] = kLocked;
        }
        b.bu[idx] = p.u[t];  // Tile.backupDisplacement
        b.bv[idx] = p.v[t];
        b.done[idx] = -1;
    }
}

constexpr int kSweepThreads = 512;

__global__ void __launch_bounds__(kSweepThreads) validate_sweep_kernel(ValidateParams vp, ValidateBufs b) {
    constexpr int T = kSweepThreads, NW = T / 32;
    const int pair = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int cnt = vp.ni * vp.nj;
    const PairView p = pair_view(b, vp, pair);
    int *list = b.list + (long)pair * cnt;
    int *done = b.done + (long)pair * cnt;
    __shared__ int s_warp[NW];
    __shared__ int s_count, s_corr;

    // open tiles in spiral order
    if (tid == 0) s_count = 0;
    __syncthreads();
    for (int r0 = 0; r0 < cnt; r0 += T) {
        const int r = r0 + tid;
        const int t = r < cnt ? b.order[r] : 0;
        const bool open = r < cnt && !(p.state[t] & kLocked);
        const unsigned m = __ballot_sync(0xffffffffu, open);
        if (lane == 0) s_warp[warp] = __popc(m);
        __syncthreads();
        int before = s_count;
        for (int w = 0; w < warp; w++) before += s_warp[w];
        if (open) list[before + __popc(m & ((1u << lane) - 1u))] = t;
        __syncthreads();
        if (tid == 0) {
            int add = 0;
            for (int w = 0; w < NW; w++) add += s_warp[w];
            s_count += add;
        }
        __syncthreads();
    }
    const int L = s_count;

    int sweeps = 0, round = 0;
    if (L > 0) {
        for (;;) {
            const int start = round;
            if (tid == 0) s_corr = 0;
            __syncthreads();
            for (;;) {  // rounds of this sweep
                int mine = 0;
                bool left = false;
                for (int q = tid; q < L; q += T) {
                    const int t = list[q];
                    if (done[t] >= start) continue;
                    const int ti = t / vp.nj, tj = t - ti * vp.nj;
                    const int rt = b.rank[t];
                    bool ready = true;
                    for (int a = -1; a <= 1 && ready; a++)
                        for (int c = -1; c <= 1; c++) {
                            const int i = ti + a, j = tj + c;
                            if ((a == 0 && c == 0) || i < 0 || i >= vp.ni || j < 0 || j >= vp.nj) continue;
                            const int nq = i * vp.nj + j;
                            if ((p.state[nq] & kLocked) || b.rank[nq] > rt) continue;
                            const int dn = done[nq];
                            // processed in an earlier round of this sweep (not this one)
                            if (dn < start || dn >= round) { ready = false; break; }
                        }
                    if (!ready) { left = true; continue; }
                    if (visit_open_tile(p, t, vp.threshold, vp.epsilon0)) atomicAdd(&s_corr, 1);
                    done[t] = round;
                    mine++;
                }
                const int active = __syncthreads_count(mine > 0);
                const int any_left = __syncthreads_or(left);
                round++;
                if (!any_left) break;
                if (active < 4) {
                    // a chain of adjacent open tiles: finish the sweep in spiral order
                    if (tid == 0) {
                        for (int q = 0; q < L; q++) {
                            const int t = list[q];
                            if (done[t] >= start) continue;
                            if (visit_open_tile(p, t, vp.threshold, vp.epsilon0)) s_corr++;
                            done[t] = round;
                        }
                    }
                    round++;
                    __syncthreads();
                    break;
                }
            }
            sweeps++;
            __syncthreads();
            const int corrected = s_corr;
            __syncthreads();
            if (corrected == 0) break;
            if (!vp.iterate_until_no_corrections && sweeps >= vp.max_iterations) break;
            if (sweeps >= kMaxValidationSweeps) break;  // bound for iterate-until-no-corrections
        }
        // still-invalid vectors are set to 0 (VectorValidatorJob.java:378-388, replaceDisplacement)
        for (int q = tid; q < L; q += T) {
            const int t = list[q];
            if ((p.state[t] & kInvalid) && replace_ok(p, t, 0.0f, 0.0f)) {
                p.u[t] = 0.0f;
                p.v[t] = 0.0f;
            }
        }
    } else {
        sweeps = 1;  // one sweep that found nothing to do
    }
    if (tid == 0 && b.sweeps != nullptr) b.sweeps[pair] = sweeps;
}

}  // namespace

void spiral_order(int ni, int nj, int *order) {
    // circularVisitor: rings around the centre, each visited right, down, left, up
    int start_i = ni / 2, start_j = nj / 2;
    int side_i = 2, side_j = 2;
    if (ni != start_i * 2) side_i = 1; else start_i--;
    if (nj != start_j * 2) side_j = 1; else start_j--;
    const long total = (long)ni * nj;
    long visited = 0;
    auto visit = [&](int i, int j) {
        // each in-range cell is reached exactly once: rings are disjoint
        if (i >= 0 && i < ni && j >= 0 && j < nj) order[visited++] = i * nj + j;
    };
    while (visited < total) {
        const int right = side_j > 1 ? side_j - 1 : 0;
        const int down = side_i > 1 ? side_i - 1 : 0;
        const int left = side_j > 1 ? side_j - 1 : 0;
        const int up = side_i > 2 ? side_i - 2 : 0;
        int i = start_i, j = start_j;
        visit(i, j);
        for (int o = 0; o < right; o++) visit(i, ++j);
        for (int o = 0; o < down; o++) visit(++i, j);
        if (down > 0) {
            for (int o = 0; o < left; o++) visit(i, --j);
            for (int o = 0; o < up; o++) visit(--i, j);
        }
        side_i += 2;
        side_j += 2;
        start_i--;
        start_j--;
    }
}

cudaError_t launch_validate(cudaStream_t s, int pairs, const ValidateParams &vp, const ValidateBufs &b) {
    const long total = (long)vp.ni * vp.nj * pairs;
    if (total <= 0) return cudaSuccess;
    long blocks = (total + 255) / 256;
    if (blocks > 65535L * 16) blocks = 65535L * 16;
    validate_init_kernel<<<(unsigned)blocks, 256, 0, s>>>(vp, b, pairs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    validate_sweep_kernel<<<pairs, kSweepThreads, 0, s>>>(vp, b);
    return cudaGetLastError();
}

}  // namespace qlpiv
