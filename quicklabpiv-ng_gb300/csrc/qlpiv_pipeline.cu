// Adaptive multi-pass PIV on the device (host orchestration) and the C ABI of the
// stages around the correlation: grids, velocity inheritance, displacement field,
// image warping.  Declarations and reference citations: include/qlpiv.h.
//
// Level loop (LocalPIVOpenCLGpuJob.java:188-411, SimpleStrategy): for each level L
//   tiles of L (grid)          -> host, cached in the plan
//   inheritance from L-1       -> inherit kernel (level 0: zero)
//   warp / clip                -> spline + warp kernels (BothImages), or displaced B
//                                 origins (no warping)
//   xcorr + peak + sub-pixel   -> K1, which also accumulates the increment into the
//                                 level's tile displacements
//   validation (optional)      -> multi-peak normalised-median validation and replacement
//                                 (VectorValidatorJob, qlpiv_validate.cu)
// Everything stays on the device; only the last level's displacements leave it.
#include <cuda_runtime.h>

#include <algorithm>

#include <cstring>
#include <vector>

#include "qlpiv_adaptive.h"
#include "qlpiv_dense.h"
#include "qlpiv_handle.h"
#include "qlpiv_internal.h"
#include "qlpiv_validate.h"
#include "qlpiv_xcorr.cuh"

namespace qlpiv {

struct LevelPlan {
    qlpiv_grid g{};
    std::vector<int32_t> tops, lefts;
    std::vector<double> cy, cx;      // tile centres (top + N/2 - 0.5), double
    std::vector<float2> kfy, kfx;    // their spline knot factors (double-words)
    std::vector<float> cyf, cxf;     // same, float
    DevBuf d_kfy, d_kfx, d_cyf, d_cxf;  // knot factors of the spline solves (knot_factors), float knots
    DevBuf d_fi, d_at, d_al, d_bt, d_bl;  // flattened work list, pairs x count
    DevBuf d_u, d_v;                       // tile displacements, pairs x count
    DevBuf coef;                           // 6 doubles + 2 float4 per tile and pair
    DevBuf d_rows;                         // inheritance stage 1: 2 x pairs x tiles_i x parent tiles_j
    DevBuf d_inh;                          // Direct / Area / Distance tables: tiles_i + tiles_j int2
    // validation (allocated only when the descriptor asks for it)
    DevBuf d_tops, d_lefts, d_order, d_rank;  // grid rows / columns, spiral order and rank
    DevBuf d_bu, d_bv, d_puv, d_npk, d_state, d_list, d_done, d_sweeps;
    DevBuf d_tiles, d_tmax;  // micro / mini warping: warped tiles (A then B) and their maxima
    long count() const { return (long)g.tiles_i * g.tiles_j; }
};

struct AdaptivePlan {
    qlpiv_adaptive_desc desc{};
    int pixel_type = -1, height = 0, width = 0, pairs = 0;
    std::vector<LevelPlan> levels;
    DevBuf warped;        // 2 x pairs x height x width pixels
    DevBuf warped_table;  // pairs qlpiv_frame entries
    DevBuf host_frames;   // images uploaded by qlpiv_piv_adaptive (host variant)
    DevBuf host_table;
    // optical flow after PIV: kFlowLanes pairs in flight, each lane with its own planes (FlowBufs)
    // and stream, forked from and joined back into the handle's stream
    static constexpr int kFlowLanes = 4;
    DevBuf flow[kFlowLanes];
    cudaStream_t flow_side[kFlowLanes] = {};
    cudaEvent_t flow_fork = nullptr, flow_done[kFlowLanes] = {};
    DevBuf flow_dense;    // dense field of the host variant, 2 x pairs x height x width
    DevBuf mp_batch;      // batched multi-peak replay of the correlation passes: batches,
    DevBuf mp_slots;      //   their claim bitmask (zeroed at allocation, zero between launches)
    DevBuf mp_retry;      //   and the list of IAs to run again (1 + tiles of the largest level)
    long mp_units = 0;
    DevBuf stab_list;     // tile stabilisation: two lists of 1 + stab_cap ints (EVALUATING tiles)
    DevBuf stab_vec;      //   and the increments of the last pass (stab_cap vectors)
    long stab_cap = 0;
};

void destroy_plan(AdaptivePlan *p) {
    if (!p) return;
    for (LevelPlan &l : p->levels)
        for (DevBuf *b : {&l.d_kfy, &l.d_kfx, &l.d_cyf, &l.d_cxf, &l.d_fi, &l.d_at, &l.d_al, &l.d_bt,
                          &l.d_bl, &l.d_u, &l.d_v, &l.coef, &l.d_rows, &l.d_inh, &l.d_tops, &l.d_lefts, &l.d_order,
                          &l.d_rank, &l.d_bu, &l.d_bv, &l.d_puv, &l.d_npk, &l.d_state, &l.d_list, &l.d_done,
                          &l.d_sweeps, &l.d_tiles, &l.d_tmax})
            b->release();
    for (DevBuf *b : {&p->warped, &p->warped_table, &p->host_frames, &p->host_table, &p->flow_dense,
                      &p->mp_batch, &p->mp_slots, &p->mp_retry, &p->stab_list, &p->stab_vec})
        b->release();
    for (int k = 0; k < AdaptivePlan::kFlowLanes; k++) {
        p->flow[k].release();
        if (p->flow_side[k]) cudaStreamDestroy(p->flow_side[k]);
        if (p->flow_done[k]) cudaEventDestroy(p->flow_done[k]);
    }
    if (p->flow_fork) cudaEventDestroy(p->flow_fork);
    delete p;
}


static float full_scale(int pixel_type) { return pixel_type == QLPIV_PIX_U8 ? 255.0f : 65535.0f; }

// Micro / mini per-tile warping modes: image mode (1 first, 2 second, 3 both) and mini flag.
static bool per_tile_warp(int m) { return m >= QLPIV_WARP_FIRST_MICRO && m <= QLPIV_WARP_BOTH_MINI; }
// Full-image bilinear warping (BiLinearImageWarpingStrategy): image mode 1 first, 2 second, 3 both.
static bool full_warp(int m) { return m >= QLPIV_WARP_BOTH_BILINEAR && m <= QLPIV_WARP_SECOND_BILINEAR; }
static int full_image_mode(int m) {
    return m == QLPIV_WARP_BOTH_BILINEAR ? 3 : (m == QLPIV_WARP_FIRST_BILINEAR ? 1 : 2);
}
static int tile_image_mode(int m) { return (m - QLPIV_WARP_FIRST_MICRO) % 3 + 1; }
// The correlation passes replay their multi-peak lists in batches (mp_batched).
static bool batched_replay(const qlpiv_adaptive_desc &d) {
    return d.validation == QLPIV_VALIDATE_MULTIPEAK_MEDIAN && d.num_peaks >= 1 && d.num_peaks <= 4 &&
           (d.subpix_mode == QLPIV_SUBPIX_NONE || d.subpix_mode == QLPIV_SUBPIX_GAUSS3);
}
static bool tile_mini(int m) { return m >= QLPIV_WARP_FIRST_MINI; }

static qlpiv_status check_adaptive(const qlpiv_adaptive_desc *d, int pixel_type, int height, int width) {
    if (!d) return fail(QLPIV_E_ARG, "adaptive descriptor is NULL");
    if (pixel_type != QLPIV_PIX_U8 && pixel_type != QLPIV_PIX_U16)
        return fail(QLPIV_E_ARG, "adaptive PIV takes u8 or u16 images");
    if (height <= 0 || width <= 0) return fail(QLPIV_E_SHAPE, "image size %d x %d", height, width);
    if (d->ia_end <= 0 || d->ia_start < d->ia_end || d->ia_start % d->ia_end != 0)
        return fail(QLPIV_E_ARG, "IA start %d must be a multiple of IA end %d", d->ia_start, d->ia_end);
    int r = d->ia_start / d->ia_end;
    if ((r & (r - 1)) != 0) return fail(QLPIV_E_ARG, "IA start / end ratio is not a power of two");
    for (int n = d->ia_start; n >= d->ia_end; n >>= 1)
        if (!xcorr_size_supported(n)) return fail(QLPIV_E_SHAPE, "IA size %d is not supported (16, 32, 64, 128)", n);
    if (d->warp_mode != QLPIV_WARP_NONE && !full_warp(d->warp_mode) && !per_tile_warp(d->warp_mode))
        return fail(QLPIV_E_ARG, "unknown warp mode %d", d->warp_mode);
    if (d->norm_mode != QLPIV_NORM_MAX_A && d->norm_mode != QLPIV_NORM_OWN_MAX && d->norm_mode != QLPIV_NORM_NONE)
        return fail(QLPIV_E_ARG, "unknown normalisation mode %d", d->norm_mode);
    if (d->max_mode != QLPIV_MAX_COMPUTE && d->max_mode != QLPIV_MAX_FIXED)
        return fail(QLPIV_E_ARG, "max mode %d not valid for adaptive PIV", d->max_mode);
    if (qlpiv_status st = check_subpix(d->subpix_mode, d->subpix_pixels, d->subpix_iterations)) return st;
    if (d->inherit_mode < QLPIV_INHERIT_BICUBIC_SPLINE || d->inherit_mode > QLPIV_INHERIT_DISTANCE)
        return fail(QLPIV_E_ARG, "unknown velocity inheritance mode %d", d->inherit_mode);
    if (!(d->overlap_factor >= 0.1f && d->overlap_factor <= 0.9f))
        return fail(QLPIV_E_ARG, "Overlap factor must greater than 1/10 and less than 9/10");
    if (d->validation < QLPIV_VALIDATE_NONE || d->validation > QLPIV_VALIDATE_MEDIAN)
        return fail(QLPIV_E_ARG, "unknown validation mode %d", d->validation);
    if (d->clipping_mode < QLPIV_CLIP_ALLOWED || d->clipping_mode > QLPIV_CLIP_NO_OUT_OF_BOUND)
        return fail(QLPIV_E_ARG, "unknown clipping mode %d", d->clipping_mode);
    if (d->superposition_start < 0) return fail(QLPIV_E_ARG, "superposition start level %d < 0", d->superposition_start);
    if (d->stable_mode != QLPIV_STABLE_SIMPLE && d->stable_mode != QLPIV_STABLE_MAX_DISPLACEMENT)
        return fail(QLPIV_E_ARG, "unknown tile stabilisation mode %d", d->stable_mode);
    if (d->stable_mode == QLPIV_STABLE_MAX_DISPLACEMENT) {
        if (d->stable_max_retries < 1 || !(d->stable_max_displacement >= 0.0f))
            return fail(QLPIV_E_ARG, "stabilisation needs max retries >= 1 and a maximum displacement >= 0");
        if (d->validation != QLPIV_VALIDATE_NONE)
            return fail(QLPIV_E_ARG, "tile stabilisation with vector validation is not supported");
        if (per_tile_warp(d->warp_mode))
            return fail(QLPIV_E_ARG, "tile stabilisation with micro / mini warping is not supported");
    }
    if (d->validation == QLPIV_VALIDATE_MULTIPEAK_MEDIAN) {
        for (int n = d->ia_start; n >= d->ia_end; n >>= 1)
            if (!multipeak_supported(n, d->num_peaks, d->peak_kernel))
                return fail(QLPIV_E_ARG, "multi-peak search: %d peaks with cell width %d not supported for IA %d "
                            "(1..%d peaks, cell width >= 2)", d->num_peaks, d->peak_kernel, n, QLPIV_MAX_PEAKS);
    }
    if (d->validation != QLPIV_VALIDATE_NONE) {
        if (!(d->median_threshold > 0.0f) || !(d->median_epsilon0 >= 0.0f))
            return fail(QLPIV_E_ARG, "validation threshold must be > 0 and epsilon0 >= 0");
        if (d->max_correction_iterations < 0) return fail(QLPIV_E_ARG, "max correction iterations < 0");
    }
    return QLPIV_OK;
}

// Strategies of the validation model: the multi-peak model k, every other model one.
static int validation_strategies(const qlpiv_adaptive_desc &d) {
    return d.validation == QLPIV_VALIDATE_MULTIPEAK_MEDIAN ? d.num_peaks : 1;
}

// Per child row and per child column tables of the Direct / Area / Distance inheritance
// (cni row entries, then cnj column entries; Direct needs none).  The reference's serial walk
// keeps a parent reference row across child rows and a reference column that restarts at 0 on
// every child row; on separable grids both advance independently:
//   Area      (first, last) parent index overlapping the child span.  The walk moves the
//             reference by one parent per child tile before scanning, and throws when one move
//             is not enough, when the child lies before the reference, or when a row move and a
//             column move fall on the same tile (Area.java:76-104, 121-131).
//   Distance  (p, past): p the last parent whose centre is at or before the child centre (0
//             when none is, the last parent at most), past = the centre of parent p lies after
//             the child centre (DistanceGeneric.java:77-166, 168-176).
static qlpiv_status inherit_tables(int mode, int pn, int pni, int pnj, const int32_t *ptops, const int32_t *plefts,
                                   int cn, int cni, int cnj, const int32_t *ctops, const int32_t *clefts,
                                   std::vector<int2> &tab) {
    tab.assign((size_t)cni + cnj, make_int2(0, 0));
    if (mode == QLPIV_INHERIT_DIRECT) {
        if (cni < 2 * pni || cnj < 2 * pnj)
            return fail(QLPIV_E_SHAPE, "Direct inheritance needs at least 2 x %d by 2 x %d child tiles, got %d x %d",
                        pni, pnj, cni, cnj);
        return QLPIV_OK;
    }
    if (mode == QLPIV_INHERIT_AREA) {
        // relation of a parent span to a child span: 0 overlap, +1 parent before, -1 parent after
        auto rel = [&](int p, int c) { return span_overlap(p, pn, c, cn) > 0 ? 0 : (p <= c ? 1 : -1); };
        bool row_moved = false, col0_moved = false;
        for (int axis = 0; axis < 2; axis++) {
            const int np = axis == 0 ? pni : pnj, nc = axis == 0 ? cni : cnj;
            const int32_t *ps = axis == 0 ? ptops : plefts, *cs = axis == 0 ? ctops : clefts;
            int ref = 0;
            for (int k = 0; k < nc; k++) {
                int r = rel(ps[ref], cs[k]);
                if (r < 0) return fail(QLPIV_E_SHAPE, "Area inheritance: child tile %d lies before its parent", k);
                if (r > 0) {
                    if (ref + 1 == np) return fail(QLPIV_E_SHAPE, "Area inheritance: no parent tile past child %d", k);
                    ref++;
                    if (axis == 0) row_moved = true;
                    else if (k == 0) col0_moved = true;
                    if (rel(ps[ref], cs[k]) != 0)
                        return fail(QLPIV_E_SHAPE, "Area inheritance: child %d skips a parent tile", k);
                }
                int last = ref;
                while (last + 1 < np && rel(ps[last + 1], cs[k]) == 0) last++;
                tab[(size_t)(axis == 0 ? k : cni + k)] = make_int2(ref, last);
            }
        }
        if (row_moved && col0_moved)
            return fail(QLPIV_E_SHAPE, "Area inheritance: reference tile moves right and down at once");
        return QLPIV_OK;
    }
    if (mode == QLPIV_INHERIT_DISTANCE) {
        const float half_p = (float)pn / 2.0f, half_c = (float)cn / 2.0f;
        for (int axis = 0; axis < 2; axis++) {
            const int np = axis == 0 ? pni : pnj, nc = axis == 0 ? cni : cnj;
            const int32_t *ps = axis == 0 ? ptops : plefts, *cs = axis == 0 ? ctops : clefts;
            int ref = 0;
            for (int k = 0; k < nc; k++) {
                const float c = (float)cs[k] + half_c;
                while (ref + 1 < np && (float)ps[ref + 1] + half_p <= c) ref++;
                const int past = (float)ps[ref] + half_p > c ? 1 : 0;
                tab[(size_t)(axis == 0 ? k : cni + k)] = make_int2(ref, past);
            }
        }
        return QLPIV_OK;
    }
    return fail(QLPIV_E_ARG, "inheritance mode %d has no tables", mode);
}

// Spiral visit order of a grid and the rank of every tile in it.
static void spiral_rank(int ni, int nj, std::vector<int32_t> &order, std::vector<int32_t> &rank) {
    const long cnt = (long)ni * nj;
    order.resize(cnt);
    rank.resize(cnt);
    spiral_order(ni, nj, order.data());
    for (long r = 0; r < cnt; r++) rank[order[r]] = (int32_t)r;
}

static int level_count(const qlpiv_adaptive_desc *d) {
    int k = 0;
    for (int n = d->ia_start; n >= d->ia_end; n >>= 1) k++;
    return k;
}

static cudaError_t upload(DevBuf &b, const void *src, size_t bytes, cudaStream_t s) {
    cudaError_t e = b.ensure(bytes);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, s);
}

// (Re)builds the plan for this geometry.  Host arrays uploaded here are consumed by
// the stream before the next rebuild (the caller synchronises on rebuild).
static qlpiv_status build_plan_inner(qlpiv_handle *h, const qlpiv_adaptive_desc *d, int pixel_type, int height,
                                     int width, int pairs) {
    AdaptivePlan *p = h->plan;
    if (p && p->pixel_type == pixel_type && p->height == height && p->width == width && p->pairs == pairs &&
        std::memcmp(&p->desc, d, sizeof(*d)) == 0)
        return QLPIV_OK;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "plan rebuild");
    if (p) destroy_plan(p);
    h->plan = p = new AdaptivePlan();
    p->desc = *d;
    p->pixel_type = pixel_type;
    p->height = height;
    p->width = width;
    p->pairs = pairs;
    const int nlev = level_count(d);
    p->levels.resize(nlev);
    for (int lv = 0; lv < nlev; lv++) {
        LevelPlan &L = p->levels[lv];
        if (grid_level(height, width, d->margins, d->ia_start, lv, d->overlap_factor, d->superposition_start, &L.g,
                       nullptr, nullptr, 0) < -1)
            return fail(QLPIV_E_SHAPE, "image too small for IA %d at level %d", d->ia_start >> lv, lv);
        if ((full_warp(d->warp_mode) || per_tile_warp(d->warp_mode)) && lv > 0 &&
            (L.g.tiles_i < 3 || L.g.tiles_j < 3))
            return fail(QLPIV_E_SHAPE, "level %d has %d x %d tiles: the warp spline needs at least 3 per axis", lv,
                        L.g.tiles_i, L.g.tiles_j);
        L.tops.resize(L.g.tiles_i);
        L.lefts.resize(L.g.tiles_j);
        grid_level(height, width, d->margins, d->ia_start, lv, d->overlap_factor, d->superposition_start, &L.g,
                   L.tops.data(), L.lefts.data(), 1 << 30);
        const int n = L.g.n, ni = L.g.tiles_i, nj = L.g.tiles_j;
        L.cyf.resize(ni);
        L.cxf.resize(nj);
        L.cy.resize(ni);
        L.cx.resize(nj);
        for (int i = 0; i < ni; i++) {
            L.cyf[i] = (float)L.tops[i] + (float)n / 2.0f - 0.5f;
            L.cy[i] = (double)L.cyf[i];
        }
        for (int j = 0; j < nj; j++) {
            L.cxf[j] = (float)L.lefts[j] + (float)n / 2.0f - 0.5f;
            L.cx[j] = (double)L.cxf[j];
        }
        const long cnt = L.count(), total = cnt * pairs;
        std::vector<int32_t> fi(total), at(total), al(total);
        for (int q = 0; q < pairs; q++)
            for (int i = 0; i < ni; i++)
                for (int j = 0; j < nj; j++) {
                    const long k = (long)q * cnt + (long)i * nj + j;
                    fi[k] = q;
                    at[k] = L.tops[i];
                    al[k] = L.lefts[j];
                }
        cudaStream_t s = h->stream;
        L.kfy.resize((size_t)KF_ARRAYS * ni);
        L.kfx.resize((size_t)KF_ARRAYS * nj);
        knot_factors_dw(L.cy.data(), ni, L.kfy.data());
        knot_factors_dw(L.cx.data(), nj, L.kfx.data());
        if ((e = upload(L.d_kfy, L.kfy.data(), sizeof(float2) * L.kfy.size(), s)) != cudaSuccess ||
            (e = upload(L.d_kfx, L.kfx.data(), sizeof(float2) * L.kfx.size(), s)) != cudaSuccess ||
            (e = upload(L.d_cyf, L.cyf.data(), sizeof(float) * ni, s)) != cudaSuccess ||
            (e = upload(L.d_cxf, L.cxf.data(), sizeof(float) * nj, s)) != cudaSuccess ||
            (e = upload(L.d_fi, fi.data(), sizeof(int32_t) * total, s)) != cudaSuccess ||
            (e = upload(L.d_at, at.data(), sizeof(int32_t) * total, s)) != cudaSuccess ||
            (e = upload(L.d_al, al.data(), sizeof(int32_t) * total, s)) != cudaSuccess ||
            (e = L.d_bt.ensure(sizeof(int32_t) * total)) != cudaSuccess ||
            (e = L.d_bl.ensure(sizeof(int32_t) * total)) != cudaSuccess ||
            (e = L.d_u.ensure(sizeof(float) * total)) != cudaSuccess ||
            (e = L.d_v.ensure(sizeof(float) * total)) != cudaSuccess ||
            (e = L.coef.ensure(spline_coef_bytes(total))) != cudaSuccess ||
            (lv > 0 && (e = L.d_rows.ensure(sizeof(float) * 2 * (long)pairs * ni *
                                            p->levels[lv - 1].g.tiles_j)) != cudaSuccess))
            return cuda_fail(e, "adaptive plan");
        if ((e = upload(L.d_tops, L.tops.data(), sizeof(int32_t) * ni, s)) != cudaSuccess ||
            (e = upload(L.d_lefts, L.lefts.data(), sizeof(int32_t) * nj, s)) != cudaSuccess)
            return cuda_fail(e, "grid upload");
        std::vector<int2> inh;
        if (lv > 0 && d->inherit_mode != QLPIV_INHERIT_BICUBIC_SPLINE) {
            const LevelPlan &P = p->levels[lv - 1];
            if (qlpiv_status st = inherit_tables(d->inherit_mode, P.g.n, P.g.tiles_i, P.g.tiles_j, P.tops.data(),
                                                 P.lefts.data(), n, ni, nj, L.tops.data(), L.lefts.data(), inh))
                return st;
            if ((e = upload(L.d_inh, inh.data(), sizeof(int2) * inh.size(), s)) != cudaSuccess)
                return cuda_fail(e, "inheritance tables");
        }
        std::vector<int32_t> order, rank;
        if (d->validation != QLPIV_VALIDATE_NONE) {
            spiral_rank(ni, nj, order, rank);
            const long k = validation_strategies(*d);
            if ((e = upload(L.d_order, order.data(), sizeof(int32_t) * cnt, s)) != cudaSuccess ||
                (e = upload(L.d_rank, rank.data(), sizeof(int32_t) * cnt, s)) != cudaSuccess ||
                (e = L.d_bu.ensure(sizeof(float) * total)) != cudaSuccess ||
                (e = L.d_bv.ensure(sizeof(float) * total)) != cudaSuccess ||
                (e = L.d_puv.ensure(sizeof(float2) * total * k)) != cudaSuccess ||
                (e = L.d_npk.ensure(total)) != cudaSuccess || (e = L.d_state.ensure(total)) != cudaSuccess ||
                (e = L.d_list.ensure(sizeof(int32_t) * total)) != cudaSuccess ||
                (e = L.d_done.ensure(sizeof(int32_t) * total)) != cudaSuccess ||
                (e = L.d_sweeps.ensure(sizeof(int32_t) * pairs)) != cudaSuccess)
                return cuda_fail(e, "validation buffers");
        }
        if (per_tile_warp(d->warp_mode) && lv > 0) {
            const size_t tb = (size_t)total * n * n * pixel_bytes(pixel_type);
            if ((e = L.d_tiles.ensure(2 * tb)) != cudaSuccess ||
                (e = L.d_tmax.ensure(sizeof(float) * 2 * total)) != cudaSuccess)
                return cuda_fail(e, "warped tile buffers");
        }
        // the host vectors above die at scope exit: make the copies complete first
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "adaptive plan upload");
    }
    if (d->stable_mode == QLPIV_STABLE_MAX_DISPLACEMENT && d->stable_max_retries > 1) {
        long most = 0;
        for (const LevelPlan &l : p->levels) most = l.count() * pairs > most ? l.count() * pairs : most;
        if ((e = p->stab_list.ensure(sizeof(int) * 2 * (size_t)(1 + most))) != cudaSuccess ||
            (e = p->stab_vec.ensure(sizeof(qlpiv_vector) * (size_t)most)) != cudaSuccess)
            return cuda_fail(e, "stabilisation buffers");
        p->stab_cap = most;
    }
    if (batched_replay(*d)) {
        long units = 0, most = 0;
        for (const LevelPlan &l : p->levels) most = l.count() * pairs > most ? l.count() * pairs : most;
        const size_t batch_bytes = xcorr_batch_bytes(h->num_sms, &units);
        const size_t slot_bytes = xcorr_batch_slot_bytes(units);
        if ((e = p->mp_batch.ensure(batch_bytes)) != cudaSuccess ||
            (e = p->mp_slots.ensure(slot_bytes)) != cudaSuccess ||
            (e = cudaMemsetAsync(p->mp_slots.p, 0, slot_bytes, h->stream)) != cudaSuccess ||
            (e = p->mp_retry.ensure(sizeof(int) * (size_t)(1 + most))) != cudaSuccess)
            return cuda_fail(e, "multi-peak batch buffers");
        p->mp_units = units;
    }
    if (full_warp(d->warp_mode)) {
        const size_t img = (size_t)height * width * pixel_bytes(pixel_type);
        const size_t stride = (img + 255) & ~(size_t)255;
        if ((e = p->warped.ensure(2 * stride * pairs)) != cudaSuccess ||
            (e = p->warped_table.ensure(sizeof(qlpiv_frame) * pairs)) != cudaSuccess)
            return cuda_fail(e, "warp buffers");
        std::vector<qlpiv_frame> t(pairs);
        char *base = p->warped.as<char>();
        for (int q = 0; q < pairs; q++)
            t[q] = {base + 2 * q * stride, base + (2 * q + 1) * stride, height, width, (int64_t)width};
        if ((e = cudaMemcpyAsync(p->warped_table.p, t.data(), sizeof(qlpiv_frame) * pairs, cudaMemcpyHostToDevice,
                                 h->stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(h->stream)) != cudaSuccess)
            return cuda_fail(e, "warp table");
    }
    return QLPIV_OK;
}

static qlpiv_status build_plan(qlpiv_handle *h, const qlpiv_adaptive_desc *d, int pixel_type, int height, int width,
                               int pairs) {
    qlpiv_status st = build_plan_inner(h, d, pixel_type, height, width, pairs);
    if (st != QLPIV_OK && h->plan) {  // never leave a half-built plan behind
        destroy_plan(h->plan);
        h->plan = nullptr;
    }
    return st;
}

// Stage timing: events recorded around a stage's launches when profiling is on.
struct StageScope {
    qlpiv_handle *h;
    StageEvent ev{};
    bool on;
    StageScope(qlpiv_handle *h_, const char *stage, int level, int ia_side, long launches, long items)
        : h(h_), on(h_->profiling) {
        if (!on) return;
        ev.stage = stage;
        ev.level = level;
        ev.ia_side = ia_side;
        ev.launches = launches;
        ev.items = items;
        if (cudaEventCreate(&ev.begin) != cudaSuccess || cudaEventCreate(&ev.end) != cudaSuccess) {
            on = false;
            return;
        }
        cudaEventRecord(ev.begin, h->stream);
    }
    ~StageScope() {
        if (!on) return;
        cudaEventRecord(ev.end, h->stream);
        h->prof_pending.push_back(ev);
    }
};

static SplineCoef coef_of(LevelPlan &L, int pairs) { return spline_coef_at(L.coef.p, L.count() * pairs); }

// Queues the whole level loop; the last level's displacements end in levels.back().d_u/d_v.
static qlpiv_status run_levels(qlpiv_handle *h, const qlpiv_frame *frames_dev) {
    AdaptivePlan *p = h->plan;
    const qlpiv_adaptive_desc &d = p->desc;
    cudaStream_t s = h->stream;
    cudaError_t e;
    const int pairs = p->pairs;
    const float fm = d.fixed_max > 0.0f ? d.fixed_max : full_scale(p->pixel_type);
    for (size_t lv = 0; lv < p->levels.size(); lv++) {
        LevelPlan &L = p->levels[lv];
        const long total = L.count() * pairs;
        float *u = L.d_u.as<float>(), *v = L.d_v.as<float>();
        if (lv == 0) {
            if ((e = cudaMemsetAsync(u, 0, sizeof(float) * total, s)) != cudaSuccess ||
                (e = cudaMemsetAsync(v, 0, sizeof(float) * total, s)) != cudaSuccess)
                return cuda_fail(e, "level 0 reset");
        } else {
            LevelPlan &P = p->levels[lv - 1];
            const bool spline = d.inherit_mode == QLPIV_INHERIT_BICUBIC_SPLINE;
            StageScope sc(h, "inherit", (int)lv, L.g.n, spline ? 2 : 1, total);
            float *ru = L.d_rows.as<float>(), *rv = ru + (long)pairs * L.g.tiles_i * P.g.tiles_j;
            if (spline)
                e = launch_inherit(s, pairs, P.d_cyf.as<float>(), P.g.tiles_i, P.d_cxf.as<float>(), P.g.tiles_j,
                                   P.d_u.as<float>(), P.d_v.as<float>(), L.d_cyf.as<float>(), L.g.tiles_i,
                                   L.d_cxf.as<float>(), L.g.tiles_j, d.warp_mode == QLPIV_WARP_NONE, ru, rv, u, v);
            else
                e = launch_inherit_tiles(s, pairs, d.inherit_mode, P.g.n, P.g.tiles_i, P.g.tiles_j, P.d_tops.as<int>(),
                                         P.d_lefts.as<int>(), P.d_u.as<float>(), P.d_v.as<float>(), L.g.n,
                                         L.g.tiles_i, L.g.tiles_j, L.d_tops.as<int>(), L.d_lefts.as<int>(),
                                         L.d_inh.as<int2>(), d.warp_mode == QLPIV_WARP_NONE, u, v);
            if (e != cudaSuccess) return cuda_fail(e, "inheritance");
            h->launches += spline ? 2 : 1;
            if (d.clipping_mode == QLPIV_CLIP_NO_OUT_OF_BOUND) {
                // the child tiles take the inherited value through Tile.accumulateDisplacement
                if ((e = launch_clip_inherited(s, total, L.d_at.as<int>(), L.d_al.as<int>(), L.g.n, p->height,
                                               p->width, u, v)) != cudaSuccess)
                    return cuda_fail(e, "inheritance clipping");
                h->launches++;
            }
        }
        // tile stabilisation: pass r of the level (InterAreaDisplacementStableStrategy repeats the
        // warp and the correlation of the tiles still EVALUATING, listed on the device; a pass
        // whose list is empty does nothing)
        const bool stab = d.stable_mode == QLPIV_STABLE_MAX_DISPLACEMENT && d.stable_max_retries > 1;
        const int passes = stab ? d.stable_max_retries : 1;
        int *lists[2] = {p->stab_list.as<int>(), p->stab_list.as<int>() + 1 + p->stab_cap};
        const bool validate = d.validation != QLPIV_VALIDATE_NONE;
        for (int pass = 1; pass <= passes; pass++) {
            const int *list = pass == 1 ? nullptr : lists[pass & 1];  // EVALUATING tiles after pass - 1
            const qlpiv_frame *src = frames_dev;
            const int *bt = L.d_at.as<int>(), *bl = L.d_al.as<int>();
            const bool tiles = per_tile_warp(d.warp_mode) && lv > 0;
            if (tiles) {
                StageScope sc(h, "tile-warp", (int)lv, L.g.n, 1, total);
                const size_t tb = (size_t)total * L.g.n * L.g.n * pixel_bytes(p->pixel_type);
                char *ta = L.d_tiles.as<char>();
                float *mx = L.d_tmax.as<float>();
                if ((e = launch_tile_warp(s, p->pixel_type, pairs, frames_dev, L.g.n, L.g.tiles_i, L.g.tiles_j,
                                          L.d_tops.as<int>(), L.d_lefts.as<int>(), u, v, tile_image_mode(d.warp_mode),
                                          tile_mini(d.warp_mode), fm, ta, ta + tb, mx, mx + total)) != cudaSuccess)
                    return cuda_fail(e, "tile warp");
                h->launches++;
            } else if (per_tile_warp(d.warp_mode)) {
                // level 0: both tiles clipped at the grid (the displacements are zero)
            } else if (full_warp(d.warp_mode)) {
                if (lv > 0) {  // no warping at the first level: displacements are all zero
                    SplineCoef c = coef_of(L, pairs);
                    {
                        StageScope sc(h, "spline", (int)lv, L.g.n, 1, total);
                        if ((e = launch_spline(s, pairs, L.d_kfy.as<float2>(), L.g.tiles_i, L.d_kfx.as<float2>(),
                                               L.g.tiles_j, u, v, c, list)) != cudaSuccess)
                            return cuda_fail(e, "spline");
                    }
                    {
                        StageScope sc(h, "warp", (int)lv, L.g.n, 1, (long)pairs * p->height * p->width);
                        if ((e = launch_warp(s, p->pixel_type, pairs, p->height, p->width, frames_dev,
                                             p->warped_table.as<qlpiv_frame>(), L.d_cyf.as<float>(), L.g.tiles_i,
                                             L.d_cxf.as<float>(), L.g.tiles_j, c, d.int16_warp_quirk,
                                             full_image_mode(d.warp_mode), list)) != cudaSuccess)
                            return cuda_fail(e, "warp");
                    }
                    h->launches += 2;
                    src = p->warped_table.as<qlpiv_frame>();
                }
            } else {
                StageScope sc(h, "origins", (int)lv, L.g.n, 1, total);
                if ((e = launch_displaced_origins(s, total, L.d_at.as<int>(), L.d_al.as<int>(), u, v, L.d_bt.as<int>(),
                                                  L.d_bl.as<int>())) != cudaSuccess)
                    return cuda_fail(e, "displaced origins");
                h->launches++;
                bt = L.d_bt.as<int>();
                bl = L.d_bl.as<int>();
            }
            IaJob job{};
            job.frames = src;
            job.frame_idx = L.d_fi.as<int>();
            job.num_frames = pairs;
            job.a_top = L.d_at.as<int>();
            job.a_left = L.d_al.as<int>();
            job.b_top = bt;
            job.b_left = bl;
            job.count = total;
            job.norm_mode = d.norm_mode;
            job.max_mode = d.max_mode;
            job.fixed_max_a = job.fixed_max_b = fm;
            // FirstImage / SecondImage: tiles cut from the warped (or, at level 0, the whole) frame keep
            // the fixed maximum, tiles clipped from the other frame their own (Image.clipImageMatrix)
            if (d.max_mode == QLPIV_MAX_FIXED && d.warp_mode == QLPIV_WARP_FIRST_BILINEAR) job.max_mode = QLPIV_MAX_FIXED_A;
            if (d.max_mode == QLPIV_MAX_FIXED && d.warp_mode == QLPIV_WARP_SECOND_BILINEAR) job.max_mode = QLPIV_MAX_FIXED_B;
            if (per_tile_warp(d.warp_mode)) {
                job.max_mode = QLPIV_MAX_COMPUTE;  // level 0: clipped tiles
                if (tiles) {  // the warped tiles, contiguous, with their maxima
                    const size_t tb = (size_t)total * L.g.n * L.g.n * pixel_bytes(p->pixel_type);
                    job.frames = nullptr;
                    job.frame_idx = nullptr;
                    job.img_a = L.d_tiles.p;
                    job.img_b = L.d_tiles.as<char>() + tb;
                    job.pitch_a = job.pitch_b = L.g.n;
                    job.h = (int)(total * L.g.n);
                    job.w = L.g.n;
                    job.a_top = job.a_left = job.b_top = job.b_left = nullptr;
                    job.max_mode = QLPIV_MAX_GIVEN;
                    job.max_a = L.d_tmax.as<float>();
                    job.max_b = L.d_tmax.as<float>() + total;
                }
            }
            job.subpix = d.subpix_mode;
            job.subpix_pixels = d.subpix_mode >= QLPIV_SUBPIX_GAUSS_LM ? d.subpix_pixels : 0;
            job.subpix_iters = d.subpix_iterations;
            job.acc_u = u;
            job.acc_v = v;
            if (d.clipping_mode == QLPIV_CLIP_NO_OUT_OF_BOUND) {
                job.clip_top = L.d_at.as<int>();
                job.clip_left = L.d_al.as<int>();
                job.clip_n = L.g.n;
                job.clip_h = p->height;
                job.clip_w = p->width;
            }
            if (d.validation == QLPIV_VALIDATE_MULTIPEAK_MEDIAN) {
                // the multi-peak model selects FindMaximumMultiPeaks for every level (the others keep
                // FindMaximumFromCenter)
                job.num_peaks = d.num_peaks;
                job.peak_kernel = d.peak_kernel;
                job.peak_uv = L.d_puv.as<float2>();
                job.npeaks = L.d_npk.as<uint8_t>();
                if (p->mp_units > 0) {
                    job.mp_batch = p->mp_batch.as<MpBatch>();
                    job.mp_batch_units = p->mp_units;
                    job.mp_slots = p->mp_slots.as<unsigned>();
                    job.mp_retry = p->mp_retry.as<int>();
                }
            }
            if (stab) {
                job.ia_list = list;
                job.out = p->stab_vec.as<qlpiv_vector>();
            }
            int nk = 1;
            {
                StageScope sc(h, "xcorr", (int)lv, L.g.n, 1, total);
                if ((e = launch_xcorr(job, L.g.n, p->pixel_type, s, h->num_sms, &nk)) != cudaSuccess)
                    return cuda_fail(e, "xcorr");
            }
            h->launches += nk;
            if (stab && pass < passes) {
                if ((e = launch_stable_update(s, pass, passes, d.stable_max_displacement, job.out, list, total,
                                              lists[(pass + 1) & 1])) != cudaSuccess)
                    return cuda_fail(e, "tile stabilisation");
                h->launches++;
            }
        }
        if (validate) {
            StageScope sc(h, "validate", (int)lv, L.g.n, 2, total);
            ValidateParams vp{L.g.tiles_i, L.g.tiles_j, validation_strategies(d), d.median_threshold,
                              d.median_epsilon0, d.max_correction_iterations, d.iterate_until_no_corrections,
                              d.validation, 0, 0, 0};
            if (d.clipping_mode == QLPIV_CLIP_NO_OUT_OF_BOUND) {
                vp.clip_n = L.g.n;
                vp.clip_h = p->height;
                vp.clip_w = p->width;
            }
            ValidateBufs vb{u, v, L.d_bu.as<float>(), L.d_bv.as<float>(), L.d_puv.as<float2>(),
                            L.d_npk.as<uint8_t>(), L.d_state.as<uint8_t>(), L.d_tops.as<int>(), L.d_lefts.as<int>(),
                            L.d_order.as<int>(), L.d_rank.as<int>(), L.d_list.as<int>(), L.d_done.as<int>(),
                            L.d_sweeps.as<int>()};
            if ((e = launch_validate(s, pairs, vp, vb)) != cudaSuccess) return cuda_fail(e, "validation");
            h->launches += 2;
        }
    }
    return QLPIV_OK;
}

static qlpiv_status check_host_frames(const qlpiv_frame *frames, int num_pairs, int height, int width) {
    for (int q = 0; q < num_pairs; q++)
        if (!frames[q].img_a || !frames[q].img_b || frames[q].height != height || frames[q].width != width ||
            frames[q].pitch < width)
            return fail(QLPIV_E_SHAPE, "frame %d: NULL image or size differs from %d x %d", q, height, width);
    return QLPIV_OK;
}

// Copies host frame pairs into the plan's frame buffers (packed rows) and their table; the
// table's host staging is kept in `t` until the caller synchronises.
static qlpiv_status upload_host_frames(qlpiv_handle *h, const qlpiv_frame *frames, std::vector<qlpiv_frame> &t) {
    AdaptivePlan *p = h->plan;
    cudaStream_t s = h->stream;
    const int num_pairs = p->pairs, height = p->height, width = p->width;
    const size_t pb = pixel_bytes(p->pixel_type), row = (size_t)width * pb, img = row * height;
    const size_t stride = (img + 255) & ~(size_t)255;
    cudaError_t e;
    if ((e = p->host_frames.ensure(2 * stride * num_pairs)) != cudaSuccess ||
        (e = p->host_table.ensure(sizeof(qlpiv_frame) * num_pairs)) != cudaSuccess)
        return cuda_fail(e, "frame buffers");
    t.resize(num_pairs);
    char *base = p->host_frames.as<char>();
    // rows packed in the host image (pitch == width): one linear copy per image
    auto upload = [&](char *d, const void *src, size_t spitch) {
        return spitch == row ? cudaMemcpyAsync(d, src, img, cudaMemcpyHostToDevice, s)
                             : cudaMemcpy2DAsync(d, row, src, spitch, row, height, cudaMemcpyHostToDevice, s);
    };
    for (int q = 0; q < num_pairs; q++) {
        char *da = base + 2 * q * stride, *db = base + (2 * q + 1) * stride;
        const size_t spitch = (size_t)frames[q].pitch * pb;
        if ((e = upload(da, frames[q].img_a, spitch)) != cudaSuccess ||
            (e = upload(db, frames[q].img_b, spitch)) != cudaSuccess)
            return cuda_fail(e, "frame upload");
        t[q] = {da, db, height, width, (int64_t)width};
    }
    if ((e = cudaMemcpyAsync(p->host_table.p, t.data(), sizeof(qlpiv_frame) * num_pairs, cudaMemcpyHostToDevice,
                             s)) != cudaSuccess)
        return cuda_fail(e, "frame table upload");
    return QLPIV_OK;
}

// Device bytes the adaptive plan of `pairs` pairs allocates (the buffers of build_plan_inner, each
// rounded to 256 B) plus the device copies of host frames: the request server's admission estimate.
size_t plan_device_bytes(const qlpiv_adaptive_desc *d, int pixel_type, int height, int width, int pairs) {
    auto al = [](size_t x) { return ((x < 256 ? 256 : x) + 255) & ~(size_t)255; };
    size_t total = 0, most = 0;
    const int nlev = level_count(d);
    int prev_nj = 0;
    for (int lv = 0; lv < nlev; lv++) {
        qlpiv_grid g{};
        if (grid_level(height, width, d->margins, d->ia_start, lv, d->overlap_factor, d->superposition_start, &g,
                       nullptr, nullptr, 0) < -1)
            return 0;
        most = (size_t)g.tiles_i * g.tiles_j * pairs > most ? (size_t)g.tiles_i * g.tiles_j * pairs : most;
        const size_t ni = g.tiles_i, nj = g.tiles_j, cnt = ni * nj, tot = cnt * pairs;
        total += al(8 * KF_ARRAYS * ni) + al(8 * KF_ARRAYS * nj) + al(4 * ni) + al(4 * nj);
        total += 5 * al(4 * tot) + 2 * al(4 * tot) + al(spline_coef_bytes((long)tot));
        if (lv > 0) total += al(8 * (size_t)pairs * ni * prev_nj);
        if (lv > 0 && d->inherit_mode != QLPIV_INHERIT_BICUBIC_SPLINE) total += al(8 * (ni + nj));
        total += al(4 * ni) + al(4 * nj);
        if (per_tile_warp(d->warp_mode) && lv > 0)
            total += al(2 * tot * g.n * g.n * pixel_bytes(pixel_type)) + al(8 * tot);
        if (d->validation != QLPIV_VALIDATE_NONE) {
            const size_t k = validation_strategies(*d);
            total += 2 * al(4 * cnt) + 2 * al(4 * tot) + al(8 * tot * k) + 2 * al(tot) + 2 * al(4 * tot) +
                     al(4 * (size_t)pairs);
        }
        prev_nj = (int)nj;
    }
    const size_t img = (size_t)height * width * pixel_bytes(pixel_type);
    const size_t stride = (img + 255) & ~(size_t)255;
    total += al(2 * stride * pairs) + al(sizeof(qlpiv_frame) * pairs);  // frames copied from the host
    if (full_warp(d->warp_mode)) total += al(2 * stride * pairs) + al(sizeof(qlpiv_frame) * pairs);
    if (d->stable_mode == QLPIV_STABLE_MAX_DISPLACEMENT && d->stable_max_retries > 1)
        total += al(sizeof(int) * 2 * (1 + most)) + al(sizeof(qlpiv_vector) * most);
    if (batched_replay(*d)) {
        int dev = 0, sms = 0;
        long units = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
            total += al(xcorr_batch_bytes(sms, &units)) + al(xcorr_batch_slot_bytes(units));
        total += al(sizeof(int) * (1 + most));
    }
    return total;
}

// Queues one host frame pair (pinned memory, rows of `pitch` elements) through the adaptive loop
// on the handle's stream and the last level's displacements into pinned out_u / out_v; does not
// wait.  The frames and the results stay valid until the stream passes this point.
qlpiv_status queue_adaptive_pinned(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int pixel_type, int height,
                                   int width, const void *img_a, const void *img_b, long pitch, float *out_u,
                                   float *out_v) {
    qlpiv_status st = check_adaptive(desc, pixel_type, height, width);
    if (st != QLPIV_OK) return st;
    if ((st = build_plan(h, desc, pixel_type, height, width, 1)) != QLPIV_OK) return st;
    qlpiv_frame f{img_a, img_b, height, width, (int64_t)pitch};
    std::vector<qlpiv_frame> t;
    if ((st = upload_host_frames(h, &f, t)) != QLPIV_OK) return st;
    if ((st = run_levels(h, h->plan->host_table.as<qlpiv_frame>())) != QLPIV_OK) return st;
    LevelPlan &L = h->plan->levels.back();
    const size_t bytes = sizeof(float) * L.count();
    cudaError_t e;
    if ((e = cudaMemcpyAsync(out_u, L.d_u.p, bytes, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(out_v, L.d_v.p, bytes, cudaMemcpyDeviceToHost, h->stream)) != cudaSuccess)
        return cuda_fail(e, "result download");
    return QLPIV_OK;
}

// Releases the handle's cached adaptive plan (its device memory) after the stream drains.
void drop_plan(qlpiv_handle *h) {
    if (!h->plan) return;
    cudaStreamSynchronize(h->stream);
    destroy_plan(h->plan);
    h->plan = nullptr;
}

}  // namespace qlpiv

using namespace qlpiv;

extern "C" {

qlpiv_status qlpiv_grid_superposition(int height, int width, const int margins[4], int ia_start, int level,
                                      float overlap_factor, qlpiv_grid *grid, int32_t *tops, int32_t *lefts,
                                      int cap) {
    if (!grid || !margins) return fail(QLPIV_E_ARG, "NULL argument");
    const int r = qlpiv::grid_superposition(height, width, margins, ia_start, level, overlap_factor, grid, tops, lefts,
                                            cap);
    if (r == -2) return fail(QLPIV_E_ARG, "Overlap factor must greater than 1/10 and less than 9/10");
    if (r == -3) return fail(QLPIV_E_SHAPE, "no IA of size %d fits the image", ia_start >> level);
    if (r == -1) return fail(QLPIV_E_SHAPE, "grid larger than the given capacity %d", cap);
    return QLPIV_OK;
}

qlpiv_status qlpiv_grid_nosuperposition(int height, int width, const int margins[4], int ia_start, int level,
                                        qlpiv_grid *grid, int32_t *tops, int32_t *lefts, int cap) {
    if (!grid || !margins) return fail(QLPIV_E_ARG, "NULL argument");
    const int r = qlpiv::grid_nosuperposition(height, width, margins, ia_start, level, grid, tops, lefts, cap);
    if (r == -3) return fail(QLPIV_E_SHAPE, "no IA of size %d fits the image", ia_start >> level);
    if (r == -1) return fail(QLPIV_E_SHAPE, "grid larger than the given capacity %d", cap);
    return QLPIV_OK;
}

qlpiv_status qlpiv_grid_level(int height, int width, const int margins[4], int ia_start, int level,
                              float overlap_factor, int superposition_start, qlpiv_grid *grid, int32_t *tops,
                              int32_t *lefts, int cap) {
    if (!grid || !margins) return fail(QLPIV_E_ARG, "NULL argument");
    if (superposition_start < 0) return fail(QLPIV_E_ARG, "superposition start level %d < 0", superposition_start);
    const int r = qlpiv::grid_level(height, width, margins, ia_start, level, overlap_factor, superposition_start, grid,
                                    tops, lefts, cap);
    if (r == -2) return fail(QLPIV_E_ARG, "Overlap factor must greater than 1/10 and less than 9/10");
    if (r == -3) return fail(QLPIV_E_SHAPE, "no IA of size %d fits the image", ia_start >> level);
    if (r == -1) return fail(QLPIV_E_SHAPE, "grid larger than the given capacity %d", cap);
    return QLPIV_OK;
}

qlpiv_status qlpiv_adaptive_levels(const qlpiv_adaptive_desc *desc, int height, int width, int *levels,
                                   qlpiv_grid *grids, int max_levels) {
    if (!levels) return fail(QLPIV_E_ARG, "levels is NULL");
    qlpiv_status st = check_adaptive(desc, QLPIV_PIX_U8, height, width);
    if (st != QLPIV_OK) return st;
    *levels = level_count(desc);
    if (grids) {
        for (int lv = 0; lv < *levels && lv < max_levels; lv++)
            if (qlpiv::grid_level(height, width, desc->margins, desc->ia_start, lv, desc->overlap_factor,
                                  desc->superposition_start, &grids[lv], nullptr, nullptr, 0) < -1)
                return fail(QLPIV_E_SHAPE, "image too small for level %d", lv);
    }
    return QLPIV_OK;
}

qlpiv_status qlpiv_inherit(qlpiv_handle *h, int pni, int pnj, const double *p_ci, const double *p_cj, const float *pu,
                           const float *pv, int cni, int cnj, const float *c_ci, const float *c_cj, int round_int,
                           float *cu, float *cv) {
    if (!h || !p_ci || !p_cj || !pu || !pv || !c_ci || !c_cj || !cu || !cv) return fail(QLPIV_E_ARG, "NULL argument");
    if (pni < 1 || pnj < 1 || cni < 1 || cnj < 1) return fail(QLPIV_E_SHAPE, "empty grid");
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaStream_t s = h->stream;
    const long pc = (long)pni * pnj, cc = (long)cni * cnj;
    std::vector<float> fpy(p_ci, p_ci + pni), fpx(p_cj, p_cj + pnj);  // tile centres are exact in float
    DevBuf *b = h->scratch;
    cudaError_t e;
    if ((e = upload(b[0], fpy.data(), sizeof(float) * pni, s)) != cudaSuccess ||
        (e = upload(b[1], fpx.data(), sizeof(float) * pnj, s)) != cudaSuccess ||
        (e = upload(b[2], pu, sizeof(float) * pc, s)) != cudaSuccess ||
        (e = upload(b[3], pv, sizeof(float) * pc, s)) != cudaSuccess ||
        (e = upload(b[4], c_ci, sizeof(float) * cni, s)) != cudaSuccess ||
        (e = upload(b[5], c_cj, sizeof(float) * cnj, s)) != cudaSuccess ||
        (e = b[6].ensure(sizeof(float) * 2 * cc)) != cudaSuccess ||
        (e = b[7].ensure(sizeof(float) * 2 * (long)cni * pnj)) != cudaSuccess)
        return cuda_fail(e, "inherit upload");
    float *out = b[6].as<float>(), *rows = b[7].as<float>();
    if ((e = launch_inherit(s, 1, b[0].as<float>(), pni, b[1].as<float>(), pnj, b[2].as<float>(), b[3].as<float>(),
                            b[4].as<float>(), cni, b[5].as<float>(), cnj, round_int, rows, rows + (long)cni * pnj,
                            out, out + cc)) != cudaSuccess)
        return cuda_fail(e, "inherit");
    h->launches += 2;
    if ((e = cudaMemcpyAsync(cu, out, sizeof(float) * cc, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(cv, out + cc, sizeof(float) * cc, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "inherit download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_inherit_tiles(qlpiv_handle *h, int mode, int pn, int pni, int pnj, const int32_t *p_tops,
                                 const int32_t *p_lefts, const float *pu, const float *pv, int cn, int cni, int cnj,
                                 const int32_t *c_tops, const int32_t *c_lefts, int round_int, float *cu, float *cv) {
    if (!h || !p_tops || !p_lefts || !pu || !pv || !c_tops || !c_lefts || !cu || !cv)
        return fail(QLPIV_E_ARG, "NULL argument");
    if (mode < QLPIV_INHERIT_DIRECT || mode > QLPIV_INHERIT_DISTANCE)
        return fail(QLPIV_E_ARG, "inheritance mode %d (Direct, Area or Distance)", mode);
    if (pni < 1 || pnj < 1 || cni < 1 || cnj < 1 || pn < 1 || cn < 1) return fail(QLPIV_E_SHAPE, "empty grid");
    std::vector<int2> tab;
    if (qlpiv_status st = inherit_tables(mode, pn, pni, pnj, p_tops, p_lefts, cn, cni, cnj, c_tops, c_lefts, tab))
        return st;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaStream_t s = h->stream;
    const long pc = (long)pni * pnj, cc = (long)cni * cnj;
    DevBuf *b = h->scratch;
    cudaError_t e;
    if ((e = upload(b[0], p_tops, sizeof(int32_t) * pni, s)) != cudaSuccess ||
        (e = upload(b[1], p_lefts, sizeof(int32_t) * pnj, s)) != cudaSuccess ||
        (e = upload(b[2], pu, sizeof(float) * pc, s)) != cudaSuccess ||
        (e = upload(b[3], pv, sizeof(float) * pc, s)) != cudaSuccess ||
        (e = upload(b[4], c_tops, sizeof(int32_t) * cni, s)) != cudaSuccess ||
        (e = upload(b[5], c_lefts, sizeof(int32_t) * cnj, s)) != cudaSuccess ||
        (e = upload(b[7], tab.data(), sizeof(int2) * tab.size(), s)) != cudaSuccess ||
        (e = b[6].ensure(sizeof(float) * 2 * cc)) != cudaSuccess)
        return cuda_fail(e, "inherit upload");
    float *out = b[6].as<float>();
    if ((e = launch_inherit_tiles(s, 1, mode, pn, pni, pnj, b[0].as<int>(), b[1].as<int>(), b[2].as<float>(),
                                  b[3].as<float>(), cn, cni, cnj, b[4].as<int>(), b[5].as<int>(), b[7].as<int2>(),
                                  round_int, out, out + cc)) != cudaSuccess)
        return cuda_fail(e, "inherit");
    h->launches += 1;
    if ((e = cudaMemcpyAsync(cu, out, sizeof(float) * cc, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(cv, out + cc, sizeof(float) * cc, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "inherit download");
    return QLPIV_OK;
}

// Shared set-up of qlpiv_displacement_field / qlpiv_warp_pair: knot factors (double, for the
// solve), float knots (for the evaluation) and displacements uploaded, spline nodes computed.
// Uses scratch[2..5] and scratch[8] (float knots: ni row knots then nj column knots).
static qlpiv_status field_setup(qlpiv_handle *h, int ni, int nj, const double *ci, const double *cj, const float *u,
                                const float *v, SplineCoef *coef) {
    cudaStream_t s = h->stream;
    DevBuf *b = h->scratch;
    const long cnt = (long)ni * nj;
    std::vector<float> fk(ni + nj);
    for (int i = 0; i < ni; i++) fk[i] = (float)ci[i];
    for (int j = 0; j < nj; j++) fk[ni + j] = (float)cj[j];
    std::vector<float2> kf((size_t)KF_ARRAYS * (ni + nj));
    knot_factors_dw(ci, ni, kf.data());
    knot_factors_dw(cj, nj, kf.data() + (size_t)KF_ARRAYS * ni);
    cudaError_t e;
    if ((e = upload(b[2], u, sizeof(float) * cnt, s)) != cudaSuccess ||
        (e = upload(b[3], v, sizeof(float) * cnt, s)) != cudaSuccess ||
        (e = upload(b[4], kf.data(), sizeof(float2) * kf.size(), s)) != cudaSuccess ||
        (e = b[5].ensure(spline_coef_bytes(cnt))) != cudaSuccess ||
        (e = upload(b[8], fk.data(), sizeof(float) * (ni + nj), s)) != cudaSuccess)
        return cuda_fail(e, "field upload");
    *coef = spline_coef_at(b[5].p, cnt);
    if ((e = launch_spline(s, 1, b[4].as<float2>(), ni, b[4].as<float2>() + (size_t)KF_ARRAYS * ni, nj,
                           b[2].as<float>(), b[3].as<float>(), *coef)) != cudaSuccess)
        return cuda_fail(e, "spline");
    h->launches += 1;
    // the host staging must outlive this function's vectors: wait for the uploads
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "field set-up");
    return QLPIV_OK;
}

qlpiv_status qlpiv_displacement_field(qlpiv_handle *h, int height, int width, int ni, int nj, const double *ci,
                                      const double *cj, const float *u, const float *v, float *fu, float *fv) {
    if (!h || !ci || !cj || !u || !v || !fu || !fv) return fail(QLPIV_E_ARG, "NULL argument");
    if (ni < 3 || nj < 3) return fail(QLPIV_E_SHAPE, "the spline needs at least 3 tiles per axis");
    if (height <= 0 || width <= 0) return fail(QLPIV_E_SHAPE, "image size %d x %d", height, width);
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    SplineCoef coef;
    qlpiv_status st = field_setup(h, ni, nj, ci, cj, u, v, &coef);
    if (st != QLPIV_OK) return st;
    cudaStream_t s = h->stream;
    DevBuf *b = h->scratch;
    const size_t px = (size_t)height * width;
    cudaError_t e;
    if ((e = b[6].ensure(sizeof(float) * px)) != cudaSuccess || (e = b[7].ensure(sizeof(float) * px)) != cudaSuccess)
        return cuda_fail(e, "field buffers");
    if ((e = launch_field(s, height, width, b[8].as<float>(), ni, b[8].as<float>() + ni, nj, coef, b[6].as<float>(),
                          b[7].as<float>())) != cudaSuccess)
        return cuda_fail(e, "field");
    h->launches++;
    if ((e = cudaMemcpyAsync(fu, b[6].p, sizeof(float) * px, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(fv, b[7].p, sizeof(float) * px, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "field download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_warp_pair(qlpiv_handle *h, int pixel_type, int warp_mode, const void *img_a, const void *img_b,
                             int height, int width, int ni, int nj, const double *ci, const double *cj, const float *u,
                             const float *v, int int16_quirk, void *out_a, void *out_b) {
    if (!h || !img_a || !img_b || !ci || !cj || !u || !v || !out_a || !out_b) return fail(QLPIV_E_ARG, "NULL argument");
    if (!full_warp(warp_mode)) return fail(QLPIV_E_ARG, "warp mode %d is not a full-image bilinear warp", warp_mode);
    if (pixel_type != QLPIV_PIX_U8 && pixel_type != QLPIV_PIX_U16) return fail(QLPIV_E_ARG, "u8 or u16 images only");
    if (ni < 3 || nj < 3) return fail(QLPIV_E_SHAPE, "the spline needs at least 3 tiles per axis");
    if (height <= 0 || width <= 0) return fail(QLPIV_E_SHAPE, "image size %d x %d", height, width);
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    SplineCoef coef;
    qlpiv_status st = field_setup(h, ni, nj, ci, cj, u, v, &coef);
    if (st != QLPIV_OK) return st;
    cudaStream_t s = h->stream;
    const size_t bytes = (size_t)height * width * pixel_bytes(pixel_type);
    const size_t stride = (bytes + 255) & ~(size_t)255;
    cudaError_t e;
    if ((e = h->tiles_a.ensure(4 * stride)) != cudaSuccess || (e = h->frames.ensure(2 * sizeof(qlpiv_frame))) !=
        cudaSuccess)
        return cuda_fail(e, "warp buffers");
    char *base = h->tiles_a.as<char>();
    qlpiv_frame t[2] = {{base, base + stride, height, width, (int64_t)width},
                        {base + 2 * stride, base + 3 * stride, height, width, (int64_t)width}};
    if ((e = cudaMemcpyAsync(base, img_a, bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(base + stride, img_b, bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(h->frames.p, t, sizeof(t), cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "warp upload");
    const qlpiv_frame *dt = h->frames.as<qlpiv_frame>();
    DevBuf *b = h->scratch;
    if ((e = launch_warp(s, pixel_type, 1, height, width, dt, dt + 1, b[8].as<float>(), ni, b[8].as<float>() + ni, nj,
                         coef, int16_quirk, full_image_mode(warp_mode))) != cudaSuccess)
        return cuda_fail(e, "warp");
    h->launches++;
    if ((e = cudaMemcpyAsync(out_a, base + 2 * stride, bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(out_b, base + 3 * stride, bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "warp download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_tile_warp(qlpiv_handle *h, int pixel_type, const void *img_a, const void *img_b, int height,
                             int width, int n, int ni, int nj, const int32_t *tops, const int32_t *lefts,
                             const float *u, const float *v, int warp_mode, float full_max, void *tiles_a,
                             void *tiles_b, float *max_a, float *max_b) {
    if (!h || !img_a || !img_b || !tops || !lefts || !u || !v || !tiles_a || !tiles_b || !max_a || !max_b)
        return fail(QLPIV_E_ARG, "NULL argument");
    if (pixel_type != QLPIV_PIX_U8 && pixel_type != QLPIV_PIX_U16) return fail(QLPIV_E_ARG, "u8 or u16 images only");
    if (!per_tile_warp(warp_mode)) return fail(QLPIV_E_ARG, "warp mode %d is not a micro / mini mode", warp_mode);
    if (ni < 3 || nj < 3) return fail(QLPIV_E_SHAPE, "the spline needs at least 3 tiles per axis");
    if (height <= 0 || width <= 0 || n <= 0 || n > 64) return fail(QLPIV_E_SHAPE, "image %d x %d, tile %d", height, width, n);
    for (int i = 0; i < ni; i++)
        if (tops[i] < 0 || tops[i] + n > height) return fail(QLPIV_E_SHAPE, "tile row %d leaves the image", i);
    for (int j = 0; j < nj; j++)
        if (lefts[j] < 0 || lefts[j] + n > width) return fail(QLPIV_E_SHAPE, "tile column %d leaves the image", j);
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaStream_t s = h->stream;
    const size_t pb = pixel_bytes(pixel_type), bytes = (size_t)height * width * pb;
    const size_t stride = (bytes + 255) & ~(size_t)255;
    const long cnt = (long)ni * nj;
    const size_t tb = (size_t)cnt * n * n * pb;
    DevBuf *b = h->scratch;
    cudaError_t e;
    if ((e = h->tiles_a.ensure(2 * stride)) != cudaSuccess || (e = h->frames.ensure(sizeof(qlpiv_frame))) != cudaSuccess ||
        (e = b[0].ensure(sizeof(int32_t) * (ni + nj))) != cudaSuccess ||
        (e = b[1].ensure(sizeof(float) * 2 * cnt)) != cudaSuccess || (e = b[2].ensure(2 * tb)) != cudaSuccess ||
        (e = b[3].ensure(sizeof(float) * 2 * cnt)) != cudaSuccess)
        return cuda_fail(e, "tile warp buffers");
    char *base = h->tiles_a.as<char>();
    const qlpiv_frame t{base, base + stride, height, width, (int64_t)width};
    int32_t *dtl = b[0].as<int32_t>();
    float *duv = b[1].as<float>(), *dmx = b[3].as<float>();
    char *dtiles = b[2].as<char>();
    if ((e = cudaMemcpyAsync(base, img_a, bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(base + stride, img_b, bytes, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(h->frames.p, &t, sizeof(t), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dtl, tops, sizeof(int32_t) * ni, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dtl + ni, lefts, sizeof(int32_t) * nj, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(duv, u, sizeof(float) * cnt, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(duv + cnt, v, sizeof(float) * cnt, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "tile warp upload");
    if ((e = launch_tile_warp(s, pixel_type, 1, h->frames.as<qlpiv_frame>(), n, ni, nj, dtl, dtl + ni, duv, duv + cnt,
                              tile_image_mode(warp_mode), tile_mini(warp_mode), full_max, dtiles, dtiles + tb, dmx,
                              dmx + cnt)) != cudaSuccess)
        return cuda_fail(e, "tile warp");
    h->launches++;
    if ((e = cudaMemcpyAsync(tiles_a, dtiles, tb, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(tiles_b, dtiles + tb, tb, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(max_a, dmx, sizeof(float) * cnt, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(max_b, dmx + cnt, sizeof(float) * cnt, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "tile warp download");
    return QLPIV_OK;
}

qlpiv_status qlpiv_piv_adaptive_device(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int pixel_type, int height,
                                       int width, int num_pairs, const qlpiv_frame *frames, float *out_u,
                                       float *out_v) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    qlpiv_status st = check_adaptive(desc, pixel_type, height, width);
    if (st != QLPIV_OK) return st;
    if (num_pairs < 0) return fail(QLPIV_E_ARG, "num_pairs < 0");
    if (num_pairs == 0) return QLPIV_OK;
    if (!frames || !out_u || !out_v) return fail(QLPIV_E_ARG, "NULL frame table or output");
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    if ((st = build_plan(h, desc, pixel_type, height, width, num_pairs)) != QLPIV_OK) return st;
    if ((st = run_levels(h, frames)) != QLPIV_OK) return st;
    LevelPlan &L = h->plan->levels.back();
    const size_t bytes = sizeof(float) * L.count() * num_pairs;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(out_u, L.d_u.p, bytes, cudaMemcpyDeviceToDevice, h->stream)) != cudaSuccess ||
        (e = cudaMemcpyAsync(out_v, L.d_v.p, bytes, cudaMemcpyDeviceToDevice, h->stream)) != cudaSuccess)
        return cuda_fail(e, "adaptive output");
    return QLPIV_OK;
}

// Queues the optical flow after PIV of every pair on the last level's tiles (in place in
// d_u/d_v).  frames: host-side copy of the device frame table (image pointers per pair).
// dense_u/dense_v: device, pairs x height x width, or NULL.
static qlpiv_status queue_flow(qlpiv_handle *h, const qlpiv_flow_desc &flow, const qlpiv_frame *frames,
                               float *dense_u, float *dense_v, std::vector<float> &weights) {
    AdaptivePlan *p = h->plan;
    qlpiv_flow_desc fd = flow;
    fd.clipping_mode = p->desc.clipping_mode;  // one PIVInputParameters clipping mode for every stage
    LevelPlan &L = p->levels.back();
    cudaStream_t s = h->stream;
    const int ni = L.g.tiles_i, nj = L.g.tiles_j;
    const long cnt = L.count(), np = (long)p->height * p->width;
    // pairs run on up to kFlowLanes streams at once (one lane with the stage profiler, whose
    // events sit on the handle's stream)
    const int lanes = h->profiling ? 1 : std::min(p->pairs, AdaptivePlan::kFlowLanes);
    FlowBufs fb[AdaptivePlan::kFlowLanes];
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < lanes && e == cudaSuccess; k++) {
        if ((e = flow_buffers(p->flow[k], p->height, p->width, ni, nj, fd.iterations_ls, &fb[k])) != cudaSuccess ||
            (e = upload_flow_weights(s, fd, fb[k], weights)) != cudaSuccess)
            break;
        if (lanes > 1 && !p->flow_side[k] &&
            ((e = cudaStreamCreateWithFlags(&p->flow_side[k], cudaStreamNonBlocking)) != cudaSuccess ||
             (e = cudaEventCreateWithFlags(&p->flow_done[k], cudaEventDisableTiming)) != cudaSuccess))
            break;
    }
    if (e == cudaSuccess && lanes > 1 && !p->flow_fork)
        e = cudaEventCreateWithFlags(&p->flow_fork, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "flow buffers");
    struct MarkCtx {
        qlpiv_handle *h;
        int level, n;
        long items;
        StageEvent ev;
    } mc{h, (int)p->levels.size() - 1, L.g.n, np, {}};
    auto on_mark = [](void *c, const char *stage, bool begin) {
        MarkCtx *m = static_cast<MarkCtx *>(c);
        if (begin) {
            m->ev = StageEvent{stage, m->level, m->n, 0, m->items, nullptr, nullptr};
            if (cudaEventCreate(&m->ev.begin) != cudaSuccess || cudaEventCreate(&m->ev.end) != cudaSuccess) return;
            cudaEventRecord(m->ev.begin, m->h->stream);
        } else if (m->ev.end) {
            cudaEventRecord(m->ev.end, m->h->stream);
            m->h->prof_pending.push_back(m->ev);
            m->ev.end = nullptr;
        }
    };
    const FlowMarks marks{on_mark, &mc};
    // the splines of every pair's final tile displacements in one launch set (the warp of this
    // level used the inherited displacements; the coefficients are free again)
    const SplineCoef all = coef_of(L, p->pairs);
    if (h->profiling) on_mark(&mc, "flow:spline", true);
    if ((e = launch_spline(s, p->pairs, L.d_kfy.as<float2>(), ni, L.d_kfx.as<float2>(), nj, L.d_u.as<float>(),
                           L.d_v.as<float>(), all)) != cudaSuccess)
        return cuda_fail(e, "flow spline");
    if (h->profiling) on_mark(&mc, "flow:spline", false);
    h->launches += 1;
    if (lanes > 1) {
        if ((e = cudaEventRecord(p->flow_fork, s)) != cudaSuccess) return cuda_fail(e, "flow fork");
        for (int k = 0; k < lanes; k++)
            if ((e = cudaStreamWaitEvent(p->flow_side[k], p->flow_fork, 0)) != cudaSuccess)
                return cuda_fail(e, "flow fork");
    }
    for (int q = 0; q < p->pairs; q++) {
        long launches = 0;
        const long off = (long)q * cnt;
        const SplineCoef pc = spline_coef_offset(all, off);
        const int k = q % lanes;
        cudaStream_t ls = lanes > 1 ? p->flow_side[k] : s;
        if ((e = run_flow(ls, fd, p->pixel_type, frames[q].img_a, frames[q].img_b, frames[q].pitch, p->height,
                          p->width, L.g.n, ni, nj, L.d_kfy.as<float2>(), L.d_kfx.as<float2>(), L.d_cyf.as<float>(),
                          L.d_cxf.as<float>(), L.d_tops.as<int>(), L.d_lefts.as<int>(), L.d_u.as<float>() + q * cnt,
                          L.d_v.as<float>() + q * cnt, dense_u ? dense_u + q * np : nullptr,
                          dense_v ? dense_v + q * np : nullptr, fb[k], &launches,
                          h->profiling ? &marks : nullptr, &pc)) != cudaSuccess)
            return cuda_fail(e, "optical flow after PIV");
        h->launches += launches;
    }
    if (lanes > 1)
        for (int k = 0; k < lanes; k++)
            if ((e = cudaEventRecord(p->flow_done[k], p->flow_side[k])) != cudaSuccess ||
                (e = cudaStreamWaitEvent(s, p->flow_done[k], 0)) != cudaSuccess)
                return cuda_fail(e, "flow join");
    return QLPIV_OK;
}

static qlpiv_status check_flow_grid(qlpiv_handle *h) {
    LevelPlan &L = h->plan->levels.back();
    if (L.g.tiles_i < 3 || L.g.tiles_j < 3)
        return fail(QLPIV_E_SHAPE, "last level has %d x %d tiles: the flow spline needs at least 3 per axis",
                    L.g.tiles_i, L.g.tiles_j);
    return QLPIV_OK;
}

qlpiv_status qlpiv_piv_adaptive(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int pixel_type, int height,
                                int width, int num_pairs, const qlpiv_frame *frames, float *out_u, float *out_v) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    qlpiv_status st = check_adaptive(desc, pixel_type, height, width);
    if (st != QLPIV_OK) return st;
    if (num_pairs < 0) return fail(QLPIV_E_ARG, "num_pairs < 0");
    if (num_pairs == 0) return QLPIV_OK;
    if (!frames || !out_u || !out_v) return fail(QLPIV_E_ARG, "NULL frame table or output");
    if ((st = check_host_frames(frames, num_pairs, height, width)) != QLPIV_OK) return st;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    if ((st = build_plan(h, desc, pixel_type, height, width, num_pairs)) != QLPIV_OK) return st;
    AdaptivePlan *p = h->plan;
    cudaStream_t s = h->stream;
    cudaError_t e;
    std::vector<qlpiv_frame> t;
    if ((st = upload_host_frames(h, frames, t)) != QLPIV_OK) return st;
    if ((st = run_levels(h, p->host_table.as<qlpiv_frame>())) != QLPIV_OK) return st;
    LevelPlan &L = p->levels.back();
    const size_t bytes = sizeof(float) * L.count() * num_pairs;
    if ((e = cudaMemcpyAsync(out_u, L.d_u.p, bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(out_v, L.d_v.p, bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "adaptive PIV");
    return QLPIV_OK;
}

qlpiv_status qlpiv_piv_flow(qlpiv_handle *h, const qlpiv_adaptive_desc *piv, const qlpiv_flow_desc *flow,
                            int pixel_type, int height, int width, int num_pairs, const qlpiv_frame *frames,
                            float *out_u, float *out_v, float *dense_u, float *dense_v) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    qlpiv_status st = check_adaptive(piv, pixel_type, height, width);
    if (st != QLPIV_OK) return st;
    if (const char *m = check_flow_desc(flow, height, width)) return fail(QLPIV_E_ARG, "%s", m);
    if (num_pairs < 0) return fail(QLPIV_E_ARG, "num_pairs < 0");
    if (num_pairs == 0) return QLPIV_OK;
    if (!frames || !out_u || !out_v) return fail(QLPIV_E_ARG, "NULL frame table or output");
    if ((st = check_host_frames(frames, num_pairs, height, width)) != QLPIV_OK) return st;
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    if ((st = build_plan(h, piv, pixel_type, height, width, num_pairs)) != QLPIV_OK) return st;
    if ((st = check_flow_grid(h)) != QLPIV_OK) return st;
    AdaptivePlan *p = h->plan;
    cudaStream_t s = h->stream;
    cudaError_t e;
    std::vector<qlpiv_frame> t;
    std::vector<float> weights;
    if ((st = upload_host_frames(h, frames, t)) != QLPIV_OK) return st;
    if ((st = run_levels(h, p->host_table.as<qlpiv_frame>())) != QLPIV_OK) return st;
    const size_t np = (size_t)height * width;
    float *du = nullptr, *dv = nullptr;
    if (dense_u || dense_v) {
        if ((e = p->flow_dense.ensure(sizeof(float) * 2 * np * num_pairs)) != cudaSuccess)
            return cuda_fail(e, "dense field buffer");
        du = p->flow_dense.as<float>();
        dv = du + np * num_pairs;
    }
    if ((st = queue_flow(h, *flow, t.data(), du, dv, weights)) != QLPIV_OK) return st;
    LevelPlan &L = p->levels.back();
    const size_t bytes = sizeof(float) * L.count() * num_pairs, db = sizeof(float) * np * num_pairs;
    if ((e = cudaMemcpyAsync(out_u, L.d_u.p, bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(out_v, L.d_v.p, bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (dense_u && (e = cudaMemcpyAsync(dense_u, du, db, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
        (dense_v && (e = cudaMemcpyAsync(dense_v, dv, db, cudaMemcpyDeviceToHost, s)) != cudaSuccess) ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "PIV with optical flow");
    return QLPIV_OK;
}

qlpiv_status qlpiv_piv_flow_device(qlpiv_handle *h, const qlpiv_adaptive_desc *piv, const qlpiv_flow_desc *flow,
                                   int pixel_type, int height, int width, int num_pairs, const qlpiv_frame *frames,
                                   float *out_u, float *out_v, float *dense_u, float *dense_v) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    qlpiv_status st = check_adaptive(piv, pixel_type, height, width);
    if (st != QLPIV_OK) return st;
    if (const char *m = check_flow_desc(flow, height, width)) return fail(QLPIV_E_ARG, "%s", m);
    if (num_pairs < 0) return fail(QLPIV_E_ARG, "num_pairs < 0");
    if (num_pairs == 0) return QLPIV_OK;
    if (!frames || !out_u || !out_v) return fail(QLPIV_E_ARG, "NULL frame table or output");
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    if ((st = build_plan(h, piv, pixel_type, height, width, num_pairs)) != QLPIV_OK) return st;
    if ((st = check_flow_grid(h)) != QLPIV_OK) return st;
    AdaptivePlan *p = h->plan;
    cudaStream_t s = h->stream;
    cudaError_t e;
    // the flow stages take image pointers on the host side: read the device table once
    std::vector<qlpiv_frame> t(num_pairs);
    std::vector<float> weights;
    if ((e = cudaMemcpyAsync(t.data(), frames, sizeof(qlpiv_frame) * num_pairs, cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "frame table read");
    for (int q = 0; q < num_pairs; q++)
        if (!t[q].img_a || !t[q].img_b || t[q].height != height || t[q].width != width || t[q].pitch < width)
            return fail(QLPIV_E_SHAPE, "frame %d: NULL image or size differs from %d x %d", q, height, width);
    if ((st = run_levels(h, frames)) != QLPIV_OK) return st;
    if ((st = queue_flow(h, *flow, t.data(), dense_u, dense_v, weights)) != QLPIV_OK) return st;
    LevelPlan &L = p->levels.back();
    const size_t bytes = sizeof(float) * L.count() * num_pairs;
    if ((e = cudaMemcpyAsync(out_u, L.d_u.p, bytes, cudaMemcpyDeviceToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(out_v, L.d_v.p, bytes, cudaMemcpyDeviceToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "PIV with optical flow output");
    // the filter weights' host staging must outlive the queued upload
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "PIV with optical flow");
    return QLPIV_OK;
}

// VectorValidatorJob.compute on host arrays for one frame; clip_n > 0 applies NoOutOfBoundClipping
// to the replacements (tile side clip_n, image clip_h x clip_w).
static qlpiv_status validate_host(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int clip_n, int clip_h,
                                  int clip_w, int ni, int nj, const int32_t *tops, const int32_t *lefts, float *u,
                                  float *v, const float *peak_u, const float *peak_v, const int32_t *npeaks,
                                  uint8_t *invalid_out) {
    if (!h || !desc || !tops || !lefts || !u || !v) return fail(QLPIV_E_ARG, "NULL argument");
    if (ni < 1 || nj < 1) return fail(QLPIV_E_SHAPE, "empty grid");
    const int model = desc->validation;
    if (model < QLPIV_VALIDATE_MULTIPEAK_MEDIAN || model > QLPIV_VALIDATE_MEDIAN)
        return fail(QLPIV_E_ARG, "unknown validation model %d", model);
    const bool multi = model == QLPIV_VALIDATE_MULTIPEAK_MEDIAN;
    if (multi && (!peak_u || !peak_v || !npeaks))
        return fail(QLPIV_E_ARG, "the multi-peak model needs peak_u, peak_v and npeaks");
    const int k = multi ? desc->num_peaks : 1;
    if (k < 1 || k > QLPIV_MAX_PEAKS) return fail(QLPIV_E_ARG, "num_peaks must be in 1..%d", QLPIV_MAX_PEAKS);
    if (!(desc->median_threshold > 0.0f) || !(desc->median_epsilon0 >= 0.0f))
        return fail(QLPIV_E_ARG, "validation threshold must be > 0 and epsilon0 >= 0");
    const long cnt = (long)ni * nj;
    std::vector<float2> puv(cnt * k, make_float2(0.0f, 0.0f));
    std::vector<uint8_t> npk(cnt, 1);
    if (multi)
        for (long t = 0; t < cnt; t++) {
            if (npeaks[t] < 0 || npeaks[t] > k)
                return fail(QLPIV_E_ARG, "npeaks[%ld] = %d outside 0..%d", t, npeaks[t], k);
            npk[t] = (uint8_t)npeaks[t];
            for (int q = 0; q < k; q++) puv[t * k + q] = make_float2(peak_u[t * k + q], peak_v[t * k + q]);
        }
    std::vector<int32_t> order, rank;
    spiral_rank(ni, nj, order, rank);
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaStream_t s = h->stream;
    // one scratch buffer carved into the per-tile arrays (256-byte aligned pieces)
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t sz_f = al(sizeof(float) * cnt), sz_i = al(sizeof(int32_t) * cnt), sz_b = al(cnt);
    const size_t sz_p = al(sizeof(float2) * cnt * k), sz_t = al(sizeof(int32_t) * ni), sz_l = al(sizeof(int32_t) * nj);
    const size_t total = 4 * sz_f + sz_p + 2 * sz_b + 4 * sz_i + sz_t + sz_l + 256;
    DevBuf &b = h->scratch[11];
    cudaError_t e = b.ensure(total);
    if (e != cudaSuccess) return cuda_fail(e, "validation scratch");
    char *c = b.as<char>();
    float *du = (float *)c; c += sz_f;
    float *dv = (float *)c; c += sz_f;
    float *dbu = (float *)c; c += sz_f;
    float *dbv = (float *)c; c += sz_f;
    float2 *dpuv = (float2 *)c; c += sz_p;
    uint8_t *dnpk = (uint8_t *)c; c += sz_b;
    uint8_t *dst = (uint8_t *)c; c += sz_b;
    int32_t *dorder = (int32_t *)c; c += sz_i;
    int32_t *drank = (int32_t *)c; c += sz_i;
    int32_t *dlist = (int32_t *)c; c += sz_i;
    int32_t *ddone = (int32_t *)c; c += sz_i;
    int32_t *dtops = (int32_t *)c; c += sz_t;
    int32_t *dlefts = (int32_t *)c; c += sz_l;
    int32_t *dsweeps = (int32_t *)c;
    if ((e = cudaMemcpyAsync(du, u, sizeof(float) * cnt, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dv, v, sizeof(float) * cnt, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dpuv, puv.data(), sizeof(float2) * cnt * k, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dnpk, npk.data(), cnt, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dorder, order.data(), sizeof(int32_t) * cnt, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(drank, rank.data(), sizeof(int32_t) * cnt, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dtops, tops, sizeof(int32_t) * ni, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dlefts, lefts, sizeof(int32_t) * nj, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return cuda_fail(e, "validation upload");
    ValidateParams vp{ni, nj, k, desc->median_threshold, desc->median_epsilon0, desc->max_correction_iterations,
                      desc->iterate_until_no_corrections, model, clip_n, clip_h, clip_w};
    ValidateBufs vb{du, dv, dbu, dbv, dpuv, dnpk, dst, dtops, dlefts, dorder, drank, dlist, ddone, dsweeps};
    if ((e = launch_validate(s, 1, vp, vb)) != cudaSuccess) return cuda_fail(e, "validation");
    h->launches += 2;
    std::vector<uint8_t> state(cnt);
    if ((e = cudaMemcpyAsync(u, du, sizeof(float) * cnt, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(v, dv, sizeof(float) * cnt, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(state.data(), dst, cnt, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "validation download");
    if (invalid_out)
        for (long t = 0; t < cnt; t++) invalid_out[t] = state[t] & 1u;
    return QLPIV_OK;
}

qlpiv_status qlpiv_validate(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int ni, int nj, const int32_t *tops,
                            const int32_t *lefts, float *u, float *v, const float *peak_u, const float *peak_v,
                            const int32_t *npeaks, uint8_t *invalid_out) {
    if (desc && desc->clipping_mode == QLPIV_CLIP_NO_OUT_OF_BOUND)
        return fail(QLPIV_E_ARG, "NoOutOfBoundClipping needs the tile side and image size: use qlpiv_validate_tiles");
    return validate_host(h, desc, 0, 0, 0, ni, nj, tops, lefts, u, v, peak_u, peak_v, npeaks, invalid_out);
}

qlpiv_status qlpiv_validate_tiles(qlpiv_handle *h, const qlpiv_adaptive_desc *desc, int n, int height, int width,
                                  int ni, int nj, const int32_t *tops, const int32_t *lefts, float *u, float *v,
                                  const float *peak_u, const float *peak_v, const int32_t *npeaks,
                                  uint8_t *invalid_out) {
    if (!desc) return fail(QLPIV_E_ARG, "NULL argument");
    if (desc->clipping_mode < QLPIV_CLIP_ALLOWED || desc->clipping_mode > QLPIV_CLIP_NO_OUT_OF_BOUND)
        return fail(QLPIV_E_ARG, "unknown clipping mode %d", desc->clipping_mode);
    if (n < 1 || height < 1 || width < 1) return fail(QLPIV_E_SHAPE, "tile side and image size must be positive");
    const bool clip = desc->clipping_mode == QLPIV_CLIP_NO_OUT_OF_BOUND;
    return validate_host(h, desc, clip ? n : 0, clip ? height : 0, clip ? width : 0, ni, nj, tops, lefts, u, v,
                         peak_u, peak_v, npeaks, invalid_out);
}

qlpiv_status qlpiv_profile_enable(qlpiv_handle *h, int enable) {
    if (!h) return fail(QLPIV_E_ARG, "handle is NULL");
    std::lock_guard<std::mutex> lock(h->mu);
    h->profiling = enable != 0;
    return QLPIV_OK;
}

qlpiv_status qlpiv_profile_read(qlpiv_handle *h, qlpiv_stage_time *out, int cap, int *count) {
    if (!h || !count) return fail(QLPIV_E_ARG, "NULL argument");
    std::lock_guard<std::mutex> lock(h->mu);
    DeviceScope ds(h->device);
    if (ds.err != cudaSuccess) return cuda_fail(ds.err, "cudaSetDevice");
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "profile read");
    for (StageEvent &ev : h->prof_pending) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ev.begin, ev.end);
        cudaEventDestroy(ev.begin);
        cudaEventDestroy(ev.end);
        bool found = false;
        for (StageTotal &t : h->prof_totals)
            if (t.stage == ev.stage && t.level == ev.level) {
                t.launches += ev.launches;
                t.items += ev.items;
                t.ms += ms;
                found = true;
                break;
            }
        if (!found) h->prof_totals.push_back({ev.stage, ev.level, ev.ia_side, ev.launches, ev.items, (double)ms});
    }
    h->prof_pending.clear();
    const int n = (int)h->prof_totals.size();
    *count = n;
    if (out) {
        for (int k = 0; k < n && k < cap; k++) {
            const StageTotal &t = h->prof_totals[k];
            std::memset(out[k].stage, 0, sizeof(out[k].stage));
            std::strncpy(out[k].stage, t.stage.c_str(), sizeof(out[k].stage) - 1);
            out[k].level = t.level;
            out[k].ia_side = t.ia_side;
            out[k].launches = t.launches;
            out[k].items = t.items;
            out[k].ms = t.ms;
        }
    }
    h->prof_totals.clear();
    return QLPIV_OK;
}

}  // extern "C"
