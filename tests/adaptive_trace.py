"""Stage-by-stage trace of the adaptive PIV loop, for parity tests at full workload size.

`gpu_trace` drives the library's stage entry points (inheritance, full-image warp, one
correlation pass, validation) level by level on one frame pair and records every
intermediate; the sequence is the one `per_call.piv_adaptive_per_call` runs, which gives
displacements bit-identical to the fused device pipeline (tests/test_gpu_per_call.py).

`check_stages` feeds each recorded stage input to the CPU oracle and compares stage by stage,
so that a difference is charged to the stage that made it, never to an upstream one:

* inheritance and the float displacement field / warp: bit-identical to the oracle's float
  formulation; the warp through the FP64 field differs only on pixels whose bilinear value
  sits on a rounding boundary (counted);
* correlation pass: every peak slot against the FP64 oracle on the same (GPU-warped) frames:
  integer peaks identical except exact ties, sub-pixel within 1e-3 px;
* validation: bit-identical to the oracle validator given the same vectors.

The loop is the reference's LocalPIVOpenCLGpuJob level loop
(S/jobs/LocalPIVOpenCLGpuJob.java:188-411), S/ = src/main/java/pt/quickLabPIV/.
"""
import numpy as np

from parity import BORDER, SUBPIX_TOL, TIE_REL


def _java_round(x):
    return np.floor(x + np.float32(0.5)).astype(np.int32)


def clip_inside(tops, lefts, n, h, w, u, v):
    """Tile.accumulateDisplacement / replaceDisplacement bounds under NoOutOfBoundClipping
    (S/iareas/Tile.java:103-136): per tile of the (tops x lefts) grid, whether (u, v) rounded
    (floor(x + 0.5f)) keeps the tile inside the h x w image by the reference's test."""
    ru = np.floor(u + np.float32(0.5))
    rv = np.floor(v + np.float32(0.5))
    t = np.asarray(tops, np.float32)[:, None]
    l_ = np.asarray(lefts, np.float32)[None, :]
    return ~((t + ru < 0) | (t + np.float32(n) + ru >= np.float32(h)) | (l_ + rv < 0) |
             (l_ + np.float32(n) + rv >= np.float32(w)))


def gpu_trace(qp, handle, img_a, img_b, desc):
    """Per-level records of the adaptive loop run through the library's stage calls."""
    a = np.ascontiguousarray(img_a)
    b = np.ascontiguousarray(img_b)
    h, w = a.shape
    levels = qp.adaptive_levels(desc, h, w)
    fm = desc.fixed_max if desc.fixed_max > 0 else (255.0 if a.dtype == np.uint8 else 65535.0)
    validate = desc.validation != 0
    multi = desc.validation == qp.VALIDATE_MULTIPEAK_MEDIAN
    clip = desc.clipping_mode == qp.CLIP_NO_OUT_OF_BOUND
    pass_kw = dict(norm_mode=desc.norm_mode, max_mode=desc.max_mode, fixed_max=(fm, fm),
                   subpix_mode=desc.subpix_mode)
    if multi:
        pass_kw.update(num_peaks=desc.num_peaks, peak_kernel=desc.peak_kernel)
    warp = desc.warp_mode == qp.WARP_BOTH_BILINEAR
    assert desc.warp_mode in (qp.WARP_NONE, qp.WARP_BOTH_BILINEAR) and desc.inherit_mode == 0
    recs = []
    prev = None
    for lv, g in enumerate(levels):
        st = qp.grid.level(h, w, desc.ia_start, lv, desc.overlap_factor, list(desc.margins),
                           superposition_start=desc.superposition_start)
        n = st.n
        tops = np.asarray(st.tops, np.int32)
        lefts = np.asarray(st.lefts, np.int32)
        cy, cx = st.centres()
        ni, nj = len(tops), len(lefts)
        rec = dict(level=lv, n=n, tops=tops, lefts=lefts, cy=cy, cx=cx, wa=a, wb=b)
        if prev is None:
            u0 = np.zeros((ni, nj), np.float32)
            v0 = np.zeros((ni, nj), np.float32)
        else:
            u0, v0 = handle.inherit(prev["cy"], prev["cx"], prev["u"], prev["v"], cy, cx,
                                    round_int=not warp)
            rec["u_inh"], rec["v_inh"] = u0, v0
            if clip:   # the new tiles take the inherited value through accumulateDisplacement
                u0 = np.float32(0.0) + u0
                v0 = np.float32(0.0) + v0
                ok = clip_inside(tops, lefts, n, h, w, u0, v0)
                u0 = np.where(ok, u0, np.float32(0.0)).astype(np.float32)
                v0 = np.where(ok, v0, np.float32(0.0)).astype(np.float32)
        rec["u_in"], rec["v_in"] = u0, v0
        at = np.repeat(tops, nj)
        al = np.tile(lefts, ni)
        bt, bl = at, al
        if warp and lv > 0:
            rec["wa"], rec["wb"] = handle.warp_pair(a, b, cy.astype(np.float64), cx.astype(np.float64), u0, v0,
                                                    int16_quirk=bool(desc.int16_warp_quirk))
        elif not warp:
            bt = _java_round(at.astype(np.float32) + u0.ravel())
            bl = _java_round(al.astype(np.float32) + v0.ravel())
        rec["at"], rec["al"], rec["bt"], rec["bl"] = at, al, bt, bl
        vec = handle.piv_pass(rec["wa"], rec["wb"], n, at, al, bt, bl, **pass_kw)
        if vec.ndim == 1:
            vec = vec[:, None]
        rec["vec"] = vec
        main = vec[:, 0]
        ua = (u0.ravel() + main["u"]).reshape(ni, nj).astype(np.float32)
        va = (v0.ravel() + main["v"]).reshape(ni, nj).astype(np.float32)
        if clip:   # accumulateDisplacement drops an increment that moves the tile out of the image
            ok = clip_inside(tops, lefts, n, h, w, ua, va)
            ua = np.where(ok, ua, u0)
            va = np.where(ok, va, v0)
        rec["u_acc"], rec["v_acc"] = ua, va
        if validate:
            if multi:
                present = (vec["flags"] & qp.F_ABSENT) == 0
                npk = present.sum(axis=1).astype(np.int32).reshape(ni, nj)
                k = desc.num_peaks
                pk = (vec["u"].reshape(ni, nj, k), vec["v"].reshape(ni, nj, k), npk)
            else:
                npk = np.ones((ni, nj), np.int32)
                pk = (None, None, None)
            rec["npk"] = npk
            u, v, inv = handle.validate(tops, lefts, ua, va, *pk, desc, n=n, height=h, width=w)
        else:
            u, v, inv = ua, va, np.zeros((ni, nj), np.uint8)
        rec["u"], rec["v"], rec["invalid"] = u, v, inv
        recs.append(rec)
        prev = rec
    return recs


def _tile_planes64(oracle, wa, wb, n, at, al, bt, bl, k, fixed):
    ta, ma = oracle.clip_tile(wa, int(at[k]), int(al[k]), n)
    tb, mb = oracle.clip_tile(wb, int(bt[k]), int(bl[k]), n)
    if fixed is not None:
        ma, mb = fixed
    else:
        mb = ma
    return oracle.xcorr_fft(ta, tb, ma, mb, normalize=True, precision=64)


def compare_pass(oracle, rec, desc, fixed, nthreads=None):
    """One level's correlation pass (every peak slot) against the FP64 oracle on the same frames."""
    n = rec["n"]
    vec = rec["vec"]
    k = vec.shape[1]
    if desc.validation == 1:
        ref, npk = oracle.piv_pass_multi(rec["wa"], rec["wb"], n, rec["at"], rec["al"], rec["bt"], rec["bl"],
                                         norm_mode=oracle.NORM_FIXED if fixed else oracle.NORM_MAX_A,
                                         fixed_max=fixed or (255.0, 255.0), precision=64,
                                         kernel_width=desc.peak_kernel, num_peaks=k, nthreads=nthreads)
    else:
        ref = oracle.piv_pass(rec["wa"], rec["wb"], n, rec["at"], rec["al"], rec["bt"], rec["bl"],
                              norm_mode=oracle.NORM_FIXED if fixed else oracle.NORM_MAX_A,
                              fixed_max=fixed or (255.0, 255.0), precision=64, nthreads=nthreads)[:, None]
    gi = np.stack([vec["peak_i"], vec["peak_j"]], -1).astype(np.int32)
    ri = np.stack([ref["peak_i"], ref["peak_j"]], -1).astype(np.int32)
    absent_g = (vec["flags"] & 32) != 0
    absent_r = (ref["flags"] & 32) != 0
    differ = (gi != ri).any(-1) | (absent_g != absent_r)
    ties = 0
    tie_ias = set()
    for ia in np.nonzero(differ.any(1))[0]:
        p = _tile_planes64(oracle, rec["wa"], rec["wb"], n, rec["at"], rec["al"], rec["bt"], rec["bl"], ia, fixed)
        # an IA's peak list differs only through exact ties: every GPU peak value equals the
        # FP64 value at the oracle's peak of the same rank within the FP32 rounding level
        for s in np.nonzero(differ[ia])[0]:
            if absent_g[ia, s] or absent_r[ia, s]:
                vg = float(vec["peak_value"][ia, s]) if not absent_g[ia, s] else 0.0
                vr = float(ref["peak_value"][ia, s]) if not absent_r[ia, s] else 0.0
            else:
                vg = p[gi[ia, s, 0], gi[ia, s, 1]]
                vr = p[ri[ia, s, 0], ri[ia, s, 1]]
            if abs(vg - vr) > TIE_REL * max(abs(vr), abs(vg), 1e-30):
                raise AssertionError(f"level {rec['level']} IA {ia} slot {s}: GPU peak {tuple(gi[ia, s])} "
                                     f"(fp64 {vg}) vs oracle {tuple(ri[ia, s])} ({vr})")
        ties += 1
        tie_ias.add(int(ia))
    same = ~differ & ~absent_g
    d_i = np.abs(ref["sub_i"].astype(np.float64) - ref["peak_i"])
    d_j = np.abs(ref["sub_j"].astype(np.float64) - ref["peak_j"])
    border = (np.abs(d_i - 1.0) < BORDER) | (np.abs(d_j - 1.0) < BORDER)
    # an IA with a tie anywhere in its list may order its later slots differently
    for ia in tie_ias:
        same[ia, :] = False
    cmp = same & ~border
    err = np.maximum(np.abs(vec["u"].astype(np.float64) - ref["u64"]), np.abs(vec["v"].astype(np.float64) - ref["v64"]))
    # A flat peak (a weak secondary peak) magnifies the plane's rounding through the fit: such a
    # slot may exceed 1e-3 px, but never the error that the plane tolerance (1e-5 of the plane
    # maximum) propagates through the 3-point fit's derivatives at the FP64 stencil.
    flat = 0
    for ia, sl in np.argwhere(cmp & (err > SUBPIX_TOL)):
        p = _tile_planes64(oracle, rec["wa"], rec["wb"], n, rec["at"], rec["al"], rec["bt"], rec["bl"], ia, fixed)
        bound = gauss3_error_bound(p, int(ri[ia, sl, 0]), int(ri[ia, sl, 1]), 1e-5 * float(np.abs(p).max()))
        if not err[ia, sl] <= max(SUBPIX_TOL, bound):
            raise AssertionError(f"level {rec['level']} IA {ia} slot {sl}: sub-pixel error {err[ia, sl]:.3e} px "
                                 f"(conditioning bound {bound:.3e})")
        flat += 1
        cmp[ia, sl] = False
    worst = float(err[cmp].max(initial=0.0))
    return {"level": rec["level"], "n": n, "ias": int(vec.shape[0]), "slots": int(cmp.size),
            "compared": int(cmp.sum()), "tie_ias": ties, "border": int((same & border).sum()),
            "flat_peaks": flat, "max_err_px": worst,
            "p99_err_px": float(np.quantile(err[cmp], 0.99)) if cmp.any() else 0.0}


def gauss3_error_bound(plane, i, j, eps):
    """Largest change of the 3-point Gaussian (or parabolic fallback) sub-pixel position of the
    peak at (i, j) when every stencil value moves by up to eps: first-order, summed over the
    three values of each axis (Gaussian1DPolynomialInterpolator's formulas, +1e-8 included)."""
    d = plane.shape[0]
    if i < 1 or j < 1 or i + 1 >= d or j + 1 >= d:
        return 0.0
    worst = 0.0
    for ys in ((plane[i - 1, j], plane[i, j], plane[i + 1, j]), (plane[i, j - 1], plane[i, j], plane[i, j + 1])):
        y = np.asarray(ys, np.float64) + 1e-8
        if (y > 0).all():
            lg = np.log(y)
            num = lg[0] - lg[2]
            den = 2 * lg[0] - 4 * lg[1] + 2 * lg[2]
            g = np.array([(den - 2 * num) / den ** 2, 4 * num / den ** 2, (-den - 2 * num) / den ** 2]) / y
        else:
            num = y[0] - y[2]
            den = 2 * y[0] - 4 * y[1] + 2 * y[2]
            g = np.array([(den - 2 * num) / den ** 2, 4 * num / den ** 2, (-den - 2 * num) / den ** 2])
        worst = max(worst, float(np.abs(g).sum()) * eps)
    return worst


def check_stages(qp, oracle, recs, desc, cfg=None, nthreads=None):
    """Stage-by-stage parity of a gpu_trace; returns a list of per-level summaries."""
    fixed = None
    if desc.max_mode == qp.MAX_FIXED:
        fm = desc.fixed_max if desc.fixed_max > 0 else (255.0 if recs[0]["wa"].dtype == np.uint8 else 65535.0)
        fixed = (fm, fm)
    warp = desc.warp_mode == qp.WARP_BOTH_BILINEAR
    out = []
    prev = None
    for rec in recs:
        s = {}
        h, w = rec["wa"].shape
        if prev is not None:
            ou, ov = oracle.inherit(prev["cy"].astype(np.float64), prev["cx"].astype(np.float64), prev["u"], prev["v"],
                                    rec["cy"], rec["cx"], not warp)
            assert ou.tobytes() == rec["u_inh"].tobytes() and ov.tobytes() == rec["v_inh"].tobytes(), \
                f"level {rec['level']}: inheritance differs from the oracle"
            if warp:
                ys = rec["cy"].astype(np.float64)
                xs = rec["cx"].astype(np.float64)
                fu, fv = oracle.displacement_field(ys, xs, rec["u_in"], rec["v_in"], h, w)
                a0, b0 = recs[0]["wa"], recs[0]["wb"]
                oa, ob = oracle.warp_both(a0, b0, fu, fv, int16_quirk=bool(desc.int16_warp_quirk))
                assert oa.tobytes() == rec["wa"].tobytes() and ob.tobytes() == rec["wb"].tobytes(), \
                    f"level {rec['level']}: warped frames differ from the oracle's float formulation"
                du, dv = oracle.displacement_field(ys, xs, rec["u_in"], rec["v_in"], h, w, precision=64)
                s["field_err_px"] = float(max(np.abs(fu - du).max(), np.abs(fv - dv).max()))
                da, db = oracle.warp_both(a0, b0, du, dv, int16_quirk=bool(desc.int16_warp_quirk))
                s["warp_pixels_vs_fp64_field"] = int((da != oa).sum() + (db != ob).sum())
                s["warp_max_level_diff"] = int(max(np.abs(da.astype(np.int64) - oa).max(),
                                                   np.abs(db.astype(np.int64) - ob).max()))
        s.update(compare_pass(oracle, rec, desc, fixed, nthreads))
        if desc.validation and cfg is not None:
            k = rec["vec"].shape[1]
            ni, nj = rec["u_acc"].shape
            lcfg = type(cfg).from_buffer_copy(cfg)
            if desc.clipping_mode == 2:
                lcfg.clip_n, lcfg.clip_h, lcfg.clip_w = rec["n"], h, w
            vu, vv, vinv, _ = oracle.validate(rec["tops"], rec["lefts"], rec["u_acc"], rec["v_acc"],
                                              rec["vec"]["u"].reshape(ni, nj, k), rec["vec"]["v"].reshape(ni, nj, k),
                                              rec["npk"], lcfg)
            assert vu.tobytes() == rec["u"].tobytes() and vv.tobytes() == rec["v"].tobytes(), \
                f"level {rec['level']}: validated field differs from the oracle validator"
            assert np.array_equal(vinv.astype(bool), rec["invalid"].astype(bool))
            s["invalid_after_validation"] = int(rec["invalid"].astype(bool).sum())
        out.append(s)
        prev = rec
    return out


def oracle_levels(oracle, img_a, img_b, recs, desc, sched, cfg=None, fixed_max=None, warp=True):
    """The FP64 oracle pipeline run independently from the raw frames, with its per-level inputs
    rebuilt from its own validated fields: inherited (u_in, v_in), warped frames (or displaced B
    origins), accumulated and final (u, v), main peaks.  The rebuilt accumulation is checked
    against the pipeline's own vectors, so the intermediates are the pipeline's."""
    n0, n1, ofac = sched
    clip = desc.clipping_mode == 2
    res = oracle.piv_adaptive(img_a, img_b, n0, n1, ofac, fixed_max=fixed_max, precision=64, validation=cfg,
                              return_levels=True, warp=warp, clip_mode=desc.clipping_mode,
                              superposition_start=desc.superposition_start)
    vec = res[1]
    luv = res[2] if cfg is not None else None
    h, w = img_a.shape
    out = []
    off = 0
    prev = None
    for rec in recs:
        ni, nj = len(rec["tops"]), len(rec["lefts"])
        cnt = ni * nj
        lv = {}
        if prev is None:
            u_in = np.zeros((ni, nj), np.float32)
            v_in = np.zeros((ni, nj), np.float32)
        else:
            u_in, v_in = oracle.inherit(prev["cy"].astype(np.float64), prev["cx"].astype(np.float64), prev["u"],
                                        prev["v"], rec["cy"], rec["cx"], not warp, precision=64)
            if clip:
                ok = clip_inside(rec["tops"], rec["lefts"], rec["n"], h, w, u_in, v_in)
                u_in = np.where(ok, np.float32(0.0) + u_in, np.float32(0.0)).astype(np.float32)
                v_in = np.where(ok, np.float32(0.0) + v_in, np.float32(0.0)).astype(np.float32)
        lv["u_in"], lv["v_in"] = u_in, v_in
        wa, wb = img_a, img_b
        if warp and prev is not None:
            du, dv = oracle.displacement_field(rec["cy"].astype(np.float64), rec["cx"].astype(np.float64), u_in, v_in,
                                               h, w, precision=64)
            wa, wb = oracle.warp_both(img_a, img_b, du, dv, int16_quirk=bool(desc.int16_warp_quirk))
        lv["wa"], lv["wb"] = wa, wb
        at = np.repeat(rec["tops"], nj)
        al = np.tile(rec["lefts"], ni)
        lv["bt"] = at if warp else _java_round(at.astype(np.float32) + u_in.ravel())
        lv["bl"] = al if warp else _java_round(al.astype(np.float32) + v_in.ravel())
        v0 = vec[off:off + cnt]
        lv["peak"] = np.stack([v0["peak_i"], v0["peak_j"]], -1)
        ua = (u_in.ravel().astype(np.float64) + v0["u64"]).astype(np.float32).reshape(ni, nj)
        va = (v_in.ravel().astype(np.float64) + v0["v64"]).astype(np.float32).reshape(ni, nj)
        lv["u_acc_raw"], lv["v_acc_raw"] = ua, va
        if clip:
            ok = clip_inside(rec["tops"], rec["lefts"], rec["n"], h, w, ua, va)
            ua = np.where(ok, ua, u_in)
            va = np.where(ok, va, v_in)
        lv["u_acc"], lv["v_acc"] = ua, va
        if luv is not None:
            lv["u"] = luv[2 * off:2 * off + cnt].reshape(ni, nj)
            lv["v"] = luv[2 * off + cnt:2 * off + 2 * cnt].reshape(ni, nj)
        else:
            lv["u"], lv["v"] = ua, va
        lv["cy"], lv["cx"] = rec["cy"], rec["cx"]
        out.append(lv)
        prev = lv
        off += cnt
    if luv is None:
        fu, fv = res[0]
        assert fu.tobytes() == out[-1]["u"].tobytes() and fv.tobytes() == out[-1]["v"].tobytes(), \
            "rebuilt FP64 intermediates do not reproduce the oracle pipeline"
    return out


def cascade_report(recs, olv, desc, tol=1e-3, same_in=1e-4):
    """Classifies every last-level vector whose GPU and FP64 displacements differ by more than
    `tol`: its inputs at the last level differ (inherited value by more than `same_in`, a pixel of
    its warped A or B tile, or its displaced B origin), validation replaced it in either run, or its
    integer peak is a tie.  A vector with none of these causes is 'unexplained'; per level, the
    count of differing vectors and of their causes."""
    levels = []
    for rec, lv in zip(recs, olv):
        n = rec["n"]
        h, w = rec["wa"].shape
        err = np.maximum(np.abs(rec["u"] - lv["u"]), np.abs(rec["v"] - lv["v"])).ravel()
        d_in = np.maximum(np.abs(rec["u_in"] - lv["u_in"]), np.abs(rec["v_in"] - lv["v_in"])).ravel()
        replaced = ((rec["u"] != rec["u_acc"]) | (rec["v"] != rec["v_acc"]) |
                    (lv["u"] != lv["u_acc"]) | (lv["v"] != lv["v_acc"])).ravel()
        gpeak = np.stack([rec["vec"]["peak_i"][:, 0], rec["vec"]["peak_j"][:, 0]], -1)
        tie = (gpeak != lv["peak"]).any(-1)
        pix_a = rec["wa"] != lv["wa"]
        pix_b = rec["wb"] != lv["wb"]
        refusal_flip = np.zeros(err.size, bool)
        if desc.clipping_mode == 2:
            # NoOutOfBoundClipping: the two runs refused the increment differently (its rounded
            # sum sits on a .5 boundary)
            ng_u = (rec["u_in"].ravel() + rec["vec"]["u"][:, 0]).reshape(rec["u_in"].shape)
            ng_v = (rec["v_in"].ravel() + rec["vec"]["v"][:, 0]).reshape(rec["u_in"].shape)
            ok_g = clip_inside(rec["tops"], rec["lefts"], n, h, w, ng_u, ng_v)
            ok_o = clip_inside(rec["tops"], rec["lefts"], n, h, w, lv["u_acc_raw"], lv["v_acc_raw"])
            refusal_flip = (ok_g != ok_o).ravel()
        causes = {"inherited": 0, "pixels": 0, "validation": 0, "tie": 0, "clipping": 0, "unexplained": 0}
        unexplained = []
        for k in np.nonzero(err > tol)[0]:
            t, l_ = int(rec["at"][k]), int(rec["al"][k])
            bt, bl = int(rec["bt"][k]), int(rec["bl"][k])
            ra = pix_a[max(t, 0):max(min(t + n, h), 0), max(l_, 0):max(min(l_ + n, w), 0)].any()
            rb = pix_b[max(bt, 0):max(min(bt + n, h), 0), max(bl, 0):max(min(bl + n, w), 0)].any()
            origin = bt != int(lv["bt"][k]) or bl != int(lv["bl"][k])
            if d_in[k] > same_in:
                causes["inherited"] += 1
            elif ra or rb or origin:
                causes["pixels"] += 1
            elif replaced[k]:
                causes["validation"] += 1
            elif refusal_flip[k]:
                causes["clipping"] += 1
            elif tie[k]:
                causes["tie"] += 1
            else:
                causes["unexplained"] += 1
                unexplained.append(int(k))
        levels.append({"level": rec["level"], "vectors": int(err.size), "over_tol": int((err > tol).sum()),
                       "max_px": float(err.max()), "causes": causes, "unexplained_ias": unexplained[:10]})
    return levels
