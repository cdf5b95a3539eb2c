"""Plain per-call GPU path: the adaptive PIV loop of one frame pair driven stage by stage from
the host, every stage one synchronous library call on host arrays (inputs copied in, results
copied out), no batching across pairs and no device-resident state between stages.

This is how the reference drives its GPU jobs (`LocalPIVOpenCLGpuJob.java:188-411`: per pair and
per level, the warp, the correlation job and the validator each take host data and return host
data), and it is the denominator of the batched path's speed-up.  It runs the same kernels as
`Handle.piv_adaptive` and gives bit-identical displacements.
"""
import numpy as np

from . import (CLIP_NO_OUT_OF_BOUND, F_ABSENT, MAX_COMPUTE, MAX_FIXED, MAX_FIXED_A, MAX_FIXED_B, VALIDATE_MULTIPEAK_MEDIAN,
               VALIDATE_NONE, WARP_BOTH_BILINEAR, WARP_BOTH_MINI, WARP_FIRST_BILINEAR, WARP_FIRST_MICRO, WARP_NONE,
               WARP_SECOND_BILINEAR, adaptive_levels, grid)


def _java_round(x):
    return np.floor(x + np.float32(0.5)).astype(np.int32)


def _inside(tops, lefts, n, h, w, u, v):
    """Tile.accumulateDisplacement / replaceDisplacement bounds under NoOutOfBoundClipping
    (S/iareas/Tile.java:103-136): per tile, whether (u, v) rounded keeps the tile inside."""
    ru = np.floor(u + np.float32(0.5))
    rv = np.floor(v + np.float32(0.5))
    t = tops.astype(np.float32)[:, None]
    l_ = lefts.astype(np.float32)[None, :]
    return ~((t + ru < 0) | (t + np.float32(n) + ru >= np.float32(h)) | (l_ + rv < 0) |
             (l_ + np.float32(n) + rv >= np.float32(w)))


def piv_adaptive_per_call(handle, img_a, img_b, desc):
    """Adaptive multi-pass PIV of one pair, one library call per stage; returns (u, v) of the
    last level shaped (tiles_i, tiles_j)."""
    a = np.ascontiguousarray(img_a)
    b = np.ascontiguousarray(img_b)
    h, w = a.shape
    levels = adaptive_levels(desc, h, w)
    fm = desc.fixed_max if desc.fixed_max > 0 else (255.0 if a.dtype == np.uint8 else 65535.0)
    validate = desc.validation != VALIDATE_NONE
    multi = desc.validation == VALIDATE_MULTIPEAK_MEDIAN
    clip = desc.clipping_mode == CLIP_NO_OUT_OF_BOUND
    max_mode = desc.max_mode
    if max_mode == MAX_FIXED and desc.warp_mode == WARP_FIRST_BILINEAR:
        max_mode = MAX_FIXED_A     # tiles of the warped first frame keep the fixed maximum
    if max_mode == MAX_FIXED and desc.warp_mode == WARP_SECOND_BILINEAR:
        max_mode = MAX_FIXED_B
    pass_kw = dict(norm_mode=desc.norm_mode, max_mode=max_mode, fixed_max=(fm, fm),
                   subpix_mode=desc.subpix_mode)
    if multi:
        pass_kw.update(num_peaks=desc.num_peaks, peak_kernel=desc.peak_kernel)
    margins = list(desc.margins)
    prev = None
    for lv, g in enumerate(levels):
        n = g["n"]
        st = grid.level(h, w, desc.ia_start, lv, desc.overlap_factor, margins,
                        superposition_start=desc.superposition_start)
        assert (st.n, st.tiles_i, st.tiles_j) == (n, g["tiles_i"], g["tiles_j"])
        tops = np.asarray(st.tops, np.int32)
        lefts = np.asarray(st.lefts, np.int32)
        cy, cx = st.centres()
        ni, nj = len(tops), len(lefts)
        if prev is None:
            u = np.zeros((ni, nj), np.float32)
            v = np.zeros((ni, nj), np.float32)
        else:
            pcy, pcx, pu, pv, pn, ptops, plefts = prev
            rnd = desc.warp_mode == WARP_NONE
            if desc.inherit_mode == 0:
                u, v = handle.inherit(pcy, pcx, pu, pv, cy, cx, round_int=rnd)
            else:
                u, v = handle.inherit_tiles(desc.inherit_mode, pn, ptops, plefts, pu, pv, n, tops, lefts,
                                            round_int=rnd)
            if clip:   # the new tiles take the inherited value through accumulateDisplacement
                u = np.float32(0.0) + u
                v = np.float32(0.0) + v
                ok = _inside(tops, lefts, n, h, w, u, v)
                u = np.where(ok, u, np.float32(0.0)).astype(np.float32)
                v = np.where(ok, v, np.float32(0.0)).astype(np.float32)
        at = np.repeat(tops, nj)
        al = np.tile(lefts, ni)
        src_a, src_b = a, b
        bt, bl = at, al
        per_tile = WARP_FIRST_MICRO <= desc.warp_mode <= WARP_BOTH_MINI
        if per_tile:
            if lv > 0:   # warped tiles with their maxima, through the tile entry points
                ta, tb, ma, mb = handle.tile_warp(a, b, n, tops, lefts, u, v, desc.warp_mode, fm)
                tkw = dict(norm_mode=desc.norm_mode, subpix_mode=desc.subpix_mode)
                vec = handle.xcorr_multipeaks(ta, tb, ma, mb, num_peaks=desc.num_peaks, peak_kernel=desc.peak_kernel,
                                              **tkw) if multi else handle.xcorr_peaks(ta, tb, ma, mb, **tkw)
            else:        # level 0: both tiles clipped with their own maxima
                vec = handle.piv_pass(a, b, n, at, al, **dict(pass_kw, max_mode=MAX_COMPUTE))
        elif desc.warp_mode in (WARP_BOTH_BILINEAR, WARP_FIRST_BILINEAR, WARP_SECOND_BILINEAR):
            if lv > 0:
                src_a, src_b = handle.warp_pair(a, b, cy.astype(np.float64), cx.astype(np.float64), u, v,
                                                int16_quirk=bool(desc.int16_warp_quirk), warp_mode=desc.warp_mode)
        else:
            bt = _java_round(at.astype(np.float32) + u.ravel())
            bl = _java_round(al.astype(np.float32) + v.ravel())
        if not per_tile:
            vec = handle.piv_pass(src_a, src_b, n, at, al, bt, bl, **pass_kw)
        main = vec[:, 0] if vec.ndim == 2 else vec
        nu = (u.ravel() + main["u"]).reshape(ni, nj).astype(np.float32)
        nv = (v.ravel() + main["v"]).reshape(ni, nj).astype(np.float32)
        if clip:   # accumulateDisplacement drops an increment that moves the tile out of the image
            ok = _inside(tops, lefts, n, h, w, nu, nv)
            nu = np.where(ok, nu, u)
            nv = np.where(ok, nv, v)
        u, v = nu, nv
        if validate:
            if multi:
                present = (vec["flags"] & F_ABSENT) == 0
                npk = present.sum(axis=1).astype(np.int32).reshape(ni, nj)
                k = desc.num_peaks
                pk = (vec["u"].reshape(ni, nj, k), vec["v"].reshape(ni, nj, k), npk)
            else:
                pk = (None, None, None)
            u, v, _ = handle.validate(tops, lefts, u, v, *pk, desc, n=n, height=h, width=w)
        prev = (cy, cx, u, v, n, tops, lefts)
    return prev[2], prev[3]
