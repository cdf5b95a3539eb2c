"""ctypes front-end of the CPU oracle (oracle/qlpiv_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
legs of bench.py, as the checker or the timed CPU baseline.  The product never
imports this module.
"""
import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libqlpiv_oracle.so"

# orc_vector (48 bytes): the product's qlpiv_vector (first 32 bytes) plus the
# double-precision displacement of the FP64 twin.
VECTOR_DTYPE = np.dtype([
    ("u", "<f4"), ("v", "<f4"), ("sub_i", "<f4"), ("sub_j", "<f4"),
    ("peak_value", "<f4"), ("min_floor", "<f4"), ("peak_i", "<i2"), ("peak_j", "<i2"),
    ("flags", "<u4"), ("u64", "<f8"), ("v64", "<f8"),
])

F_SUB_I, F_SUB_J, F_PARABOLIC, F_EDGE, F_NO_PEAK = 1, 2, 4, 8, 16

NORM_MAX_A, NORM_OWN_MAX, NORM_FIXED, NORM_NONE = 0, 1, 2, 3

_lib = None


class ValidCfg(ctypes.Structure):
    """orc_valid_cfg: validation model and settings.  model 1: multi-peak normalised median
    (num_peaks strategies); 2 / 3: difference validator without / with bilinear replacement;
    4 / 5: normalised median without / with bilinear replacement.  clip_n / clip_h / clip_w:
    NoOutOfBoundClipping bounds of the replacements (clip_n 0: clipping allowed)."""
    _fields_ = [("enabled", ctypes.c_int), ("num_peaks", ctypes.c_int), ("kernel_width", ctypes.c_int),
                ("threshold", ctypes.c_float), ("epsilon0", ctypes.c_float), ("max_iterations", ctypes.c_int),
                ("iterate_until_no_corrections", ctypes.c_int), ("model", ctypes.c_int), ("clip_n", ctypes.c_int),
                ("clip_h", ctypes.c_int), ("clip_w", ctypes.c_int)]


MODEL_MULTIPEAK_MEDIAN, MODEL_DIFFERENCE_ONLY, MODEL_DIFFERENCE, MODEL_MEDIAN_ONLY, MODEL_MEDIAN = 1, 2, 3, 4, 5


def valid_cfg(num_peaks=3, kernel_width=3, threshold=2.0, epsilon0=0.1, max_iterations=2,
              iterate_until_no_corrections=False, model=MODEL_MULTIPEAK_MEDIAN, clip=None):
    """clip: None (clipping allowed) or (tile side, image height, image width) for
    NoOutOfBoundClipping."""
    cn, ch, cw = clip if clip is not None else (0, 0, 0)
    return ValidCfg(1, num_peaks if model == MODEL_MULTIPEAK_MEDIAN else 1, kernel_width, threshold, epsilon0,
                    max_iterations, int(iterate_until_no_corrections), model, cn, ch, cw)


def build(force=False):
    """Compile the oracle with its Makefile (gcc only; seconds)."""
    src = [HERE / "qlpiv_oracle.c", HERE / "qlpiv_oracle_adaptive.c", HERE / "qlpiv_oracle_validate.c", HERE / "qlpiv_oracle_dense.c",
           HERE / "oracle_types.h", HERE / "oracle_impl.h", HERE / "oracle_interp_impl.h", HERE / "oracle_dense_impl.h",
           HERE / "Makefile"]
    if not force and LIB_PATH.exists() and all(LIB_PATH.stat().st_mtime >= s.stat().st_mtime for s in src):
        return LIB_PATH
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        vp = ctypes.c_void_p
        c_int, c_float, c_long = ctypes.c_int, ctypes.c_float, ctypes.c_long
        L.orc_xcorr_fft_f32.argtypes = [fp, fp, c_int, c_float, c_float, c_int, fp]
        L.orc_xcorr_fft_f64.argtypes = [fp, fp, c_int, c_float, c_float, c_int, dp]
        L.orc_xcorr_direct_f64.argtypes = [fp, fp, c_int, c_float, c_float, c_int, dp]
        L.orc_find_max_from_center_f32.argtypes = [fp, c_int, c_int, ip, ip, fp, fp]
        L.orc_find_max_from_center_f64.argtypes = [dp, c_int, c_int, ip, ip, dp, dp]
        L.orc_subpixel_gauss3_f32.argtypes = [fp, c_int, c_int, c_int, c_int, fp, fp, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_gauss_lm_fit.argtypes = [dp, dp, c_int, dp]
        L.orc_gauss_lm_fit.restype = c_int
        L.orc_hongwei_guo_fit.argtypes = [fp, fp, c_int, c_int, fp, fp]
        L.orc_hongwei_guo_fit.restype = c_int
        L.orc_subpixel_lm.argtypes = [fp, c_int, c_int, c_int, c_int, c_float, fp, fp, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_subpixel_hg.argtypes = [fp, c_int, c_int, c_int, c_int, c_int, c_float, fp, fp, fp,
                                      ctypes.POINTER(ctypes.c_uint32)]
        L.orc_subpixel_gauss3_f64.argtypes = [dp, c_int, c_int, c_int, c_int, dp, dp, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_clip_tile.argtypes = [vp, c_int, c_int, c_int, c_int, c_int, c_int, fp]
        L.orc_clip_tile.restype = c_float
        L.orc_grid_superposition.argtypes = [c_int] * 8 + [c_float, vp, ip, ip, c_int]
        L.orc_grid_nosuperposition.argtypes = [c_int] * 8 + [vp, ip, ip, c_int]
        L.orc_piv_pass.argtypes = [vp, vp, c_int, c_int, c_int, c_int, c_long, ip, ip, ip, ip, c_int,
                                   c_float, c_float, c_int, c_int, vp, c_int]
        L.orc_displacement_field.argtypes = [dp, c_int, dp, c_int, fp, fp, c_int, c_int, c_int, fp, fp]
        L.orc_tile_warp.argtypes = [vp, vp, c_int, c_int, c_int, c_int, c_int, c_int, ip, ip, fp, fp, c_int, c_int,
                                    c_float, vp, vp, vp, vp]
        L.orc_displacement_field_off.argtypes = [dp, c_int, dp, c_int, fp, fp, c_int, c_int, c_int, c_float, c_float,
                                                 fp, fp]
        L.orc_warp_both.argtypes = [vp, vp, c_int, c_int, c_int, fp, fp, c_int, vp, vp]
        L.orc_warp_full.argtypes = [vp, vp, c_int, c_int, c_int, fp, fp, c_int, c_int, vp, vp]
        L.orc_inherit.argtypes = [dp, c_int, dp, c_int, fp, fp, fp, c_int, fp, c_int, c_int, c_int, fp, fp]
        L.orc_piv_adaptive.argtypes = [vp, vp, c_int, c_int, c_int, c_int, c_int, c_float, c_int, c_int, c_float,
                                       c_int, c_int, c_int, fp, fp, ip, ip, vp]
        L.orc_piv_pass_multi.argtypes = [vp, vp, c_int, c_int, c_int, c_int, c_long, ip, ip, ip, ip, c_int,
                                         c_float, c_float, c_int, c_int, c_int, c_int, vp, ip, c_int]
        L.orc_find_max_multipeaks_f32.argtypes = [fp, c_int, c_int, c_int, c_int, ip, ip, fp, fp]
        L.orc_mp_list_run.argtypes = [c_int, c_int, c_int, fp, ip, ip, fp, ip, ip]
        L.orc_spiral_order.argtypes = [c_int, c_int, ip]
        L.orc_validate.argtypes = [c_int, c_int, ip, ip, fp, fp, fp, fp, ip, c_int, ctypes.POINTER(ValidCfg), vp]
        L.orc_piv_adaptive_ex.argtypes = [vp, vp, c_int, c_int, c_int, c_int, c_int, c_float, c_int, c_int, c_int,
                                          c_int, c_float, c_int, c_int, c_int, ctypes.POINTER(ValidCfg), fp, fp, ip,
                                          ip, vp, vp, vp, c_int, c_int, c_float]
        L.orc_inherit_tiles.argtypes = [c_int, c_int, c_int, c_int, ip, ip, fp, fp, c_int, c_int, c_int, ip, ip, c_int,
                                        fp, fp]
        L.orc_area_overlap.argtypes = [c_int, c_int, c_int, c_int, c_int, c_int, ip]
        L.orc_area_overlap.restype = c_float
        for sfx, real in (("", c_float), ("_f64", ctypes.c_double)):
            getattr(L, "orc_gauss_kernel" + sfx).argtypes = [c_float, c_int, vp]
            getattr(L, "orc_gauss_filter" + sfx).argtypes = [vp, c_int, c_int, vp, c_int, vp]
            getattr(L, "orc_normalize" + sfx).argtypes = [vp, c_long, vp]
            getattr(L, "orc_dense_lk" + sfx).argtypes = [vp, vp, c_int, c_int, vp, vp, c_int, c_int, c_int]
            getattr(L, "orc_liu_shen" + sfx).argtypes = [vp, vp, c_int, c_int, vp, vp, real, c_int, c_int, vp, vp,
                                                         vp]
            getattr(L, "orc_flow_after_piv" + sfx).argtypes = [fp, fp, c_int, c_int, c_int, c_int, c_int, ip, ip, fp,
                                                               fp, c_int, c_float, c_int, c_float, c_int, c_int, c_int,
                                                               c_float, c_int, c_int, c_int, c_int, c_int, vp, vp]
            getattr(L, "orc_dense_lk_pyramid" + sfx).argtypes = [vp, vp, c_int, c_int, vp, vp, c_int, c_int, c_int,
                                                                 c_int]
        L.orc_vector_size.restype = c_int
        assert L.orc_vector_size() == VECTOR_DTYPE.itemsize
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def xcorr_fft(ta, tb, max_a, max_b, normalize=True, precision=32):
    """(2N-1)^2 correlation plane by the restated SimpleFFT path."""
    ta, tb = _f32(ta), _f32(tb)
    n = ta.shape[0]
    d = 2 * n - 1
    if precision == 32:
        out = np.zeros((d, d), np.float32)
        lib().orc_xcorr_fft_f32(_ptr(ta, ctypes.c_float), _ptr(tb, ctypes.c_float), n, max_a, max_b,
                                int(normalize), _ptr(out, ctypes.c_float))
    else:
        out = np.zeros((d, d), np.float64)
        lib().orc_xcorr_fft_f64(_ptr(ta, ctypes.c_float), _ptr(tb, ctypes.c_float), n, max_a, max_b,
                                int(normalize), _ptr(out, ctypes.c_double))
    return out


def xcorr_direct(ta, tb, max_a, max_b, normalize=True):
    ta, tb = _f32(ta), _f32(tb)
    n = ta.shape[0]
    out = np.zeros((2 * n - 1, 2 * n - 1), np.float64)
    lib().orc_xcorr_direct_f64(_ptr(ta, ctypes.c_float), _ptr(tb, ctypes.c_float), n, max_a, max_b,
                               int(normalize), _ptr(out, ctypes.c_double))
    return out


def find_max_from_center(plane):
    plane = np.ascontiguousarray(plane)
    di, dj = plane.shape
    oi, oj = ctypes.c_int(), ctypes.c_int()
    if plane.dtype == np.float32:
        ov, om = ctypes.c_float(), ctypes.c_float()
        lib().orc_find_max_from_center_f32(_ptr(plane, ctypes.c_float), di, dj, ctypes.byref(oi),
                                           ctypes.byref(oj), ctypes.byref(ov), ctypes.byref(om))
    else:
        plane = plane.astype(np.float64)
        ov, om = ctypes.c_double(), ctypes.c_double()
        lib().orc_find_max_from_center_f64(_ptr(plane, ctypes.c_double), di, dj, ctypes.byref(oi),
                                           ctypes.byref(oj), ctypes.byref(ov), ctypes.byref(om))
    return oi.value, oj.value, ov.value, om.value


SUBPIX_NONE, SUBPIX_GAUSS3, SUBPIX_GAUSS_LM, SUBPIX_HONGWEI_GUO = 0, 1, 2, 3


def subpix_code(mode, pixels=3, iterations=20):
    """The packed sub-pixel argument of the oracle's passes."""
    return int(mode) | (int(pixels) << 8) | (int(iterations) << 16)


def gauss_lm_fit(x, y):
    """Least-squares Gaussian mean of (x, y) (Levenberg-Marquardt), or None."""
    x, y = _f64(x), _f64(y)
    m = ctypes.c_double()
    ok = lib().orc_gauss_lm_fit(_ptr(x, ctypes.c_double), _ptr(y, ctypes.c_double), len(x), ctypes.byref(m))
    return m.value if ok else None


def hongwei_guo_fit(xs, ys, iterations):
    """Hongwei Guo weighted log fit: (mean, amplitude) or None when singular."""
    xs, ys = _f32(xs), _f32(ys)
    m, a = ctypes.c_float(), ctypes.c_float()
    ok = lib().orc_hongwei_guo_fit(_ptr(xs, ctypes.c_float), _ptr(ys, ctypes.c_float), len(xs), iterations,
                                   ctypes.byref(m), ctypes.byref(a))
    return (m.value, a.value) if ok else None


def subpixel_lm(plane, mi, mj, pixels, min_floor=0.0):
    """Gaussian1DInterpolator on a float plane: (sub_i, sub_j, flags)."""
    plane = _f32(plane)
    si, sj, fl = ctypes.c_float(), ctypes.c_float(), ctypes.c_uint32()
    lib().orc_subpixel_lm(_ptr(plane, ctypes.c_float), plane.shape[0], mi, mj, pixels, min_floor, ctypes.byref(si),
                          ctypes.byref(sj), ctypes.byref(fl))
    return si.value, sj.value, fl.value


def subpixel_hg(plane, mi, mj, pixels, iterations, peak_value, min_floor=0.0):
    """Gaussian1DHongweiGuoInterpolator on a float plane: (sub_i, sub_j, peak_value, flags)."""
    plane = _f32(plane)
    si, sj, fl = ctypes.c_float(), ctypes.c_float(), ctypes.c_uint32()
    pv = ctypes.c_float(peak_value)
    lib().orc_subpixel_hg(_ptr(plane, ctypes.c_float), plane.shape[0], mi, mj, pixels, iterations, min_floor,
                          ctypes.byref(si), ctypes.byref(sj), ctypes.byref(pv), ctypes.byref(fl))
    return si.value, sj.value, pv.value, fl.value


def subpixel_gauss3(plane, mi, mj):
    plane = np.ascontiguousarray(plane)
    di, dj = plane.shape
    fl = ctypes.c_uint32()
    if plane.dtype == np.float32:
        pi, pj = ctypes.c_float(), ctypes.c_float()
        lib().orc_subpixel_gauss3_f32(_ptr(plane, ctypes.c_float), di, dj, mi, mj, ctypes.byref(pi),
                                      ctypes.byref(pj), ctypes.byref(fl))
    else:
        plane = plane.astype(np.float64)
        pi, pj = ctypes.c_double(), ctypes.c_double()
        lib().orc_subpixel_gauss3_f64(_ptr(plane, ctypes.c_double), di, dj, mi, mj, ctypes.byref(pi),
                                      ctypes.byref(pj), ctypes.byref(fl))
    return pi.value, pj.value, fl.value


def clip_tile(img, top, left, n):
    img = np.ascontiguousarray(img)
    tile = np.zeros((n, n), np.float32)
    mx = lib().orc_clip_tile(img.ctypes.data, img.shape[0], img.shape[1], img.dtype.itemsize, top, left, n,
                             _ptr(tile, ctypes.c_float))
    return tile, mx


class _Grid(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in
                ("n", "tiles_i", "tiles_j", "margin_top", "margin_left", "margin_bottom", "margin_right")]


def level_grid(h, w, n_start, level, overlap_factor=0.5, margins=(0, 0, 0, 0), superposition_start=0):
    """Grid of one level under the mixed division: NoSuperPosition before superposition_start,
    then SuperPosition restarted with IA n_start >> superposition_start
    (AdaptiveInterAreaStrategyMixedSuperPosition.java:31-92)."""
    if level < superposition_start:
        return grid(h, w, n_start, level, overlap_factor, margins, superposition=False)
    return grid(h, w, n_start >> superposition_start, level - superposition_start, overlap_factor, margins)


def grid(h, w, n_start, level=0, overlap_factor=0.5, margins=(0, 0, 0, 0), superposition=True):
    """IA grid of one adaptive level.  margins = (top, bottom, left, right).
    Returns (dict of grid scalars, tops[tiles_i], lefts[tiles_j])."""
    cap = 65536
    tops = np.zeros(cap, np.int32)
    lefts = np.zeros(cap, np.int32)
    g = _Grid()
    mt, mb, ml, mr = margins
    if superposition:
        rc = lib().orc_grid_superposition(h, w, mt, mb, ml, mr, n_start, level, overlap_factor, ctypes.byref(g),
                                          _ptr(tops, ctypes.c_int), _ptr(lefts, ctypes.c_int), cap)
    else:
        rc = lib().orc_grid_nosuperposition(h, w, mt, mb, ml, mr, n_start, level, ctypes.byref(g),
                                            _ptr(tops, ctypes.c_int), _ptr(lefts, ctypes.c_int), cap)
    if rc != 0:
        raise ValueError("grid too large")
    d = {k: getattr(g, k) for k, _ in _Grid._fields_}
    return d, tops[:g.tiles_i].copy(), lefts[:g.tiles_j].copy()


def piv_pass(img_a, img_b, n, a_top, a_left, b_top=None, b_left=None, norm_mode=NORM_MAX_A,
             fixed_max=(255.0, 255.0), subpix=True, precision=32, nthreads=None):
    """One correlation pass over all IAs (vectors in IA order)."""
    img_a = np.ascontiguousarray(img_a)
    img_b = np.ascontiguousarray(img_b)
    assert img_a.dtype == img_b.dtype and img_a.dtype in (np.uint8, np.uint16)
    a_top = np.ascontiguousarray(a_top, np.int32)
    a_left = np.ascontiguousarray(a_left, np.int32)
    b_top = a_top if b_top is None else np.ascontiguousarray(b_top, np.int32)
    b_left = a_left if b_left is None else np.ascontiguousarray(b_left, np.int32)
    count = a_top.shape[0]
    out = np.zeros(count, VECTOR_DTYPE)
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    lib().orc_piv_pass(img_a.ctypes.data, img_b.ctypes.data, img_a.shape[0], img_a.shape[1], img_a.dtype.itemsize,
                       n, count, _ptr(a_top, ctypes.c_int), _ptr(a_left, ctypes.c_int), _ptr(b_top, ctypes.c_int),
                       _ptr(b_left, ctypes.c_int), norm_mode, fixed_max[0], fixed_max[1], int(subpix),
                       0 if precision == 32 else 1, out.ctypes.data, nthreads)
    return out


def grid_origins(h, w, n, overlap_factor=0.5, level=0, n_start=None, margins=(0, 0, 0, 0), superposition=True):
    """Flattened (row-major) tile origins of one grid."""
    g, tops, lefts = grid(h, w, n if n_start is None else n_start, level, overlap_factor, margins, superposition)
    tt, ll = np.meshgrid(tops, lefts, indexing="ij")
    return g, tt.ravel().astype(np.int32), ll.ravel().astype(np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


WARP_FIRST_BILINEAR, WARP_SECOND_BILINEAR = 2, 3
WARP_FIRST_MICRO, WARP_SECOND_MICRO, WARP_BOTH_MICRO, WARP_FIRST_MINI, WARP_SECOND_MINI, WARP_BOTH_MINI = range(4, 10)


def tile_warp(img_a, img_b, n, tops, lefts, u, v, warp_mode, full_max):
    """Micro / mini per-tile warping: (tiles_a, tiles_b, max_a, max_b), float tiles."""
    img_a, img_b = np.ascontiguousarray(img_a), np.ascontiguousarray(img_b)
    tops = np.ascontiguousarray(tops, np.int32)
    lefts = np.ascontiguousarray(lefts, np.int32)
    u, v = _f32(u), _f32(v)
    cnt = len(tops) * len(lefts)
    ta = np.zeros((cnt, n, n), np.float32)
    tb = np.zeros_like(ta)
    ma = np.zeros(cnt, np.float32)
    mb = np.zeros(cnt, np.float32)
    lib().orc_tile_warp(img_a.ctypes.data, img_b.ctypes.data, img_a.shape[0], img_a.shape[1], img_a.dtype.itemsize, n,
                        len(tops), len(lefts), _ptr(tops, ctypes.c_int), _ptr(lefts, ctypes.c_int),
                        _ptr(u, ctypes.c_float), _ptr(v, ctypes.c_float), (warp_mode - 4) % 3 + 1,
                        int(warp_mode >= 7), float(full_max), ta.ctypes.data, tb.ctypes.data, ma.ctypes.data,
                        mb.ctypes.data)
    return ta, tb, ma, mb


def displacement_field(ys, xs, u, v, h, w, precision=32, offset=0.0):
    """Per-pixel (u, v) from tile displacements at tile centres (bicubic spline), evaluated
    in float (precision=32, the CUDA formulation) or double, pixel (i, j) at (i, j) + offset."""
    ys, xs = _f64(ys), _f64(xs)
    u, v = _f32(u), _f32(v)
    fu = np.zeros((h, w), np.float32)
    fv = np.zeros((h, w), np.float32)
    lib().orc_displacement_field_off(_ptr(ys, ctypes.c_double), len(ys), _ptr(xs, ctypes.c_double), len(xs),
                                     _ptr(u, ctypes.c_float), _ptr(v, ctypes.c_float), h, w,
                                     0 if precision == 32 else 1, offset, offset, _ptr(fu, ctypes.c_float),
                                     _ptr(fv, ctypes.c_float))
    return fu, fv


def warp_both(img_a, img_b, fu, fv, int16_quirk=False, image_mode=3):
    """Full-image warp: image_mode 3 both frames by half the field, 1 frame A, 2 frame B by the
    whole field (the other frame copied)."""
    img_a, img_b = np.ascontiguousarray(img_a), np.ascontiguousarray(img_b)
    fu, fv = _f32(fu), _f32(fv)
    oa, ob = np.zeros_like(img_a), np.zeros_like(img_b)
    lib().orc_warp_full(img_a.ctypes.data, img_b.ctypes.data, img_a.shape[0], img_a.shape[1], img_a.dtype.itemsize,
                        _ptr(fu, ctypes.c_float), _ptr(fv, ctypes.c_float), int(int16_quirk), int(image_mode),
                        oa.ctypes.data, ob.ctypes.data)
    return oa, ob


def inherit(py, px, pu, pv, cy, cx, round_int=False, precision=32):
    py, px = _f64(py), _f64(px)
    pu, pv, cy, cx = _f32(pu), _f32(pv), _f32(cy), _f32(cx)
    cu = np.zeros((len(cy), len(cx)), np.float32)
    cv = np.zeros((len(cy), len(cx)), np.float32)
    lib().orc_inherit(_ptr(py, ctypes.c_double), len(py), _ptr(px, ctypes.c_double), len(px), _ptr(pu, ctypes.c_float),
                      _ptr(pv, ctypes.c_float), _ptr(cy, ctypes.c_float), len(cy), _ptr(cx, ctypes.c_float), len(cx),
                      int(round_int), 0 if precision == 32 else 1, _ptr(cu, ctypes.c_float),
                      _ptr(cv, ctypes.c_float))
    return cu, cv


INHERIT_BICUBIC_SPLINE, INHERIT_DIRECT, INHERIT_AREA, INHERIT_DISTANCE = range(4)


def inherit_tiles(mode, pn, p_tops, p_lefts, pu, pv, cn, c_tops, c_lefts, round_int=False):
    """Direct / Area / Distance inheritance by the reference's serial walk; raises ValueError
    where the reference throws."""
    p_tops = np.ascontiguousarray(p_tops, np.int32)
    p_lefts = np.ascontiguousarray(p_lefts, np.int32)
    c_tops = np.ascontiguousarray(c_tops, np.int32)
    c_lefts = np.ascontiguousarray(c_lefts, np.int32)
    pu, pv = _f32(pu), _f32(pv)
    cu = np.zeros((len(c_tops), len(c_lefts)), np.float32)
    cv = np.zeros_like(cu)
    rc = lib().orc_inherit_tiles(mode, pn, len(p_tops), len(p_lefts), _ptr(p_tops, ctypes.c_int),
                                 _ptr(p_lefts, ctypes.c_int), _ptr(pu, ctypes.c_float), _ptr(pv, ctypes.c_float), cn,
                                 len(c_tops), len(c_lefts), _ptr(c_tops, ctypes.c_int), _ptr(c_lefts, ctypes.c_int),
                                 int(round_int), _ptr(cu, ctypes.c_float), _ptr(cv, ctypes.c_float))
    if rc != 0:
        raise ValueError(f"the reference's inheritance walk throws here (code {rc})")
    return cu, cv


def area_overlap(parent_top, parent_left, pn, top, left, n):
    """checkOverlappingFactor: (factor, up, down, left, right)."""
    fl = ctypes.c_int()
    f = lib().orc_area_overlap(parent_top, parent_left, pn, top, left, n, ctypes.byref(fl))
    return float(f), bool(fl.value & 1), bool(fl.value & 2), bool(fl.value & 4), bool(fl.value & 8)


CLIP_ALLOWED, CLIP_LOGGED, CLIP_NO_OUT_OF_BOUND = 0, 1, 2


def piv_adaptive(img_a, img_b, n_start, n_end, overlap_factor, norm_mode=NORM_MAX_A, fixed_max=None,
                 int16_quirk=False, precision=32, nthreads=None, return_levels=False, warp=True, validation=None,
                 inherit=INHERIT_BICUBIC_SPLINE, clip_mode=CLIP_ALLOWED, superposition_start=0, stable_max=None,
                 stable_retries=1):
    """Adaptive multi-pass PIV (warp: False none, True BothImages bilinear, or a micro / mini mode
    4..9 as WARP_*); returns (u, v) of
    the last level, shaped (tiles_i, tiles_j), and optionally all levels' vectors.
    superposition_start: the mixed division's first SuperPosition level (level_grid).
    stable_max / stable_retries: InterAreaDisplacementStableStrategy (passes repeated per level
    while a tile's increment exceeds stable_max, at most stable_retries passes; no validation).
    validation: a ValidCfg (multi-peak finder + normalised-median validation per level);
    with return_levels the result also carries every level's validated (u, v) and
    invalid flags."""
    img_a, img_b = np.ascontiguousarray(img_a), np.ascontiguousarray(img_b)
    h, w = img_a.shape
    cap = 65536 * 16
    u = np.zeros(cap, np.float32)
    v = np.zeros(cap, np.float32)
    ni, nj = ctypes.c_int(), ctypes.c_int()
    total = 0
    lv, n = 0, n_start
    while n >= n_end:
        g, _, _ = level_grid(h, w, n_start, lv, overlap_factor, superposition_start=superposition_start)
        total += g["tiles_i"] * g["tiles_j"]
        n >>= 1
        lv += 1
    vec = np.zeros(total, VECTOR_DTYPE) if return_levels else None
    luv = np.zeros(2 * total, np.float32) if return_levels else None
    linv = np.zeros(total, np.uint8) if return_levels else None
    cfg = validation if validation is not None else ValidCfg(0, 0, 0, 0.0, 0.0, 0, 0, 0, 0, 0, 0)
    rc = lib().orc_piv_adaptive_ex(img_a.ctypes.data, img_b.ctypes.data, h, w, img_a.dtype.itemsize, n_start, n_end,
                                   overlap_factor, int(warp), int(inherit), int(clip_mode), norm_mode,
                                   float(fixed_max or 0.0),
                                   int(int16_quirk),
                                   0 if precision == 32 else 1, nthreads or (os.cpu_count() or 1), ctypes.byref(cfg),
                                   _ptr(u, ctypes.c_float), _ptr(v, ctypes.c_float), ctypes.byref(ni),
                                   ctypes.byref(nj), vec.ctypes.data if vec is not None else None,
                                   luv.ctypes.data if luv is not None else None,
                                   linv.ctypes.data if linv is not None else None, int(superposition_start),
                                   int(stable_retries) if stable_max is not None else 1,
                                   float(stable_max or 0.0))
    if rc != 0:
        raise ValueError("adaptive PIV failed")
    shape = (ni.value, nj.value)
    out = (u[:ni.value * nj.value].reshape(shape).copy(), v[:ni.value * nj.value].reshape(shape).copy())
    if not return_levels:
        return out
    if validation is None:
        return out, vec
    return out, vec, luv, linv


def piv_pass_multi(img_a, img_b, n, a_top, a_left, b_top=None, b_left=None, norm_mode=NORM_MAX_A,
                   fixed_max=(255.0, 255.0), subpix=True, precision=32, kernel_width=3, num_peaks=3, nthreads=None):
    """One pass with FindMaximumMultiPeaks: vectors shaped (count, num_peaks), largest
    peak first, and the number of peaks found per IA."""
    img_a = np.ascontiguousarray(img_a)
    img_b = np.ascontiguousarray(img_b)
    assert img_a.dtype == img_b.dtype and img_a.dtype in (np.uint8, np.uint16)
    a_top = np.ascontiguousarray(a_top, np.int32)
    a_left = np.ascontiguousarray(a_left, np.int32)
    b_top = a_top if b_top is None else np.ascontiguousarray(b_top, np.int32)
    b_left = a_left if b_left is None else np.ascontiguousarray(b_left, np.int32)
    count = a_top.shape[0]
    out = np.zeros((count, num_peaks), VECTOR_DTYPE)
    npk = np.zeros(count, np.int32)
    rc = lib().orc_piv_pass_multi(img_a.ctypes.data, img_b.ctypes.data, img_a.shape[0], img_a.shape[1],
                                  img_a.dtype.itemsize, n, count, _ptr(a_top, ctypes.c_int),
                                  _ptr(a_left, ctypes.c_int), _ptr(b_top, ctypes.c_int), _ptr(b_left, ctypes.c_int),
                                  norm_mode, fixed_max[0], fixed_max[1], int(subpix), 0 if precision == 32 else 1,
                                  kernel_width, num_peaks, out.ctypes.data, _ptr(npk, ctypes.c_int),
                                  nthreads or (os.cpu_count() or 1))
    if rc != 0:
        raise ValueError("bad multi-peak settings")
    return out, npk


def find_max_multipeaks(plane, kernel_width, num_peaks):
    """FindMaximumMultiPeaks on one plane: [(i, j, value), ...] largest first, minFloor."""
    p = _f32(plane)
    oi = np.zeros(64, np.int32)
    oj = np.zeros(64, np.int32)
    ov = np.zeros(64, np.float32)
    mf = np.zeros(1, np.float32)
    n = lib().orc_find_max_multipeaks_f32(_ptr(p, ctypes.c_float), p.shape[0], p.shape[1], kernel_width, num_peaks,
                                          _ptr(oi, ctypes.c_int), _ptr(oj, ctypes.c_int), _ptr(ov, ctypes.c_float),
                                          _ptr(mf, ctypes.c_float))
    if n < 0:
        raise ValueError("bad multi-peak settings")
    return [(int(oi[r]), int(oj[r]), float(ov[r])) for r in range(n)], float(mf[0])


def mp_list_run(max_size, kernel_width, entries):
    """SimpleFixedLengthFloatLinkedList: addInAscendOrder of every (value, i, j); returns the
    list in ascending order."""
    v = _f32([e[0] for e in entries])
    i = np.ascontiguousarray([e[1] for e in entries], np.int32)
    j = np.ascontiguousarray([e[2] for e in entries], np.int32)
    ov = np.zeros(65, np.float32)
    oi = np.zeros(65, np.int32)
    oj = np.zeros(65, np.int32)
    n = lib().orc_mp_list_run(max_size, kernel_width, len(entries), _ptr(v, ctypes.c_float), _ptr(i, ctypes.c_int),
                              _ptr(j, ctypes.c_int), _ptr(ov, ctypes.c_float), _ptr(oi, ctypes.c_int),
                              _ptr(oj, ctypes.c_int))
    return [(float(ov[r]), int(oi[r]), int(oj[r])) for r in range(n)]


def spiral_order(ni, nj):
    """VectorValidatorJob.circularVisitor visit order (flat tile indices)."""
    order = np.zeros(ni * nj, np.int32)
    n = lib().orc_spiral_order(ni, nj, _ptr(order, ctypes.c_int))
    return order[:n]


def validate(tops, lefts, u, v, peak_u, peak_v, npeaks, cfg):
    """Multi-peak normalised-median validation of one frame's tiles.  u, v: (ni, nj)
    accumulated displacements (main peak included); peak_u/peak_v: (ni, nj, k) peak
    increments; npeaks: (ni, nj).  Returns validated (u, v), invalid flags, sweeps."""
    u = _f32(u).copy()
    v = _f32(v).copy()
    ni, nj = u.shape
    k = peak_u.shape[-1]
    tops = np.ascontiguousarray(tops, np.int32)
    lefts = np.ascontiguousarray(lefts, np.int32)
    pu, pv = _f32(peak_u), _f32(peak_v)
    npk = np.ascontiguousarray(npeaks, np.int32)
    inv = np.zeros((ni, nj), np.uint8)
    sweeps = lib().orc_validate(ni, nj, _ptr(tops, ctypes.c_int), _ptr(lefts, ctypes.c_int), _ptr(u, ctypes.c_float),
                                _ptr(v, ctypes.c_float), _ptr(pu, ctypes.c_float), _ptr(pv, ctypes.c_float),
                                _ptr(npk, ctypes.c_int), k, ctypes.byref(cfg), inv.ctypes.data)
    return u, v, inv, sweeps


# ---------------- dense optical flow stages ----------------

def _real(a, precision):
    return np.ascontiguousarray(a, np.float32 if precision == 32 else np.float64)


def _rptr(a):
    return a.ctypes.data


def _fn(name, precision):
    return getattr(lib(), name if precision == 32 else name + "_f64")


def gauss_kernel(sigma, px, precision=32):
    """GaussianFilter2D.createKernel weights (float, or unrounded double for precision=64)."""
    k = np.zeros(px, np.float32 if precision == 32 else np.float64)
    _fn("orc_gauss_kernel", precision)(ctypes.c_float(sigma), px, _rptr(k))
    return k


def gauss_filter(img, sigma, px, precision=32):
    """GaussianFilter2D.applyFilter of a 2-D image (any numeric dtype) -> float32 (float64 for the
    FP64 twin)."""
    a = _real(img, precision)
    k = gauss_kernel(sigma, px, precision)
    out = np.zeros_like(a)
    _fn("orc_gauss_filter", precision)(_rptr(a), a.shape[0], a.shape[1], _rptr(k), px, _rptr(out))
    return out


def normalize(img, precision=32):
    a = _real(img, precision)
    out = np.zeros_like(a)
    _fn("orc_normalize", precision)(_rptr(a), ctypes.c_long(a.size), _rptr(out))
    return out


def dense_lk(img_a, img_b, us, vs, window, iterations, half_pixel=False, precision=32):
    """Dense Lucas-Kanade: returns refined (us, vs) (columns, rows)."""
    a, b = _real(img_a, precision), _real(img_b, precision)
    u, v = _real(us, precision).copy(), _real(vs, precision).copy()
    _fn("orc_dense_lk", precision)(_rptr(a), _rptr(b), a.shape[0], a.shape[1], _rptr(u), _rptr(v), window,
                                   iterations, int(half_pixel))
    return u, v


def dense_lk_pyramid(img_a, img_b, us, vs, window, iterations, half_pixel=False, levels=2, precision=32):
    """Dense Lucas-Kanade coarse to fine over `levels` 2 x 2 box-averaged levels (this library's own
    design): returns refined (us, vs) (columns, rows)."""
    a, b = _real(img_a, precision), _real(img_b, precision)
    u, v = _real(us, precision).copy(), _real(vs, precision).copy()
    _fn("orc_dense_lk_pyramid", precision)(_rptr(a), _rptr(b), a.shape[0], a.shape[1], _rptr(u), _rptr(v), window,
                                           iterations, int(half_pixel), levels)
    return u, v


def liu_shen(ls_a, ls_b, us, vs, lam, iterations, half_pixel=False, intermediates=False, precision=32):
    """Liu-Shen passes on (us, vs); with intermediates also the fixed terms (12 planes: w, IIx,
    IIy, II, Ixt, Iyt, A11, A12, A22, B11, B12, B22) and every pass's (unew, vnew)."""
    a, b = _real(ls_a, precision), _real(ls_b, precision)
    u, v = _real(us, precision).copy(), _real(vs, precision).copy()
    h, w = a.shape
    dt = a.dtype
    fixed = np.zeros((12, h, w), dt) if intermediates else None
    un = np.zeros((iterations, h, w), dt) if intermediates else None
    vn = np.zeros((iterations, h, w), dt) if intermediates else None
    lam_c = ctypes.c_float(lam) if precision == 32 else ctypes.c_double(lam)
    passes = _fn("orc_liu_shen", precision)(_rptr(a), _rptr(b), h, w, _rptr(u), _rptr(v), lam_c, iterations,
                                            int(half_pixel), fixed.ctypes.data if fixed is not None else None,
                                            un.ctypes.data if un is not None else None,
                                            vn.ctypes.data if vn is not None else None)
    if intermediates:
        return u, v, passes, fixed, un, vn
    return u, v


def flow_after_piv(img_a, img_b, n, tops, lefts, tu, tv, mode=2, sigma_lk=2.0, px_lk=3, sigma_ls=0.48, px_ls=5,
                   window=27, iterations_lk=5, lam=4.0, iterations_ls=60, dense_export=True, ignore_piv=0,
                   pyramid_levels=0, precision=32, clip_mode=CLIP_ALLOWED):
    """Optical flow after PIV on the last step's tile grid: returns updated tile (u, v)
    (rows, columns) and the dense field (rows, columns; float64 for precision=64, the FP64
    twin).  ignore_piv: 0 none, 1 IgnoreU, 2 IgnoreV, 3 IgnoreUV, 4 Auto, 5 AutoSmall."""
    a, b = _f32(img_a), _f32(img_b)
    h, w = a.shape
    tops = np.ascontiguousarray(tops, np.int32)
    lefts = np.ascontiguousarray(lefts, np.int32)
    u = np.array(tu, np.float32, order="C", copy=True)
    v = np.array(tv, np.float32, order="C", copy=True)
    dt = np.float32 if precision == 32 else np.float64
    du = np.zeros((h, w), dt)
    dv = np.zeros((h, w), dt)
    _fn("orc_flow_after_piv", precision)(_ptr(a, ctypes.c_float), _ptr(b, ctypes.c_float), h, w, n, len(tops),
                                         len(lefts), _ptr(tops, ctypes.c_int), _ptr(lefts, ctypes.c_int),
                                         _ptr(u, ctypes.c_float), _ptr(v, ctypes.c_float), mode, sigma_lk, px_lk,
                                         sigma_ls, px_ls, window, iterations_lk, lam, iterations_ls,
                                         int(dense_export), int(ignore_piv), int(pyramid_levels), int(clip_mode),
                                         du.ctypes.data, dv.ctypes.data)
    return u, v, du, dv

