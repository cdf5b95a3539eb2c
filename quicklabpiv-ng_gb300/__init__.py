"""quicklabpiv-ng_gb300: GB300-native FFT-PIV hot path of QuickLabPIV-ng.

The compute path is libqlpiv_gpu.so (hand-written sm_103a CUDA behind the C ABI of
include/qlpiv.h).  This package is the Python host side of that boundary: a ctypes
binding (`Handle`) and mirrors of the reference's stage plugins (`jobs`, `grid`).
There is no CPU fallback: without the built library every entry point raises.
"""
import ctypes
import os
from pathlib import Path

import numpy as np

from . import build as _build

PKG = Path(__file__).resolve().parent
LIB_PATH = _build.LIB

# include/qlpiv.h enums
OK, E_ARG, E_SHAPE, E_OOM, E_CUDA, E_TIMEOUT, E_CANCELLED, E_UNSUPPORTED, E_NO_DEVICE = range(9)
PIX_U8, PIX_U16, PIX_F32 = 0, 1, 2
NORM_MAX_A, NORM_OWN_MAX, NORM_NONE = 0, 1, 3
MAX_COMPUTE, MAX_GIVEN, MAX_FIXED, MAX_FIXED_A, MAX_FIXED_B = 0, 1, 2, 3, 4
SUBPIX_NONE, SUBPIX_GAUSS3, SUBPIX_GAUSS_LM, SUBPIX_HONGWEI_GUO = 0, 1, 2, 3
MAX_SUBPIX_PIXELS = 15
F_SUB_I, F_SUB_J, F_PARABOLIC, F_EDGE, F_NO_PEAK, F_ABSENT, F_FLOOR = 1, 2, 4, 8, 16, 32, 64
MAX_PEAKS = 16
VALIDATE_NONE, VALIDATE_MULTIPEAK_MEDIAN = 0, 1
VALIDATE_DIFFERENCE_ONLY, VALIDATE_DIFFERENCE, VALIDATE_MEDIAN_ONLY, VALIDATE_MEDIAN = 2, 3, 4, 5

VECTOR_DTYPE = np.dtype([
    ("u", "<f4"), ("v", "<f4"), ("sub_i", "<f4"), ("sub_j", "<f4"),
    ("peak_value", "<f4"), ("min_floor", "<f4"), ("peak_i", "<i2"), ("peak_j", "<i2"), ("flags", "<u4"),
])
assert VECTOR_DTYPE.itemsize == 32

SUPPORTED_IA = (16, 32, 64, 128)

_STATUS_NAMES = {OK: "OK", E_ARG: "E_ARG", E_SHAPE: "E_SHAPE", E_OOM: "E_OOM", E_CUDA: "E_CUDA",
                 E_TIMEOUT: "E_TIMEOUT", E_CANCELLED: "E_CANCELLED", E_UNSUPPORTED: "E_UNSUPPORTED",
                 E_NO_DEVICE: "E_NO_DEVICE"}


class QlpivError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class PassDesc(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("norm_mode", ctypes.c_int), ("max_mode", ctypes.c_int),
                ("fixed_max_a", ctypes.c_float), ("fixed_max_b", ctypes.c_float), ("subpix_mode", ctypes.c_int),
                ("num_peaks", ctypes.c_int), ("peak_kernel", ctypes.c_int), ("subpix_pixels", ctypes.c_int),
                ("subpix_iterations", ctypes.c_int), ("reserved", ctypes.c_int * 2)]


class Frame(ctypes.Structure):
    _fields_ = [("img_a", ctypes.c_void_p), ("img_b", ctypes.c_void_p), ("height", ctypes.c_int32),
                ("width", ctypes.c_int32), ("pitch", ctypes.c_int64)]


FRAME_DTYPE = np.dtype([("img_a", "<u8"), ("img_b", "<u8"), ("height", "<i4"), ("width", "<i4"), ("pitch", "<i8")])
assert FRAME_DTYPE.itemsize == 32


class Grid(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int) for k in
                ("n", "tiles_i", "tiles_j", "margin_top", "margin_left", "margin_bottom", "margin_right")]


WARP_NONE, WARP_BOTH_BILINEAR, WARP_FIRST_BILINEAR, WARP_SECOND_BILINEAR = 0, 1, 2, 3
WARP_FIRST_MICRO, WARP_SECOND_MICRO, WARP_BOTH_MICRO, WARP_FIRST_MINI, WARP_SECOND_MINI, WARP_BOTH_MINI = range(4, 10)


class AdaptiveDesc(ctypes.Structure):
    _fields_ = [("ia_start", ctypes.c_int), ("ia_end", ctypes.c_int), ("overlap_factor", ctypes.c_float),
                ("margins", ctypes.c_int * 4), ("warp_mode", ctypes.c_int), ("norm_mode", ctypes.c_int),
                ("max_mode", ctypes.c_int), ("fixed_max", ctypes.c_float), ("subpix_mode", ctypes.c_int),
                ("int16_warp_quirk", ctypes.c_int), ("validation", ctypes.c_int), ("num_peaks", ctypes.c_int),
                ("peak_kernel", ctypes.c_int), ("median_threshold", ctypes.c_float),
                ("median_epsilon0", ctypes.c_float), ("max_correction_iterations", ctypes.c_int),
                ("iterate_until_no_corrections", ctypes.c_int), ("subpix_pixels", ctypes.c_int),
                ("subpix_iterations", ctypes.c_int), ("inherit_mode", ctypes.c_int), ("clipping_mode", ctypes.c_int),
                ("superposition_start", ctypes.c_int), ("stable_mode", ctypes.c_int),
                ("stable_max_displacement", ctypes.c_float), ("stable_max_retries", ctypes.c_int),
                ("reserved", ctypes.c_int * 5)]


STABLE_SIMPLE, STABLE_MAX_DISPLACEMENT = 0, 1
# mixed batch plans: autotune modes and schedules
AUTOTUNE_OFF, AUTOTUNE_ON, AUTOTUNE_PERSISTENT = 0, 1, 2
SCHEDULE_PER_SIZE, SCHEDULE_PERSISTENT = 0, 1


CLIP_ALLOWED, CLIP_LOGGED, CLIP_NO_OUT_OF_BOUND = 0, 1, 2


def adaptive_desc(ia_start, ia_end, overlap_factor, margins=(0, 0, 0, 0), warp_mode=WARP_BOTH_BILINEAR,
                  norm_mode=NORM_MAX_A, max_mode=MAX_FIXED, fixed_max=0.0, subpix_mode=SUBPIX_GAUSS3,
                  int16_warp_quirk=False, validation=None, subpix_pixels=3, subpix_iterations=20,
                  inherit_mode=0, clipping_mode=CLIP_ALLOWED, superposition_start=0, stable_max_displacement=None,
                  stable_max_retries=0):
    """Adaptive PIV parameters; the defaults follow the reference's BothImages bilinear
    warping (tiles copied from the warped image keep the full-scale maximum).
    superposition_start: the level from which the interrogation areas overlap (the mixed
    division; 0: SuperPosition throughout, >= the level count: NoSuperPosition).
    stable_max_displacement / stable_max_retries: InterAreaDisplacementStableStrategy (a level's
    tiles are correlated again while their increment exceeds the maximum, at most
    stable_max_retries passes); None: one correlation per level.
    validation: None, or a dict with keys model (VALIDATE_*; default the multi-peak
    normalised-median model), num_peaks, peak_kernel, threshold, epsilon0, max_iterations,
    iterate_until (see multipeak_validation() and validation_model()).  clipping_mode:
    CLIP_ALLOWED, CLIP_LOGGED or CLIP_NO_OUT_OF_BOUND (ClippingModeEnum)."""
    d = AdaptiveDesc()
    d.ia_start, d.ia_end, d.overlap_factor = ia_start, ia_end, overlap_factor
    d.margins[:] = list(margins)
    d.warp_mode, d.norm_mode, d.max_mode, d.fixed_max = warp_mode, norm_mode, max_mode, fixed_max
    d.subpix_mode, d.int16_warp_quirk = subpix_mode, int(int16_warp_quirk)
    d.subpix_pixels, d.subpix_iterations = subpix_pixels, subpix_iterations
    d.inherit_mode = inherit_mode
    d.clipping_mode = clipping_mode
    d.superposition_start = superposition_start
    if stable_max_displacement is not None:
        d.stable_mode = STABLE_MAX_DISPLACEMENT
        d.stable_max_displacement = stable_max_displacement
        d.stable_max_retries = stable_max_retries
    if validation is not None:
        set_validation(d, **validation)
    return d


def multipeak_validation(num_peaks=3, peak_kernel=3, threshold=2.0, epsilon0=0.1, max_iterations=2,
                         iterate_until=False):
    """Settings of VelocityValidationOptionsMultiPeakNormalizedMedianModel plus the
    validator job's iteration settings."""
    return dict(num_peaks=num_peaks, peak_kernel=peak_kernel, threshold=threshold, epsilon0=epsilon0,
                max_iterations=max_iterations, iterate_until=iterate_until)


def validation_model(model, threshold=2.0, epsilon0=0.1, max_iterations=2, iterate_until=False):
    """Settings of the four single-strategy models (VALIDATE_DIFFERENCE_ONLY, VALIDATE_DIFFERENCE,
    VALIDATE_MEDIAN_ONLY, VALIDATE_MEDIAN; FindMaximumFromCenter peaks)."""
    return dict(model=model, num_peaks=1, peak_kernel=3, threshold=threshold, epsilon0=epsilon0,
                max_iterations=max_iterations, iterate_until=iterate_until)


def set_validation(d, num_peaks=3, peak_kernel=3, threshold=2.0, epsilon0=0.1, max_iterations=2,
                   iterate_until=False, model=None):
    d.validation = VALIDATE_MULTIPEAK_MEDIAN if model is None else model
    d.num_peaks, d.peak_kernel = num_peaks, peak_kernel
    d.median_threshold, d.median_epsilon0 = threshold, epsilon0
    d.max_correction_iterations, d.iterate_until_no_corrections = max_iterations, int(iterate_until)
    return d


FLOW_LUCAS_KANADE, FLOW_LIU_SHEN = 1, 2
INHERIT_BICUBIC_SPLINE, INHERIT_DIRECT, INHERIT_AREA, INHERIT_DISTANCE = range(4)
IGNORE_PIV_NONE, IGNORE_PIV_U, IGNORE_PIV_V, IGNORE_PIV_UV, IGNORE_PIV_AUTO, IGNORE_PIV_AUTO_SMALL = range(6)


class FlowDesc(ctypes.Structure):
    _fields_ = [("mode", ctypes.c_int), ("filter_sigma_lk", ctypes.c_float), ("filter_px_lk", ctypes.c_int),
                ("filter_sigma_ls", ctypes.c_float), ("filter_px_ls", ctypes.c_int), ("window_lk", ctypes.c_int),
                ("iterations_lk", ctypes.c_int), ("lambda_ls", ctypes.c_float), ("iterations_ls", ctypes.c_int),
                ("dense_export", ctypes.c_int), ("ignore_piv", ctypes.c_int), ("pyramid_levels", ctypes.c_int),
                ("clipping_mode", ctypes.c_int), ("reserved", ctypes.c_int * 3)]


def flow_desc(mode=FLOW_LUCAS_KANADE, filter_sigma_lk=2.0, filter_px_lk=3, filter_sigma_ls=0.48, filter_px_ls=5,
              window_lk=27, iterations_lk=5, lambda_ls=4.0, iterations_ls=60, dense_export=False, ignore_piv=0,
              pyramid_levels=0, clipping_mode=CLIP_ALLOWED):
    """Optical flow after PIV (OpticalFlowAfterPIV Lucas-Kanade or Liu-Shen interpolator
    options); dense_export selects whole-pixel evaluation and the dense field export.
    pyramid_levels > 1 runs the Lucas-Kanade stage coarse to fine over that many 2 x 2
    box-averaged levels (an extension: the reference runs it at full resolution only)."""
    d = FlowDesc()
    d.mode, d.filter_sigma_lk, d.filter_px_lk = mode, filter_sigma_lk, filter_px_lk
    d.filter_sigma_ls, d.filter_px_ls, d.window_lk, d.iterations_lk = filter_sigma_ls, filter_px_ls, window_lk, \
        iterations_lk
    d.lambda_ls, d.iterations_ls, d.dense_export = lambda_ls, iterations_ls, int(dense_export)
    d.ignore_piv, d.pyramid_levels = ignore_piv, pyramid_levels
    d.clipping_mode = clipping_mode
    return d


class StageTime(ctypes.Structure):
    _fields_ = [("stage", ctypes.c_char * 24), ("level", ctypes.c_int), ("ia_side", ctypes.c_int),
                ("launches", ctypes.c_long), ("items", ctypes.c_long), ("ms", ctypes.c_double)]


class Params(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("reserved", ctypes.c_int * 7)]


class ServerParams(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("slots", ctypes.c_int), ("hbm_budget", ctypes.c_int64),
                ("staging_bytes", ctypes.c_int64), ("submit_timeout_ms", ctypes.c_int), ("reserved", ctypes.c_int * 7)]


class Request(ctypes.Structure):
    _fields_ = [("schedule", ctypes.POINTER(AdaptiveDesc)), ("pixel_type", ctypes.c_int), ("height", ctypes.c_int),
                ("width", ctypes.c_int), ("pitch", ctypes.c_int64), ("img_a", ctypes.c_void_p),
                ("img_b", ctypes.c_void_p), ("out_u", ctypes.c_void_p), ("out_v", ctypes.c_void_p)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("tiles_i", ctypes.c_int), ("tiles_j", ctypes.c_int),
                ("queue_ms", ctypes.c_double), ("device_ms", ctypes.c_double), ("total_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in ("submitted", "completed", "failed", "pending", "in_flight",
                                              "device_bytes_in_flight", "hbm_budget")] + \
               [("reserved", ctypes.c_int64 * 4)]


class MatExportParams(ctypes.Structure):
    _fields_ = [("image_width", ctypes.c_int), ("image_height", ctypes.c_int), ("ia_start", ctypes.c_int),
                ("ia_end", ctypes.c_int), ("overlap_factor", ctypes.c_float), ("frames", ctypes.c_int),
                ("swap_uv", ctypes.c_int), ("mark_invalid_as_nan", ctypes.c_int),
                ("export_date", ctypes.c_char_p), ("layout", ctypes.c_int), ("maps_per_file", ctypes.c_int),
                ("reserved", ctypes.c_int * 2)]


class MatVelocityMap(ctypes.Structure):
    _fields_ = [("ia_height", ctypes.c_int), ("ia_width", ctypes.c_int), ("adaptive_step", ctypes.c_int),
                ("tiles_i", ctypes.c_int), ("tiles_j", ctypes.c_int), ("margins", ctypes.c_int * 4),
                ("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("invalid", ctypes.c_void_p)]


# C ABI symbol table: name -> (restype, argtypes).  Kept beside include/qlpiv.h.
_vp, _i, _l, _f = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_float
_SIGNATURES = {
    "qlpiv_abi_version": (_i, []),
    "qlpiv_last_error": (ctypes.c_char_p, []),
    "qlpiv_create": (_i, [ctypes.POINTER(Params), ctypes.POINTER(_vp)]),
    "qlpiv_destroy": (_i, [_vp]),
    "qlpiv_synchronize": (_i, [_vp]),
    "qlpiv_launch_count": (_l, [_vp]),
    "qlpiv_xcorr_planes": (_i, [_vp, _i, _l, _i, _vp, _vp, _vp, _vp, _i, _vp]),
    "qlpiv_xcorr_peaks": (_i, [_vp, _i, _l, _i, _vp, _vp, _vp, _vp, _i, _i, _vp]),
    "qlpiv_xcorr_multipeaks": (_i, [_vp, _i, _l, _i, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp]),
    "qlpiv_probe_division": (_i, [_i, ctypes.POINTER(ctypes.c_int64)]),
    "qlpiv_validate": (_i, [_vp, ctypes.POINTER(AdaptiveDesc), _i, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qlpiv_validate_tiles": (_i, [_vp, ctypes.POINTER(AdaptiveDesc), _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp,
                                  _vp, _vp]),
    "qlpiv_pass": (_i, [_vp, ctypes.POINTER(PassDesc), _vp, _vp, _i, _i, _i, _l, _vp, _vp, _vp, _vp, _vp]),
    "qlpiv_pass_device": (_i, [_vp, ctypes.POINTER(PassDesc), _vp, _vp, _i, _i, _i, _l, _vp, _vp, _vp, _vp, _vp]),
    "qlpiv_pass_batch": (_i, [_vp, ctypes.POINTER(PassDesc), _i, _i, _vp, _l, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qlpiv_pass_batch_device": (_i, [_vp, ctypes.POINTER(PassDesc), _i, _i, _vp, _l, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qlpiv_get_stream": (_i, [_vp, ctypes.POINTER(_vp)]),
    "qlpiv_set_stream": (_i, [_vp, _vp]),
    "qlpiv_measure_fp32_peak": (_i, [_i, ctypes.POINTER(ctypes.c_double)]),
    "qlpiv_grid_superposition": (_i, [_i, _i, _vp, _i, _i, _f, ctypes.POINTER(Grid), _vp, _vp, _i]),
    "qlpiv_grid_nosuperposition": (_i, [_i, _i, _vp, _i, _i, ctypes.POINTER(Grid), _vp, _vp, _i]),
    "qlpiv_grid_level": (_i, [_i, _i, _vp, _i, _i, ctypes.c_float, _i, ctypes.POINTER(Grid), _vp, _vp, _i]),
    "qlpiv_adaptive_levels": (_i, [ctypes.POINTER(AdaptiveDesc), _i, _i, ctypes.POINTER(_i), _vp, _i]),
    "qlpiv_inherit": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _i, _vp, _vp]),
    "qlpiv_inherit_tiles": (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _i, _i, _i, _vp, _vp, _i, _vp, _vp]),
    "qlpiv_displacement_field": (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "qlpiv_warp_pair": (_i, [_vp, _i, _i, _vp, _vp, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _i, _vp, _vp]),
    "qlpiv_tile_warp": (_i, [_vp, _i, _vp, _vp, _i, _i, _i, _i, _i, _vp, _vp, _vp, _vp, _i, _f, _vp, _vp, _vp, _vp]),
    "qlpiv_piv_adaptive": (_i, [_vp, ctypes.POINTER(AdaptiveDesc), _i, _i, _i, _i, _vp, _vp, _vp]),
    "qlpiv_piv_adaptive_device": (_i, [_vp, ctypes.POINTER(AdaptiveDesc), _i, _i, _i, _i, _vp, _vp, _vp]),
    "qlpiv_inherit_noalloc": (_i, [_i, _vp, _i, _i, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _i, _vp, _vp]),
    "qlpiv_gaussian_filter": (_i, [_vp, _i, _vp, _i, _i, _f, _i, _vp]),
    "qlpiv_normalize": (_i, [_vp, _vp, _i, _i, _vp]),
    "qlpiv_dense_lk": (_i, [_vp, _vp, _vp, _i, _i, _vp, _vp, _i, _i, _i]),
    "qlpiv_liu_shen": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _vp, _vp, _i, _i, _f, _i, _i]),
    "qlpiv_flow_after_piv": (_i, [_vp, ctypes.POINTER(FlowDesc), _i, _vp, _vp, _i, _i, _i, _i, _i, _vp, _vp, _vp,
                                  _vp, _vp, _vp]),
    "qlpiv_piv_flow": (_i, [_vp, ctypes.POINTER(AdaptiveDesc), ctypes.POINTER(FlowDesc), _i, _i, _i, _i, _vp, _vp,
                            _vp, _vp, _vp]),
    "qlpiv_piv_flow_device": (_i, [_vp, ctypes.POINTER(AdaptiveDesc), ctypes.POINTER(FlowDesc), _i, _i, _i, _i, _vp,
                                   _vp, _vp, _vp, _vp]),
    "qlpiv_mixed_plan_create": (_i, [_vp, ctypes.POINTER(PassDesc), _i, _i, _vp, _vp, _vp, _i, ctypes.POINTER(_vp)]),
    "qlpiv_mixed_plan_info": (_i, [_vp, ctypes.POINTER(ctypes.c_int64), _vp, _vp, _vp]),
    "qlpiv_mixed_plan_schedule": (_i, [_vp, ctypes.POINTER(ctypes.c_int32)]),
    "qlpiv_adaptive_batch_create": (_i, [_vp, _i, _i, _vp, _vp, _i, _vp, ctypes.POINTER(_vp)]),
    "qlpiv_adaptive_batch_info": (_i, [_vp, ctypes.POINTER(ctypes.c_int64), _vp, _vp,
                                       ctypes.POINTER(ctypes.c_int32)]),
    "qlpiv_adaptive_batch_run": (_i, [_vp, _vp, ctypes.POINTER(_vp), ctypes.POINTER(_vp)]),
    "qlpiv_adaptive_batch_download": (_i, [_vp, _vp, _vp, _vp]),
    "qlpiv_adaptive_batch_destroy": (_i, [_vp]),
    "qlpiv_mixed_plan_run": (_i, [_vp, _vp, ctypes.POINTER(_vp)]),
    "qlpiv_mixed_plan_download": (_i, [_vp, _vp, _vp]),
    "qlpiv_mixed_plan_destroy": (_i, [_vp]),
    "qlpiv_server_create": (_i, [ctypes.POINTER(ServerParams), ctypes.POINTER(_vp)]),
    "qlpiv_server_destroy": (_i, [_vp]),
    "qlpiv_submit": (_i, [_vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    "qlpiv_poll": (_i, [_vp, ctypes.c_uint64, ctypes.POINTER(Result), _i]),
    "qlpiv_server_stats_read": (_i, [_vp, ctypes.POINTER(ServerStats)]),
    "qlpiv_adaptive_plan_bytes": (_i, [ctypes.POINTER(AdaptiveDesc), _i, _i, _i, _i, ctypes.POINTER(ctypes.c_int64)]),
    "qlpiv_tiff_info": (_i, [ctypes.c_char_p, ctypes.POINTER(_i), ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "qlpiv_tiff_read": (_i, [ctypes.c_char_p, _vp, ctypes.c_int64]),
    "qlpiv_mat_export": (_i, [ctypes.c_char_p, ctypes.POINTER(MatExportParams), _i, ctypes.POINTER(MatVelocityMap)]),
    "qlpiv_probe_log": (_i, [_i, _vp, _l, _vp, _vp]),
    "qlpiv_profile_enable": (_i, [_vp, _i]),
    "qlpiv_profile_read": (_i, [_vp, _vp, _i, ctypes.POINTER(_i)]),
}

_lib = None


def load_library(path=None):
    """Load libqlpiv_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python quicklabpiv-ng_gb300/build.py` "
                           "(or __graft_entry__.build()); there is no CPU fallback")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.qlpiv_abi_version() != 5:
        raise RuntimeError("libqlpiv_gpu.so ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def exported_symbols():
    return list(_SIGNATURES)


def _check(status):
    if status != OK:
        raise QlpivError(status, load_library().qlpiv_last_error().decode())


def library_grid(height, width, ia_start, level, overlap_factor, margins=(0, 0, 0, 0), superposition=True,
                 superposition_start=None):
    """IA grid computed by the library (host code of libqlpiv_gpu.so); with superposition_start,
    the mixed division's grid of that level (qlpiv_grid_level)."""
    lib = load_library()
    g = Grid()
    m = (ctypes.c_int * 4)(*margins)
    cap = 1 << 16
    tops = np.zeros(cap, np.int32)
    lefts = np.zeros(cap, np.int32)
    if superposition_start is not None:
        _check(lib.qlpiv_grid_level(height, width, m, ia_start, level, overlap_factor, superposition_start,
                                    ctypes.byref(g), _addr(tops), _addr(lefts), cap))
    elif superposition:
        _check(lib.qlpiv_grid_superposition(height, width, m, ia_start, level, overlap_factor, ctypes.byref(g),
                                            _addr(tops), _addr(lefts), cap))
    else:
        _check(lib.qlpiv_grid_nosuperposition(height, width, m, ia_start, level, ctypes.byref(g), _addr(tops),
                                              _addr(lefts), cap))
    return {k: getattr(g, k) for k, _ in Grid._fields_}, tops[:g.tiles_i].copy(), lefts[:g.tiles_j].copy()


def adaptive_levels(desc, height, width):
    lib = load_library()
    n = ctypes.c_int()
    grids = (Grid * 16)()
    _check(lib.qlpiv_adaptive_levels(ctypes.byref(desc), height, width, ctypes.byref(n), grids, 16))
    return [{k: getattr(grids[i], k) for k, _ in Grid._fields_} for i in range(n.value)]


NOALLOC_MAX_ROWS = 524288


def inherit_noalloc(device, stream, p_ci, p_cj, pu, pv, c_ci, c_cj, cu, cv, pni, pnj, cni, cnj, round_int=False):
    """qlpiv_inherit_noalloc: every array a device buffer (torch tensor or address);
    queued on `stream` (cudaStream_t as int, 0 = legacy default stream).  Tensors are checked
    (CUDA, on `device`, float32, contiguous, sized for the grids) before the call; raw
    addresses are the caller's responsibility."""
    args = (p_ci, p_cj, pu, pv, c_ci, c_cj, cu, cv)
    sizes = (pni, pnj, pni * pnj, pni * pnj, cni, cnj, cni * cnj, cni * cnj)
    names = ("p_ci", "p_cj", "pu", "pv", "c_ci", "c_cj", "cu", "cv")
    for x, size, name in zip(args, sizes, names):
        if isinstance(x, int):
            continue
        if not getattr(x, "is_cuda", False) or x.device.index != device:
            raise ValueError(f"{name} must be a CUDA tensor on device {device}")
        if str(x.dtype) != "torch.float32" or not x.is_contiguous():
            raise ValueError(f"{name} must be a contiguous float32 tensor")
        if x.numel() != size:
            raise ValueError(f"{name} has {x.numel()} elements, the grids need {size}")
    a = [x if isinstance(x, int) else _addr(x) for x in args]
    _check(load_library().qlpiv_inherit_noalloc(device, stream or None, pni, pnj, a[0], a[1], a[2], a[3], cni, cnj,
                                                a[4], a[5], int(round_int), a[6], a[7]))


def probe_division(device=0):
    """Quotients of the IA-16 kernel's normalisation division that differ from IEEE division over
    every integer pixel value and integer maximum below 65536 (0 expected)."""
    n = ctypes.c_int64()
    _check(load_library().qlpiv_probe_division(device, ctypes.byref(n)))
    return n.value


def probe_log(x, device=0):
    """(fit logarithm, CUDA double log) of positive floats x, evaluated on the device."""
    x = np.ascontiguousarray(x, np.float32)
    mine = np.empty(x.size, np.float64)
    ref = np.empty(x.size, np.float64)
    _check(load_library().qlpiv_probe_log(device, _addr(x), x.size, _addr(mine), _addr(ref)))
    return mine, ref


def measure_fp32_peak(device=0):
    """Live FP32 FMA throughput (TFLOP/s) of the device."""
    t = ctypes.c_double()
    _check(load_library().qlpiv_measure_fp32_peak(device, ctypes.byref(t)))
    return t.value


def pixel_type_of(dtype):
    dtype = np.dtype(dtype)
    if dtype == np.uint8:
        return PIX_U8
    if dtype == np.uint16:
        return PIX_U16
    if dtype == np.float32:
        return PIX_F32
    raise ValueError(f"unsupported pixel dtype {dtype}")


def _addr(x):
    """Address of a contiguous numpy array or torch tensor."""
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


class Handle:
    """One device context of the library (qlpiv_create / qlpiv_destroy)."""

    def __init__(self, device=0):
        lib = load_library()
        self._lib = lib
        p = Params()
        p.device = device
        h = ctypes.c_void_p()
        _check(lib.qlpiv_create(ctypes.byref(p), ctypes.byref(h)))
        self._h = h
        self.device = device

    def close(self):
        if getattr(self, "_h", None):
            self._lib.qlpiv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def launches(self):
        return self._lib.qlpiv_launch_count(self._h)

    def synchronize(self):
        _check(self._lib.qlpiv_synchronize(self._h))

    @property
    def stream(self):
        """cudaStream_t (as an int) the handle queues work on."""
        s = ctypes.c_void_p()
        _check(self._lib.qlpiv_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def set_stream(self, stream):
        _check(self._lib.qlpiv_set_stream(self._h, stream))

    def profile(self, enable=True):
        _check(self._lib.qlpiv_profile_enable(self._h, int(enable)))

    def profile_read(self):
        """Per (stage, level) device time accumulated since the last read."""
        n = ctypes.c_int()
        buf = (StageTime * 64)()
        _check(self._lib.qlpiv_profile_read(self._h, buf, 64, ctypes.byref(n)))
        return [{"stage": buf[k].stage.decode(), "level": buf[k].level, "ia_side": buf[k].ia_side,
                 "launches": buf[k].launches, "items": buf[k].items, "ms": buf[k].ms} for k in range(min(n.value, 64))]

    # -- tile API (Job<List<Tile>, XCorrelationResults>) -------------------------
    @staticmethod
    def _tiles(tiles_a, tiles_b):
        ta = np.ascontiguousarray(tiles_a)
        tb = np.ascontiguousarray(tiles_b)
        if ta.ndim == 2:
            ta, tb = ta[None], tb[None]
        if ta.shape != tb.shape or ta.ndim != 3 or ta.shape[1] != ta.shape[2] or ta.dtype != tb.dtype:
            raise ValueError("tiles must be two (count, n, n) arrays of one dtype")
        return ta, tb

    @staticmethod
    def _maxes(max_a, max_b, count):
        if max_a is None and max_b is None:
            return None, None
        ma = np.ascontiguousarray(np.broadcast_to(np.asarray(max_a, np.float32), (count,)))
        mb = np.ascontiguousarray(np.broadcast_to(np.asarray(max_b, np.float32), (count,)))
        return ma, mb

    def xcorr_planes(self, tiles_a, tiles_b, max_a=None, max_b=None, norm_mode=NORM_MAX_A):
        ta, tb = self._tiles(tiles_a, tiles_b)
        count, n = ta.shape[0], ta.shape[1]
        ma, mb = self._maxes(max_a, max_b, count)
        d = 2 * n - 1
        out = np.empty((count, d, d), np.float32)
        _check(self._lib.qlpiv_xcorr_planes(self._h, n, count, pixel_type_of(ta.dtype), _addr(ta), _addr(tb),
                                            _addr(ma), _addr(mb), norm_mode, _addr(out)))
        return out

    def xcorr_peaks(self, tiles_a, tiles_b, max_a=None, max_b=None, norm_mode=NORM_MAX_A, subpix_mode=SUBPIX_GAUSS3):
        ta, tb = self._tiles(tiles_a, tiles_b)
        count, n = ta.shape[0], ta.shape[1]
        ma, mb = self._maxes(max_a, max_b, count)
        out = np.empty(count, VECTOR_DTYPE)
        _check(self._lib.qlpiv_xcorr_peaks(self._h, n, count, pixel_type_of(ta.dtype), _addr(ta), _addr(tb),
                                           _addr(ma), _addr(mb), norm_mode, subpix_mode, _addr(out)))
        return out

    def xcorr_multipeaks(self, tiles_a, tiles_b, max_a=None, max_b=None, norm_mode=NORM_MAX_A,
                         subpix_mode=SUBPIX_GAUSS3, num_peaks=3, peak_kernel=3):
        """FindMaximumMultiPeaks on every tile pair: vectors shaped (count, num_peaks),
        largest peak first (absent slots flagged F_ABSENT)."""
        ta, tb = self._tiles(tiles_a, tiles_b)
        count, n = ta.shape[0], ta.shape[1]
        ma, mb = self._maxes(max_a, max_b, count)
        out = np.empty((count, num_peaks), VECTOR_DTYPE)
        _check(self._lib.qlpiv_xcorr_multipeaks(self._h, n, count, pixel_type_of(ta.dtype), _addr(ta), _addr(tb),
                                                _addr(ma), _addr(mb), norm_mode, subpix_mode, num_peaks, peak_kernel,
                                                _addr(out)))
        return out

    # -- frame API ---------------------------------------------------------------
    @staticmethod
    def desc(n, norm_mode=NORM_MAX_A, max_mode=MAX_COMPUTE, fixed_max=(255.0, 255.0), subpix_mode=SUBPIX_GAUSS3,
             num_peaks=0, peak_kernel=3, subpix_pixels=3, subpix_iterations=20):
        """Pass descriptor; num_peaks > 0 selects FindMaximumMultiPeaks (num_peaks vectors
        per IA); subpix_pixels / subpix_iterations configure the P-point interpolators."""
        d = PassDesc()
        d.n, d.norm_mode, d.max_mode = n, norm_mode, max_mode
        d.fixed_max_a, d.fixed_max_b = fixed_max
        d.subpix_mode = subpix_mode
        d.num_peaks, d.peak_kernel = num_peaks, peak_kernel
        d.subpix_pixels, d.subpix_iterations = subpix_pixels, subpix_iterations
        return d

    @staticmethod
    def _out_vectors(count, d):
        return np.empty(count, VECTOR_DTYPE) if d.num_peaks == 0 else np.empty((count, d.num_peaks), VECTOR_DTYPE)

    def piv_pass(self, img_a, img_b, n, a_top, a_left, b_top=None, b_left=None, **kw):
        """One correlation pass over host images; origins per IA (int32)."""
        ia = np.ascontiguousarray(img_a)
        ib = np.ascontiguousarray(img_b)
        if ia.shape != ib.shape or ia.dtype != ib.dtype or ia.ndim != 2:
            raise ValueError("images must be two 2-D arrays of one shape and dtype")
        at = np.ascontiguousarray(a_top, np.int32)
        al = np.ascontiguousarray(a_left, np.int32)
        bt = at if b_top is None else np.ascontiguousarray(b_top, np.int32)
        bl = al if b_left is None else np.ascontiguousarray(b_left, np.int32)
        count = at.shape[0]
        if not (al.shape[0] == bt.shape[0] == bl.shape[0] == count):
            raise ValueError("origin arrays differ in length")
        d = self.desc(n, **kw)
        out = self._out_vectors(count, d)
        _check(self._lib.qlpiv_pass(self._h, ctypes.byref(d), _addr(ia), _addr(ib), ia.shape[0], ia.shape[1],
                                    pixel_type_of(ia.dtype), count, _addr(at), _addr(al), _addr(bt), _addr(bl),
                                    _addr(out)))
        return out

    def piv_pass_device(self, img_a, img_b, height, width, pixel_type, n, count, a_top, a_left, b_top, b_left, out,
                        **kw):
        """Queue one pass on device-resident buffers (torch tensors or raw addresses);
        does not wait."""
        d = self.desc(n, **kw)
        a = [x if isinstance(x, int) else _addr(x) for x in (img_a, img_b, a_top, a_left, b_top, b_left, out)]
        _check(self._lib.qlpiv_pass_device(self._h, ctypes.byref(d), a[0], a[1], height, width, pixel_type, count,
                                           a[2], a[3], a[4], a[5], a[6]))

    def piv_pass_batch(self, frames_a, frames_b, n, frame_of_ia, a_top, a_left, b_top=None, b_left=None, **kw):
        """Batched pass over host image pairs (lists of 2-D arrays, sizes may differ)."""
        if len(frames_a) != len(frames_b):
            raise ValueError("frames_a and frames_b differ in length")
        fa = [np.ascontiguousarray(x) for x in frames_a]
        fb = [np.ascontiguousarray(x) for x in frames_b]
        dt = fa[0].dtype
        table = (Frame * len(fa))()
        for k, (x, y) in enumerate(zip(fa, fb)):
            if x.shape != y.shape or x.dtype != dt or y.dtype != dt:
                raise ValueError("all frames must share the pixel dtype and pair shapes must match")
            table[k] = Frame(x.ctypes.data, y.ctypes.data, x.shape[0], x.shape[1], x.shape[1])
        fi = np.ascontiguousarray(frame_of_ia, np.int32)
        at = np.ascontiguousarray(a_top, np.int32)
        al = np.ascontiguousarray(a_left, np.int32)
        bt = at if b_top is None else np.ascontiguousarray(b_top, np.int32)
        bl = al if b_left is None else np.ascontiguousarray(b_left, np.int32)
        d = self.desc(n, **kw)
        out = self._out_vectors(len(at), d)
        _check(self._lib.qlpiv_pass_batch(self._h, ctypes.byref(d), pixel_type_of(dt), len(fa), table, len(at),
                                          _addr(fi), _addr(at), _addr(al), _addr(bt), _addr(bl), _addr(out)))
        return out

    def piv_pass_batch_device(self, pixel_type, num_frames, frames, n, count, frame_of_ia, a_top, a_left, b_top,
                              b_left, out, **kw):
        """Queue a batched pass; every argument is a device buffer (torch tensor or address)."""
        d = self.desc(n, **kw)
        a = [x if isinstance(x, int) else _addr(x) for x in (frames, frame_of_ia, a_top, a_left, b_top, b_left, out)]
        _check(self._lib.qlpiv_pass_batch_device(self._h, ctypes.byref(d), pixel_type, num_frames, a[0], count, a[1],
                                                 a[2], a[3], a[4], a[5], a[6]))

    # -- stages between passes --------------------------------------------------
    def inherit(self, p_ci, p_cj, pu, pv, c_ci, c_cj, round_int=False):
        """Velocity inheritance from a parent grid to a child grid (host arrays)."""
        p_ci = np.ascontiguousarray(p_ci, np.float64)
        p_cj = np.ascontiguousarray(p_cj, np.float64)
        pu = np.ascontiguousarray(pu, np.float32)
        pv = np.ascontiguousarray(pv, np.float32)
        c_ci = np.ascontiguousarray(c_ci, np.float32)
        c_cj = np.ascontiguousarray(c_cj, np.float32)
        cu = np.empty((len(c_ci), len(c_cj)), np.float32)
        cv = np.empty_like(cu)
        _check(self._lib.qlpiv_inherit(self._h, len(p_ci), len(p_cj), _addr(p_ci), _addr(p_cj), _addr(pu), _addr(pv),
                                       len(c_ci), len(c_cj), _addr(c_ci), _addr(c_cj), int(round_int), _addr(cu),
                                       _addr(cv)))
        return cu, cv

    def inherit_tiles(self, mode, pn, p_tops, p_lefts, pu, pv, cn, c_tops, c_lefts, round_int=False):
        """Direct / Area / Distance velocity inheritance between two grids (host arrays)."""
        p_tops = np.ascontiguousarray(p_tops, np.int32)
        p_lefts = np.ascontiguousarray(p_lefts, np.int32)
        c_tops = np.ascontiguousarray(c_tops, np.int32)
        c_lefts = np.ascontiguousarray(c_lefts, np.int32)
        pu = np.ascontiguousarray(pu, np.float32)
        pv = np.ascontiguousarray(pv, np.float32)
        cu = np.empty((len(c_tops), len(c_lefts)), np.float32)
        cv = np.empty_like(cu)
        _check(self._lib.qlpiv_inherit_tiles(self._h, mode, pn, len(p_tops), len(p_lefts), _addr(p_tops),
                                             _addr(p_lefts), _addr(pu), _addr(pv), cn, len(c_tops), len(c_lefts),
                                             _addr(c_tops), _addr(c_lefts), int(round_int), _addr(cu), _addr(cv)))
        return cu, cv

    def displacement_field(self, ci, cj, u, v, height, width):
        ci = np.ascontiguousarray(ci, np.float64)
        cj = np.ascontiguousarray(cj, np.float64)
        u = np.ascontiguousarray(u, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        fu = np.empty((height, width), np.float32)
        fv = np.empty_like(fu)
        _check(self._lib.qlpiv_displacement_field(self._h, height, width, len(ci), len(cj), _addr(ci), _addr(cj),
                                                  _addr(u), _addr(v), _addr(fu), _addr(fv)))
        return fu, fv

    def warp_pair(self, img_a, img_b, ci, cj, u, v, int16_quirk=False, warp_mode=None):
        """Full-image bilinear warp of one pair (BothImages by default, or WARP_FIRST_BILINEAR /
        WARP_SECOND_BILINEAR); the frame that is not warped comes back unchanged."""
        ia = np.ascontiguousarray(img_a)
        ib = np.ascontiguousarray(img_b)
        ci = np.ascontiguousarray(ci, np.float64)
        cj = np.ascontiguousarray(cj, np.float64)
        u = np.ascontiguousarray(u, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        oa = np.empty_like(ia)
        ob = np.empty_like(ib)
        mode = WARP_BOTH_BILINEAR if warp_mode is None else warp_mode
        _check(self._lib.qlpiv_warp_pair(self._h, pixel_type_of(ia.dtype), mode, _addr(ia), _addr(ib), ia.shape[0],
                                         ia.shape[1], len(ci), len(cj), _addr(ci), _addr(cj), _addr(u), _addr(v),
                                         int(int16_quirk), _addr(oa), _addr(ob)))
        return oa, ob

    def tile_warp(self, img_a, img_b, n, tops, lefts, u, v, warp_mode, full_max):
        """Micro / mini per-tile warping of one pair: (tiles_a, tiles_b, max_a, max_b), tiles
        shaped (len(tops) * len(lefts), n, n) in the image's dtype."""
        ia = np.ascontiguousarray(img_a)
        ib = np.ascontiguousarray(img_b, ia.dtype)
        tops = np.ascontiguousarray(tops, np.int32)
        lefts = np.ascontiguousarray(lefts, np.int32)
        u = np.ascontiguousarray(u, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        cnt = len(tops) * len(lefts)
        ta = np.empty((cnt, n, n), ia.dtype)
        tb = np.empty_like(ta)
        ma = np.empty(cnt, np.float32)
        mb = np.empty(cnt, np.float32)
        _check(self._lib.qlpiv_tile_warp(self._h, pixel_type_of(ia.dtype), _addr(ia), _addr(ib), ia.shape[0],
                                         ia.shape[1], n, len(tops), len(lefts), _addr(tops), _addr(lefts), _addr(u),
                                         _addr(v), int(warp_mode), float(full_max), _addr(ta), _addr(tb), _addr(ma),
                                         _addr(mb)))
        return ta, tb, ma, mb

    def validate(self, tops, lefts, u, v, peak_u, peak_v, npeaks, desc, n=None, height=None, width=None):
        """Vector validation of one frame's tiles (host arrays) with desc.validation's model:
        u, v (ni, nj) with the main peak accumulated; for the multi-peak model peak_u/peak_v
        (ni, nj, k) and npeaks (ni, nj), for the others None.  With the tile side n and the
        image size (required by desc.clipping_mode CLIP_NO_OUT_OF_BOUND) the call goes through
        qlpiv_validate_tiles.  Returns validated copies of (u, v) and the invalid flags."""
        u = np.array(u, np.float32, order="C", copy=True)
        v = np.array(v, np.float32, order="C", copy=True)
        ni, nj = u.shape
        multi = desc.validation == VALIDATE_MULTIPEAK_MEDIAN
        if multi:
            pu = np.ascontiguousarray(peak_u, np.float32)
            pv = np.ascontiguousarray(peak_v, np.float32)
            if pu.shape != (ni, nj, desc.num_peaks) or pv.shape != pu.shape:
                raise ValueError("peak arrays must be (ni, nj, num_peaks)")
            npk = np.ascontiguousarray(npeaks, np.int32)
            pk = (_addr(pu), _addr(pv), _addr(npk))
        else:
            pk = (None, None, None)
        tops = np.ascontiguousarray(tops, np.int32)
        lefts = np.ascontiguousarray(lefts, np.int32)
        inv = np.empty((ni, nj), np.uint8)
        if n is None:
            _check(self._lib.qlpiv_validate(self._h, ctypes.byref(desc), ni, nj, _addr(tops), _addr(lefts), _addr(u),
                                            _addr(v), *pk, _addr(inv)))
        else:
            _check(self._lib.qlpiv_validate_tiles(self._h, ctypes.byref(desc), n, height, width, ni, nj, _addr(tops),
                                                  _addr(lefts), _addr(u), _addr(v), *pk, _addr(inv)))
        return u, v, inv

    # -- dense optical flow ------------------------------------------------------
    def gaussian_filter(self, img, sigma, kernel_px):
        """GaussianFilter2D of a 2-D u8 / u16 / f32 image -> float32."""
        a = np.ascontiguousarray(img)
        out = np.empty(a.shape, np.float32)
        _check(self._lib.qlpiv_gaussian_filter(self._h, pixel_type_of(a.dtype), _addr(a), a.shape[0], a.shape[1],
                                               float(sigma), int(kernel_px), _addr(out)))
        return out

    def normalize(self, img):
        a = np.ascontiguousarray(img, np.float32)
        out = np.empty_like(a)
        _check(self._lib.qlpiv_normalize(self._h, _addr(a), a.shape[0], a.shape[1], _addr(out)))
        return out

    def dense_lk(self, img_a, img_b, us, vs, window, iterations, half_pixel=False):
        """Dense Lucas-Kanade; returns refined (us, vs) (columns, rows)."""
        a = np.ascontiguousarray(img_a, np.float32)
        b = np.ascontiguousarray(img_b, np.float32)
        u = np.array(us, np.float32, order="C", copy=True)
        v = np.array(vs, np.float32, order="C", copy=True)
        _check(self._lib.qlpiv_dense_lk(self._h, _addr(a), _addr(b), a.shape[0], a.shape[1], _addr(u), _addr(v),
                                        int(window), int(iterations), int(half_pixel)))
        return u, v

    def liu_shen(self, ls_a, ls_b, us, vs, lam, iterations_ls, lk_a=None, lk_b=None, window=27, iterations_lk=0,
                 half_pixel=False):
        """Lucas-Kanade pass (iterations_lk > 0) then Liu-Shen passes; returns (us, vs)."""
        la = np.ascontiguousarray(ls_a, np.float32)
        lb = np.ascontiguousarray(ls_b, np.float32)
        ka = np.ascontiguousarray(lk_a, np.float32) if lk_a is not None else None
        kb = np.ascontiguousarray(lk_b, np.float32) if lk_b is not None else None
        u = np.array(us, np.float32, order="C", copy=True)
        v = np.array(vs, np.float32, order="C", copy=True)
        _check(self._lib.qlpiv_liu_shen(self._h, _addr(ka), _addr(kb), _addr(la), _addr(lb), la.shape[0], la.shape[1],
                                        _addr(u), _addr(v), int(window), int(iterations_lk), float(lam),
                                        int(iterations_ls), int(half_pixel)))
        return u, v

    def flow_after_piv(self, img_a, img_b, n, tops, lefts, tile_u, tile_v, desc, dense=True):
        """Optical flow after PIV of one frame pair on a tile grid (side n, rows tops, columns
        lefts); returns (tile_u, tile_v) and, with dense, the dense field (u, v) (rows, columns)."""
        a = np.ascontiguousarray(img_a)
        b = np.ascontiguousarray(img_b, a.dtype)
        tops = np.ascontiguousarray(tops, np.int32)
        lefts = np.ascontiguousarray(lefts, np.int32)
        tu = np.array(tile_u, np.float32, order="C", copy=True)
        tv = np.array(tile_v, np.float32, order="C", copy=True)
        if tu.shape != (len(tops), len(lefts)) or tv.shape != tu.shape:
            raise ValueError("tile displacements must be (len(tops), len(lefts))")
        du = np.empty(a.shape, np.float32) if dense else None
        dv = np.empty(a.shape, np.float32) if dense else None
        _check(self._lib.qlpiv_flow_after_piv(self._h, ctypes.byref(desc), pixel_type_of(a.dtype), _addr(a), _addr(b),
                                              a.shape[0], a.shape[1], int(n), len(tops), len(lefts), _addr(tops),
                                              _addr(lefts), _addr(tu), _addr(tv), _addr(du), _addr(dv)))
        return (tu, tv, du, dv) if dense else (tu, tv)

    def piv_flow(self, frames_a, frames_b, desc, flow, dense=False):
        """Adaptive PIV followed by the optical flow after PIV of every pair; returns (u, v)
        shaped (pairs, tiles_i, tiles_j), plus the dense fields (pairs, h, w) with dense."""
        fa = [np.ascontiguousarray(x) for x in frames_a]
        fb = [np.ascontiguousarray(x) for x in frames_b]
        h, w = fa[0].shape
        dt = fa[0].dtype
        table = (Frame * len(fa))()
        for k, (x, y) in enumerate(zip(fa, fb)):
            if x.shape != (h, w) or y.shape != (h, w) or x.dtype != dt or y.dtype != dt:
                raise ValueError("all frames must share shape and dtype")
            table[k] = Frame(x.ctypes.data, y.ctypes.data, h, w, w)
        last = adaptive_levels(desc, h, w)[-1]
        u = np.empty((len(fa), last["tiles_i"], last["tiles_j"]), np.float32)
        v = np.empty_like(u)
        du = np.empty((len(fa), h, w), np.float32) if dense else None
        dv = np.empty((len(fa), h, w), np.float32) if dense else None
        _check(self._lib.qlpiv_piv_flow(self._h, ctypes.byref(desc), ctypes.byref(flow), pixel_type_of(dt), h, w,
                                        len(fa), table, _addr(u), _addr(v), _addr(du), _addr(dv)))
        return (u, v, du, dv) if dense else (u, v)

    def piv_flow_device(self, desc, flow, pixel_type, height, width, num_pairs, frames, out_u, out_v, dense_u=None,
                        dense_v=None):
        """Queue adaptive PIV plus optical flow over a device frame table into device outputs."""
        a = [x if isinstance(x, int) or x is None else _addr(x) for x in (frames, out_u, out_v, dense_u, dense_v)]
        _check(self._lib.qlpiv_piv_flow_device(self._h, ctypes.byref(desc), ctypes.byref(flow), pixel_type, height,
                                               width, num_pairs, *a))

    def piv_adaptive(self, frames_a, frames_b, desc):
        """Adaptive multi-pass PIV of image pairs of one size; returns (u, v) of the last
        level shaped (pairs, tiles_i, tiles_j)."""
        fa = [np.ascontiguousarray(x) for x in frames_a]
        fb = [np.ascontiguousarray(x) for x in frames_b]
        h, w = fa[0].shape
        dt = fa[0].dtype
        table = (Frame * len(fa))()
        for k, (x, y) in enumerate(zip(fa, fb)):
            if x.shape != (h, w) or y.shape != (h, w) or x.dtype != dt or y.dtype != dt:
                raise ValueError("all frames must share shape and dtype")
            table[k] = Frame(x.ctypes.data, y.ctypes.data, h, w, w)
        last = adaptive_levels(desc, h, w)[-1]
        u = np.empty((len(fa), last["tiles_i"], last["tiles_j"]), np.float32)
        v = np.empty_like(u)
        _check(self._lib.qlpiv_piv_adaptive(self._h, ctypes.byref(desc), pixel_type_of(dt), h, w, len(fa), table,
                                            _addr(u), _addr(v)))
        return u, v

    def piv_adaptive_device(self, desc, pixel_type, height, width, num_pairs, frames, out_u, out_v):
        """Queue adaptive PIV over a device frame table into device outputs."""
        a = [x if isinstance(x, int) else _addr(x) for x in (frames, out_u, out_v)]
        _check(self._lib.qlpiv_piv_adaptive_device(self._h, ctypes.byref(desc), pixel_type, height, width, num_pairs,
                                                   a[0], a[1], a[2]))


def adaptive_plan_bytes(desc, pixel_type, height, width, pairs=1):
    """Device bytes of an adaptive plan (the request server's admission estimate)."""
    b = ctypes.c_int64()
    _check(load_library().qlpiv_adaptive_plan_bytes(ctypes.byref(desc), pixel_type, height, width, pairs,
                                                    ctypes.byref(b)))
    return b.value


def tiff_info(path):
    """(height, width, bits_per_sample) of a baseline greyscale TIFF."""
    h, w, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(load_library().qlpiv_tiff_info(os.fsencode(path), ctypes.byref(h), ctypes.byref(w), ctypes.byref(b)))
    return h.value, w.value, b.value


def read_tiff(path):
    """Decode a baseline greyscale TIFF (8 or 16 bits, uncompressed or PackBits) to a uint8 /
    uint16 array, the frame reader of S/jobs/ImageReaderJob.java:81-115."""
    h, w, b = tiff_info(path)
    out = np.empty((h, w), np.uint8 if b == 8 else np.uint16)
    _check(load_library().qlpiv_tiff_read(os.fsencode(path), out.ctypes.data, out.nbytes))
    return out


MAT_RUN, MAT_STEP, MAT_DENSE = 0, 1, 2


def export_mat(path, maps, image_height, image_width, ia_start, ia_end, overlap_factor, swap_uv=False,
               mark_invalid_as_nan=False, export_date=None, layout=MAT_RUN, maps_per_file=0):
    """Write the vector maps as a MATLAB level-5 file with the variables of
    S/exporter/StructMultiFrameFloatVelocityExporter.java.

    maps: one dict per IA size with u (row displacements) and v (column displacements), frames x
    tiles_i x tiles_j float32, ia (height, width), margins (top, left, bottom, right), optionally
    adaptive_step (MAT_STEP layout) and invalid (same shape, bool).  MAT_RUN (the end-of-run
    export) stores the column displacement as `u` unless swap_uv, as PIVMap does.
    maps_per_file: split the frames into volumes (path with _MV0.mat, volume k as _MV<k>.mat)."""
    keep, table = [], (MatVelocityMap * max(1, len(maps)))()
    frames = None
    for k, m in enumerate(maps):
        u = np.ascontiguousarray(m["u"], np.float32)
        v = np.ascontiguousarray(m["v"], np.float32)
        if u.ndim == 2:
            u, v = u[None], v[None]
        if u.shape != v.shape or u.ndim != 3:
            raise ValueError("u and v must be frames x tiles_i x tiles_j")
        if frames is not None and u.shape[0] != frames:
            raise ValueError("every map needs the same number of frames")
        frames = u.shape[0]
        inv = m.get("invalid")
        inv = None if inv is None else np.ascontiguousarray(np.asarray(inv).reshape(u.shape), np.uint8)
        keep += [u, v, inv]
        e = table[k]
        e.ia_height, e.ia_width = (int(x) for x in m["ia"])
        e.adaptive_step = int(m.get("adaptive_step", 0))
        e.tiles_i, e.tiles_j = u.shape[1], u.shape[2]
        e.margins[:] = [int(x) for x in m.get("margins", (0, 0, 0, 0))]
        e.u, e.v = u.ctypes.data, v.ctypes.data
        e.invalid = None if inv is None else inv.ctypes.data
    p = MatExportParams(image_width=image_width, image_height=image_height, ia_start=ia_start, ia_end=ia_end,
                        overlap_factor=overlap_factor, frames=1 if frames is None else frames, swap_uv=int(bool(swap_uv)),
                        mark_invalid_as_nan=int(bool(mark_invalid_as_nan)), layout=layout,
                        export_date=None if export_date is None else export_date.encode(),
                        maps_per_file=int(maps_per_file))
    _check(load_library().qlpiv_mat_export(os.fsencode(path), ctypes.byref(p), len(maps), table))


def export_adaptive_mat(path, desc, height, width, u, v, invalid=None, **kw):
    """Export piv_adaptive's final vector maps (pairs x tiles_i x tiles_j) with the last level's
    IA size, margins and adaptive step, as the reference exports a PIV run's result map."""
    levels = adaptive_levels(desc, height, width)
    g = levels[-1]
    m = dict(u=u, v=v, ia=(g["n"], g["n"]), adaptive_step=len(levels) - 1, invalid=invalid,
             margins=(g["margin_top"], g["margin_left"], g["margin_bottom"], g["margin_right"]))
    export_mat(path, [m], height, width, desc.ia_start, desc.ia_end, desc.overlap_factor, **kw)


def export_dense_mat(path, desc, height, width, dense_u, dense_v, **kw):
    """Export a dense flow field (pairs x height x width, rows / columns as qlpiv_flow_after_piv
    returns it) in the reference's dense layout: one `velocities` struct over the pixels inside
    the last level's margins."""
    g = adaptive_levels(desc, height, width)[-1]
    m = dict(u=dense_u, v=dense_v, ia=(g["n"], g["n"]),
             margins=(g["margin_top"], g["margin_left"], g["margin_bottom"], g["margin_right"]))
    export_mat(path, [m], height, width, desc.ia_start, desc.ia_end, desc.overlap_factor, layout=MAT_DENSE, **kw)


class AdaptiveBatch:
    """Adaptive batch (qlpiv_adaptive_batch_*): pairs of uneven sizes, each with its own adaptive
    schedule (schedules[schedule_of_pair[q]]), one graph launch per batch; pairs of one size and
    schedule share a group.  frames: FRAME_DTYPE table of device images."""

    def __init__(self, handle, frames, pixel_type, schedules, schedule_of_pair):
        self._h = handle
        self._lib = handle._lib
        table = np.ascontiguousarray(frames, FRAME_DTYPE)
        self.num_pairs = len(table)
        descs = (AdaptiveDesc * len(schedules))(*schedules)
        sidx = np.ascontiguousarray(schedule_of_pair, np.int32)
        p = ctypes.c_void_p()
        _check(self._lib.qlpiv_adaptive_batch_create(handle._h, pixel_type, self.num_pairs, table.ctypes.data,
                                                     descs, len(schedules), _addr(sidx), ctypes.byref(p)))
        self._p = p
        tot = ctypes.c_int64()
        groups = ctypes.c_int32()
        self.pair_offset = np.empty(self.num_pairs + 1, np.int64)
        self.tiles = np.empty((self.num_pairs, 2), np.int32)
        _check(self._lib.qlpiv_adaptive_batch_info(p, ctypes.byref(tot), _addr(self.pair_offset),
                                                   _addr(self.tiles), ctypes.byref(groups)))
        self.total = tot.value
        self.groups = groups.value

    def run(self):
        """Queues the batch on the handle's stream; returns the device addresses of (u, v)."""
        u, v = ctypes.c_void_p(), ctypes.c_void_p()
        _check(self._lib.qlpiv_adaptive_batch_run(self._h._h, self._p, ctypes.byref(u), ctypes.byref(v)))
        return u.value, v.value

    def displacements(self):
        u = np.empty(self.total, np.float32)
        v = np.empty(self.total, np.float32)
        _check(self._lib.qlpiv_adaptive_batch_download(self._h._h, self._p, _addr(u), _addr(v)))
        return u, v

    def pair(self, arr, q):
        ti, tj = int(self.tiles[q][0]), int(self.tiles[q][1])
        o = int(self.pair_offset[q])
        return arr[o:o + ti * tj].reshape(ti, tj)

    def close(self):
        if getattr(self, "_p", None):
            self._lib.qlpiv_adaptive_batch_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MixedPlan:
    """Mixed batch plan (qlpiv_mixed_plan_*): pairs of uneven sizes, each with its own IA size
    and overlap, one graph launch per batch.  frames: FRAME_DTYPE table of device images;
    autotune: AUTOTUNE_OFF / AUTOTUNE_ON (True) / AUTOTUNE_PERSISTENT.  `schedule` is the one
    the graph runs (SCHEDULE_PER_SIZE or SCHEDULE_PERSISTENT)."""

    def __init__(self, handle, frames, ia_sizes, overlap_factors, pixel_type, autotune=True, **desc_kw):
        self._h = handle
        self._lib = handle._lib
        table = np.ascontiguousarray(frames, FRAME_DTYPE)
        sizes = np.ascontiguousarray(ia_sizes, np.int32)
        ofac = np.ascontiguousarray(overlap_factors, np.float32)
        self.num_pairs = len(table)
        d = Handle.desc(16, **desc_kw)
        p = ctypes.c_void_p()
        _check(self._lib.qlpiv_mixed_plan_create(handle._h, ctypes.byref(d), pixel_type, self.num_pairs,
                                                 table.ctypes.data, _addr(sizes), _addr(ofac), int(autotune),
                                                 ctypes.byref(p)))
        self._p = p
        tot = ctypes.c_int64()
        self.pair_offset = np.empty(self.num_pairs + 1, np.int64)
        self.tiles = np.empty((self.num_pairs, 2), np.int32)
        self.waves = np.empty(4, np.int32)
        _check(self._lib.qlpiv_mixed_plan_info(p, ctypes.byref(tot), _addr(self.pair_offset), _addr(self.tiles),
                                               _addr(self.waves)))
        self.total = tot.value
        sched = ctypes.c_int32()
        _check(self._lib.qlpiv_mixed_plan_schedule(p, ctypes.byref(sched)))
        self.schedule = sched.value

    def run(self):
        """Queues the batch on the handle's stream; returns the device address of the vectors."""
        out = ctypes.c_void_p()
        _check(self._lib.qlpiv_mixed_plan_run(self._h._h, self._p, ctypes.byref(out)))
        return out.value

    def vectors(self):
        out = np.empty(self.total, VECTOR_DTYPE)
        _check(self._lib.qlpiv_mixed_plan_download(self._h._h, self._p, _addr(out)))
        return out

    def pair_vectors(self, vec, q):
        ti, tj = int(self.tiles[q][0]), int(self.tiles[q][1])
        o = int(self.pair_offset[q])
        return vec[o:o + ti * tj].reshape(ti, tj)

    def close(self):
        if getattr(self, "_p", None):
            self._lib.qlpiv_mixed_plan_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request server (qlpiv_server_*): submit frame pairs of any size with their own adaptive
    schedule from any thread, poll for the displacements."""

    def __init__(self, device=0, slots=0, hbm_budget=0, staging_bytes=0, submit_timeout_ms=0):
        lib = load_library()
        self._lib = lib
        p = ServerParams()
        p.device, p.slots, p.hbm_budget, p.staging_bytes, p.submit_timeout_ms = (device, slots, hbm_budget,
                                                                                  staging_bytes, submit_timeout_ms)
        s = ctypes.c_void_p()
        _check(lib.qlpiv_server_create(ctypes.byref(p), ctypes.byref(s)))
        self._s = s
        self._outs = {}

    def close(self):
        if getattr(self, "_s", None):
            self._lib.qlpiv_server_destroy(self._s)
            self._s = None
            self._outs.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, img_a, img_b, desc):
        """Queues one pair (2-D u8 / u16 arrays of one shape); returns the ticket."""
        a = np.ascontiguousarray(img_a)
        b = np.ascontiguousarray(img_b, a.dtype)
        h, w = a.shape
        last = adaptive_levels(desc, h, w)[-1]
        u = np.empty((last["tiles_i"], last["tiles_j"]), np.float32)
        v = np.empty_like(u)
        r = Request()
        keep_desc = AdaptiveDesc.from_buffer_copy(desc)
        r.schedule = ctypes.pointer(keep_desc)
        r.pixel_type, r.height, r.width, r.pitch = pixel_type_of(a.dtype), h, w, w
        r.img_a, r.img_b, r.out_u, r.out_v = a.ctypes.data, b.ctypes.data, u.ctypes.data, v.ctypes.data
        t = ctypes.c_uint64()
        _check(self._lib.qlpiv_submit(self._s, ctypes.byref(r), ctypes.byref(t)))
        self._outs[t.value] = (u, v)   # the library writes them before poll reports the ticket done
        return t.value

    def poll(self, ticket, timeout_ms=-1):
        """None while the request runs (timeout); else (u, v, info); raises on a failed request."""
        res = Result()
        st = self._lib.qlpiv_poll(self._s, ctypes.c_uint64(ticket), ctypes.byref(res), int(timeout_ms))
        if st == E_TIMEOUT:
            return None
        _check(st)
        u, v = self._outs.pop(ticket)
        info = {"queue_ms": res.queue_ms, "device_ms": res.device_ms, "total_ms": res.total_ms,
                "tiles": (res.tiles_i, res.tiles_j)}
        if res.status != OK:
            raise QlpivError(res.status, self._lib.qlpiv_last_error().decode())
        return u, v, info

    def stats(self):
        st = ServerStats()
        _check(self._lib.qlpiv_server_stats_read(self._s, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_ if k != "reserved"}


from . import grid, jobs, per_call, synth  # noqa: E402,F401
