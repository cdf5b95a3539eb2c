"""Parity criteria shared by the GPU tests.

Integer peaks: bit-exact against the FP64 oracle except exact ties, where a tie is two
candidate cells whose FP64 correlation values differ by less than TIE_REL * peak (the
FP32 rounding level of the reference path itself).  Sub-pixel displacement: within
SUBPIX_TOL px of the FP64 oracle, for IAs whose integer peaks agree.  The acceptance
test |delta| <= 1 px of the 3-point fit is a threshold; IAs whose FP64 delta lies
within BORDER of it are not compared.
"""
import numpy as np

TIE_REL = 2e-6
SUBPIX_TOL = 1e-3
BORDER = 1e-3


def tile_pairs(oracle, img_a, img_b, n, a_top, a_left, b_top, b_left, idx):
    out = []
    for k in idx:
        ta, ma = oracle.clip_tile(img_a, int(a_top[k]), int(a_left[k]), n)
        tb, mb = oracle.clip_tile(img_b, int(b_top[k]), int(b_left[k]), n)
        out.append((ta, tb, ma, mb))
    return out


def compare_vectors(oracle, gpu, ref64, img_a, img_b, n, a_top, a_left, b_top, b_left, norm_mode,
                    fixed_max=(255.0, 255.0)):
    """Returns a dict of counts; raises AssertionError with details on a parity break."""
    gi = np.stack([gpu["peak_i"], gpu["peak_j"]], 1).astype(np.int32)
    ri = np.stack([ref64["peak_i"], ref64["peak_j"]], 1).astype(np.int32)
    mism = np.nonzero((gi != ri).any(1))[0]
    ties = 0
    for k in mism:
        ta, ma = oracle.clip_tile(img_a, int(a_top[k]), int(a_left[k]), n)
        tb, mb = oracle.clip_tile(img_b, int(b_top[k]), int(b_left[k]), n)
        if norm_mode == oracle.NORM_MAX_A:
            mb = ma
        elif norm_mode == oracle.NORM_FIXED:
            ma, mb = fixed_max
        p = oracle.xcorr_fft(ta, tb, ma, mb, normalize=norm_mode != oracle.NORM_NONE, precision=64)
        vg = p[gi[k, 0], gi[k, 1]]
        vr = p[ri[k, 0], ri[k, 1]]
        if abs(vg - vr) <= TIE_REL * max(abs(vr), 1e-30):
            ties += 1
            continue
        raise AssertionError(f"IA {k}: GPU peak {tuple(gi[k])} (fp64 value {vg}) vs oracle {tuple(ri[k])} ({vr})")
    same = np.ones(len(gpu), bool)
    same[mism] = False
    # flags describing the fit outcome must agree where the peaks agree
    fl_mask = 0x1F
    dflag = (gpu["flags"] & fl_mask) != (ref64["flags"] & fl_mask)
    d_i = np.abs(ref64["sub_i"].astype(np.float64) - ref64["peak_i"])
    d_j = np.abs(ref64["sub_j"].astype(np.float64) - ref64["peak_j"])
    border = (np.abs(d_i - 1.0) < BORDER) | (np.abs(d_j - 1.0) < BORDER)
    bad_flags = np.nonzero(same & dflag & ~border)[0]
    if len(bad_flags):
        k = bad_flags[0]
        raise AssertionError(f"IA {k}: flags {gpu['flags'][k]} vs oracle {ref64['flags'][k]}")
    cmp = same & ~border
    eu = np.abs(gpu["u"].astype(np.float64) - ref64["u64"])[cmp]
    ev = np.abs(gpu["v"].astype(np.float64) - ref64["v64"])[cmp]
    worst = float(max(eu.max(initial=0.0), ev.max(initial=0.0)))
    if worst > SUBPIX_TOL:
        k = np.nonzero(cmp)[0][np.argmax(np.maximum(np.abs(gpu["u"] - ref64["u64"])[cmp],
                                                    np.abs(gpu["v"] - ref64["v64"])[cmp]))]
        raise AssertionError(f"sub-pixel error {worst:.3e} px > {SUBPIX_TOL} at IA {k}: gpu ({gpu['u'][k]}, "
                             f"{gpu['v'][k]}) fp64 ({ref64['u64'][k]}, {ref64['v64'][k]})")
    return {"count": len(gpu), "ties": ties, "compared": int(cmp.sum()), "max_err_px": worst}
