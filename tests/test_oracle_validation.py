"""Pins the oracle's multi-peak search and vector validation.

Known answers from the reference's own tests:
  * tests/pt/quickLabPIV/util/SimpleFixedLengthFloatLinkedListTests.java:99-400 -- the sorted,
    adjacency-suppressing peak list (3 entries, kernel width 5);
  * tests/pt/quickLabPIV/maximum/FindMaximumMultiPeakTests.java:24-158 -- 10x10 plane, 4 peaks,
    3x3 cells.
The reference has no test of the validator or the replacements; those are checked against
a second, independent restatement (tests/validation_ref.py) and by properties.
"""
import numpy as np
import pytest

import validation_ref as vref
from validation_cases import smooth_case


# ---- SimpleFixedLengthFloatLinkedList.addInAscendOrder known answers (3 entries, kw 5) ----
BASE = [(70, 1, 5), (30, 3, 1), (50, 8, 9)]
LIST_KATS = [
    (BASE, [(30, 3, 1), (50, 8, 9), (70, 1, 5)]),
    (BASE + [(55, 8, 8)], [(30, 3, 1), (55, 8, 8), (70, 1, 5)]),
    (BASE + [(35, 4, 1)], [(35, 4, 1), (50, 8, 9), (70, 1, 5)]),
    (BASE + [(75, 1, 6)], [(30, 3, 1), (50, 8, 9), (75, 1, 6)]),
    ([(70, 7, 1), (30, 3, 3), (50, 8, 9), (55, 5, 6)], [(55, 5, 6), (70, 7, 1)]),
    (BASE + [(49, 7, 9)], [(30, 3, 1), (50, 8, 9), (70, 1, 5)]),
    (BASE + [(29, 3, 2)], [(30, 3, 1), (50, 8, 9), (70, 1, 5)]),
    (BASE + [(69, 2, 4)], [(30, 3, 1), (50, 8, 9), (70, 1, 5)]),
    (BASE + [(70, 2, 4)], [(30, 3, 1), (50, 8, 9), (70, 1, 5)]),
    ([(70, 2, 3)], [(70, 2, 3)]),
]


@pytest.mark.parametrize("entries,expected", LIST_KATS)
def test_peak_list_known_answers(oracle, entries, expected):
    got = oracle.mp_list_run(3, 5, entries)
    assert [(float(v), i, j) for v, i, j in expected] == got
    ref = vref.PeakList(3, 5)
    for e in entries:
        ref.add(*e)
    assert [(float(v), i, j) for v, i, j in ref.items] == got


def test_multipeak_known_answer(oracle):
    m = np.full((10, 10), 12.0, np.float32)
    m[3, 6] = 15.0
    m[4, 5] = 16.0
    m[9, 4] = 13.0
    peaks, _ = oracle.find_max_multipeaks(m, 3, 4)
    assert peaks[0] == (4, 5, 16.0)       # 15 at (3, 6) is suppressed next to 16
    assert peaks[1] == (9, 4, 13.0)
    assert peaks[2][2] == 12.0
    assert vref.find_max_multipeaks(m, 3, 4)[0] == peaks


@pytest.mark.parametrize("d,kw,k", [(31, 3, 3), (63, 3, 4), (31, 5, 2), (15, 3, 1), (7, 3, 6), (127, 3, 3),
                                    (10, 4, 5)])
def test_multipeak_matches_independent_restatement(oracle, d, kw, k):
    rng = np.random.default_rng(d * 100 + kw * 10 + k)
    for trial in range(6):
        m = rng.normal(0.0, 1.0, (d, d)).astype(np.float32)
        if trial % 3 == 1:
            m = np.abs(m)                        # plane of positives, like a real correlation
        if trial % 3 == 2:
            m = np.round(m * 2).astype(np.float32)   # many ties and zero cells (stale positions)
        for _ in range(3):
            m[rng.integers(d), rng.integers(d)] += rng.uniform(3, 6)
        got, mf = oracle.find_max_multipeaks(m, kw, k)
        exp, emf = vref.find_max_multipeaks(m, kw, k)
        assert got == exp, (trial, got, exp)
        assert mf == emf == float(m.min())


def test_multipeak_pass_peak0_is_the_plane_maximum(oracle, rankine_pair):
    a, b = rankine_pair
    g, tops, lefts = oracle.grid_origins(a.shape[0], a.shape[1], 32, 0.5)
    sel = slice(0, None, 7)
    vec, npk = oracle.piv_pass_multi(a, b, 32, tops[sel], lefts[sel], num_peaks=3, kernel_width=3)
    assert (npk == 3).all()
    for r, (t, l) in enumerate(zip(tops[sel], lefts[sel])):
        ta, ma = oracle.clip_tile(a, int(t), int(l), 32)
        tb, _ = oracle.clip_tile(b, int(t), int(l), 32)
        plane = oracle.xcorr_fft(ta, tb, ma, ma)
        peaks, mf = oracle.find_max_multipeaks(plane, 3, 3)
        assert [(p[0], p[1]) for p in peaks] == [(int(x["peak_i"]), int(x["peak_j"])) for x in vec[r]]
        assert peaks[0][2] == float(plane.max())
        assert vec[r][0]["min_floor"] == mf == float(plane.min())
        # secondary peaks are never larger and never adjacent to a larger one
        vals = [p[2] for p in peaks]
        assert vals == sorted(vals, reverse=True)


@pytest.mark.parametrize("ni,nj", [(1, 1), (1, 5), (2, 3), (3, 3), (4, 4), (5, 8), (7, 6), (61, 61), (64, 63)])
def test_spiral_order(oracle, ni, nj):
    got = oracle.spiral_order(ni, nj).tolist()
    assert sorted(got) == list(range(ni * nj))
    assert got == vref.spiral_order(ni, nj)
    ci = (ni - 1) // 2
    cj = (nj - 1) // 2
    assert got[0] == ci * nj + cj


@pytest.mark.parametrize("seed", range(8))
@pytest.mark.parametrize("k", [1, 2, 3])
def test_validation_matches_independent_restatement(oracle, seed, k):
    rng = np.random.default_rng(seed * 31 + k)
    ni, nj = [(9, 11), (12, 12), (5, 7), (16, 13)][seed % 4]
    outliers = [3, 8, 20, 1][seed % 4]
    tops, lefts, u, v, pu, pv, npk, _, _ = smooth_case(rng, ni, nj, k, outliers)
    iterate_until = seed % 3 == 0
    cfg = oracle.valid_cfg(num_peaks=k, threshold=2.0, epsilon0=0.1, max_iterations=1 + seed % 3,
                           iterate_until_no_corrections=iterate_until)
    gu, gv, ginv, gs = oracle.validate(tops, lefts, u, v, pu, pv, npk, cfg)
    eu, ev, einv, es = vref.validate(tops, lefts, u, v, pu, pv, npk, k, 2.0, 0.1, 1 + seed % 3, iterate_until)
    assert gs == es
    np.testing.assert_array_equal(ginv, einv)
    np.testing.assert_array_equal(gu.view(np.uint32), eu.view(np.uint32))
    np.testing.assert_array_equal(gv.view(np.uint32), ev.view(np.uint32))


def test_validation_keeps_a_smooth_field(oracle):
    rng = np.random.default_rng(5)
    tops, lefts, u, v, pu, pv, npk, _, _ = smooth_case(rng, 10, 10, 3, 0)
    gu, gv, inv, sweeps = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg())
    assert not inv.any() and sweeps == 1
    np.testing.assert_array_equal(gu, u)
    np.testing.assert_array_equal(gv, v)


def test_validation_repairs_isolated_outliers(oracle):
    rng = np.random.default_rng(11)
    tops, lefts, u, v, pu, pv, npk, tu, tv = smooth_case(rng, 14, 14, 3, 6)
    gu, gv, inv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(num_peaks=3))
    assert not inv.any()
    # every repaired vector is back near the smooth field (secondary peak or interpolation)
    assert np.abs(gu - tu).max() < 0.5 and np.abs(gv - tv).max() < 0.5


def test_validation_secondary_peak_is_exact(oracle):
    rng = np.random.default_rng(2)
    tops, lefts, u, v, pu, pv, npk, tu, tv = smooth_case(rng, 9, 9, 2, 0)
    u[4, 4] += 7.0
    v[4, 4] -= 5.0
    pu[4, 4, 1] = pu[4, 4, 0] - 7.0
    pv[4, 4, 1] = pv[4, 4, 0] + 5.0
    gu, gv, inv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(num_peaks=2))
    assert not inv.any()
    f = np.float32
    assert gu[4, 4] == f(f(u[4, 4] - pu[4, 4, 0]) + pu[4, 4, 1])
    assert gv[4, 4] == f(f(v[4, 4] - pv[4, 4, 0]) + pv[4, 4, 1])


def test_validation_bilinear_fallback(oracle):
    rng = np.random.default_rng(3)
    tops, lefts, u, v, pu, pv, npk, tu, tv = smooth_case(rng, 9, 9, 1, 0)
    u[:] = 1.0
    v[:] = -2.0
    u[4, 4] = 9.0
    gu, gv, inv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(num_peaks=1))
    assert not inv.any()
    assert gu[4, 4] == 1.0 and gv[4, 4] == -2.0


def test_validation_zeroes_what_it_cannot_repair(oracle):
    # a 1x2 grid: every tile's lone neighbour is itself invalid after the first sweep
    tops = np.array([0], np.int32)
    lefts = np.array([0, 16], np.int32)
    u = np.array([[0.0, 50.0]], np.float32)
    v = np.zeros((1, 2), np.float32)
    pu = np.zeros((1, 2, 1), np.float32)
    pv = np.zeros((1, 2, 1), np.float32)
    npk = np.ones((1, 2), np.int32)
    gu, gv, inv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(num_peaks=1))
    eu, ev, einv, _ = vref.validate(tops, lefts, u, v, pu, pv, npk, 1, 2.0, 0.1, 2)
    np.testing.assert_array_equal(inv, einv)
    np.testing.assert_array_equal(gu, eu)
    assert (gu[inv == 1] == 0).all()


def _tile_grid(oracle, h, w, n):
    _, tops, lefts = oracle.grid(h, w, n, 0, 0.5)
    return tops, lefts


def test_micro_warp_integer_displacement_is_a_shift(oracle):
    """Micro warping by a whole-pixel displacement cuts the tiles at the displaced origins
    (BiLinearImageMicroAndMiniWarpingStrategy: floor(u) moves the tile, the fraction warps)."""
    rng = np.random.default_rng(4)
    a = rng.integers(0, 255, (96, 112)).astype(np.uint8)
    b = rng.integers(0, 255, (96, 112)).astype(np.uint8)
    n = 16
    tops, lefts = _tile_grid(oracle, 96, 112, n)
    cnt = len(tops) * len(lefts)
    u = np.full(cnt, 4.0, np.float32)
    v = np.full(cnt, -2.0, np.float32)
    for mode in (oracle.WARP_FIRST_MICRO, oracle.WARP_SECOND_MICRO, oracle.WARP_BOTH_MICRO):
        ta, tb, ma, mb = oracle.tile_warp(a, b, n, tops, lefts, u, v, mode, 255.0)
        for k in range(cnt):
            t, l = tops[k // len(lefts)], lefts[k % len(lefts)]
            da, db = {oracle.WARP_FIRST_MICRO: ((-4, 2), (0, 0)), oracle.WARP_SECOND_MICRO: ((0, 0), (4, -2)),
                      oracle.WARP_BOTH_MICRO: ((-2, 1), (2, -1))}[mode]

            def cut(img, dy, dx):
                y0, x0 = t + dy, l + dx
                out = np.zeros((n, n), np.float32)
                for i in range(n):
                    for j in range(n):
                        yy = min(max(y0 + i, 0), 95)
                        xx = min(max(x0 + j, 0), 111)
                        out[i, j] = img[yy, xx]
                return out
            np.testing.assert_array_equal(ta[k], cut(a, *da))
            np.testing.assert_array_equal(tb[k], cut(b, *db))
            assert ma[k] == (max(16, a[t:t + n, l:l + n].max()) if mode == oracle.WARP_SECOND_MICRO else 255.0)
            assert mb[k] == (max(16, b[t:t + n, l:l + n].max()) if mode == oracle.WARP_FIRST_MICRO else 255.0)


def test_mini_warp_of_a_uniform_field_equals_micro(oracle):
    """With every tile displaced alike the mini spline is flat: mini == micro."""
    rng = np.random.default_rng(5)
    a = rng.integers(0, 4095, (128, 128)).astype(np.uint16)
    b = rng.integers(0, 4095, (128, 128)).astype(np.uint16)
    n = 32
    tops, lefts = _tile_grid(oracle, 128, 128, n)
    cnt = len(tops) * len(lefts)
    u = np.full(cnt, 1.375, np.float32)
    v = np.full(cnt, -0.625, np.float32)
    for micro, mini in ((oracle.WARP_FIRST_MICRO, oracle.WARP_FIRST_MINI),
                        (oracle.WARP_SECOND_MICRO, oracle.WARP_SECOND_MINI),
                        (oracle.WARP_BOTH_MICRO, oracle.WARP_BOTH_MINI)):
        r1 = oracle.tile_warp(a, b, n, tops, lefts, u, v, micro, 4095.0)
        r2 = oracle.tile_warp(a, b, n, tops, lefts, u, v, mini, 4095.0)
        for x, y in zip(r1, r2):
            np.testing.assert_array_equal(x, y)


# ---- the four single-strategy models and NoOutOfBoundClipping of the replacements ----

def _clip_geometry(tops, lefts, n=16):
    """An image whose last tile row touches the bottom edge and whose last column ends 2 px
    inside the right edge, so that replacements near the borders are refused."""
    return n, int(tops[-1]) + n, int(lefts[-1]) + n + 2


@pytest.mark.parametrize("model", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("clip", [False, True])
@pytest.mark.parametrize("seed", range(4))
def test_validation_models_match_independent_restatement(oracle, model, clip, seed):
    rng = np.random.default_rng(100 + seed * 7 + model)
    k = 3 if model == 1 else 1
    ni, nj = [(9, 11), (12, 12), (5, 7), (16, 13)][seed]
    tops, lefts, u, v, pu, pv, npk, _, _ = smooth_case(rng, ni, nj, k, [3, 8, 20, 1][seed])
    geo = _clip_geometry(tops, lefts) if clip else None
    thr = 1.5 if model in (2, 3) else 2.0
    cfg = oracle.valid_cfg(num_peaks=k, threshold=thr, epsilon0=0.1, max_iterations=2, model=model, clip=geo)
    gu, gv, ginv, gs = oracle.validate(tops, lefts, u, v, pu, pv, npk, cfg)
    eu, ev, einv, es = vref.validate(tops, lefts, u, v, pu, pv, npk, k, thr, 0.1, 2, False, model=model, clip=geo)
    assert gs == es
    np.testing.assert_array_equal(ginv, einv)
    np.testing.assert_array_equal(gu.view(np.uint32), eu.view(np.uint32))
    np.testing.assert_array_equal(gv.view(np.uint32), ev.view(np.uint32))


def test_difference_models_never_validate(oracle):
    """Every tile starts invalid and the difference validator only looks at valid top-left, top
    and left neighbours, so no tile is ever validated: every vector ends at 0, except where
    NoOutOfBoundClipping refuses the 0 (tiles touching the bottom edge keep their value)."""
    rng = np.random.default_rng(3)
    tops, lefts, u, v, pu, pv, npk, _, _ = smooth_case(rng, 9, 10, 1, 0)
    for model in (2, 3):
        gu, gv, inv, sweeps = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(model=model))
        assert inv.all() and not gu.any() and not gv.any() and sweeps == 1
        geo = _clip_geometry(tops, lefts)
        cu, cv, inv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(model=model, clip=geo))
        assert inv.all()
        assert np.array_equal(cu[-1], u[-1]) and np.array_equal(cv[-1], v[-1])   # 0 refused on the last row
        assert not cu[:-1].any() and not cv[:-1].any()


def test_median_only_zeroes_without_replacing(oracle):
    rng = np.random.default_rng(4)
    tops, lefts, u, v, pu, pv, npk, tu, tv = smooth_case(rng, 12, 12, 1, 6)
    ou, ov, inv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(model=4))
    assert inv.sum() >= 6
    assert not ou[inv.astype(bool)].any()
    assert np.array_equal(ou[~inv.astype(bool)], u[~inv.astype(bool)])
    bu, bv, binv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(model=5))
    assert binv.sum() < inv.sum()                     # bilinear replacement repairs most of them
    fixed = inv.astype(bool) & ~binv.astype(bool)
    assert np.abs(bu[fixed] - tu[fixed]).max() < 1.0


def test_clipping_refuses_replacements_that_leave_the_image(oracle):
    """Bilinear replacement of an outlier on the bottom row under NoOutOfBoundClipping: the value
    is refused (the tile touches the bottom edge), the revalidation finds the outlier again, and
    the final zeroing is refused too: the vector keeps its value and stays invalid."""
    rng = np.random.default_rng(9)
    tops, lefts, u, v, pu, pv, npk, _, _ = smooth_case(rng, 8, 8, 1, 0)
    u[-1, 3] += 7.0
    geo = _clip_geometry(tops, lefts)
    au, av, ainv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(model=5))
    cu, cv, cinv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, oracle.valid_cfg(model=5, clip=geo))
    assert abs(au[-1, 3] - u[-1, 3]) > 5.0            # allowed: replaced by the neighbours' estimate
    assert cu[-1, 3] == u[-1, 3] and cinv[-1, 3]      # every replacement refused
