"""Pins the oracle's dense optical-flow stages to the reference's fixtures.

* Gaussian prefilter: testFiles/GaussianFilter2D_3px_2.0f_rankine_vortex01_0.matFloat and
  ..._5px_0.48f_rankine_vortex01_0_1.matFloat (GaussianFilter2DTest: 4e-5 and 1e-4), on an
  interior window and on 6-pixel bands along every border (the padding rules).
* Dense Lucas-Kanade: testFiles/Python_denseLucasKanade_PyrLvs2_Fs2_0_Iter5_64x64.matFloat, window
  27, 1/4/5 iterations (DenseLucasKanadeGpuJTPPythonTest: 6e-3 on every pixel).
* Liu-Shen: testFiles/Python_with_JavaLK_denseLiuShen_lambda4_Rankine_vortex_64x64.matFloat, lambda 4,
  5 passes from the Java Lucas-Kanade field (DenseLiuShenGpuJTPTest: fixed terms 1e-5, new vectors
  1e-3 per pass).
"""
import numpy as np
import pytest

from conftest import GOLDEN


@pytest.fixture(scope="module")
def dense():
    return np.load(GOLDEN / "dense_golden.npz")


def test_gauss_kernel_normalised(oracle):
    for sigma, px in [(2.0, 3), (0.48, 5), (1.0, 7)]:
        k = oracle.gauss_kernel(sigma, px)
        assert abs(float(k.sum()) - 1.0) < 1e-6
        assert np.array_equal(k, k[::-1])


@pytest.mark.parametrize("sigma,px,tol,which", [(2.0, 3, 4e-5, ("f1_0", "a")), (0.48, 5, 1e-4, ("f2_0", "a")),
                                                (0.48, 5, 1e-4, ("f2_1", "b"))])
def test_gauss_filter_matches_reference(oracle, rankine_pair, sigma, px, tol, which):
    name, src = which
    img = rankine_pair[0] if src == "a" else rankine_pair[1]
    out = oracle.gauss_filter(img, sigma, px)
    win = np.load(GOLDEN / "filter_golden.npz")
    r0, r1, c0, c1 = win["window"]
    assert np.abs(out[r0:r1, c0:c1] - win[name]).max() <= tol
    e = np.load(GOLDEN / "filter_edges.npz")
    assert np.abs(out[:6] - e[f"{name}_top"]).max() <= tol
    assert np.abs(out[-6:] - e[f"{name}_bottom"]).max() <= tol
    assert np.abs(out[:, :6] - e[f"{name}_left"]).max() <= tol
    assert np.abs(out[:, -6:] - e[f"{name}_right"]).max() <= tol


def test_gauss_filter_right_padding_rule(oracle):
    # the right border is padded with the last values in order, not mirrored: a ramp shows it
    img = np.tile(np.arange(8, dtype=np.float32) ** 2, (3, 1))
    out = oracle.gauss_filter(img, 0.8, 5)
    k = oracle.gauss_kernel(0.8, 5)
    row = img[0]
    padded = np.concatenate([row[1::-1], row, row[-2:]])     # left: mirror with edge, right: copy
    f32 = np.float32
    exp = []
    for j in range(8):
        acc = f32(0)
        for q in range(5):
            acc = f32(acc + f32(padded[j + 4 - q] * k[q]))
        exp.append(acc)
    # the column pass of a constant column returns the row value (weights sum to 1 within rounding)
    assert np.abs(out[1] - np.array(exp, np.float32)).max() < 1e-4


def test_normalize(oracle):
    a = np.array([[0.0, 2.0], [4.0, 1.0]], np.float32)
    assert np.array_equal(oracle.normalize(a), a / np.float32(4.0))


@pytest.mark.parametrize("iters", [1, 4, 5])
def test_dense_lk_matches_python_fixture(oracle, dense, iters):
    a, b = dense["lk_imageA"], dense["lk_imageB"]
    u0, v0 = dense[f"lk_beforeLK2nd{iters}_u"], dense[f"lk_beforeLK2nd{iters}_v"]
    u, v = oracle.dense_lk(a, b, u0, v0, 27, iters, half_pixel=False)
    assert np.abs(u - dense[f"lk_afterLK2nd{iters}_u"]).max() <= 6e-3
    assert np.abs(v - dense[f"lk_afterLK2nd{iters}_v"]).max() <= 6e-3
    assert np.abs(u - u0).max() > 1e-2      # the iterations moved the field


def test_liu_shen_matches_python_fixture(oracle, dense):
    la, lb = dense["ls_Im1LS_Filtered"], dense["ls_Im2LS_Filtered"]
    us, vs = dense["ls_uLK"], dense["ls_vLK"]
    u, v, passes, fixed, un, vn = oracle.liu_shen(la, lb, us, vs, 4.0, 5, half_pixel=False, intermediates=True)
    assert passes == 5
    for q, name in enumerate(["cmtx", "IIx", "IIy", "II", "Ixt", "Iyt", "A11", "A12", "A22", "B11", "B12", "B22"]):
        assert np.abs(fixed[q] - dense[f"ls_{name}"]).max() <= 1e-5, name
    for k in range(5):
        assert np.abs(un[k] - dense[f"ls_unews{k}"]).max() <= 1e-3, k
        assert np.abs(vn[k] - dense[f"ls_vnews{k}"]).max() <= 1e-3, k
    # output orientation: columns <- vnew, rows <- unew of the last pass
    assert np.array_equal(u, vn[-1]) and np.array_equal(v, un[-1])


def _flow_case(oracle, h=96, w=112, n=16, seed=0):
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 255, (h, w)).astype(np.uint8)
    b = np.roll(a, (1, 2), axis=(0, 1))
    _, tops, lefts = oracle.grid(h, w, n, 0, 0.5)
    tu = rng.normal(1.0, 0.2, (len(tops), len(lefts))).astype(np.float32)
    tv = rng.normal(2.0, 0.2, (len(tops), len(lefts))).astype(np.float32)
    return a, b, tops, lefts, tu, tv


@pytest.mark.parametrize("mode,dense", [(1, False), (1, True), (2, False), (2, True)])
def test_flow_after_piv_is_the_stage_composition(oracle, mode, dense):
    """orc_flow_after_piv equals the pinned stages chained by hand (DenseLucasKanade /
    DenseLiuShen AparapiJobInterpolator.interpolate(stepTilesA, stepTilesB))."""
    n = 16
    a, b, tops, lefts, tu, tv = _flow_case(oracle, n=n)
    h, w = a.shape
    u, v, du, dv = oracle.flow_after_piv(a, b, n, tops, lefts, tu, tv, mode=mode, iterations_ls=12,
                                         dense_export=dense)
    ys = (tops + n / 2.0 - 0.5).astype(np.float32)
    xs = (lefts + n / 2.0 - 0.5).astype(np.float32)
    fu, fv = oracle.displacement_field(ys, xs, tu, tv, h, w, offset=0.0 if dense else 0.5)
    us, vs = oracle.dense_lk(oracle.gauss_filter(a, 2.0, 3), oracle.gauss_filter(b, 2.0, 3), fv, fu, 27, 5,
                             half_pixel=not dense)
    if mode == 2:
        la = oracle.normalize(oracle.gauss_filter(a, 0.48, 5))
        lb = oracle.normalize(oracle.gauss_filter(b, 0.48, 5))
        us, vs = oracle.liu_shen(la, lb, us, vs, 4.0, 12, half_pixel=not dense)
    np.testing.assert_array_equal(du, vs)
    np.testing.assert_array_equal(dv, us)
    ci = tops + n // 2 - 1
    cj = lefts + n // 2 - 1
    if dense:
        def avg(f):
            return (((f[np.ix_(ci, cj)] + f[np.ix_(ci, cj + 1)]) + f[np.ix_(ci + 1, cj)]) +
                    f[np.ix_(ci + 1, cj + 1)]) / np.float32(4.0)
        eu, ev = avg(vs), avg(us)
    else:
        eu, ev = vs[np.ix_(ci, cj)], us[np.ix_(ci, cj)]
    np.testing.assert_array_equal(u, eu)
    np.testing.assert_array_equal(v, ev)


def test_flow_after_piv_still_images_stay_still(oracle):
    a, _, tops, lefts, tu, tv = _flow_case(oracle, seed=3)
    z = np.zeros_like(tu)
    u, v, du, dv = oracle.flow_after_piv(a, a, 16, tops, lefts, z, z, mode=2, iterations_ls=5)
    assert not u.any() and not v.any() and not du.any() and not dv.any()


@pytest.mark.parametrize("mode", [1, 2, 3, 4, 5])
def test_flow_after_piv_ignore_piv_modes(oracle, mode):
    """ignorePIVBaseDisplacements: the PIV field handed to Lucas-Kanade, checked through a run
    with one LK iteration on identical images (no motion: LK keeps the field where it starts)."""
    n = 16
    a, _, tops, lefts, tu, tv = _flow_case(oracle, n=n, seed=mode)
    tu = tu * 3.0
    h, w = a.shape
    ys = (tops + n / 2.0 - 0.5).astype(np.float32)
    xs = (lefts + n / 2.0 - 0.5).astype(np.float32)
    fu, fv = oracle.displacement_field(ys, xs, tu, tv, h, w, offset=0.5)
    if mode in (4, 5):
        lim = np.float32(3.0 if mode == 4 else 0.9)
        fu = np.where(np.abs(fu) < lim, np.float32(0), fu)
        fv = np.where(np.abs(fv) < lim, np.float32(0), fv)
    if mode in (2, 3):
        fu = np.full_like(fu, 0.5)
    if mode in (1, 3):
        fv = np.full_like(fv, 0.5)
    us, vs = oracle.dense_lk(oracle.gauss_filter(a, 2.0, 3), oracle.gauss_filter(a, 2.0, 3), fv, fu, 27, 1,
                             half_pixel=True)
    u, v, du, dv = oracle.flow_after_piv(a, a, n, tops, lefts, tu, tv, mode=1, iterations_lk=1, dense_export=False,
                                         ignore_piv=mode)
    np.testing.assert_array_equal(du, vs)
    np.testing.assert_array_equal(dv, us)


def _pyr_down(f, scale):
    """2 x 2 box average, ((a + b) + (c + d)) * 0.25 * scale in float32."""
    h2, w2 = f.shape[0] // 2, f.shape[1] // 2
    g = f[:2 * h2, :2 * w2]
    t = (g[0::2, 0::2] + g[0::2, 1::2]) + (g[1::2, 0::2] + g[1::2, 1::2])
    return ((t * np.float32(0.25)) * np.float32(scale)).astype(np.float32)


def _pyr_up(f, h, w):
    si = np.minimum(np.arange(h) >> 1, f.shape[0] - 1)
    sj = np.minimum(np.arange(w) >> 1, f.shape[1] - 1)
    return (np.float32(2.0) * f[np.ix_(si, sj)]).astype(np.float32)


@pytest.mark.parametrize("levels,shape,half", [(2, (64, 72), False), (3, (67, 81), True), (2, (45, 38), True)])
def test_lk_pyramid_is_the_level_composition(oracle, levels, shape, half):
    """orc_dense_lk_pyramid equals down-sampling, coarse LK, nearest up-sampling and finer LK
    chained by hand (odd sides drop their last row / column)."""
    rng = np.random.default_rng(levels)
    h, w = shape
    a = oracle.gauss_filter(rng.integers(0, 255, (h, w)).astype(np.float32), 1.5, 3)
    b = np.roll(a, (2, -3), axis=(0, 1))
    us = rng.normal(0.0, 0.5, (h, w)).astype(np.float32)
    vs = rng.normal(0.0, 0.5, (h, w)).astype(np.float32)
    la, lb, lu, lv = [a], [b], [us], [vs]
    for _ in range(1, levels):
        la.append(_pyr_down(la[-1], 1.0))
        lb.append(_pyr_down(lb[-1], 1.0))
        lu.append(_pyr_down(lu[-1], 0.5))
        lv.append(_pyr_down(lv[-1], 0.5))
    u, v = lu[-1], lv[-1]
    for lev in range(levels - 1, -1, -1):
        if lev < levels - 1:
            u = _pyr_up(u, *la[lev].shape)
            v = _pyr_up(v, *la[lev].shape)
        u, v = oracle.dense_lk(la[lev], lb[lev], u, v, 9, 3, half_pixel=half)
    pu, pv = oracle.dense_lk_pyramid(a, b, us, vs, 9, 3, half_pixel=half, levels=levels)
    np.testing.assert_array_equal(pu, u)
    np.testing.assert_array_equal(pv, v)
    one = oracle.dense_lk_pyramid(a, b, us, vs, 9, 3, half_pixel=half, levels=1)
    np.testing.assert_array_equal(one[0], oracle.dense_lk(a, b, us, vs, 9, 3, half_pixel=half)[0])


def test_lk_pyramid_recovers_a_larger_shift(oracle):
    """From a zero start, a 6-pixel shift of smooth particles is beyond a 9-pixel window at full
    resolution but within reach at the coarser levels."""
    rng = np.random.default_rng(5)
    h, w = 96, 96
    a = oracle.gauss_filter((rng.random((h, w)) < 0.05).astype(np.float32) * 200.0, 2.0, 5)
    b = np.roll(a, (0, 6), axis=(0, 1))
    z = np.zeros((h, w), np.float32)
    inner = (slice(24, 72), slice(24, 72))
    u1, _ = oracle.dense_lk_pyramid(a, b, z, z, 9, 5, levels=1)
    u3, v3 = oracle.dense_lk_pyramid(a, b, z, z, 9, 5, levels=3)
    e1 = np.median(np.abs(u1[inner] - 6.0))
    e3 = np.median(np.abs(u3[inner] - 6.0))
    assert e3 < 0.5 and e3 < e1
    assert np.median(np.abs(v3[inner])) < 0.5


def test_flow_after_piv_pyramid_levels(oracle):
    """pyramid_levels 0 and 1 are the reference's full-resolution flow; 2 differs."""
    n = 16
    a, b, tops, lefts, tu, tv = _flow_case(oracle, n=n)
    r0 = oracle.flow_after_piv(a, b, n, tops, lefts, tu, tv, mode=1)
    r1 = oracle.flow_after_piv(a, b, n, tops, lefts, tu, tv, mode=1, pyramid_levels=1)
    r2 = oracle.flow_after_piv(a, b, n, tops, lefts, tu, tv, mode=1, pyramid_levels=2)
    for x, y in zip(r0, r1):
        np.testing.assert_array_equal(x, y)
    assert not np.array_equal(r0[2], r2[2])


# ---- the FP64 twin of the dense stages (error reference of the CUDA dense flow) ----

@pytest.mark.parametrize("sigma,px,tol,which", [(2.0, 3, 4e-5, ("f1_0", "a")), (0.48, 5, 1e-4, ("f2_0", "a"))])
def test_gauss_filter_fp64_twin_matches_reference(oracle, rankine_pair, sigma, px, tol, which):
    name, src = which
    img = rankine_pair[0] if src == "a" else rankine_pair[1]
    out64 = oracle.gauss_filter(img, sigma, px, precision=64)
    assert out64.dtype == np.float64
    win = np.load(GOLDEN / "filter_golden.npz")
    r0, r1, c0, c1 = win["window"]
    assert np.abs(out64[r0:r1, c0:c1] - win[name]).max() <= tol
    out32 = oracle.gauss_filter(img, sigma, px)
    assert np.abs(out32 - out64).max() <= 1e-4 * max(1.0, float(np.abs(out64).max()))
    k64 = oracle.gauss_kernel(sigma, px, precision=64)
    assert abs(float(k64.sum()) - 1.0) < 1e-14


@pytest.mark.parametrize("iters", [1, 5])
def test_dense_lk_fp64_twin_matches_python_fixture(oracle, dense, iters):
    a, b = dense["lk_imageA"], dense["lk_imageB"]
    u0, v0 = dense[f"lk_beforeLK2nd{iters}_u"], dense[f"lk_beforeLK2nd{iters}_v"]
    u, v = oracle.dense_lk(a, b, u0, v0, 27, iters, half_pixel=False, precision=64)
    assert u.dtype == np.float64
    assert np.abs(u - dense[f"lk_afterLK2nd{iters}_u"]).max() <= 6e-3
    assert np.abs(v - dense[f"lk_afterLK2nd{iters}_v"]).max() <= 6e-3
    u32, v32 = oracle.dense_lk(a, b, u0, v0, 27, iters, half_pixel=False)
    assert np.sqrt(np.mean((u32 - u) ** 2 + (v32 - v) ** 2)) <= 1e-4


def test_liu_shen_fp64_twin_matches_python_fixture(oracle, dense):
    la, lb = dense["ls_Im1LS_Filtered"], dense["ls_Im2LS_Filtered"]
    us, vs = dense["ls_uLK"], dense["ls_vLK"]
    u, v, passes, fixed, un, vn = oracle.liu_shen(la, lb, us, vs, 4.0, 5, half_pixel=False, intermediates=True,
                                                  precision=64)
    assert passes == 5 and fixed.dtype == np.float64
    for q, name in enumerate(["cmtx", "IIx", "IIy", "II", "Ixt", "Iyt", "A11", "A12", "A22", "B11", "B12", "B22"]):
        assert np.abs(fixed[q] - dense[f"ls_{name}"]).max() <= 1e-5, name
    for k in range(5):
        assert np.abs(un[k] - dense[f"ls_unews{k}"]).max() <= 1e-3, k
        assert np.abs(vn[k] - dense[f"ls_vnews{k}"]).max() <= 1e-3, k


@pytest.mark.parametrize("mode,dense_export,levels", [(1, False, 0), (2, True, 2)])
def test_flow_after_piv_fp64_twin_close_to_float(oracle, mode, dense_export, levels):
    """The float path (the reference's arithmetic) stays within 1e-4 px RMS of its FP64 twin."""
    n = 16
    a, b, tops, lefts, tu, tv = _flow_case(oracle, n=n)
    kw = dict(mode=mode, iterations_ls=12, dense_export=dense_export, pyramid_levels=levels)
    u, v, du, dv = oracle.flow_after_piv(a, b, n, tops, lefts, tu, tv, **kw)
    u64, v64, du64, dv64 = oracle.flow_after_piv(a, b, n, tops, lefts, tu, tv, precision=64, **kw)
    assert du64.dtype == np.float64 and u64.dtype == np.float32
    assert np.sqrt(np.mean((du - du64) ** 2 + (dv - dv64) ** 2)) <= 1e-4
    assert np.abs(du - du64).max() > 0.0      # a separate double-precision run, not the float path
