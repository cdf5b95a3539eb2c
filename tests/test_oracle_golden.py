"""Pins the CPU oracle to the reference's own golden vectors and known-answer tests.

Sources (QuickLabPIV-ng, read once by tests/golden/make_golden.py):
  * resources/fftBenchmark/gpuFFTBenchmarkValidationData.matFloat -- correlation planes of
    the 512x512 Rankine pair, 16x16 IAs without overlap, each tile normalised by its own
    max; checked by S/jobs/GpuFFTBenchmarkJob.java:307-337 at 1e-2 absolute.
  * tests/pt/quickLabPIV/xcorr/FastRealFFTXCorrTests.java: 4x4 real-pair FFT xcorr equals the
    by-definition xcorr within 1e-3.
  * tests/pt/quickLabPIV/images/ImageCrossCorrelationRealFFTParStdJobTests.java:232-576: the
    synthetic pair shifted by 10 px; FindMaximumFromCenter lands at D/2 -+ 10 for 64 and 128
    pixel tiles in the four quadrants.
  * tests/pt/quickLabPIV/iareas/AdaptiveInterArea*GeometryTests.java: IA grid geometry.
  * tests/pt/quickLabPIV/interpolators/Gaussian1DInterpolatorAdvanced3Pixels*Test.java: analytic
    Gaussian peaks recovered within 8e-3 px by the 3-point fit.
"""
import numpy as np
import pytest

from conftest import GOLDEN


def test_bitreverse_equals_perfect_shuffle(oracle):
    # SimpleFFT.perfectShuffleFFTInput (S/jobs/xcorr/SimpleFFT.java:32-69), restated as the
    # swap procedure on an index array; the oracle and the kernels use bit reversal.
    for n in [2 ** k for k in range(1, 10)]:
        arr = list(range(n))
        osf, ods = 1, n
        while ods > 2:
            for osi in range(osf):
                oo = osi * ods
                sf, ds = 1, ods
                while ds > 2:
                    for si in range(sf):
                        io = si * ds
                        for i in range(0, ds // 2, 2):
                            s, d = oo + io + i + 1, oo + io + ds // 2 + i
                            arr[s], arr[d] = arr[d], arr[s]
                    ds >>= 1
                    sf <<= 1
            ods >>= 1
            osf <<= 1
        bits = n.bit_length() - 1
        rev = [int(format(k, f"0{bits}b")[::-1], 2) if bits else 0 for k in range(n)]
        assert arr == rev, n


def test_gpu_fft_benchmark_golden(oracle, rankine_pair):
    a, b = rankine_pair
    g = np.load(GOLDEN / "gpu_fft_golden.npz")
    for idx, plane in zip(g["index"], g["planes"]):
        ti, tj = divmod(int(idx), 32)
        ta, ma = oracle.clip_tile(a, ti * 16, tj * 16, 16)
        tb, mb = oracle.clip_tile(b, ti * 16, tj * 16, 16)
        p32 = oracle.xcorr_fft(ta, tb, ma, mb, precision=32)
        p64 = oracle.xcorr_fft(ta, tb, ma, mb, precision=64)
        assert np.abs(p32 - plane).max() <= 1e-2, idx
        assert np.abs(p64 - plane).max() <= 1e-2, idx
        # the CPU-path normalisation (both tiles by A's max) is a different plane
        if mb != ma:
            assert np.abs(oracle.xcorr_fft(ta, tb, ma, ma) - plane).max() > 1e-2


def test_fast_real_fft_xcorr_4x4_kat(oracle):
    f = np.zeros((4, 4), np.float32)
    g = np.zeros((4, 4), np.float32)
    f[:3, :3] = [[6, 6, 6], [7, 6, 6], [7, 7, 6]]
    g[:3, :3] = [[5, 5, 6], [6, 6, 7], [7, 7, 7]]
    p = oracle.xcorr_fft(f, g, 1.0, 1.0, normalize=False)
    ref = oracle.xcorr_direct(f, g, 1.0, 1.0, normalize=False)
    assert np.abs(p - ref).max() <= 1e-3
    # by-definition helper: R(s) = sum_m f(m) g(m+s), zero shift at index N-1
    assert ref[3, 3] == pytest.approx(float((f * g).sum()))


@pytest.mark.parametrize("n", [64, 128])
@pytest.mark.parametrize("quadrant,top,left,di,dj", [
    ("top_left", "320-n", "320-n", -10, -10),
    ("bottom_left", "320", "320-n", 10, -10),
    ("top_right", "320-n", "320", -10, 10),
    ("bottom_right", "320", "320", 10, 10),
])
def test_shift_kat(oracle, n, quadrant, top, left, di, dj):
    d = np.load(GOLDEN / "shift_kat.npz")
    t0, l0 = eval(top, {"n": n}), eval(left, {"n": n})
    ta, ma = oracle.clip_tile(d["img1"], t0, l0, n)
    tb, mb = oracle.clip_tile(d["img2"], t0, l0, n)
    for norm in (True, False):
        plane = oracle.xcorr_fft(ta, tb, ma, mb, normalize=norm)
        i, j, _, _ = oracle.find_max_from_center(plane)
        dd = 2 * n - 1
        assert (i, j) == (dd // 2 + di, dd // 2 + dj), (quadrant, norm)


def test_find_max_tie_break(oracle):
    # equal values: the cell closest to (D/2+1, D/2+1) wins; among equal distances the
    # first in scan order wins (centre column, centre row, then quadrants).
    d = 9
    p = np.ones((d, d), np.float32)
    c = d // 2 + 1
    p[c - 1, c] = 5.0
    p[c + 1, c] = 5.0
    i, j, v, mn = oracle.find_max_from_center(p)
    assert (i, j, v, mn) == (c - 1, c, 5.0, 1.0)
    p[:] = 1.0
    p[2, 2] = 7.0
    p[c + 2, c + 2] = 7.0     # closer to the centre than (2,2)
    assert oracle.find_max_from_center(p)[:2] == (c + 2, c + 2)
    p[:] = 1.0
    p[0, :] = 9.0             # row 0 / column 0 are never visited
    p[:, 0] = 9.0
    p[3, 6] = 2.0
    assert oracle.find_max_from_center(p)[:3] == (3, 6, 2.0)


def _gauss_plane(d, ui, uj, sigma=1.2):
    ii, jj = np.meshgrid(np.arange(d), np.arange(d), indexing="ij")
    return (1000.0 * np.exp(-((ii - ui) ** 2 + (jj - uj) ** 2) / (2 * sigma ** 2)) + 1e-3).astype(np.float32)


@pytest.mark.parametrize("ui,uj", [(15.3, 14.8), (15.0, 15.0), (16.45, 13.55), (12.1, 18.9)])
def test_gaussian3_kat(oracle, ui, uj):
    # analytic Gaussian with known centre (GaussianTestHelper style), 8e-3 px tolerance
    p = _gauss_plane(31, ui, uj)
    i, j, _, _ = oracle.find_max_from_center(p)
    pi, pj, fl = oracle.subpixel_gauss3(p, i, j)
    assert abs(pi - ui) < 8e-3 and abs(pj - uj) < 8e-3
    assert fl & oracle.F_SUB_I and fl & oracle.F_SUB_J


def test_gaussian3_edges(oracle):
    p = _gauss_plane(31, 29.7, 15.0)
    pi, pj, fl = oracle.subpixel_gauss3(p, 30, 15)
    assert fl & oracle.F_EDGE and (pi, pj) == (30.0, 15.0)
    pi, pj, fl = oracle.subpixel_gauss3(p, 0, 0)
    assert fl & oracle.F_NO_PEAK
    q = _gauss_plane(31, 15.2, 15.0)
    q[14, 15] = -1.0   # negative stencil value -> parabolic fallback
    pi, pj, fl = oracle.subpixel_gauss3(q, 15, 15)
    assert fl & oracle.F_PARABOLIC


# AdaptiveInterAreaSuperPositionGeometryTests.simpleIASuperPositionValidationTest1Pass:
# 139x139 image, margins 16, overlap factor 1/3, IA 64 -> 32: level 0 keeps margins 16.
def test_grid_superposition_kat(oracle):
    g, tops, lefts = oracle.grid(139, 139, 64, level=0, overlap_factor=1.0 / 3.0, margins=(16, 16, 16, 16))
    assert (g["n"], g["margin_top"], g["margin_bottom"], g["margin_left"], g["margin_right"]) == (64, 16, 16, 16, 16)
    inc = np.float32(64) * np.float32(1.0 / 3.0)
    exp_n = 0
    x = np.float32(0.0)
    while x <= 139 - 32 - 64 + 0.01:
        exp_n += 1
        x = np.float32(x + inc)
    assert g["tiles_i"] == exp_n == g["tiles_j"]
    assert list(tops) == [16 + int(np.floor(np.float32(k * inc) + np.float32(0.5))) for k in range(exp_n)]


def test_grid_counts_for_configs(oracle):
    # 512x512, IA 32 at 50 %: 31x31 = 961 vectors; 1024x1024 IA 64->32->16 at 75 %:
    # 61^2, 125^2, 253^2 (83,355 vectors over three passes)
    g, _, _ = oracle.grid(512, 512, 32, 0, 0.5)
    assert g["tiles_i"] * g["tiles_j"] == 961
    counts = [oracle.grid(1024, 1024, 64, lv, 0.25)[0] for lv in range(3)]
    assert [c["tiles_i"] for c in counts] == [61, 125, 253]
    g, tops, lefts = oracle.grid(512, 512, 16, 0, 0.5, superposition=False)
    assert (g["tiles_i"], g["tiles_j"], tops[1], lefts[31]) == (32, 32, 16, 496)


def test_piv_pass_matches_single_ia(oracle, rankine_pair):
    a, b = rankine_pair
    g, tt, ll = oracle.grid_origins(512, 512, 32, 0.5)
    out = oracle.piv_pass(a, b, 32, tt, ll, nthreads=4)
    k = 500
    ta, ma = oracle.clip_tile(a, tt[k], ll[k], 32)
    tb, _ = oracle.clip_tile(b, tt[k], ll[k], 32)
    plane = oracle.xcorr_fft(ta, tb, ma, ma)
    i, j, v, mn = oracle.find_max_from_center(plane)
    pi, pj, fl = oracle.subpixel_gauss3(plane, i, j)
    r = out[k]
    assert (r["peak_i"], r["peak_j"], r["peak_value"], r["min_floor"], r["flags"]) == (i, j, np.float32(v), np.float32(mn), fl)
    assert r["u"] == np.float32(np.float32(pi) - np.float32(31))
    # the vortex field is smooth: most vectors are within a few px
    assert np.median(np.abs(out["u"])) < 8


def _akima5_np(x, y, t):
    d = np.diff(y) / np.diff(x)
    w = np.r_[0.0, np.abs(np.diff(d))]
    fd = np.zeros(5)
    fd[2] = ((w[3] * d[1] + w[1] * d[2]) / (w[3] + w[1]) if w[3] + w[1] > 0
             else ((x[3] - x[2]) * d[1] + (x[2] - x[1]) * d[2]) / (x[3] - x[1]))
    for at, (i0, i1, i2) in ((0, (0, 1, 2)), (1, (0, 1, 2)), (3, (2, 3, 4)), (4, (2, 3, 4))):
        c = np.polyfit(x[[i0, i1, i2]], y[[i0, i1, i2]], 2)
        fd[at] = 2 * c[0] * x[at] + c[1]
    k = int(min(max(np.searchsorted(x, t, side="right") - 1, 0), 3))
    h = x[k + 1] - x[k]
    s = t - x[k]
    c2 = (3 * (y[k + 1] - y[k]) / h - 2 * fd[k] - fd[k + 1]) / h
    c3 = (2 * (y[k] - y[k + 1]) / h + fd[k] + fd[k + 1]) / h ** 2
    return y[k] + s * (fd[k] + s * (c2 + s * c3))


def test_inherit_fp64_matches_independent_akima(oracle):
    """B-inherit has no reference fixture: the oracle's double Akima (5x5 window) is
    checked against an independent numpy implementation (parabola derivatives by polyfit)."""
    rng = np.random.default_rng(5)
    py = np.arange(9) * 16.0 + 31.5
    px = np.arange(11) * 16.0 + 31.5
    pu = rng.standard_normal((9, 11)).astype(np.float32)
    cy = (np.arange(17) * 8.0 + 15.5).astype(np.float32)
    cx = (np.arange(21) * 8.0 + 15.5).astype(np.float32)
    cu, _ = oracle.inherit(py, px, pu, pu, cy, cx, precision=64)

    def window(v, c):
        lo = np.searchsorted(v, c, side="right")
        r = (lo - 1) - 2 if lo > 0 and v[lo - 1] == c else lo - 2
        return min(max(r, 0), len(v) - 5)

    for i in range(len(cy)):
        for j in range(len(cx)):
            y = float(np.clip(cy[i], py[0], py[-1]))
            x = float(np.clip(cx[j], px[0], px[-1]))
            wi, wj = window(py, y), window(px, x)
            row = [_akima5_np(py[wi:wi + 5], pu[wi:wi + 5, wj + b].astype(float), y) for b in range(5)]
            ref = _akima5_np(px[wj:wj + 5], np.array(row), x)
            assert abs(cu[i, j] - ref) < 2e-6, (i, j)


def test_field_fp64_matches_independent_spline(oracle):
    """B-field: natural cubic splines (scipy) for the knot derivatives and an explicit
    bicubic Hermite patch, compared with the oracle's double evaluation."""
    interp = pytest.importorskip("scipy.interpolate")
    rng = np.random.default_rng(6)
    ys = np.arange(7) * 8.0 + 7.5
    xs = np.arange(9) * 8.0 + 7.5
    f = rng.standard_normal((7, 9)).astype(np.float32)
    h, w = 64, 80
    fu, _ = oracle.displacement_field(ys, xs, f, f, h, w, precision=64)
    fd = f.astype(float)
    fy = np.stack([interp.CubicSpline(ys, fd[:, j], bc_type="natural")(ys, 1) for j in range(9)], 1)
    fx = np.stack([interp.CubicSpline(xs, fd[i, :], bc_type="natural")(xs, 1) for i in range(7)], 0)
    fyx = np.zeros_like(fd)
    for i in range(7):
        for j in range(9):
            ni, pi = min(i + 1, 6), max(i - 1, 0)
            nj, pj = min(j + 1, 8), max(j - 1, 0)
            fyx[i, j] = (fd[ni, nj] - fd[ni, pj] - fd[pi, nj] + fd[pi, pj]) / ((ys[ni] - ys[pi]) * (xs[nj] - xs[pj]))

    def basis(t):
        return np.array([2 * t ** 3 - 3 * t ** 2 + 1, -2 * t ** 3 + 3 * t ** 2]), np.array([t ** 3 - 2 * t ** 2 + t,
                                                                                           t ** 3 - t ** 2])
    for (yy, xx) in [(0, 0), (10, 13), (20, 33), (40, 70), (63, 79), (31, 44)]:
        y = float(np.clip(yy, ys[0], ys[-1]))
        x = float(np.clip(xx, xs[0], xs[-1]))
        i = min(int(np.searchsorted(ys, y, side="right") - 1), 5)
        j = min(int(np.searchsorted(xs, x, side="right") - 1), 7)
        dy, dx = ys[i + 1] - ys[i], xs[j + 1] - xs[j]
        a0, a1 = basis((y - ys[i]) / dy)
        b0, b1 = basis((x - xs[j]) / dx)
        val = 0.0
        for a in range(2):
            for b in range(2):
                val += (fd[i + a, j + b] * a0[a] * b0[b] + fy[i + a, j + b] * dy * a1[a] * b0[b]
                        + fx[i + a, j + b] * dx * a0[a] * b1[b] + fyx[i + a, j + b] * dy * dx * a1[a] * b1[b])
        assert abs(fu[int(yy), int(xx)] - val) < 1e-6, (yy, xx)
