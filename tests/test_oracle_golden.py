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
