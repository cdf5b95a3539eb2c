"""P-point sub-pixel interpolators in K1 against the CPU oracle.

* On the kernel's own correlation planes (qlpiv_xcorr_planes of the same tiles) the oracle's
  Gaussian least-squares / Hongwei Guo fits must give the kernel's sub-pixel peaks within 2e-5 px
  (both fit in double from the same float samples; libm and CUDA exp/log differ in the last bits),
  with the same flags and (Hongwei Guo) peak value.
* Frame passes against the oracle's FP64 pass: integer peaks identical except ties, sub-pixel
  displacements within 1e-3 px.
"""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def qp():
    pkg = load_package()
    pkg.build.build()
    pkg.load_library()
    return pkg


@pytest.fixture(scope="module")
def handle(qp):
    h = qp.Handle(0)
    yield h
    h.close()


def _frames(qp, n, seed, bits=8):
    h, w = 6 * n, 7 * n
    flow = qp.synth.Flow(vmax=min(5.0, n / 5), rc=2.5 * n, shear=0.004)
    a, b = qp.synth.particle_pair((h, w), flow, ppp=0.025, diam=2.6, diam_sd=0.4, bits=bits, seed=seed)
    tops, lefts = np.meshgrid(np.arange(0, h - n + 1, n // 2), np.arange(0, w - n + 1, n // 2), indexing="ij")
    return a, b, tops.ravel().astype(np.int32), lefts.ravel().astype(np.int32)


MODES = [(2, 3, 20), (2, 5, 20), (2, 7, 20), (3, 3, 20), (3, 5, 20), (3, 7, 10), (3, 9, 30)]


def _close(x, y, tol):
    both_nan = np.isnan(x) & np.isnan(y)
    return both_nan | (np.abs(x - y) <= tol)


@pytest.mark.parametrize("n", [16, 32, 64, 128])
@pytest.mark.parametrize("mode,pixels,iters", MODES)
def test_ppoint_fit_matches_oracle_on_kernel_planes(qp, handle, oracle, n, mode, pixels, iters):
    a, b, tops, lefts = _frames(qp, n, seed=n + 7 * pixels + mode)
    vec = handle.piv_pass(a, b, n, tops, lefts, subpix_mode=mode, subpix_pixels=pixels, subpix_iterations=iters)
    ta = np.stack([a[t:t + n, l:l + n] for t, l in zip(tops, lefts)])
    tb = np.stack([b[t:t + n, l:l + n] for t, l in zip(tops, lefts)])
    planes = handle.xcorr_planes(ta, tb)
    ref = handle.piv_pass(a, b, n, tops, lefts, subpix_mode=qp.SUBPIX_NONE)
    assert (vec["peak_i"] == ref["peak_i"]).all() and (vec["peak_j"] == ref["peak_j"]).all()
    fitted = 0
    for r in range(len(vec)):
        pi, pj = int(vec[r]["peak_i"]), int(vec[r]["peak_j"])
        mf = float(vec[r]["min_floor"])
        if mode == qp.SUBPIX_GAUSS_LM:
            si, sj, fl = oracle.subpixel_lm(planes[r], pi, pj, pixels, mf)
            pv = float(ref[r]["peak_value"])
        else:
            si, sj, pv, fl = oracle.subpixel_hg(planes[r], pi, pj, pixels, iters, float(ref[r]["peak_value"]), mf)
        assert int(vec[r]["flags"]) == fl, r
        assert _close(np.float32(vec[r]["sub_i"]), np.float32(si), 2e-5), (r, vec[r]["sub_i"], si)
        assert _close(np.float32(vec[r]["sub_j"]), np.float32(sj), 2e-5), (r, vec[r]["sub_j"], sj)
        assert _close(np.float32(vec[r]["peak_value"]), np.float32(pv), 2e-5 * max(1.0, abs(pv))), r
        fitted += (fl & 3) == 3
    assert fitted >= 0.9 * len(vec)


@pytest.mark.parametrize("mode,pixels,iters", [(2, 5, 20), (3, 5, 20)])
def test_ppoint_pass_against_fp64_oracle(qp, handle, oracle, mode, pixels, iters):
    n = 32
    a, b, tops, lefts = _frames(qp, n, seed=99 + mode, bits=12)
    vec = handle.piv_pass(a, b, n, tops, lefts, subpix_mode=mode, subpix_pixels=pixels, subpix_iterations=iters,
                          max_mode=qp.MAX_COMPUTE)
    o64 = oracle.piv_pass(a, b, n, tops, lefts, subpix=oracle.subpix_code(mode, pixels, iters), precision=64)
    same = (vec["peak_i"] == o64["peak_i"]) & (vec["peak_j"] == o64["peak_j"])
    assert same.mean() >= 0.995
    err = np.hypot(vec["u"] - o64["u64"], vec["v"] - o64["v64"])
    assert np.mean(err[same] <= 1e-3) >= 0.999


def test_ppoint_with_multipeaks(qp, handle, oracle):
    n, k = 32, 3
    a, b, tops, lefts = _frames(qp, n, seed=5)
    vec = handle.piv_pass(a, b, n, tops, lefts, num_peaks=k, peak_kernel=3, subpix_mode=qp.SUBPIX_HONGWEI_GUO,
                          subpix_pixels=5, subpix_iterations=20)
    ta = np.stack([a[t:t + n, l:l + n] for t, l in zip(tops, lefts)])
    tb = np.stack([b[t:t + n, l:l + n] for t, l in zip(tops, lefts)])
    planes = handle.xcorr_planes(ta, tb)
    for r in range(0, len(vec), 7):
        peaks, mf = oracle.find_max_multipeaks(planes[r], 3, k)
        for s, (pi, pj, pv) in enumerate(peaks):
            si, sj, pv2, fl = oracle.subpixel_hg(planes[r], pi, pj, 5, 20, pv, mf)
            g = vec[r, s]
            assert (int(g["peak_i"]), int(g["peak_j"]), int(g["flags"])) == (pi, pj, fl)
            assert _close(np.float32(g["sub_i"]), np.float32(si), 2e-5)
            assert _close(np.float32(g["sub_j"]), np.float32(sj), 2e-5)


def test_ppoint_settings_rejected(qp, handle):
    a, b, tops, lefts = _frames(qp, 16, seed=1)
    for mode, p, it in [(2, 4, 20), (2, 17, 20), (2, 1, 20), (3, 5, 5), (3, 5, 51), (4, 3, 20)]:
        with pytest.raises(qp.QlpivError) as e:
            handle.piv_pass(a, b, 16, tops, lefts, subpix_mode=mode, subpix_pixels=p, subpix_iterations=it)
        assert e.value.status == qp.E_ARG
