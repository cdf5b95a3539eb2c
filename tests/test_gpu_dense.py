"""Dense optical flow stages on the GPU against the CPU oracle and the reference's fixtures.

Every stage uses the oracle's operation order with IEEE single operations and no contraction:
the Gaussian prefilter, the normalisation, dense Lucas-Kanade and Liu-Shen must be bit-identical
to the oracle; the fixture tolerances of the reference's own tests are checked as well.
"""
import numpy as np
import pytest

from conftest import GOLDEN, load_package

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


@pytest.fixture(scope="module")
def dense():
    return np.load(GOLDEN / "dense_golden.npz")


@pytest.mark.parametrize("sigma,px", [(2.0, 3), (0.48, 5), (1.3, 9)])
def test_gaussian_filter_bit_exact(qp, handle, oracle, rankine_pair, sigma, px):
    a, b = rankine_pair
    for img in (a, b, (a.astype(np.uint16) * 16), a[:200, :137].astype(np.float32) / 7.0):
        got = handle.gaussian_filter(img, sigma, px)
        exp = oracle.gauss_filter(img, sigma, px)
        assert got.tobytes() == exp.tobytes()
    win = np.load(GOLDEN / "filter_golden.npz")
    if (sigma, px) == (2.0, 3):
        r0, r1, c0, c1 = win["window"]
        assert np.abs(handle.gaussian_filter(a, sigma, px)[r0:r1, c0:c1] - win["f1_0"]).max() <= 4e-5


def test_normalize_bit_exact(qp, handle, oracle, rankine_pair):
    f = handle.gaussian_filter(rankine_pair[0], 0.48, 5)
    assert handle.normalize(f).tobytes() == oracle.normalize(f).tobytes()


@pytest.mark.parametrize("iters,half", [(1, False), (4, False), (5, False), (5, True)])
def test_dense_lk_bit_exact_and_fixture(qp, handle, oracle, dense, iters, half):
    a, b = dense["lk_imageA"], dense["lk_imageB"]
    u0, v0 = dense[f"lk_beforeLK2nd{iters}_u"], dense[f"lk_beforeLK2nd{iters}_v"]
    gu, gv = handle.dense_lk(a, b, u0, v0, 27, iters, half_pixel=half)
    ou, ov = oracle.dense_lk(a, b, u0, v0, 27, iters, half_pixel=half)
    assert gu.tobytes() == ou.tobytes() and gv.tobytes() == ov.tobytes()
    if not half:
        assert np.abs(gu - dense[f"lk_afterLK2nd{iters}_u"]).max() <= 6e-3
        assert np.abs(gv - dense[f"lk_afterLK2nd{iters}_v"]).max() <= 6e-3


def test_liu_shen_bit_exact_and_fixture(qp, handle, oracle, dense):
    la, lb = dense["ls_Im1LS_Filtered"], dense["ls_Im2LS_Filtered"]
    us, vs = dense["ls_uLK"], dense["ls_vLK"]
    for passes in (1, 4, 5):
        gu, gv = handle.liu_shen(la, lb, us, vs, 4.0, passes)
        ou, ov = oracle.liu_shen(la, lb, us, vs, 4.0, passes)
        assert gu.tobytes() == ou.tobytes() and gv.tobytes() == ov.tobytes()
        assert np.abs(gv - dense[f"ls_unews{passes - 1}"]).max() <= 1e-3
        assert np.abs(gu - dense[f"ls_vnews{passes - 1}"]).max() <= 1e-3


@pytest.mark.parametrize("half", [False, True])
def test_lk_then_liu_shen_on_a_synthetic_pair(qp, handle, oracle, half):
    flow = qp.synth.Flow(vmax=2.5, rc=30.0, shear=0.004)
    a, b = qp.synth.particle_pair((150, 211), flow, ppp=0.05, diam=2.5, diam_sd=0.3, bits=8, seed=21)
    lka, lkb = oracle.gauss_filter(a, 2.0, 3), oracle.gauss_filter(b, 2.0, 3)
    lsa, lsb = oracle.normalize(oracle.gauss_filter(a, 0.48, 5)), oracle.normalize(oracle.gauss_filter(b, 0.48, 5))
    yy, xx = np.meshgrid(np.arange(150, dtype=np.float64), np.arange(211, dtype=np.float64), indexing="ij")
    dr, dc = flow.displacement(yy, xx, (150, 211))
    us0 = (0.8 * dc).astype(np.float32)   # a rough initial field, like an upsampled PIV result
    vs0 = (0.8 * dr).astype(np.float32)
    gu, gv = handle.liu_shen(lsa, lsb, us0, vs0, 4.0, 6, lk_a=lka, lk_b=lkb, window=11, iterations_lk=5,
                             half_pixel=half)
    ku, kv = oracle.dense_lk(lka, lkb, us0, vs0, 11, 5, half_pixel=half)
    ou, ov = oracle.liu_shen(lsa, lsb, ku, kv, 4.0, 6, half_pixel=half)
    assert gu.tobytes() == ou.tobytes() and gv.tobytes() == ov.tobytes()
    # Lucas-Kanade moved the rough field toward the truth in the interior
    lu, lv = handle.dense_lk(lka, lkb, us0, vs0, 11, 5, half_pixel=half)
    inner = (slice(20, 130), slice(20, 190))
    assert np.median(np.abs(lu - dc)[inner]) < np.median(np.abs(us0 - dc)[inner])


def test_dense_settings_rejected(qp, handle, dense):
    a = dense["lk_imageA"]
    z = np.zeros_like(a)
    for win, it in [(2, 1), (33, 1), (28, 1), (27, 0)]:
        with pytest.raises(qp.QlpivError) as e:
            handle.dense_lk(a, a, z, z, win, it)
        assert e.value.status == qp.E_ARG
    with pytest.raises(qp.QlpivError):
        handle.gaussian_filter(a, 2.0, 4)
