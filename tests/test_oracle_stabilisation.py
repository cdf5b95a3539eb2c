"""The oracle's restatement of the tile stabilisation loop (InterAreaDisplacementStableStrategy,
S/iareas/InterAreaDisplacementStableStrategy.java:19-36, in the per-level loop of
S/jobs/LocalPIVOpenCLGpuJob.java:233-405).  CPU only."""
import numpy as np
import pytest

from conftest import load_package

f32 = np.float32


@pytest.fixture(scope="module")
def qp():
    return load_package()


def _pair(qp, h, w, seed, vmax=5.0):
    flow = qp.synth.Flow(vmax=vmax, rc=40.0, shear=0.01)
    return qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, diam_sd=0.2, bits=8, seed=seed)


def test_first_level_bothimages_repeats_the_same_increment(qp, oracle):
    """The BothImages strategy warps from the second level on only: at the first level every pass
    correlates the same tiles, so a tile whose increment exceeds the maximum takes it again on
    every pass until the retries run out (the reference's loop, restated)."""
    a, b = _pair(qp, 128, 160, 3)
    one = oracle.piv_adaptive(a, b, 32, 32, 0.5, fixed_max=255.0)
    du, dv = one[0].astype(np.float64), one[1].astype(np.float64)
    norm = np.sqrt(du * du + dv * dv).astype(np.float32)
    mx = float(np.median(norm))
    for retries in (2, 3):
        u, v = oracle.piv_adaptive(a, b, 32, 32, 0.5, fixed_max=255.0, stable_max=mx, stable_retries=retries)
        big = norm > f32(mx)
        assert big.any() and (~big).any()
        eu, ev = np.zeros_like(one[0]), np.zeros_like(one[1])
        for r in range(retries):
            eu = np.where(big | (r == 0), (eu + one[0]).astype(np.float32), eu)
            ev = np.where(big | (r == 0), (ev + one[1]).astype(np.float32), ev)
        assert u.tobytes() == eu.tobytes() and v.tobytes() == ev.tobytes()


def test_no_warping_repeats_displaced_tiles(qp, oracle):
    """Without warping the B tiles sit at the rounded accumulated displacement, so a repeated pass
    measures the residual from there and adds it (the reference accumulates it onto the
    non-integer displacement).  A maximum no increment reaches repeats nothing; a small one
    changes the result."""
    a, b = _pair(qp, 160, 192, 5)
    base = oracle.piv_adaptive(a, b, 32, 16, 0.5, warp=False)
    loose = oracle.piv_adaptive(a, b, 32, 16, 0.5, warp=False, stable_max=100.0, stable_retries=3)
    assert base[0].tobytes() == loose[0].tobytes() and base[1].tobytes() == loose[1].tobytes()
    r3 = oracle.piv_adaptive(a, b, 32, 16, 0.5, warp=False, stable_max=0.05, stable_retries=3)
    assert not np.array_equal(r3[0], base[0])
    # a repeated pass moves a vector by less than a pixel (a residual of the integer B-tile move)
    assert np.abs(r3[0] - base[0]).max() < 1.5


def test_stabilisation_rejects_validation_and_tile_warps(qp):
    d = qp.adaptive_desc(32, 16, 0.5, stable_max_displacement=0.1, stable_max_retries=3,
                         validation=qp.multipeak_validation())
    with pytest.raises(qp.QlpivError):
        qp.adaptive_levels(d, 256, 256)
    d = qp.adaptive_desc(32, 16, 0.5, warp_mode=qp.WARP_BOTH_MICRO, stable_max_displacement=0.1,
                         stable_max_retries=3)
    with pytest.raises(qp.QlpivError):
        qp.adaptive_levels(d, 256, 256)
    assert len(qp.adaptive_levels(qp.adaptive_desc(32, 16, 0.5, stable_max_displacement=0.1, stable_max_retries=3),
                                  256, 256)) == 2
