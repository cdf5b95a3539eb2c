"""Direct / Area / Distance velocity inheritance on the GPU against the oracle's serial walk.

The kernel evaluates each child tile independently from per-row and per-column tables; the
oracle walks the tiles like the reference.  Both use the reference's float operations in the
same order, so results must be bit-identical, and the library must reject (QLPIV_E_SHAPE)
exactly the geometries on which the walk throws.
"""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

MODES = [1, 2, 3]


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


def _level_grids(qp):
    out = []
    for (h, w) in [(97, 131), (200, 296), (512, 512)]:
        for n0 in (32, 64):
            for f in (0.25, 0.5, 1.0 / 3.0, 0.1, 0.9):
                for margins in ((0, 0, 0, 0), (3, 5, 2, 7)):
                    for sup in (True, False):
                        try:
                            gp, pt, pl = qp.library_grid(h, w, n0, 0, f, margins, sup)
                            gc, ct, cl = qp.library_grid(h, w, n0, 1, f, margins, sup)
                        except qp.QlpivError:
                            continue
                        out.append((gp["n"], pt, pl, gc["n"], ct, cl))
    return out


@pytest.mark.parametrize("mode", MODES)
def test_adaptive_grids_bit_exact(qp, handle, oracle, mode):
    rng = np.random.default_rng(mode)
    grids = _level_grids(qp)
    assert len(grids) >= 40
    for k, (pn, pt, pl, cn, ct, cl) in enumerate(grids):
        pu = rng.normal(0, 4, (len(pt), len(pl))).astype(np.float32)
        pv = rng.normal(0, 4, (len(pt), len(pl))).astype(np.float32)
        rnd = bool(k & 1)
        ou, ov = oracle.inherit_tiles(mode, pn, pt, pl, pu, pv, cn, ct, cl, round_int=rnd)
        gu, gv = handle.inherit_tiles(mode, pn, pt, pl, pu, pv, cn, ct, cl, round_int=rnd)
        assert gu.tobytes() == ou.tobytes() and gv.tobytes() == ov.tobytes(), (k, pn, len(pt), len(ct))


@pytest.mark.parametrize("mode", MODES)
def test_random_grids_and_rejections(qp, handle, oracle, mode):
    rng = np.random.default_rng(10 + mode)
    ok = rejected = 0
    for t in range(150):
        pn = int(rng.choice([16, 32, 64]))
        cn = pn // 2
        pni, pnj = int(rng.integers(1, 7)), int(rng.integers(1, 7))
        pt = np.cumsum(rng.integers(1, pn + 1, pni)) - 1 + int(rng.integers(0, 4))
        pl = np.cumsum(rng.integers(1, pn + 1, pnj)) - 1 + int(rng.integers(0, 4))
        cni, cnj = int(rng.integers(1, 12)), int(rng.integers(1, 12))
        ct = np.cumsum(rng.integers(1, cn + 1, cni)) - 1 + int(rng.integers(0, 6))
        cl = np.cumsum(rng.integers(1, cn + 1, cnj)) - 1 + int(rng.integers(0, 6))
        pu = rng.normal(0, 3, (pni, pnj)).astype(np.float32)
        pv = rng.normal(0, 3, (pni, pnj)).astype(np.float32)
        try:
            ou, ov = oracle.inherit_tiles(mode, pn, pt, pl, pu, pv, cn, ct, cl)
        except ValueError:
            with pytest.raises(qp.QlpivError) as e:
                handle.inherit_tiles(mode, pn, pt, pl, pu, pv, cn, ct, cl)
            assert e.value.status == qp.E_SHAPE
            rejected += 1
            continue
        gu, gv = handle.inherit_tiles(mode, pn, pt, pl, pu, pv, cn, ct, cl)
        assert gu.tobytes() == ou.tobytes() and gv.tobytes() == ov.tobytes(), t
        ok += 1
    assert ok >= 30
    if mode != 3:
        assert rejected >= 10


@pytest.mark.parametrize("mode,warp,bits", [(2, 1, 8), (3, 1, 12), (1, 1, 8), (2, 0, 8), (3, 6, 8)])
def test_adaptive_pipeline_with_inheritance_mode(qp, handle, oracle, mode, warp, bits):
    h, w = 320, 288
    flow = qp.synth.Flow(vmax=4.0, rc=56.0, shear=0.005)
    pairs = [qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, bits=bits, seed=500 + k + mode)
             for k in range(2)]
    fm = 255.0 if bits == 8 else 4095.0
    desc = qp.adaptive_desc(64, 16, 0.5 if warp else 0.25, warp_mode=warp, fixed_max=fm if warp else 0.0,
                            max_mode=qp.MAX_FIXED if warp else qp.MAX_COMPUTE, inherit_mode=mode)
    u, v = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    for k, (a, b) in enumerate(pairs):
        ou, ov = oracle.piv_adaptive(a, b, 64, 16, 0.5 if warp else 0.25, fixed_max=fm if warp else None,
                                     precision=32, warp=warp, inherit=mode)
        err = np.maximum(np.abs(u[k] - ou), np.abs(v[k] - ov))
        assert np.mean(err <= 1e-3) >= 0.995 and err.max() <= 5e-3, (k, float(np.mean(err <= 1e-3)),
                                                                      float(err.max()))
    pu, pv = qp.per_call.piv_adaptive_per_call(handle, pairs[0][0], pairs[0][1], desc)
    assert pu.tobytes() == u[0].tobytes() and pv.tobytes() == v[0].tobytes()


def test_inherit_tiles_rejects(qp, handle):
    pt = pl = np.array([0, 16, 32])
    pu = np.zeros((3, 3), np.float32)
    with pytest.raises(qp.QlpivError) as e:
        handle.inherit_tiles(0, 32, pt, pl, pu, pu, 16, pt, pl)       # spline: use qlpiv_inherit
    assert e.value.status == qp.E_ARG
    with pytest.raises(qp.QlpivError) as e:
        handle.inherit_tiles(1, 32, pt, pl, pu, pu, 16, pt[:2], pl)   # Direct needs 2 children per parent
    assert e.value.status == qp.E_SHAPE
    bad = qp.adaptive_desc(64, 16, 0.5, inherit_mode=7)
    a, b = qp.synth.particle_pair((256, 256), qp.synth.Flow(vmax=2.0, rc=40.0), seed=1)
    with pytest.raises(qp.QlpivError) as e:
        handle.piv_adaptive([a], [b], bad)
    assert e.value.status == qp.E_ARG
