"""qlpiv_inherit_noalloc: velocity inheritance for callers that cannot let the library
allocate device memory during a call (a Java host passing device buffers from its own pool
under a fixed memory budget, an acquisition loop that must not take cudaMalloc's implicit
synchronisation).  Its scratch is a fixed device array inside the library; the result must
equal the allocating entry point qlpiv_inherit, on two calls in a row that reuse that array.

This file is collected last so that a failing run that stops at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu


def _case(qp, seed, h, w, n_start):
    gp = qp.grid.superposition(h, w, n_start, 0, 0.25)
    gc = qp.grid.superposition(h, w, n_start, 1, 0.25)
    py, px = gp.centres()
    cy, cx = gc.centres()
    rng = np.random.default_rng(seed)
    yy, xx = np.meshgrid(py, px, indexing="ij")
    dr, dc = qp.synth.Flow(vmax=4.0, rc=40.0, shear=0.003).displacement(yy, xx, (h, w))
    pu = (dr + 0.05 * rng.standard_normal(dr.shape)).astype(np.float32)
    pv = (dc + 0.05 * rng.standard_normal(dc.shape)).astype(np.float32)
    return py, px, pu, pv, cy, cx


def test_inherit_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    qp = load_package()
    qp.build.build()
    qp.load_library()
    dev = torch.device("cuda:0")
    with qp.Handle(0) as h:
        for seed, (hh, ww, n0, rnd) in enumerate([(300, 420, 64, False), (512, 384, 32, True)]):
            py, px, pu, pv, cy, cx = _case(qp, seed, hh, ww, n0)
            ref_u, ref_v = h.inherit(py.astype(np.float64), px.astype(np.float64), pu, pv, cy, cx, rnd)
            d = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (py, px, pu, pv, cy, cx)]
            cu = torch.full((len(cy), len(cx)), np.nan, dtype=torch.float32, device=dev)
            cv = torch.full_like(cu, np.nan)
            qp.inherit_noalloc(0, 0, d[0], d[1], d[2], d[3], d[4], d[5], cu, cv, len(py), len(px), len(cy),
                               len(cx), rnd)
            torch.cuda.synchronize()
            assert cu.cpu().numpy().tobytes() == ref_u.tobytes()
            assert cv.cpu().numpy().tobytes() == ref_v.tobytes()


def test_inherit_noalloc_rejects_oversized_grids():
    torch = pytest.importorskip("torch")
    qp = load_package()
    qp.build.build()
    big = qp.NOALLOC_MAX_ROWS // 8 + 1
    buf = torch.zeros(16, dtype=torch.float32, device="cuda:0")
    with pytest.raises(qp.QlpivError) as ei:
        # the size check rejects the call on the host, before anything is queued
        qp.inherit_noalloc(0, 0, buf, buf, buf, buf, buf, buf, buf, buf, 8, big, big, 8)
    assert ei.value.status == qp.E_SHAPE
    assert "QLPIV_NOALLOC_MAX_ROWS" in str(ei.value)
