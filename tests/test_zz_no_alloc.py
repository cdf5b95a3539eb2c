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


def _run_noalloc(qp, torch, dev, case, rnd, stream=None):
    py, px, pu, pv, cy, cx = case
    d = [torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev) for a in (py, px, pu, pv, cy, cx)]
    cu = torch.full((len(cy), len(cx)), np.nan, dtype=torch.float32, device=dev)
    cv = torch.full_like(cu, np.nan)
    torch.cuda.synchronize()
    qp.inherit_noalloc(0, stream.cuda_stream if stream is not None else 0, d[0], d[1], d[2], d[3], d[4], d[5], cu,
                       cv, len(py), len(px), len(cy), len(cx), rnd)
    if stream is not None:
        stream.synchronize()
    else:
        torch.cuda.synchronize()
    return cu.cpu().numpy(), cv.cpu().numpy()


def test_inherit_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    qp = load_package()
    qp.build.build()
    qp.load_library()
    dev = torch.device("cuda:0")
    with qp.Handle(0) as h:
        for seed, (hh, ww, n0, rnd) in enumerate([(300, 420, 64, False), (512, 384, 32, True)]):
            case = _case(qp, seed, hh, ww, n0)
            py, px, pu, pv, cy, cx = case
            ref_u, ref_v = h.inherit(py.astype(np.float64), px.astype(np.float64), pu, pv, cy, cx, rnd)
            cu, cv = _run_noalloc(qp, torch, dev, case, rnd)
            assert cu.tobytes() == ref_u.tobytes()
            assert cv.tobytes() == ref_v.tobytes()


def test_inherit_noalloc_small_parent_grid_and_caller_stream():
    """A parent grid with 4 rows (too few for the spline: the outputs are zero-filled) and a
    call queued on a caller-owned stream, both byte for byte against qlpiv_inherit."""
    torch = pytest.importorskip("torch")
    qp = load_package()
    qp.build.build()
    qp.load_library()
    dev = torch.device("cuda:0")
    with qp.Handle(0) as h:
        py, px, pu, pv, cy, cx = _case(qp, 7, 300, 420, 64)
        small = (py[:4], px, pu[:4], pv[:4], cy, cx)
        ref_u, ref_v = h.inherit(py[:4].astype(np.float64), px.astype(np.float64), pu[:4], pv[:4], cy, cx, False)
        assert not ref_u.any() and not ref_v.any()
        cu, cv = _run_noalloc(qp, torch, dev, small, False)
        assert cu.tobytes() == ref_u.tobytes() and cv.tobytes() == ref_v.tobytes()
        stream = torch.cuda.Stream(device=dev)
        case = (py, px, pu, pv, cy, cx)
        ref_u, ref_v = h.inherit(py.astype(np.float64), px.astype(np.float64), pu, pv, cy, cx, False)
        for _ in range(2):
            cu, cv = _run_noalloc(qp, torch, dev, case, False, stream=stream)
            assert cu.tobytes() == ref_u.tobytes() and cv.tobytes() == ref_v.tobytes()


def test_inherit_noalloc_rejects_oversized_grids():
    torch = pytest.importorskip("torch")
    qp = load_package()
    qp.build.build()
    big = qp.NOALLOC_MAX_ROWS // 8 + 1
    buf = torch.zeros(16, dtype=torch.float32, device="cuda:0")
    p = buf.data_ptr()   # raw addresses: the library's own size check is what is tested
    with pytest.raises(qp.QlpivError) as ei:
        # the size check rejects the call on the host, before anything is queued
        qp.inherit_noalloc(0, 0, p, p, p, p, p, p, p, p, 8, big, big, 8)
    assert ei.value.status == qp.E_SHAPE
    assert "QLPIV_NOALLOC_MAX_ROWS" in str(ei.value)
