"""Optical flow after PIV on the GPU against the CPU oracle.

The flow stage (prefilters, Liu-Shen normalisation, per-pixel spline field of the tile
displacements, dense Lucas-Kanade, Liu-Shen, tile replacement) runs every float operation in
the oracle's order without contraction, so tiles and dense fields must be bit-identical to
orc_flow_after_piv.  The whole PIV + flow pipeline must equal adaptive PIV followed by the flow
stage on the same tiles.
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


def _pair(qp, h, w, bits=8, seed=3):
    flow = qp.synth.Flow(vmax=3.0, rc=min(h, w) / 5.0, shear=0.01)
    a, b = qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, diam_sd=0.3, noise=2.0, bits=bits, seed=seed)
    return a, b, flow


def _tiles(oracle, flow, h, w, n, rng):
    _, tops, lefts = oracle.grid(h, w, n, 0, 0.5)
    cy = tops.astype(np.float64) + n / 2.0 - 0.5
    cx = lefts.astype(np.float64) + n / 2.0 - 0.5
    yy, xx = np.meshgrid(cy, cx, indexing="ij")
    du, dv = flow.displacement(yy, xx, (h, w))
    tu = (du + rng.normal(0.0, 0.1, du.shape)).astype(np.float32)
    tv = (dv + rng.normal(0.0, 0.1, dv.shape)).astype(np.float32)
    return tops, lefts, tu, tv


CASES = [
    # mode, dense export, sigma_lk, px_lk, window, iterations_lk, iterations_ls, bits, (h, w), n, ignore_piv
    (1, False, 2.0, 3, 27, 5, 0, 8, (192, 224), 16, 0),
    (1, True, 2.0, 3, 27, 5, 0, 8, (192, 224), 16, 0),
    (1, False, 0.0, 3, 9, 3, 0, 12, (160, 130), 32, 0),
    (2, False, 2.0, 3, 15, 2, 25, 8, (176, 160), 16, 0),
    (2, True, 1.3, 5, 27, 3, 40, 16, (128, 192), 16, 0),
    (1, False, 2.0, 3, 27, 5, 0, 8, (128, 144), 16, 1),
    (1, True, 2.0, 3, 27, 5, 0, 8, (128, 144), 16, 2),
    (2, False, 2.0, 3, 15, 3, 10, 8, (128, 144), 16, 3),
    (1, False, 2.0, 3, 27, 5, 0, 8, (128, 144), 16, 4),
    (2, True, 2.0, 3, 27, 5, 10, 8, (128, 144), 16, 5),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_flow_after_piv_bit_exact(qp, handle, oracle, case):
    mode, dense, sig, px, win, it_lk, it_ls, bits, (h, w), n, ign = CASES[case]
    a, b, flow = _pair(qp, h, w, bits=bits, seed=case + 11)
    rng = np.random.default_rng(case)
    tops, lefts, tu, tv = _tiles(oracle, flow, h, w, n, rng)
    d = qp.flow_desc(mode=mode, filter_sigma_lk=sig, filter_px_lk=px, window_lk=win, iterations_lk=it_lk,
                     iterations_ls=max(it_ls, 1), dense_export=dense, ignore_piv=ign)
    gu, gv, gdu, gdv = handle.flow_after_piv(a, b, n, tops, lefts, tu, tv, d)
    ou, ov, odu, odv = oracle.flow_after_piv(a, b, n, tops, lefts, tu, tv, mode=mode, sigma_lk=sig, px_lk=px,
                                             window=win, iterations_lk=it_lk, iterations_ls=max(it_ls, 1),
                                             dense_export=dense, ignore_piv=ign)
    assert not np.array_equal(ou, tu)               # the flow stage changed the tiles
    assert gu.tobytes() == ou.tobytes() and gv.tobytes() == ov.tobytes()
    assert gdu.tobytes() == odu.tobytes() and gdv.tobytes() == odv.tobytes()
    tu2, tv2 = handle.flow_after_piv(a, b, n, tops, lefts, tu, tv, d, dense=False)
    assert tu2.tobytes() == gu.tobytes() and tv2.tobytes() == gv.tobytes()


PYRAMID_CASES = [
    # mode, dense export, window, iterations_lk, iterations_ls, (h, w), n, pyramid levels
    (1, False, 27, 5, 0, (192, 224), 16, 2),
    (1, True, 15, 3, 0, (160, 130), 32, 3),
    (2, False, 15, 2, 10, (176, 160), 16, 2),
    (1, False, 9, 4, 0, (256, 200), 16, 4),
]


@pytest.mark.parametrize("case", range(len(PYRAMID_CASES)))
def test_flow_after_piv_pyramid_bit_exact(qp, handle, oracle, case):
    """Lucas-Kanade coarse to fine (an extension of the reference's full-resolution stage) equals
    the oracle's pyramid bit for bit, odd level sides included."""
    mode, dense, win, it_lk, it_ls, (h, w), n, levels = PYRAMID_CASES[case]
    a, b, flow = _pair(qp, h, w, seed=case + 31)
    rng = np.random.default_rng(case + 7)
    tops, lefts, tu, tv = _tiles(oracle, flow, h, w, n, rng)
    d = qp.flow_desc(mode=mode, window_lk=win, iterations_lk=it_lk, iterations_ls=max(it_ls, 1), dense_export=dense,
                     pyramid_levels=levels)
    gu, gv, gdu, gdv = handle.flow_after_piv(a, b, n, tops, lefts, tu, tv, d)
    ou, ov, odu, odv = oracle.flow_after_piv(a, b, n, tops, lefts, tu, tv, mode=mode, window=win,
                                             iterations_lk=it_lk, iterations_ls=max(it_ls, 1), dense_export=dense,
                                             pyramid_levels=levels)
    assert gdu.tobytes() == odu.tobytes() and gdv.tobytes() == odv.tobytes()
    assert gu.tobytes() == ou.tobytes() and gv.tobytes() == ov.tobytes()
    fu, fv, fdu, _ = oracle.flow_after_piv(a, b, n, tops, lefts, tu, tv, mode=mode, window=win, iterations_lk=it_lk,
                                           iterations_ls=max(it_ls, 1), dense_export=dense)
    assert not np.array_equal(fdu, odu)             # the pyramid changed the result


def test_flow_after_piv_tracks_the_flow(qp, handle, oracle):
    """Lucas-Kanade after PIV brings noisy tile displacements closer to the true flow."""
    h, w, n = 256, 256, 16
    a, b, flow = _pair(qp, h, w, seed=5)
    rng = np.random.default_rng(9)
    tops, lefts, tu, tv = _tiles(oracle, flow, h, w, n, rng)
    cy = tops + n / 2.0 - 1.0
    cx = lefts + n / 2.0 - 1.0
    yy, xx = np.meshgrid(cy, cx, indexing="ij")
    # the particles of A move by the flow at their own position: sample it half a step back
    ty, tx = flow.displacement(yy, xx, (h, w))
    inner = np.s_[3:-3, 3:-3]
    before = np.hypot(tu - ty, tv - tx)[inner]
    gu, gv = handle.flow_after_piv(a, b, n, tops, lefts, tu, tv, qp.flow_desc(), dense=False)
    after = np.hypot(gu - ty, gv - tx)[inner]
    assert np.median(after) < np.median(before)


def test_flow_descriptor_rejected(qp, handle, oracle):
    a, b, flow = _pair(qp, 96, 96)
    tops, lefts, tu, tv = _tiles(oracle, flow, 96, 96, 16, np.random.default_rng(0))
    for bad in (dict(mode=3), dict(window_lk=8), dict(window_lk=33), dict(iterations_lk=0),
                dict(mode=2, iterations_ls=0), dict(filter_px_lk=4), dict(ignore_piv=6), dict(pyramid_levels=5),
                dict(pyramid_levels=-1)):
        with pytest.raises(qp.QlpivError) as e:
            handle.flow_after_piv(a, b, 16, tops, lefts, tu, tv, qp.flow_desc(**bad))
        assert e.value.status == qp.E_ARG
    with pytest.raises(qp.QlpivError):   # tiles outside the image
        handle.flow_after_piv(a, b, 16, tops + 90, lefts, tu, tv, qp.flow_desc())
    a2, b2 = a[:56], b[:56]              # 56 >> 3 = 7 rows at the fourth level: below 8
    t2 = tops[tops + 16 <= 56]
    with pytest.raises(qp.QlpivError) as e:
        handle.flow_after_piv(a2, b2, 16, t2, lefts, tu[:len(t2)], tv[:len(t2)], qp.flow_desc(pyramid_levels=4))
    assert e.value.status == qp.E_ARG
    handle.flow_after_piv(a2, b2, 16, t2, lefts, tu[:len(t2)], tv[:len(t2)], qp.flow_desc(pyramid_levels=3))


@pytest.mark.parametrize("mode,dense", [(1, False), (2, True)])
def test_piv_flow_matches_piv_then_flow(qp, handle, oracle, mode, dense):
    h, w = 256, 288
    pairs = [_pair(qp, h, w, bits=12, seed=40 + k) for k in range(3)]
    fa, fb = [p[0] for p in pairs], [p[1] for p in pairs]
    vd = qp.multipeak_validation(num_peaks=3, peak_kernel=3, threshold=2.0, epsilon0=0.1, max_iterations=2)
    desc = qp.adaptive_desc(64, 16, 0.5, validation=vd)
    fd = qp.flow_desc(mode=mode, iterations_ls=30, dense_export=dense)
    u, v, du, dv = handle.piv_flow(fa, fb, desc, fd, dense=True)
    pu, pv = handle.piv_adaptive(fa, fb, desc)
    last = qp.adaptive_levels(desc, h, w)[-1]
    _, tops, lefts = oracle.grid(h, w, 64, len(qp.adaptive_levels(desc, h, w)) - 1, 0.5)
    assert (len(tops), len(lefts)) == (last["tiles_i"], last["tiles_j"])
    for k in range(len(pairs)):
        eu, ev, edu, edv = handle.flow_after_piv(fa[k], fb[k], last["n"], tops, lefts, pu[k], pv[k], fd)
        assert u[k].tobytes() == eu.tobytes() and v[k].tobytes() == ev.tobytes()
        assert du[k].tobytes() == edu.tobytes() and dv[k].tobytes() == edv.tobytes()
        ou, ov, odu, odv = oracle.flow_after_piv(fa[k], fb[k], last["n"], tops, lefts, pu[k], pv[k], mode=mode,
                                                 iterations_ls=30, dense_export=dense)
        assert u[k].tobytes() == ou.tobytes() and dv[k].tobytes() == odv.tobytes()
    u2, v2 = handle.piv_flow(fa, fb, desc, fd)
    assert u2.tobytes() == u.tobytes() and v2.tobytes() == v.tobytes()


def test_piv_flow_device_matches_host(qp, handle):
    torch = pytest.importorskip("torch")
    h, w = 256, 256
    pairs = [_pair(qp, h, w, bits=16, seed=70 + k) for k in range(2)]
    desc = qp.adaptive_desc(32, 16, 0.5)
    fd = qp.flow_desc(mode=2, iterations_ls=10, dense_export=True)
    u, v, du, dv = handle.piv_flow([p[0] for p in pairs], [p[1] for p in pairs], desc, fd, dense=True)
    dev = torch.device("cuda:0")
    keep = [(torch.from_numpy(a.view(np.int16)).to(dev), torch.from_numpy(b.view(np.int16)).to(dev))
            for a, b, _ in pairs]
    table = np.zeros(len(pairs), qp.FRAME_DTYPE)
    for k, (ta, tb) in enumerate(keep):
        table[k] = (ta.data_ptr(), tb.data_ptr(), h, w, w)
    ttab = torch.from_numpy(table.view(np.uint8)).to(dev)
    ou = torch.empty(u.shape, dtype=torch.float32, device=dev)
    ov = torch.empty_like(ou)
    odu = torch.empty(du.shape, dtype=torch.float32, device=dev)
    odv = torch.empty_like(odu)
    handle.piv_flow_device(desc, fd, qp.PIX_U16, h, w, len(pairs), ttab, ou, ov, odu, odv)
    handle.synchronize()
    assert ou.cpu().numpy().tobytes() == u.tobytes() and ov.cpu().numpy().tobytes() == v.tobytes()
    assert odu.cpu().numpy().tobytes() == du.tobytes() and odv.cpu().numpy().tobytes() == dv.tobytes()


def test_piv_flow_more_pairs_than_lanes(qp, handle):
    """Six pairs share the flow stage's four lanes (streams with their own planes): every pair's
    tiles and dense field equal the pair run alone."""
    h, w = 160, 192
    pairs = [_pair(qp, h, w, bits=8, seed=90 + k) for k in range(6)]
    fa, fb = [p[0] for p in pairs], [p[1] for p in pairs]
    desc = qp.adaptive_desc(32, 16, 0.5)
    fd = qp.flow_desc(mode=2, iterations_ls=12, dense_export=True)
    u, v, du, dv = handle.piv_flow(fa, fb, desc, fd, dense=True)
    for k in range(len(pairs)):
        u1, v1, du1, dv1 = handle.piv_flow([fa[k]], [fb[k]], desc, fd, dense=True)
        assert u[k].tobytes() == u1[0].tobytes() and v[k].tobytes() == v1[0].tobytes(), k
        assert du[k].tobytes() == du1[0].tobytes() and dv[k].tobytes() == dv1[0].tobytes(), k
