"""Micro / mini per-tile warping on the GPU against the CPU oracle.

The tile warp runs the oracle's float operations in the same order without contraction, so the
warped tiles and their maxima must be bit-identical; the adaptive pipeline with these modes is
compared with the oracle's pipeline (FP32 restatement and FP64 twin) like the other warp modes.
"""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

MODES = [4, 5, 6, 7, 8, 9]


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


def _case(qp, oracle, h, w, n, bits, seed):
    flow = qp.synth.Flow(vmax=5.0, rc=min(h, w) / 4.0, shear=0.01)
    a, b = qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, bits=bits, seed=seed)
    _, tops, lefts = oracle.grid(h, w, n, 0, 0.5)
    yy, xx = np.meshgrid(tops + n / 2.0, lefts + n / 2.0, indexing="ij")
    du, dv = flow.displacement(yy, xx, (h, w))
    rng = np.random.default_rng(seed)
    u = (du + rng.normal(0, 0.3, du.shape)).astype(np.float32)
    v = (dv + rng.normal(0, 0.3, dv.shape)).astype(np.float32)
    return a, b, tops, lefts, u, v


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("n,bits", [(16, 8), (32, 12), (64, 8)])
def test_tile_warp_bit_exact(qp, handle, oracle, mode, n, bits):
    h, w = 5 * n, 6 * n + 8
    a, b, tops, lefts, u, v = _case(qp, oracle, h, w, n, bits, seed=mode * 10 + n)
    full = 255.0 if bits == 8 else 4095.0
    ta, tb, ma, mb = handle.tile_warp(a, b, n, tops, lefts, u, v, mode, full)
    oa, ob, oma, omb = oracle.tile_warp(a, b, n, tops, lefts, u, v, mode, full)
    np.testing.assert_array_equal(ta.astype(np.float32), oa)
    np.testing.assert_array_equal(tb.astype(np.float32), ob)
    np.testing.assert_array_equal(ma, oma)
    np.testing.assert_array_equal(mb, omb)


def test_tile_warp_rejects_bad_arguments(qp, handle, oracle):
    a, b, tops, lefts, u, v = _case(qp, oracle, 96, 96, 16, 8, seed=1)
    with pytest.raises(qp.QlpivError):
        handle.tile_warp(a, b, 16, tops, lefts, u, v, 1, 255.0)    # not a per-tile mode
    with pytest.raises(qp.QlpivError):
        handle.tile_warp(a, b, 16, tops + 90, lefts, u, v, 6, 255.0)


@pytest.mark.parametrize("mode,bits", [(6, 8), (9, 12), (4, 8), (8, 8)])
def test_adaptive_pipeline_micro_mini(qp, handle, oracle, mode, bits):
    h, w = 320, 288
    flow = qp.synth.Flow(vmax=4.0, rc=56.0, shear=0.005)
    pairs = [qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, bits=bits, seed=300 + k + mode)
             for k in range(2)]
    fm = 255.0 if bits == 8 else 4095.0
    desc = qp.adaptive_desc(64, 16, 0.5, warp_mode=mode, fixed_max=fm)
    u, v = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    for k, (a, b) in enumerate(pairs):
        ou, ov = oracle.piv_adaptive(a, b, 64, 16, 0.5, fixed_max=fm, precision=32, warp=mode)
        err = np.maximum(np.abs(u[k] - ou), np.abs(v[k] - ov))
        assert np.mean(err <= 1e-3) >= 0.995 and err.max() <= 5e-3, (k, float(np.mean(err <= 1e-3)),
                                                                      float(err.max()))
        o64u, o64v = oracle.piv_adaptive(a, b, 64, 16, 0.5, fixed_max=fm, precision=64, warp=mode)
        err64 = np.maximum(np.abs(u[k] - o64u), np.abs(v[k] - o64v))
        assert np.mean(err64 <= 1e-3) >= 0.995 and err64.max() <= 5e-3
    # the per-call path drives the same stages one call at a time
    pu, pv = qp.per_call.piv_adaptive_per_call(handle, pairs[0][0], pairs[0][1], desc)
    assert pu.tobytes() == u[0].tobytes() and pv.tobytes() == v[0].tobytes()


def test_padded_device_frames(qp, handle):
    """Device frames whose rows are padded (pitch > width) give the packed frames' result."""
    torch = pytest.importorskip("torch")
    h, w, pad = 256, 240, 24
    pairs = [qp.synth.particle_pair((h, w), qp.synth.Flow(vmax=3.0, rc=40.0), bits=12, seed=80 + k) for k in range(2)]
    desc = qp.adaptive_desc(32, 16, 0.5)
    u1, v1 = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    dev = torch.device("cuda:0")
    keep = []
    table = np.zeros(2, qp.FRAME_DTYPE)
    for k, (a, b) in enumerate(pairs):
        pa = np.zeros((h, w + pad), np.uint16)
        pb = np.zeros((h, w + pad), np.uint16)
        pa[:, :w] = a
        pb[:, :w] = b
        ta = torch.from_numpy(pa.view(np.int16)).to(dev)
        tb = torch.from_numpy(pb.view(np.int16)).to(dev)
        keep += [ta, tb]
        table[k] = (ta.data_ptr(), tb.data_ptr(), h, w, w + pad)
    ttab = torch.from_numpy(table.view(np.uint8)).to(dev)
    ou = torch.empty(u1.size, dtype=torch.float32, device=dev)
    ov = torch.empty(v1.size, dtype=torch.float32, device=dev)
    handle.piv_adaptive_device(desc, qp.PIX_U16, h, w, 2, ttab, ou, ov)
    handle.synchronize()
    assert ou.cpu().numpy().tobytes() == u1.tobytes() and ov.cpu().numpy().tobytes() == v1.tobytes()
