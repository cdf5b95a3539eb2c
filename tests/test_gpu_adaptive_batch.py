"""Adaptive batches on the GPU: frame pairs of uneven sizes, each with its own adaptive schedule,
replayed from one captured graph (pairs of one size and schedule share a group).  Every pair's
displacements must equal the pair run alone through qlpiv_piv_adaptive, bit for bit."""
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


def _schedules(qp):
    vd = qp.multipeak_validation(num_peaks=3, peak_kernel=3, threshold=2.0, epsilon0=0.1, max_iterations=2)
    return [qp.adaptive_desc(32, 32, 0.5, warp_mode=qp.WARP_NONE),
            qp.adaptive_desc(64, 32, 0.5, warp_mode=qp.WARP_BOTH_BILINEAR),
            qp.adaptive_desc(64, 16, 0.25, warp_mode=qp.WARP_BOTH_BILINEAR, validation=vd)]


@pytest.mark.parametrize("bits", [8, 12])
def test_adaptive_batch_equals_single_pairs(qp, handle, bits):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(bits)
    shapes = [(160, 192), (256, 256), (200, 296), (384, 320)]
    sch = _schedules(qp)
    pairs, sidx = [], []
    for k in range(14):
        h, w = shapes[rng.integers(len(shapes))]
        flow = qp.synth.Flow(vmax=float(rng.uniform(1.5, 4.0)), rc=min(h, w) / 5.0, shear=0.01)
        pairs.append(qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, bits=bits, seed=500 + 10 * bits + k))
        sidx.append(int(rng.integers(len(sch))))
    dev = torch.device("cuda:0")
    view = np.uint8 if bits == 8 else np.int16
    keep, table = [], np.zeros(len(pairs), qp.FRAME_DTYPE)
    for k, (a, b) in enumerate(pairs):
        ta = torch.from_numpy(a.view(view).copy()).to(dev)
        tb = torch.from_numpy(b.view(view).copy()).to(dev)
        keep.append((ta, tb))
        table[k] = (ta.data_ptr(), tb.data_ptr(), a.shape[0], a.shape[1], a.shape[1])
    pt = qp.PIX_U8 if bits == 8 else qp.PIX_U16
    batch = qp.AdaptiveBatch(handle, table, pt, sch, sidx)
    assert batch.total == batch.pair_offset[-1]
    assert 1 < batch.groups < len(pairs)          # some pairs share a group, some groups differ
    for rep in range(2):                          # the graph replays
        batch.run()
        u, v = batch.displacements()
        for q, (a, b) in enumerate(pairs):
            u1, v1 = handle.piv_adaptive([a], [b], sch[sidx[q]])
            assert batch.pair(u, q).tobytes() == u1[0].tobytes(), (rep, q)
            assert batch.pair(v, q).tobytes() == v1[0].tobytes(), (rep, q)
    # new contents in the same device buffers: the replay reads them
    ta, tb = keep[0]
    tb.copy_(ta)
    batch.run()
    u, v = batch.displacements()
    a0 = pairs[0][0]
    u1, v1 = handle.piv_adaptive([a0], [a0], sch[sidx[0]])
    assert batch.pair(u, 0).tobytes() == u1[0].tobytes() and batch.pair(v, 0).tobytes() == v1[0].tobytes()
    batch.close()


def test_adaptive_batch_rejects(qp, handle):
    torch = pytest.importorskip("torch")
    a, b = qp.synth.particle_pair((128, 128), qp.synth.Flow(vmax=2.0, rc=30.0), bits=8, seed=9)
    ta, tb = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    table = np.zeros(1, qp.FRAME_DTYPE)
    table[0] = (ta.data_ptr(), tb.data_ptr(), 128, 128, 128)
    sch = _schedules(qp)
    with pytest.raises(qp.QlpivError) as e:
        qp.AdaptiveBatch(handle, table, qp.PIX_U8, sch, [3])
    assert e.value.status == qp.E_ARG
    with pytest.raises(qp.QlpivError) as e:
        qp.AdaptiveBatch(handle, table, qp.PIX_F32, sch, [0])
    assert e.value.status == qp.E_ARG
