"""Mixed batch plans on the GPU: pairs of uneven sizes, each with its own IA size and overlap,
one graph launch.  Every pair's vectors must equal the single-pair frame pass bit for bit."""
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


def _batch(qp, bits, count, seed):
    rng = np.random.default_rng(seed)
    shapes = [(96, 96), (128, 160), (256, 256), (200, 296), (160, 128), (384, 320)]
    pairs, sizes, ofac = [], [], []
    for k in range(count):
        h, w = shapes[rng.integers(len(shapes))]
        n = int([16, 32, 64, 128][rng.integers(4)])
        if k == 0:   # at least one IA-128 pair (the two-CTA cluster kernel)
            (h, w), n = (384, 320), 128
        if min(h, w) < 2 * n:
            n = 16
        flow = qp.synth.Flow(vmax=float(rng.uniform(1, 4)), rc=min(h, w) / 4.0)
        a, b = qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, bits=bits, seed=seed * 100 + k)
        pairs.append((a, b))
        sizes.append(n)
        ofac.append([0.5, 0.25][rng.integers(2)])
    return pairs, sizes, ofac


def _device_table(qp, pairs):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    keep, table = [], np.zeros(len(pairs), qp.FRAME_DTYPE)
    for k, (a, b) in enumerate(pairs):
        view = {np.dtype(np.uint16): np.int16, np.dtype(np.uint8): np.uint8}.get(a.dtype, a.dtype)
        ta = torch.from_numpy(a.view(view).copy()).to(dev)
        tb = torch.from_numpy(b.view(view).copy()).to(dev)
        keep.append((ta, tb))
        table[k] = (ta.data_ptr(), tb.data_ptr(), a.shape[0], a.shape[1], a.shape[1])
    return keep, table


@pytest.mark.parametrize("bits,autotune", [(8, True), (12, False)])
def test_mixed_plan_equals_single_passes(qp, handle, bits, autotune):
    pairs, sizes, ofac = _batch(qp, bits, 14, seed=bits)
    keep, table = _device_table(qp, pairs)
    pt = qp.PIX_U8 if bits == 8 else qp.PIX_U16
    plan = qp.MixedPlan(handle, table, sizes, ofac, pt, autotune=autotune)
    assert plan.total == plan.pair_offset[-1]
    if autotune:
        assert all(w in (0, 1, 2, 4, 8, 16, 32) for w in plan.waves)
    assert 128 in sizes
    plan.run()
    vec = plan.vectors()
    for q, (a, b) in enumerate(pairs):
        g = qp.grid.superposition(a.shape[0], a.shape[1], sizes[q], 0, ofac[q])
        at, al = g.origins()
        ref = handle.piv_pass(a, b, sizes[q], at, al)
        got = plan.pair_vectors(vec, q)
        assert got.shape == (g.tiles_i, g.tiles_j)
        assert got.ravel().tobytes() == ref.tobytes(), q
    # replaying the graph gives the same vectors
    plan.run()
    assert plan.vectors().tobytes() == vec.tobytes()
    # new image contents in the same device buffers: the replay reads them
    ta, tb = keep[0]
    tb.copy_(ta)
    plan.run()
    vec2 = plan.vectors()
    a0 = pairs[0][0]
    g = qp.grid.superposition(a0.shape[0], a0.shape[1], sizes[0], 0, ofac[0])
    at, al = g.origins()
    ref = handle.piv_pass(a0, a0, sizes[0], at, al)
    assert plan.pair_vectors(vec2, 0).ravel().tobytes() == ref.tobytes()
    plan.close()


def test_mixed_plan_rejects(qp, handle):
    pairs, sizes, ofac = _batch(qp, 8, 3, seed=3)
    keep, table = _device_table(qp, pairs)
    with pytest.raises(qp.QlpivError) as e:
        qp.MixedPlan(handle, table, [256, 16, 16], ofac, qp.PIX_U8)
    assert e.value.status == qp.E_SHAPE
    with pytest.raises(qp.QlpivError) as e:
        qp.MixedPlan(handle, table, sizes, ofac, qp.PIX_U8, num_peaks=3)
    assert e.value.status == qp.E_ARG


@pytest.mark.parametrize("bits,kw", [(8, {}), (12, {"max_mode": 2, "fixed_max": (4095.0, 4095.0)}),
                                     (8, {"subpix_mode": 0}), ("f32", {})])
def test_persistent_schedule_equals_single_passes(qp, handle, bits, kw):
    """IA 16 / 32 / 64 in one persistent launch (one CTA per SM drains the three work lists),
    IA 128 beside it: every pair's vectors equal its single-pair pass bit for bit (u8, 12-bit in
    u16, float32 frames)."""
    if bits == "f32":
        pairs, sizes, ofac = _batch(qp, 8, 18, seed=71)
        pairs = [(a.astype(np.float32), b.astype(np.float32)) for a, b in pairs]
        pt = qp.PIX_F32
    else:
        pairs, sizes, ofac = _batch(qp, bits, 18, seed=40 + bits + len(kw))
        pt = qp.PIX_U8 if bits == 8 else qp.PIX_U16
    keep, table = _device_table(qp, pairs)
    plan = qp.MixedPlan(handle, table, sizes, ofac, pt, autotune=qp.AUTOTUNE_PERSISTENT, **kw)
    assert plan.schedule == qp.SCHEDULE_PERSISTENT
    assert {16, 32, 64, 128} <= set(sizes)
    for rep in range(2):   # the graph replay resets the work counters
        plan.run()
        vec = plan.vectors()
        for q, (a, b) in enumerate(pairs):
            g = qp.grid.superposition(a.shape[0], a.shape[1], sizes[q], 0, ofac[q])
            at, al = g.origins()
            ref = handle.piv_pass(a, b, sizes[q], at, al, **kw)
            assert plan.pair_vectors(vec, q).ravel().tobytes() == ref.tobytes(), (rep, q)
    plan.close()


def test_autotuned_schedule(qp, handle):
    """The autotuner times both schedules and keeps one; P-point sub-pixel fits keep the per-size
    launches (the persistent kernel runs the 3-point fit only)."""
    pairs, sizes, ofac = _batch(qp, 8, 10, seed=77)
    keep, table = _device_table(qp, pairs)
    plan = qp.MixedPlan(handle, table, sizes, ofac, qp.PIX_U8, autotune=qp.AUTOTUNE_ON)
    assert plan.schedule in (qp.SCHEDULE_PER_SIZE, qp.SCHEDULE_PERSISTENT)
    plan.run()
    vec = plan.vectors()
    ref_plan = qp.MixedPlan(handle, table, sizes, ofac, qp.PIX_U8, autotune=qp.AUTOTUNE_OFF)
    assert ref_plan.schedule == qp.SCHEDULE_PER_SIZE
    ref_plan.run()
    assert ref_plan.vectors().tobytes() == vec.tobytes()
    lm = qp.MixedPlan(handle, table, sizes, ofac, qp.PIX_U8, autotune=qp.AUTOTUNE_PERSISTENT,
                      subpix_mode=qp.SUBPIX_GAUSS_LM, subpix_pixels=5)
    assert lm.schedule == qp.SCHEDULE_PER_SIZE
    for p in (plan, ref_plan, lm):
        p.close()
