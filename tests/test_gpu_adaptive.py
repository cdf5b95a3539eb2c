"""Adaptive multi-pass stages on the GPU against the CPU oracle.

Velocity inheritance, the per-pixel displacement field and the bilinear warp use the
same operation order as the oracle and are compiled without FMA contraction: they must be
bit-identical.  The whole level loop is compared with the FP64 oracle pipeline: final
displacements within 1e-3 px except where the two pipelines' integer peaks differ by an
exact tie (checked on the FP64 planes) or a warped pixel sits on a rounding boundary.
"""
import numpy as np
import pytest

from conftest import load_package

import adaptive_trace

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


def _centres(qp, h, w, n_start, level, ofac):
    g = qp.grid.superposition(h, w, n_start, level, ofac)
    cy, cx = g.centres()
    return g, cy, cx


def _smooth_field(qp, cy, cx, shape, vmax=5.0):
    yy, xx = np.meshgrid(cy, cx, indexing="ij")
    dr, dc = qp.synth.Flow(vmax=vmax, rc=40.0, shear=0.004).displacement(yy, xx, shape)
    rng = np.random.default_rng(0)
    return ((dr + 0.05 * rng.standard_normal(dr.shape)).astype(np.float32),
            (dc + 0.05 * rng.standard_normal(dc.shape)).astype(np.float32))


@pytest.mark.parametrize("round_int", [False, True])
def test_inherit_bit_exact(qp, handle, oracle, round_int):
    h, w = 300, 420
    gp, py, px = _centres(qp, h, w, 64, 0, 0.25)
    gc, cy, cx = _centres(qp, h, w, 64, 1, 0.25)
    pu, pv = _smooth_field(qp, py, px, (h, w))
    cu, cv = handle.inherit(py.astype(np.float64), px.astype(np.float64), pu, pv, cy, cx, round_int)
    ou, ov = oracle.inherit(py.astype(np.float64), px.astype(np.float64), pu, pv, cy, cx, round_int)
    assert cu.tobytes() == ou.tobytes() and cv.tobytes() == ov.tobytes()
    assert np.abs(cu).max() > 1.0
    # float evaluation stays within 1e-5 px of the double-precision interpolation
    du, dv = oracle.inherit(py.astype(np.float64), px.astype(np.float64), pu, pv, cy, cx, round_int, precision=64)
    assert np.abs(cu - du).max() <= (0.0 if round_int else 1e-5) + (1.0 if round_int else 0.0)


def test_inherit_small_parent_grid_gives_zero(qp, handle):
    py = np.arange(4, dtype=np.float64) * 8 + 7.5
    cu, cv = handle.inherit(py, py, np.ones((4, 4), np.float32), np.ones((4, 4), np.float32),
                            np.arange(7, dtype=np.float32) * 4 + 3.5, np.arange(7, dtype=np.float32) * 4 + 3.5)
    assert (cu == 0).all() and (cv == 0).all()


def test_displacement_field_bit_exact(qp, handle, oracle):
    h, w = 256, 320
    g, cy, cx = _centres(qp, h, w, 32, 0, 0.25)
    u, v = _smooth_field(qp, cy, cx, (h, w))
    fu, fv = handle.displacement_field(cy.astype(np.float64), cx.astype(np.float64), u, v, h, w)
    ou, ov = oracle.displacement_field(cy.astype(np.float64), cx.astype(np.float64), u, v, h, w)
    assert fu.tobytes() == ou.tobytes() and fv.tobytes() == ov.tobytes()
    du, dv = oracle.displacement_field(cy.astype(np.float64), cx.astype(np.float64), u, v, h, w, precision=64)
    assert np.abs(fu - du).max() < 1e-5 and np.abs(fv - dv).max() < 1e-5
    # the surface interpolates the tile values at the centres (integer-plus-half centres
    # are not pixels, so check between the 4 surrounding pixels)
    assert np.abs(fu[int(cy[3]), int(cx[5])] - u[3, 5]) < 0.5


@pytest.mark.parametrize("bits,quirk", [(8, False), (12, False), (12, True), (16, False)])
def test_warp_pair_bit_exact(qp, handle, oracle, bits, quirk):
    h, w = 200, 264
    a, b = qp.synth.particle_pair((h, w), qp.synth.Flow(vmax=4.0, rc=30.0), ppp=0.04, bits=bits, seed=bits)
    g, cy, cx = _centres(qp, h, w, 32, 1, 0.25)
    u, v = _smooth_field(qp, cy, cx, (h, w), vmax=4.0)
    wa, wb = handle.warp_pair(a, b, cy.astype(np.float64), cx.astype(np.float64), u, v, int16_quirk=quirk)
    fu, fv = oracle.displacement_field(cy.astype(np.float64), cx.astype(np.float64), u, v, h, w)
    oa, ob = oracle.warp_both(a, b, fu, fv, int16_quirk=quirk)
    assert wa.dtype == a.dtype and wa.tobytes() == oa.tobytes() and wb.tobytes() == ob.tobytes()
    assert not np.array_equal(wa, a)
    # FirstImage / SecondImage: one frame warped by the whole field, the other unchanged
    for mode, image_mode in ((qp.WARP_FIRST_BILINEAR, 1), (qp.WARP_SECOND_BILINEAR, 2)):
        wa, wb = handle.warp_pair(a, b, cy.astype(np.float64), cx.astype(np.float64), u, v, int16_quirk=quirk,
                                  warp_mode=mode)
        oa, ob = oracle.warp_both(a, b, fu, fv, int16_quirk=quirk, image_mode=image_mode)
        assert wa.tobytes() == oa.tobytes() and wb.tobytes() == ob.tobytes()
        assert np.array_equal(wb if image_mode == 1 else wa, b if image_mode == 1 else a)


@pytest.mark.parametrize("mode,bits", [(2, 8), (3, 8), (2, 12), (3, 12)])
def test_adaptive_first_second_image_warping(qp, handle, oracle, mode, bits):
    """FirstImage / SecondImage full-image warping: the warped frame's tiles keep the full-scale
    maximum, the other frame's tiles their own; against the FP32 and FP64 oracle and the per-call
    path."""
    h, w = 288, 320
    flow = qp.synth.Flow(vmax=5.0, rc=56.0, shear=0.004)
    pairs = [qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, diam_sd=0.0, bits=bits, seed=90 + k + mode)
             for k in range(2)]
    fm = 255.0 if bits == 8 else 4095.0
    desc = qp.adaptive_desc(64, 16, 0.5, warp_mode=mode, fixed_max=fm)
    u, v = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    for k, (a, b) in enumerate(pairs):
        for prec in (32, 64):
            ou, ov = oracle.piv_adaptive(a, b, 64, 16, 0.5, fixed_max=fm, precision=prec, warp=mode)
            err = np.maximum(np.abs(u[k] - ou), np.abs(v[k] - ov))
            assert np.mean(err <= 1e-3) >= 0.995 and err.max() <= 5e-3, (k, prec, float(np.mean(err <= 1e-3)),
                                                                          float(err.max()))
    pu, pv = qp.per_call.piv_adaptive_per_call(handle, pairs[0][0], pairs[0][1], desc)
    assert pu.tobytes() == u[0].tobytes() and pv.tobytes() == v[0].tobytes()


def _true_flow(qp, flow, g, shape):
    cy, cx = g.centres()
    yy, xx = np.meshgrid(cy, cx, indexing="ij")
    return flow.displacement(yy, xx, shape)


@pytest.mark.parametrize("bits,warp,tile_max", [(8, True, "full"), (12, True, "full"), (12, True, "tile"),
                                                 (8, False, "tile")])
def test_adaptive_pipeline_matches_fp64_oracle(qp, handle, oracle, bits, warp, tile_max):
    """tile_max "full": tiles cut from the warped images keep the full-scale maximum, as in
    the reference (copyMatrixRegion); with 12-bit data the v/65535*16+1 map leaves the +1
    pedestal dominant and the vectors are biased toward zero, so only parity is checked.
    "tile": the per-tile maximum (floor 16)."""
    h, w = 256, 320
    flow = qp.synth.Flow(vmax=5.0, rc=48.0, shear=0.004)
    pairs = [qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, diam_sd=0.0, bits=bits, seed=40 + k)
             for k in range(3)]
    fixed = (255.0 if bits == 8 else 65535.0) if tile_max == "full" else 0.0
    desc = qp.adaptive_desc(64, 16, 0.25, warp_mode=qp.WARP_BOTH_BILINEAR if warp else qp.WARP_NONE,
                            max_mode=qp.MAX_FIXED if fixed else qp.MAX_COMPUTE, fixed_max=fixed)
    u, v = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    g = qp.grid.superposition(h, w, 64, 2, 0.25)
    assert u.shape == (3, g.tiles_i, g.tiles_j)
    for k, (a, b) in enumerate(pairs):
        # every stage, fed the GPU's own inputs, within the criteria (ties excepted)
        recs = adaptive_trace.gpu_trace(qp, handle, a, b, desc)
        assert recs[-1]["u"].tobytes() == u[k].tobytes() and recs[-1]["v"].tobytes() == v[k].tobytes()
        adaptive_trace.check_stages(qp, oracle, recs, desc)
        # end to end against the FP64 pipeline run from the raw frames: every vector beyond
        # 1e-3 px has a cause upstream of its last correlation (its inherited value or a pixel
        # of its warped tiles differs, or an exact tie); the stages' in-tolerance differences
        # add up over the levels (the reference's own FP32 path drifts the same way)
        olv = adaptive_trace.oracle_levels(oracle, a, b, recs, desc, (64, 16, 0.25), fixed_max=fixed or None,
                                           warp=warp)
        rep = adaptive_trace.cascade_report(recs, olv, desc)
        assert all(r["causes"]["unexplained"] == 0 for r in rep), rep
        assert rep[-1]["over_tol"] <= 0.005 * rep[-1]["vectors"], rep
        if bits == 8 or tile_max == "tile":
            tr, tc = _true_flow(qp, flow, g, (h, w))
            assert np.median(np.hypot(u[k] - tr, v[k] - tc)) < 0.15


def test_adaptive_device_variant_and_repeatability(qp, handle):
    torch = pytest.importorskip("torch")
    h, w = 256, 256
    pairs = [qp.synth.particle_pair((h, w), qp.synth.Flow(vmax=3.0, rc=40.0), bits=12, seed=60 + k) for k in range(2)]
    desc = qp.adaptive_desc(32, 16, 0.25)
    u1, v1 = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    u2, v2 = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    assert u1.tobytes() == u2.tobytes() and v1.tobytes() == v2.tobytes()
    dev = torch.device("cuda:0")
    keep = [(torch.from_numpy(a.view(np.int16)).to(dev), torch.from_numpy(b.view(np.int16)).to(dev)) for a, b in pairs]
    table = np.zeros(2, qp.FRAME_DTYPE)
    for k, (ta, tb) in enumerate(keep):
        table[k] = (ta.data_ptr(), tb.data_ptr(), h, w, w)
    ttab = torch.from_numpy(table.view(np.uint8)).to(dev)
    ou = torch.empty(u1.size, dtype=torch.float32, device=dev)
    ov = torch.empty(v1.size, dtype=torch.float32, device=dev)
    handle.piv_adaptive_device(desc, qp.PIX_U16, h, w, 2, ttab, ou, ov)
    handle.synchronize()
    assert ou.cpu().numpy().tobytes() == u1.tobytes() and ov.cpu().numpy().tobytes() == v1.tobytes()


@pytest.mark.parametrize("warp", [True, False])
def test_adaptive_from_ia128(qp, handle, oracle, warp):
    """IA 128 -> 32 (the first level on the two-CTA cluster kernel) against the FP64 oracle."""
    h, w = 512, 448
    flow = qp.synth.Flow(vmax=6.0, rc=100.0, shear=0.004)
    pairs = [qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, diam_sd=0.0, bits=8, seed=70 + k)
             for k in range(2)]
    desc = qp.adaptive_desc(128, 32, 0.5, warp_mode=qp.WARP_BOTH_BILINEAR if warp else qp.WARP_NONE,
                            max_mode=qp.MAX_FIXED if warp else qp.MAX_COMPUTE, fixed_max=255.0 if warp else 0.0)
    u, v = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    for k, (a, b) in enumerate(pairs):
        recs = adaptive_trace.gpu_trace(qp, handle, a, b, desc)
        assert recs[-1]["u"].tobytes() == u[k].tobytes() and recs[-1]["v"].tobytes() == v[k].tobytes()
        adaptive_trace.check_stages(qp, oracle, recs, desc)
        olv = adaptive_trace.oracle_levels(oracle, a, b, recs, desc, (128, 32, 0.5),
                                           fixed_max=255.0 if warp else None, warp=warp)
        rep = adaptive_trace.cascade_report(recs, olv, desc)
        assert all(r["causes"]["unexplained"] == 0 for r in rep), rep
        assert rep[-1]["over_tol"] <= 0.005 * rep[-1]["vectors"], rep


@pytest.mark.parametrize("start", [1, 3])
def test_adaptive_mixed_division(qp, handle, oracle, start):
    """AdaptiveInterAreaStrategyMixedSuperPosition (S/iareas/AdaptiveInterAreaStrategyMixedSuperPosition.java:31-92):
    levels before `start` split without superposition, the rest with it, SuperPosition restarted
    at `start` (3 of 3 levels: NoSuperPosition throughout).  With warping and multi-peak
    validation: stage by stage against the oracle, end to end against the FP64 pipeline with
    every vector beyond 1e-3 px traced to an upstream cause, bit for bit against the plain
    per-call path."""
    h, w = 256, 320
    flow = qp.synth.Flow(vmax=5.0, rc=48.0, shear=0.01)
    pairs = [qp.synth.particle_pair((h, w), flow, ppp=0.02, diam=2.5, diam_sd=0.3, noise=4.0, bits=8, seed=40 + k)
             for k in range(2)]
    desc = qp.adaptive_desc(64, 16, 0.5, fixed_max=255.0, superposition_start=start,
                            validation=qp.multipeak_validation())
    u, v = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    g = qp.grid.level(h, w, 64, 2, 0.5, superposition_start=start)
    assert u.shape == (2, g.tiles_i, g.tiles_j)
    # the first level is split without superposition
    g0, plain0 = qp.grid.level(h, w, 64, 0, 0.5, superposition_start=start), qp.grid.superposition(h, w, 64, 0, 0.5)
    assert (g0.tiles_i, g0.tiles_j) != (plain0.tiles_i, plain0.tiles_j)
    cfg = oracle.valid_cfg(num_peaks=3, kernel_width=3, threshold=2.0, epsilon0=0.1, max_iterations=2)
    for q, (a, b) in enumerate(pairs):
        recs = adaptive_trace.gpu_trace(qp, handle, a, b, desc)
        assert recs[-1]["u"].tobytes() == u[q].tobytes() and recs[-1]["v"].tobytes() == v[q].tobytes()
        adaptive_trace.check_stages(qp, oracle, recs, desc, cfg)
        olv = adaptive_trace.oracle_levels(oracle, a, b, recs, desc, (64, 16, 0.5), cfg=cfg, fixed_max=255.0)
        rep = adaptive_trace.cascade_report(recs, olv, desc)
        assert all(r["causes"]["unexplained"] == 0 for r in rep), rep
    pu, pv = qp.per_call.piv_adaptive_per_call(handle, pairs[0][0], pairs[0][1], desc)
    assert pu.tobytes() == u[0].tobytes() and pv.tobytes() == v[0].tobytes()
    gy, gx = g.centres()
    yy, xx = np.meshgrid(gy, gx, indexing="ij")
    tr, tc = flow.displacement(yy, xx, (h, w))
    assert np.median(np.hypot(u[0] - tr, v[0] - tc)) < 0.3


def _shifted(qp, h, w, di, dj, seed):
    a, _ = qp.synth.particle_pair((h, w), qp.synth.Flow(vmax=0.0), ppp=0.03, diam=2.5, diam_sd=0.2, bits=8, seed=seed)
    b = np.zeros_like(a)
    b[di:, dj:] = a[:h - di, :w - dj]
    return a, b


@pytest.mark.parametrize("warp", [True, False])
def test_adaptive_stabilisation_uniform_shift(qp, handle, oracle, warp):
    """InterAreaDisplacementStableStrategy on a uniform (3, 2) px shift, every increment far from the
    1 px maximum.  BothImages: the first level repeats the same correlation (no warping there) and
    adds the increment on each of its 3 passes; the second level walks back to the shift in two.
    No warping: the displaced B tiles meet the shift on the second pass.  The device loop matches
    the oracle's on every vector and recovers the shift away from the borders."""
    h, w = 256, 288
    a, b = _shifted(qp, h, w, 3, 2, 11)
    wm = qp.WARP_BOTH_BILINEAR if warp else qp.WARP_NONE
    desc = qp.adaptive_desc(64, 32, 0.5, warp_mode=wm, fixed_max=255.0 if warp else 0.0,
                            max_mode=qp.MAX_FIXED if warp else qp.MAX_COMPUTE, stable_max_displacement=1.0,
                            stable_max_retries=3)
    u, v = handle.piv_adaptive([a], [b], desc)
    ou, ov = oracle.piv_adaptive(a, b, 64, 32, 0.5, fixed_max=255.0 if warp else None, warp=warp, stable_max=1.0,
                                 stable_retries=3)
    err = np.maximum(np.abs(u[0] - ou), np.abs(v[0] - ov))
    assert err.max() <= 1e-3, float(err.max())
    # (BothImages: full-scale tile maxima bias the level-1 correction of the 6 px the first level
    # over-accumulated by up to ~0.2 px)
    inner = (slice(1, -1), slice(1, -1))
    tol = 0.3 if warp else 1e-3
    assert np.abs(u[0][inner] - 3.0).max() < tol and np.abs(v[0][inner] - 2.0).max() < tol
    # without stabilisation the first level's single pass is all the second level inherits
    plain = qp.adaptive_desc(64, 32, 0.5, warp_mode=wm, fixed_max=255.0 if warp else 0.0,
                             max_mode=qp.MAX_FIXED if warp else qp.MAX_COMPUTE)
    pu, _ = handle.piv_adaptive([a], [b], plain)
    if warp:
        assert not np.array_equal(pu, u)


def test_adaptive_stabilisation_vortex(qp, handle, oracle):
    """Stabilisation on a vortex, three levels with BothImages warping: device and oracle loops
    agree except where an increment lies within rounding of the maximum (the pass counts can then
    differ); the result stays a vortex."""
    h, w = 256, 320
    flow = qp.synth.Flow(vmax=5.0, rc=48.0, shear=0.01)
    a, b = qp.synth.particle_pair((h, w), flow, ppp=0.02, diam=2.5, diam_sd=0.3, noise=4.0, bits=8, seed=77)
    desc = qp.adaptive_desc(64, 16, 0.5, fixed_max=255.0, stable_max_displacement=0.3, stable_max_retries=3)
    u, v = handle.piv_adaptive([a], [b], desc)
    ou, ov = oracle.piv_adaptive(a, b, 64, 16, 0.5, fixed_max=255.0, stable_max=0.3, stable_retries=3)
    err = np.maximum(np.abs(u[0] - ou), np.abs(v[0] - ov))
    assert np.mean(err <= 1e-3) >= 0.95 and np.median(err) < 1e-4, (float(np.mean(err <= 1e-3)), float(err.max()))
    g = qp.grid.superposition(h, w, 64, 2, 0.5)
    cy, cx = g.centres()
    yy, xx = np.meshgrid(cy, cx, indexing="ij")
    tr, tc = flow.displacement(yy, xx, (h, w))
    assert np.median(np.hypot(u[0] - tr, v[0] - tc)) < 0.3
