"""Clipping modes and the single-strategy validation models on the GPU against the oracle.

* ClippingModeEnum (S/ClippingModeEnum.java:9-13): under NoOutOfBoundClipping every update of a
  tile's displacement -- inheritance, the correlation increment, validation replacements and the
  zeroing of still-invalid vectors -- is refused when the rounded displacement moves the tile out
  of the image (Tile.accumulateDisplacement / replaceDisplacement, S/iareas/Tile.java:103-189).
  LoggedOutOfBoundClipping gives the AllowedOutOfBoundClipping result.
* The validation models the converter builds besides the multi-peak one
  (PIVConfigurationConverterVisitor.java:546-608): difference validator and normalised median,
  each without or with bilinear replacement, with FindMaximumFromCenter peaks.

The validator is compared with the oracle bit for bit on the same inputs; whole adaptive runs
stage by stage against the oracle (adaptive_trace.py), end to end against the FP64 pipeline
with every vector beyond 1e-3 px traced to an upstream cause, and bit for bit against the
plain per-call path.
"""
import numpy as np
import pytest

from conftest import load_package

import adaptive_trace
from validation_cases import clustered_case, smooth_case

pytestmark = pytest.mark.gpu

MODELS = [1, 2, 3, 4, 5]


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


def _vdesc(qp, model, k, clipping, threshold=2.0, iterations=2, until=False):
    d = qp.adaptive_desc(32, 16, 0.5, clipping_mode=clipping)
    if model == qp.VALIDATE_MULTIPEAK_MEDIAN:
        v = qp.multipeak_validation(num_peaks=k, peak_kernel=3, threshold=threshold, epsilon0=0.1,
                                    max_iterations=iterations, iterate_until=until)
    else:
        v = qp.validation_model(model, threshold=threshold, epsilon0=0.1, max_iterations=iterations,
                                iterate_until=until)
    qp.set_validation(d, **v)
    return d


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("clip", [False, True])
@pytest.mark.parametrize("case", range(4))
def test_validation_models_bit_exact(qp, handle, oracle, model, clip, case):
    rng = np.random.default_rng(500 + 11 * case + model)
    k = 3 if model == 1 else 1
    if case < 3:
        ni, nj = [(9, 11), (40, 33), (61, 61)][case]
        tops, lefts, u, v, pu, pv, npk, _, _ = smooth_case(rng, ni, nj, k, [3, 30, 80][case])
    else:
        tops, lefts, u, v, pu, pv, npk, _, _ = clustered_case(rng, 50, 40, k, 0.02, 12)
    n = 16
    geo = (n, int(tops[-1]) + n, int(lefts[-1]) + n + 2)   # last row touches the bottom edge
    thr = 1.5 if model in (2, 3) else 2.0
    d = _vdesc(qp, model, k, qp.CLIP_NO_OUT_OF_BOUND if clip else qp.CLIP_ALLOWED, threshold=thr,
               iterations=1 + case % 3, until=case == 2)
    peaks = (pu, pv, npk) if model == 1 else (None, None, None)
    gu, gv, ginv = handle.validate(tops, lefts, u, v, *peaks, d, n=geo[0], height=geo[1], width=geo[2])
    cfg = oracle.valid_cfg(num_peaks=k, threshold=thr, epsilon0=0.1, max_iterations=1 + case % 3,
                           iterate_until_no_corrections=case == 2, model=model, clip=geo if clip else None)
    ou, ov, oinv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, cfg)
    np.testing.assert_array_equal(ginv, oinv)
    assert gu.tobytes() == ou.tobytes() and gv.tobytes() == ov.tobytes()
    if not clip:
        # the entry point without sizes gives the same result
        hu, hv, hinv = handle.validate(tops, lefts, u, v, *peaks, d)
        assert hu.tobytes() == gu.tobytes() and hv.tobytes() == gv.tobytes()
    if model in (2, 3):
        assert ginv.all()        # the difference validator never validates a vector


def test_validate_without_sizes_refuses_clipping(qp, handle):
    rng = np.random.default_rng(1)
    tops, lefts, u, v, pu, pv, npk, _, _ = smooth_case(rng, 6, 6, 1, 1)
    d = _vdesc(qp, qp.VALIDATE_MEDIAN, 1, qp.CLIP_NO_OUT_OF_BOUND)
    with pytest.raises(qp.QlpivError):
        handle.validate(tops, lefts, u, v, None, None, None, d)


def _shifted_pair(qp, h, w, bits, seed):
    """A vortex plus a uniform 6 px downward drift: tiles near the bottom edge would leave the
    image, which NoOutOfBoundClipping refuses."""
    flow = qp.synth.Flow(vmax=4.0, rc=50.0, shear=0.004)
    a, b = qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, diam_sd=0.0, bits=bits, seed=seed)
    b = np.roll(b, 6, axis=0)
    b[:6] = 0
    return a, b


@pytest.mark.parametrize("warp", [False, True])
@pytest.mark.parametrize("model", [0, 1, 3, 5])
def test_adaptive_clipping_modes(qp, handle, oracle, warp, model):
    h, w = 256, 320
    bits = 8
    pairs = [_shifted_pair(qp, h, w, bits, 70 + k) for k in range(2)]
    k = 3 if model == 1 else 1
    out = {}
    for clipping in (qp.CLIP_ALLOWED, qp.CLIP_LOGGED, qp.CLIP_NO_OUT_OF_BOUND):
        desc = qp.adaptive_desc(64, 16, 0.25, warp_mode=qp.WARP_BOTH_BILINEAR if warp else qp.WARP_NONE,
                                max_mode=qp.MAX_FIXED if warp else qp.MAX_COMPUTE, fixed_max=255.0 if warp else 0.0,
                                clipping_mode=clipping)
        if model:
            v = (qp.multipeak_validation(num_peaks=k) if model == 1 else qp.validation_model(model))
            qp.set_validation(desc, **v)
        u, vv = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
        out[clipping] = (u, vv)
        cfg = None
        if model:
            cfg = oracle.valid_cfg(num_peaks=k, threshold=2.0, epsilon0=0.1, max_iterations=2, model=model)
        for q, (a, b) in enumerate(pairs):
            recs = adaptive_trace.gpu_trace(qp, handle, a, b, desc)
            assert recs[-1]["u"].tobytes() == u[q].tobytes() and recs[-1]["v"].tobytes() == vv[q].tobytes()
            adaptive_trace.check_stages(qp, oracle, recs, desc, cfg)
            olv = adaptive_trace.oracle_levels(oracle, a, b, recs, desc, (64, 16, 0.25), cfg=cfg,
                                               fixed_max=255.0 if warp else None, warp=warp)
            rep = adaptive_trace.cascade_report(recs, olv, desc)
            assert all(r["causes"]["unexplained"] == 0 for r in rep), rep
            assert rep[-1]["over_tol"] <= 0.01 * rep[-1]["vectors"], rep
        pu, pv = qp.per_call.piv_adaptive_per_call(handle, pairs[0][0], pairs[0][1], desc)
        assert pu.tobytes() == u[0].tobytes() and pv.tobytes() == vv[0].tobytes()
    allowed, logged, strict = out[0], out[1], out[2]
    assert allowed[0].tobytes() == logged[0].tobytes() and allowed[1].tobytes() == logged[1].tobytes()
    # the last tile row touches the bottom edge: under NoOutOfBoundClipping every downward
    # displacement of it is refused and it keeps zero (the difference model zeroes every vector
    # when clipping is allowed, and keeps the refused ones under NoOutOfBoundClipping)
    assert not np.array_equal(allowed[0], strict[0])
    assert not strict[0][0, -1].any()
    if model != 3:
        assert np.abs(allowed[0][0, -1]).max() > 2.0
    else:
        assert not allowed[0].any() and strict[0].any()


@pytest.mark.parametrize("model", [2, 3, 4, 5])
def test_adaptive_single_strategy_models(qp, handle, oracle, model):
    """Difference (never validating: every vector ends at 0) and median models, without or with
    bilinear replacement, over a whole adaptive run with outlier patches."""
    h, w = 256, 256
    flow = qp.synth.Flow(vmax=5.0, rc=48.0, shear=0.01)
    a, b = qp.synth.particle_pair((h, w), flow, ppp=0.02, diam=2.5, diam_sd=0.3, noise=4.0, bits=8, seed=17)
    c, _ = qp.synth.particle_pair((h, w), qp.synth.Flow(vmax=0.0), ppp=0.02, diam=2.5, noise=4.0, bits=8, seed=1017)
    b = b.copy()
    b[60:120, 130:190] = c[60:120, 130:190]
    desc = qp.adaptive_desc(64, 16, 0.5, fixed_max=255.0)
    qp.set_validation(desc, **qp.validation_model(model))
    u, v = handle.piv_adaptive([a], [b], desc)
    cfg = oracle.valid_cfg(threshold=2.0, epsilon0=0.1, max_iterations=2, model=model)
    recs = adaptive_trace.gpu_trace(qp, handle, a, b, desc)
    assert recs[-1]["u"].tobytes() == u[0].tobytes() and recs[-1]["v"].tobytes() == v[0].tobytes()
    adaptive_trace.check_stages(qp, oracle, recs, desc, cfg)
    olv = adaptive_trace.oracle_levels(oracle, a, b, recs, desc, (64, 16, 0.5), cfg=cfg, fixed_max=255.0)
    rep = adaptive_trace.cascade_report(recs, olv, desc)
    assert all(r["causes"]["unexplained"] == 0 for r in rep), rep
    pu, pv = qp.per_call.piv_adaptive_per_call(handle, a, b, desc)
    assert pu.tobytes() == u[0].tobytes() and pv.tobytes() == v[0].tobytes()
    if model in (2, 3):
        assert not u.any() and not v.any()
    else:
        assert np.abs(u).max() > 1.0
