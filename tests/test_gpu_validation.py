"""Multi-peak search and vector validation on the GPU against the CPU oracle.

* FindMaximumMultiPeaks: the kernel's peaks are checked against the oracle's search run on
  the kernel's own correlation planes (qlpiv_xcorr_planes): positions, values and the
  minimum floor must be identical, the sub-pixel fits within 1e-4 px.
* Validation: same inputs, same float operation order, no contraction: the validated
  displacements and invalid flags must be bit-identical to the oracle's sequential
  centre-out visit, whatever the clustering of the invalid tiles.
* The adaptive pipeline with validation is compared with the FP64 oracle pipeline.
"""
import numpy as np
import pytest

from conftest import load_package

import adaptive_trace
from validation_cases import clustered_case, smooth_case

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


def _tiles(qp, n, count, bits=8, seed=0, sparse=False):
    rng = np.random.default_rng(seed)
    h, w = 4 * n, 4 * n
    pairs = []
    for k in range(count // 9 + 1):
        a, b = qp.synth.particle_pair((h, w), qp.synth.Flow(vmax=min(4.0, n / 4), rc=n * 1.5), ppp=0.02, bits=bits,
                                      seed=seed * 100 + k)
        pairs.append((a, b))
    ta, tb = [], []
    for a, b in pairs:
        for i in range(3):
            for j in range(3):
                ta.append(a[i * n:(i + 1) * n, j * n:(j + 1) * n])
                tb.append(b[i * n + n // 2:(i + 1) * n + n // 2, j * n + n // 4:(j + 1) * n + n // 4])
    ta = np.stack(ta[:count])
    tb = np.stack(tb[:count])
    if sparse:  # mostly-zero tiles: planes full of zero cells (stale cell positions)
        mask = rng.random(ta.shape) < 0.03
        ta = np.where(mask, ta, 0).astype(ta.dtype)
        tb = np.where(rng.random(tb.shape) < 0.03, tb, 0).astype(tb.dtype)
    return ta, tb


@pytest.mark.parametrize("n,kw,k,norm,sparse", [(16, 3, 3, 0, False), (32, 3, 2, 0, False), (64, 3, 3, 0, False),
                                                (32, 2, 4, 1, False), (64, 5, 1, 0, False), (16, 7, 16, 1, False),
                                                (32, 3, 3, 3, True), (16, 2, 5, 3, True), (16, 3, 4, 1, False),
                                                (32, 3, 3, 1, False), (64, 2, 4, 0, False), (64, 3, 8, 1, False),
                                                (32, 4, 2, 0, False), (16, 3, 3, 3, True),
                                                (128, 3, 3, 0, False), (128, 2, 4, 1, False),
                                                (128, 3, 2, 3, True)])
def test_multipeaks_match_oracle_on_kernel_planes(qp, handle, oracle, n, kw, k, norm, sparse):
    ta, tb = _tiles(qp, n, 160, seed=n + kw + k, sparse=sparse)
    _check_multipeaks(qp, handle, oracle, ta, tb, n, kw, k, norm)


@pytest.mark.parametrize("n,k", [(16, 3), (32, 3), (64, 3), (16, 1), (32, 4), (64, 2)])
def test_batched_replay_reruns_are_exact(qp, handle, oracle, n, k):
    """Up to 4 peaks with the 3-point fit, the lists are replayed 32 IAs at a time from the
    records each IA stored; an IA whose list needs records that were not stored runs again per
    IA.  All-zero planes (no normalisation, empty tiles) always do: their threshold is 0.  Mixed
    with ordinary tiles in one launch, every IA must still match the oracle's search."""
    ta, tb = _tiles(qp, n, 200, seed=7 * n + k)
    zero = np.zeros(len(ta), bool)
    zero[1::3] = True
    ta = np.where(zero[:, None, None], 0, ta).astype(ta.dtype)
    tb = np.where(zero[:, None, None], 0, tb).astype(tb.dtype)
    _check_multipeaks(qp, handle, oracle, ta, tb, n, 3, k, qp.NORM_NONE)


def _check_multipeaks(qp, handle, oracle, ta, tb, n, kw, k, norm):
    planes = handle.xcorr_planes(ta, tb, norm_mode=norm)
    vec = handle.xcorr_multipeaks(ta, tb, norm_mode=norm, num_peaks=k, peak_kernel=kw)
    assert vec.shape == (len(ta), k)
    for r in range(len(ta)):
        peaks, mf = oracle.find_max_multipeaks(planes[r], kw, k)
        got = vec[r]
        present = (got["flags"] & qp.F_ABSENT) == 0
        assert int(present.sum()) == len(peaks), r
        assert not present[len(peaks):].any() and present[:len(peaks)].all()
        for s, (pi, pj, pv) in enumerate(peaks):
            assert (int(got[s]["peak_i"]), int(got[s]["peak_j"])) == (pi, pj), (r, s)
            assert got[s]["peak_value"] == np.float32(pv), (r, s)
            assert got[s]["min_floor"] == np.float32(mf)
            si, sj, _ = oracle.subpixel_gauss3(planes[r], pi, pj)
            assert abs(got[s]["sub_i"] - si) <= 1e-4 and abs(got[s]["sub_j"] - sj) <= 1e-4, (r, s)
            assert got[s]["u"] == np.float32(got[s]["sub_i"] - (n - 1))
        for s in range(len(peaks), k):
            assert got[s]["u"] == 0.0 and got[s]["v"] == 0.0


def test_multipeak_frame_pass_matches_tile_api(qp, handle, oracle, rankine_pair):
    a, b = rankine_pair
    g, tops, lefts = oracle.grid_origins(a.shape[0], a.shape[1], 32, 0.5)
    vec = handle.piv_pass(a, b, 32, tops, lefts, num_peaks=3, peak_kernel=3)
    assert vec.shape == (len(tops), 3)
    ta = np.stack([a[t:t + 32, l:l + 32] for t, l in zip(tops, lefts)])
    tb = np.stack([b[t:t + 32, l:l + 32] for t, l in zip(tops, lefts)])
    ref = handle.xcorr_multipeaks(ta, tb, num_peaks=3, peak_kernel=3)
    assert vec.tobytes() == ref.tobytes()
    # against the FP64 oracle's multi-peak pass: main peaks agree except for rare ties
    o64, npk = oracle.piv_pass_multi(a, b, 32, tops, lefts, num_peaks=3, kernel_width=3, precision=64)
    same = (vec[:, 0]["peak_i"] == o64[:, 0]["peak_i"]) & (vec[:, 0]["peak_j"] == o64[:, 0]["peak_j"])
    assert same.mean() >= 0.995
    err = np.hypot(vec[:, 0]["u"] - o64[:, 0]["u64"], vec[:, 0]["v"] - o64[:, 0]["v64"])
    assert np.all(err[same] <= 1e-3)
    batch = handle.piv_pass_batch([a], [b], 32, np.zeros(len(tops), np.int32), tops, lefts, num_peaks=3,
                                  peak_kernel=3)
    assert batch.tobytes() == vec.tobytes()


def test_multipeak_settings_rejected(qp, handle):
    ta, tb = _tiles(qp, 16, 4)
    for k, kw in [(0, 3), (17, 3), (3, 1)]:
        with pytest.raises(qp.QlpivError) as e:
            handle.xcorr_multipeaks(ta, tb, num_peaks=k, peak_kernel=kw)
        assert e.value.status == qp.E_ARG


def _desc(qp, k, iterations=2, until=False, threshold=2.0, eps0=0.1):
    d = qp.adaptive_desc(32, 16, 0.5)
    return qp.set_validation(d, num_peaks=k, peak_kernel=3, threshold=threshold, epsilon0=eps0,
                             max_iterations=iterations, iterate_until=until)


@pytest.mark.parametrize("case", range(10))
def test_validate_bit_exact(qp, handle, oracle, case):
    rng = np.random.default_rng(1000 + case)
    k = [1, 2, 3, 4][case % 4]
    if case < 5:
        ni, nj = [(9, 11), (31, 31), (61, 47), (5, 7), (125, 125)][case]
        frac = [0.05, 0.03, 0.08, 0.5, 0.02][case]
        tops, lefts, u, v, pu, pv, npk, _, _ = smooth_case(rng, ni, nj, k, int(frac * ni * nj))
    else:
        ni, nj = [(61, 61), (125, 125), (253, 253), (40, 90), (17, 17)][case - 5]
        block = [12, 30, 40, 20, 17][case - 5]
        tops, lefts, u, v, pu, pv, npk, _, _ = clustered_case(rng, ni, nj, k, 0.02, block)
    iterations, until = [(1, False), (2, False), (3, True), (2, False), (1, True)][case % 5]
    d = _desc(qp, k, iterations, until)
    gu, gv, ginv = handle.validate(tops, lefts, u, v, pu, pv, npk, d)
    cfg = oracle.valid_cfg(num_peaks=k, kernel_width=3, threshold=2.0, epsilon0=0.1, max_iterations=iterations,
                           iterate_until_no_corrections=until)
    ou, ov, oinv, _ = oracle.validate(tops, lefts, u, v, pu, pv, npk, cfg)
    assert ((ou != u) | (ov != v)).any()          # the case exercises replacement
    np.testing.assert_array_equal(ginv, oinv)
    assert gu.tobytes() == ou.tobytes() and gv.tobytes() == ov.tobytes()


def test_validate_rejects_bad_arguments(qp, handle):
    rng = np.random.default_rng(1)
    tops, lefts, u, v, pu, pv, npk, _, _ = smooth_case(rng, 6, 6, 2, 2)
    with pytest.raises(qp.QlpivError):
        handle.validate(tops, lefts, u, v, pu, pv, npk + 5, _desc(qp, 2))
    with pytest.raises(qp.QlpivError):
        handle.validate(tops, lefts, u, v, pu, pv, npk, _desc(qp, 2, threshold=0.0))


def _outlier_pair(qp, h, w, seed):
    flow = qp.synth.Flow(vmax=5.0, rc=48.0, shear=0.01)
    a, b = qp.synth.particle_pair((h, w), flow, ppp=0.02, diam=2.5, diam_sd=0.3, noise=4.0, bits=8, seed=seed)
    c, _ = qp.synth.particle_pair((h, w), qp.synth.Flow(vmax=0.0), ppp=0.02, diam=2.5, diam_sd=0.3, noise=4.0,
                                  bits=8, seed=seed + 1000)
    b = b.copy()
    b[h // 4:h // 4 + 80, w // 2:w // 2 + 80] = c[h // 4:h // 4 + 80, w // 2:w // 2 + 80]  # uncorrelated patch
    b[3 * h // 4:3 * h // 4 + 16, w // 8:w // 8 + 16] = c[3 * h // 4:3 * h // 4 + 16, w // 8:w // 8 + 16]
    return a, b, flow


def test_adaptive_pipeline_with_validation(qp, handle, oracle):
    h, w = 384, 384
    pairs = [_outlier_pair(qp, h, w, 7 + k) for k in range(3)]
    vd = qp.multipeak_validation(num_peaks=3, peak_kernel=3, threshold=2.0, epsilon0=0.1, max_iterations=2)
    desc = qp.adaptive_desc(64, 16, 0.5, fixed_max=255.0, validation=vd)
    u, v = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    u0, v0 = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs],
                                 qp.adaptive_desc(64, 16, 0.5, fixed_max=255.0))
    cfg = oracle.valid_cfg(num_peaks=3, kernel_width=3, threshold=2.0, epsilon0=0.1, max_iterations=2)
    for k, (a, b, flow) in enumerate(pairs):
        assert np.mean((u[k] != u0[k]) | (v[k] != v0[k])) > 0.03   # validation changed the field
        # every stage, fed the GPU's own inputs: peaks against FP64, validation bit for bit
        recs = adaptive_trace.gpu_trace(qp, handle, a, b, desc)
        assert recs[-1]["u"].tobytes() == u[k].tobytes() and recs[-1]["v"].tobytes() == v[k].tobytes()
        adaptive_trace.check_stages(qp, oracle, recs, desc, cfg)
        # end to end: every vector beyond 1e-3 px of the FP64 pipeline has an upstream cause
        # (inherited value, warped pixels, a validation decision or a tie)
        olv = adaptive_trace.oracle_levels(oracle, a, b, recs, desc, (64, 16, 0.5), cfg=cfg, fixed_max=255.0)
        rep = adaptive_trace.cascade_report(recs, olv, desc)
        assert all(r["causes"]["unexplained"] == 0 for r in rep), rep
        assert rep[-1]["over_tol"] <= 0.005 * rep[-1]["vectors"], rep
        fu, fv = oracle.piv_adaptive(a, b, 64, 16, 0.5, fixed_max=255.0, precision=32, validation=cfg)
        err32 = np.maximum(np.abs(u[k] - fu), np.abs(v[k] - fv))
        assert np.mean(err32 <= 1e-3) >= 0.995
    u2, v2 = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    assert u2.tobytes() == u.tobytes() and v2.tobytes() == v.tobytes()


def test_adaptive_validation_from_ia128(qp, handle, oracle):
    """Validation at an IA-128 level: the cluster kernel's multi-peak search over its plane in
    global scratch, against the FP64 and FP32 oracle."""
    h, w = 512, 448
    pairs = [_outlier_pair(qp, h, w, 21 + k) for k in range(2)]
    vd = qp.multipeak_validation(num_peaks=3, peak_kernel=3, threshold=2.0, epsilon0=0.1, max_iterations=2)
    desc = qp.adaptive_desc(128, 32, 0.5, fixed_max=255.0, validation=vd)
    u, v = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    cfg = oracle.valid_cfg(num_peaks=3, kernel_width=3, threshold=2.0, epsilon0=0.1, max_iterations=2)
    for k, (a, b, flow) in enumerate(pairs):
        recs = adaptive_trace.gpu_trace(qp, handle, a, b, desc)
        assert recs[-1]["u"].tobytes() == u[k].tobytes() and recs[-1]["v"].tobytes() == v[k].tobytes()
        adaptive_trace.check_stages(qp, oracle, recs, desc, cfg)
        olv = adaptive_trace.oracle_levels(oracle, a, b, recs, desc, (128, 32, 0.5), cfg=cfg, fixed_max=255.0)
        rep = adaptive_trace.cascade_report(recs, olv, desc)
        assert all(r["causes"]["unexplained"] == 0 for r in rep), rep
        assert rep[-1]["over_tol"] <= 0.005 * rep[-1]["vectors"], rep
        fu, fv = oracle.piv_adaptive(a, b, 128, 32, 0.5, fixed_max=255.0, precision=32, validation=cfg)
        err32 = np.maximum(np.abs(u[k] - fu), np.abs(v[k] - fv))
        assert np.mean(err32 <= 1e-3) >= 0.995
    pu, pv = qp.per_call.piv_adaptive_per_call(handle, pairs[0][0], pairs[0][1], desc)
    assert pu.tobytes() == u[0].tobytes() and pv.tobytes() == v[0].tobytes()


def test_adaptive_validation_settings_rejected(qp, handle):
    a, b, _ = _outlier_pair(qp, 128, 128, 3)
    bad = qp.adaptive_desc(32, 16, 0.5, validation=qp.multipeak_validation(num_peaks=0))
    with pytest.raises(qp.QlpivError):
        handle.piv_adaptive([a], [b], bad)
