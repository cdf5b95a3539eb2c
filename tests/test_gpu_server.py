"""Request server on the GPU: continuous batching of requests of mixed sizes and schedules.

Each request's displacements must be bit-identical to qlpiv_piv_adaptive run alone on the same
pair, whatever else is in flight; admission must respect the HBM budget; errors and timeouts
follow the C ABI's contract.
"""
import threading

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
            qp.adaptive_desc(64, 32, 0.5, warp_mode=qp.WARP_NONE),
            qp.adaptive_desc(64, 16, 0.5, warp_mode=qp.WARP_BOTH_BILINEAR),
            qp.adaptive_desc(64, 16, 0.25, warp_mode=qp.WARP_BOTH_BILINEAR, validation=vd)]


def _requests(qp, count, seed=0):
    rng = np.random.default_rng(seed)
    sizes = [(256, 256), (384, 320), (512, 512), (768, 640), (1024, 1024)]
    out = []
    for k in range(count):
        h, w = sizes[rng.integers(len(sizes))]
        bits = [8, 12][rng.integers(2)]
        flow = qp.synth.Flow(vmax=float(rng.uniform(1.0, 5.0)), rc=min(h, w) / 6.0, shear=0.003)
        a, b = qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, bits=bits, seed=500 + k)
        out.append((a, b, int(rng.integers(4))))
    return out


def test_single_request_matches_handle(qp, handle):
    a, b, _ = _requests(qp, 1, seed=3)[0]
    d = _schedules(qp)[2]
    with qp.Server(0, slots=4) as srv:
        t = srv.submit(a, b, d)
        u, v, info = srv.poll(t, timeout_ms=60000)
    eu, ev = handle.piv_adaptive([a], [b], d)
    assert u.tobytes() == eu[0].tobytes() and v.tobytes() == ev[0].tobytes()
    assert info["total_ms"] >= info["device_ms"] >= 0.0


def test_mixed_requests_same_alone_and_in_the_mix(qp, handle):
    reqs = _requests(qp, 24, seed=7)
    sch = _schedules(qp)
    alone = [handle.piv_adaptive([a], [b], sch[s]) for a, b, s in reqs]
    results = [None] * len(reqs)
    with qp.Server(0, slots=6) as srv:
        tickets = [None] * len(reqs)

        def submitter(idx):
            for k in idx:
                a, b, s = reqs[k]
                tickets[k] = srv.submit(a, b, sch[s])

        threads = [threading.Thread(target=submitter, args=(range(j, len(reqs), 3),)) for j in range(3)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        peak_in_flight = 0
        for k in range(len(reqs)):
            while True:
                r = srv.poll(tickets[k], timeout_ms=5)
                st = srv.stats()
                peak_in_flight = max(peak_in_flight, st["in_flight"])
                if r is not None:
                    results[k] = r
                    break
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
    assert peak_in_flight >= 2          # requests overlapped on the device
    for k, ((eu, ev), (u, v, _)) in enumerate(zip(alone, results)):
        assert u.tobytes() == eu[0].tobytes() and v.tobytes() == ev[0].tobytes(), k


def test_admission_respects_the_budget(qp, handle):
    reqs = _requests(qp, 10, seed=11)
    d = _schedules(qp)[2]
    need = [qp.adaptive_plan_bytes(d, qp.pixel_type_of(a.dtype), *a.shape) for a, _, _ in reqs]
    budget = int(max(need) * 1.5)
    with qp.Server(0, slots=8, hbm_budget=budget) as srv:
        tickets = [srv.submit(a, b, d) for a, b, _ in reqs]
        seen = 0
        done = {}
        while len(done) < len(tickets):
            st = srv.stats()
            assert st["device_bytes_in_flight"] <= budget
            seen = max(seen, st["in_flight"])
            for k, t in enumerate(tickets):
                if k not in done:
                    r = srv.poll(t, timeout_ms=0)
                    if r is not None:
                        done[k] = r
    for k, (a, b, _) in enumerate(reqs):
        eu, ev = handle.piv_adaptive([a], [b], d)
        assert done[k][0].tobytes() == eu[0].tobytes()


def test_server_errors(qp):
    a, b, _ = _requests(qp, 1, seed=5)[0]
    d = _schedules(qp)[1]
    need = qp.adaptive_plan_bytes(d, qp.pixel_type_of(a.dtype), *a.shape)
    with qp.Server(0, slots=2, hbm_budget=need // 2) as srv:
        with pytest.raises(qp.QlpivError) as e:      # can never fit the budget
            srv.submit(a, b, d)
        assert e.value.status == qp.E_OOM
    with qp.Server(0, slots=2) as srv:
        with pytest.raises(qp.QlpivError) as e:
            srv.poll(12345, timeout_ms=0)
        assert e.value.status == qp.E_ARG
        with pytest.raises(qp.QlpivError):           # float images are not adaptive PIV input
            srv.submit(a.astype(np.float32), b.astype(np.float32), d)
        with pytest.raises(qp.QlpivError):           # image smaller than the first IA
            srv.submit(a[:40, :40], b[:40, :40], d)
        t = srv.submit(a, b, d)
        assert srv.poll(t, timeout_ms=60000) is not None


def test_destroy_with_queued_requests(qp):
    reqs = _requests(qp, 6, seed=13)
    d = _schedules(qp)[3]
    srv = qp.Server(0, slots=1)
    for a, b, _ in reqs:
        srv.submit(a, b, d)
    srv.close()   # cancels the queued ones, waits for the one on the device
