"""The plain per-call GPU path (one library call per stage, host arrays between stages) runs the
same kernels as the device-resident adaptive pipeline: the displacements must be identical."""
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


@pytest.mark.parametrize("bits,warp,validate", [(12, True, True), (8, True, False), (8, False, False),
                                                (8, False, True), (8, 9, True), (12, 5, False)])
def test_per_call_equals_pipeline(qp, handle, bits, warp, validate):
    h, w = 320, 288
    flow = qp.synth.Flow(vmax=4.0, rc=48.0, shear=0.005)
    pairs = [qp.synth.particle_pair((h, w), flow, ppp=0.03, diam=2.5, bits=bits, seed=90 + k) for k in range(2)]
    vd = qp.multipeak_validation(num_peaks=3, peak_kernel=3, threshold=2.0, epsilon0=0.1, max_iterations=2) \
        if validate else None
    mode = warp if not isinstance(warp, bool) else (qp.WARP_BOTH_BILINEAR if warp else qp.WARP_NONE)
    desc = qp.adaptive_desc(64, 16, 0.5 if warp else 0.25, warp_mode=mode, fixed_max=65535.0 if bits > 8 else 0.0,
                            validation=vd)
    u, v = handle.piv_adaptive([p[0] for p in pairs], [p[1] for p in pairs], desc)
    for k, (a, b) in enumerate(pairs):
        pu, pv = qp.per_call.piv_adaptive_per_call(handle, a, b, desc)
        assert pu.tobytes() == u[k].tobytes() and pv.tobytes() == v[k].tobytes()
