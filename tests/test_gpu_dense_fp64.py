"""Dense optical flow of the hybrid workload against the FP64 twin of the oracle.

1024x1024 u8 vortex pair (0.05 ppp, max 3 px), one 32x32 PIV pass at 50 % overlap, then the
flow after PIV exactly as `bench.py`'s hybrid leg runs it: Lucas-Kanade over a 2-level pyramid
(prefilter sigma 2.0 / 3 px, window 27, 5 iterations per level), Liu-Shen (lambda 4, prefilter
sigma 0.48 / 5 px, 60 passes), dense export.

* The GPU's dense field equals the oracle's float restatement bit for bit at full size.
* Against the FP64 twin (the same algorithm in double, filter weights unrounded, the per-pixel
  field in double) the dense field is within 1e-4 px RMS, both for the flow stage fed the GPU's
  PIV tiles and end to end from the FP64 PIV pass.
"""
import numpy as np
import pytest

from conftest import load_package

pytestmark = pytest.mark.gpu

RMS_TOL = 1e-4


@pytest.fixture(scope="module")
def qp():
    pkg = load_package()
    pkg.build.build()
    pkg.load_library()
    return pkg


def _descs(qp):
    piv = qp.adaptive_desc(32, 32, 0.5, warp_mode=qp.WARP_NONE, norm_mode=qp.NORM_MAX_A, max_mode=qp.MAX_COMPUTE)
    flow = qp.flow_desc(mode=qp.FLOW_LIU_SHEN, filter_sigma_lk=2.0, filter_px_lk=3, window_lk=27, iterations_lk=5,
                        filter_sigma_ls=0.48, filter_px_ls=5, lambda_ls=4.0, iterations_ls=60, dense_export=True,
                        pyramid_levels=2)
    return piv, flow


def _oracle_flow(oracle, a, b, tops, lefts, tu, tv, precision):
    return oracle.flow_after_piv(a, b, 32, tops, lefts, tu, tv, mode=2, sigma_lk=2.0, px_lk=3, sigma_ls=0.48, px_ls=5,
                                 window=27, iterations_lk=5, lam=4.0, iterations_ls=60, dense_export=True,
                                 pyramid_levels=2, precision=precision)


def _rms(du, dv, ref_u, ref_v):
    eu = du.astype(np.float64) - ref_u
    ev = dv.astype(np.float64) - ref_v
    return float(np.sqrt(np.mean(eu * eu + ev * ev))), float(max(np.abs(eu).max(), np.abs(ev).max()))


def test_hybrid_dense_field_against_fp64_twin(qp, oracle):
    a, b = qp.synth.config4_pair(pair_id=0)
    piv, flow = _descs(qp)
    with qp.Handle(0) as h:
        tu, tv, du, dv = h.piv_flow([a], [b], piv, flow, dense=True)
        pu, pv = h.piv_adaptive([a], [b], piv)       # the PIV tiles the flow stage starts from
    _, tops, lefts = oracle.grid(1024, 1024, 32, 0, 0.5)
    assert pu.shape == (1, len(tops), len(lefts))

    # float restatement, same PIV tiles: bit for bit at full size
    ou, ov, odu, odv = _oracle_flow(oracle, a, b, tops, lefts, pu[0], pv[0], 32)
    assert odu.tobytes() == du[0].tobytes() and odv.tobytes() == dv[0].tobytes()
    assert ou.tobytes() == tu[0].tobytes() and ov.tobytes() == tv[0].tobytes()

    # FP64 twin of the flow stage on the GPU's PIV tiles
    _, _, wdu, wdv = _oracle_flow(oracle, a, b, tops, lefts, pu[0], pv[0], 64)
    rms, mx = _rms(du[0], dv[0], wdu, wdv)
    assert rms <= RMS_TOL, (rms, mx)

    # end to end: FP64 PIV pass, then the FP64 flow stage
    fu, fv = oracle.piv_adaptive(a, b, 32, 32, 0.5, precision=64, warp=False)
    _, _, edu, edv = _oracle_flow(oracle, a, b, tops, lefts, fu, fv, 64)
    rms_e2e, mx_e2e = _rms(du[0], dv[0], edu, edv)
    assert rms_e2e <= RMS_TOL, (rms_e2e, mx_e2e)
    # the field is the vortex, not a degenerate one
    assert np.abs(du[0]).max() > 2.0 and np.abs(dv[0]).max() > 2.0
