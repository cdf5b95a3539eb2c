"""Host-side checks that need no GPU: the C-ABI library builds, loads and exports every
symbol of include/qlpiv.h; host mirrors (IA grids, Job shape checks, synthetic data)
behave like the reference."""
import re

import numpy as np
import pytest

from conftest import ROOT, load_package


@pytest.fixture(scope="module")
def qp():
    pkg = load_package()
    pkg.build.build()
    return pkg


def header_symbols():
    text = (ROOT / "include" / "qlpiv.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(qlpiv_[a-z_0-9]+)\s*\(", text, re.M)))


def test_library_exports_header_symbols(qp):
    import ctypes
    lib = ctypes.CDLL(str(qp.LIB_PATH))
    syms = header_symbols()
    assert len(syms) >= 10
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(qp.exported_symbols()) == syms
    assert qp.load_library().qlpiv_abi_version() == 5


def test_ctypes_structs_match_header(qp, tmp_path):
    """Every ctypes / numpy mirror has the size and field offsets the C compiler gives the
    header's structs."""
    import ctypes
    import subprocess
    mirrors = {"qlpiv_pass_desc": qp.PassDesc, "qlpiv_frame": qp.Frame, "qlpiv_grid": qp.Grid,
               "qlpiv_adaptive_desc": qp.AdaptiveDesc, "qlpiv_flow_desc": qp.FlowDesc,
               "qlpiv_stage_time": qp.StageTime, "qlpiv_params": qp.Params,
               "qlpiv_server_params": qp.ServerParams, "qlpiv_request": qp.Request, "qlpiv_result": qp.Result,
               "qlpiv_server_stats": qp.ServerStats, "qlpiv_mat_export_params": qp.MatExportParams,
               "qlpiv_mat_velocity_map": qp.MatVelocityMap}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "qlpiv.h"', "int main(void) {"]
    for name, cls in mirrors.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines.append('printf("qlpiv_vector %zu\\n", sizeof(qlpiv_vector));')
    for f in qp.VECTOR_DTYPE.names:
        lines.append(f'printf("qlpiv_vector.{f} %zu\\n", offsetof(qlpiv_vector, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                        text=True).stdout.splitlines())
    for name, cls in mirrors.items():
        assert int(got[name]) == ctypes.sizeof(cls), name
        for f, _ in cls._fields_:
            assert int(got[f"{name}.{f}"]) == getattr(cls, f).offset, (name, f)
    assert int(got["qlpiv_vector"]) == qp.VECTOR_DTYPE.itemsize
    for f in qp.VECTOR_DTYPE.names:
        assert int(got[f"qlpiv_vector.{f}"]) == qp.VECTOR_DTYPE.fields[f][1], f


def test_create_without_gpu_reports_no_device(qp):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(qp.QlpivError) as ei:
        qp.Handle(0)
    assert ei.value.status in (qp.E_NO_DEVICE, qp.E_CUDA)


@pytest.mark.parametrize("h,w,n,levels,ofac,margins", [
    (512, 512, 32, 1, 0.5, (0, 0, 0, 0)),
    (1024, 1024, 64, 3, 0.25, (0, 0, 0, 0)),
    (139, 139, 64, 2, 1.0 / 3.0, (16, 16, 16, 16)),
    (600, 800, 128, 4, 0.5, (3, 5, 7, 11)),
    (2048, 1536, 16, 1, 0.75, (0, 0, 0, 0)),
])
def test_grid_mirror_matches_oracle(qp, oracle, h, w, n, levels, ofac, margins):
    for lv in range(levels):
        g = qp.grid.superposition(h, w, n, lv, ofac, margins)
        o, tops, lefts = oracle.grid(h, w, n, lv, ofac, margins)
        assert (g.n, g.tiles_i, g.tiles_j, g.margin_top, g.margin_bottom, g.margin_left, g.margin_right) == (
            o["n"], o["tiles_i"], o["tiles_j"], o["margin_top"], o["margin_bottom"], o["margin_left"],
            o["margin_right"])
        assert (g.tops == tops).all() and (g.lefts == lefts).all()
        g2 = qp.grid.nosuperposition(h, w, n, lv, margins)
        o2, t2, l2 = oracle.grid(h, w, n, lv, margins=margins, superposition=False)
        assert (g2.tiles_i, g2.tiles_j, g2.margin_top, g2.margin_left) == (o2["tiles_i"], o2["tiles_j"],
                                                                           o2["margin_top"], o2["margin_left"])
        assert (g2.tops == t2).all() and (g2.lefts == l2).all()


def test_grid_rejects_bad_overlap_and_levels(qp):
    with pytest.raises(ValueError):
        qp.grid.superposition(512, 512, 32, 0, 0.95)
    assert qp.grid.adaptive_levels(64, 16) == 3
    with pytest.raises(ValueError):
        qp.grid.adaptive_levels(48, 16)


def test_job_analyze_shape_errors(qp):
    J = qp.jobs
    job = J.CrossCorrelationGpuJob()
    t32 = J.Tile(np.zeros((32, 32), np.uint8))
    job.setInputParameters(J.JobResultEnum.JOB_RESULT_CLIPPED_TILES_A, [t32, J.Tile(np.zeros((16, 32), np.uint8))])
    job.setInputParameters(J.JobResultEnum.JOB_RESULT_CLIPPED_TILES_B, [t32, t32])
    with pytest.raises(J.JobAnalyzeException, match="along I"):
        job.analyze()
    job.setInputParameters(J.JobResultEnum.JOB_RESULT_CLIPPED_TILES_A, [J.Tile(np.zeros((32, 16), np.uint8))] * 2)
    job.setInputParameters(J.JobResultEnum.JOB_RESULT_CLIPPED_TILES_B, [J.Tile(np.zeros((32, 16), np.uint8))] * 2)
    with pytest.raises(J.JobAnalyzeException, match="square"):
        job.analyze()
    job.setInputParameters(J.JobResultEnum.JOB_RESULT_CLIPPED_TILES_A, [t32] * 3)
    job.setInputParameters(J.JobResultEnum.JOB_RESULT_CLIPPED_TILES_B, [t32] * 2)
    with pytest.raises(J.JobAnalyzeException, match="number of matrices"):
        job.analyze()
    job.setInputParameters(J.JobResultEnum.JOB_RESULT_CLIPPED_TILES_A, [J.Tile(np.zeros((24, 24), np.uint8))])
    job.setInputParameters(J.JobResultEnum.JOB_RESULT_CLIPPED_TILES_B, [J.Tile(np.zeros((24, 24), np.uint8))])
    with pytest.raises(J.JobAnalyzeException, match="not supported"):
        job.analyze()
    job.setInputParameters(J.JobResultEnum.JOB_RESULT_CLIPPED_TILES_A, [])
    job.analyze()   # empty input: nothing to do, like the reference
    job.dispose()


def test_synthetic_pair_is_seeded(qp):
    a1, b1 = qp.synth.particle_pair((64, 80), qp.synth.Flow(vmax=2.0, rc=10.0), seed=3)
    a2, b2 = qp.synth.particle_pair((64, 80), qp.synth.Flow(vmax=2.0, rc=10.0), seed=3)
    a3, _ = qp.synth.particle_pair((64, 80), qp.synth.Flow(vmax=2.0, rc=10.0), seed=4)
    assert a1.dtype == np.uint8 and (a1 == a2).all() and (b1 == b2).all() and not (a1 == a3).all()
    a, b = qp.synth.particle_pair((64, 64), qp.synth.Flow(), bits=12, seed=1)
    assert a.dtype == np.uint16 and a.max() < 4096 and a.max() > 255
    f = qp.synth.Flow(vmax=4.0, rc=64.0)
    rows, cols = np.meshgrid(np.arange(512.0), np.arange(512.0), indexing="ij")
    dr, dc = f.displacement(rows, cols, (512, 512))
    assert abs(np.hypot(dr, dc).max() - 4.0) < 0.05


def test_oracle_recovers_synthetic_flow(qp, oracle):
    """Sanity of the generator + oracle: 32 px IAs recover the vortex within 0.2 px."""
    a, b = qp.synth.config1_pair(seed=1)
    g = qp.grid.superposition(512, 512, 32, 0, 0.5)
    at, al = g.origins()
    vec = oracle.piv_pass(a, b, 32, at, al)
    cy = at + 15.5
    cx = al + 15.5
    dr, dc = qp.synth.Flow(vmax=4.0, rc=64.0).displacement(cy, cx, (512, 512))
    err = np.hypot(vec["u"] - dr, vec["v"] - dc)
    assert np.median(err) < 0.2


@pytest.mark.parametrize("h,w,n,levels,ofac,margins", [
    (512, 512, 32, 1, 0.5, (0, 0, 0, 0)),
    (1024, 1024, 64, 3, 0.25, (0, 0, 0, 0)),
    (139, 139, 64, 2, 1.0 / 3.0, (16, 16, 16, 16)),
    (600, 800, 128, 4, 0.5, (3, 5, 7, 11)),
    (777, 333, 32, 2, 0.3, (1, 2, 3, 4)),
])
def test_library_grid_matches_oracle(qp, oracle, h, w, n, levels, ofac, margins):
    """The C++ grid of libqlpiv_gpu.so (used by the device pipeline) is the reference's
    geometry; checked on the host without a GPU."""
    for lv in range(levels):
        g, tops, lefts = qp.library_grid(h, w, n, lv, ofac, margins)
        o, ot, ol = oracle.grid(h, w, n, lv, ofac, margins)
        assert g == o and (tops == ot).all() and (lefts == ol).all()
        g2, t2, l2 = qp.library_grid(h, w, n, lv, ofac, margins, superposition=False)
        o2, ot2, ol2 = oracle.grid(h, w, n, lv, margins=margins, superposition=False)
        assert g2 == o2 and (t2 == ot2).all() and (l2 == ol2).all()


@pytest.mark.parametrize("h,w,n,levels,ofac,margins", [
    (1024, 1024, 64, 3, 0.25, (0, 0, 0, 0)),
    (600, 800, 128, 4, 0.5, (3, 5, 7, 11)),
    (777, 333, 32, 2, 0.3, (1, 2, 3, 4)),
])
def test_mixed_division_grids(qp, oracle, h, w, n, levels, ofac, margins):
    """AdaptiveInterAreaStrategyMixedSuperPosition: NoSuperPosition levels before the start
    level, then SuperPosition restarted with IA n >> start.  Library, Python restatement and
    oracle agree level by level; start 0 is SuperPosition and start >= levels NoSuperPosition."""
    for start in range(levels + 1):
        for lv in range(levels):
            g, tops, lefts = qp.library_grid(h, w, n, lv, ofac, margins, superposition_start=start)
            o, ot, ol = oracle.level_grid(h, w, n, lv, ofac, margins, superposition_start=start)
            st = qp.grid.level(h, w, n, lv, ofac, margins, superposition_start=start)
            assert g == o and (tops == ot).all() and (lefts == ol).all()
            assert (np.asarray(st.tops) == tops).all() and (np.asarray(st.lefts) == lefts).all()
            assert g["n"] == n >> lv
            ref = qp.library_grid(h, w, n, lv, ofac, margins, superposition=lv >= start)
            if start in (0, levels):
                assert g == ref[0] and (tops == ref[1]).all()
        d = qp.adaptive_desc(n, n >> (levels - 1), ofac, margins=margins, superposition_start=start)
        got = qp.adaptive_levels(d, h, w)
        assert [x["tiles_i"] * x["tiles_j"] for x in got] == [
            qp.library_grid(h, w, n, lv, ofac, margins, superposition_start=start)[0]["tiles_i"] *
            qp.library_grid(h, w, n, lv, ofac, margins, superposition_start=start)[0]["tiles_j"]
            for lv in range(levels)]
    with pytest.raises(qp.QlpivError):
        qp.library_grid(h, w, n, 0, ofac, margins, superposition_start=-1)


def test_adaptive_levels_config2(qp):
    d = qp.adaptive_desc(64, 16, 0.25)
    lv = qp.adaptive_levels(d, 1024, 1024)
    assert [(g["n"], g["tiles_i"], g["tiles_j"]) for g in lv] == [(64, 61, 61), (32, 125, 125), (16, 253, 253)]
    with pytest.raises(qp.QlpivError):
        qp.adaptive_levels(qp.adaptive_desc(64, 24, 0.25), 1024, 1024)
    lv = qp.adaptive_levels(qp.adaptive_desc(128, 16, 0.25), 1024, 1024)
    assert [g["n"] for g in lv] == [128, 64, 32, 16]
    with pytest.raises(qp.QlpivError):
        qp.adaptive_levels(qp.adaptive_desc(256, 16, 0.25), 1024, 1024)   # IA 256: no kernel


def test_adaptive_plan_bytes_properties(qp):
    """The request server's admission estimate: grows with the frame size and the pair count,
    and by the warped frames and the validation buffers when those are configured."""
    d = qp.adaptive_desc(64, 16, 0.25, warp_mode=qp.WARP_NONE)
    b1 = qp.adaptive_plan_bytes(d, qp.PIX_U8, 512, 512)
    b2 = qp.adaptive_plan_bytes(d, qp.PIX_U8, 512, 512, pairs=2)
    assert 2 * 512 * 512 < b1 < b2 <= 2 * b1
    assert qp.adaptive_plan_bytes(d, qp.PIX_U16, 512, 512) - b1 >= 2 * 512 * 512   # 2 bytes per pixel
    assert qp.adaptive_plan_bytes(d, qp.PIX_U8, 1024, 1024) > 3 * b1
    dw = qp.adaptive_desc(64, 16, 0.25, warp_mode=qp.WARP_BOTH_BILINEAR)
    assert qp.adaptive_plan_bytes(dw, qp.PIX_U8, 512, 512) - b1 >= 2 * 512 * 512   # warped copies
    dv = qp.adaptive_desc(64, 16, 0.25, warp_mode=qp.WARP_NONE, validation=qp.multipeak_validation(num_peaks=3))
    assert qp.adaptive_plan_bytes(dv, qp.PIX_U8, 512, 512) > b1 + 3 * 8 * 253 * 253 // 4
    with pytest.raises(qp.QlpivError):
        qp.adaptive_plan_bytes(d, qp.PIX_F32, 512, 512)
    with pytest.raises(qp.QlpivError):
        qp.adaptive_plan_bytes(d, qp.PIX_U8, 40, 40)


def test_server_without_gpu_reports_no_device(qp):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(qp.QlpivError) as e:
        qp.Server(0)
    assert e.value.status == qp.E_NO_DEVICE


@pytest.mark.parametrize("bad", [-1, 2])
def test_batch_pass_rejects_frame_index_outside_table(qp, bad):
    """qlpiv_pass_batch checks every IA's frame index against the frame table before it touches
    the handle or the device (a bad index would otherwise make the kernel read past the
    table).  The handle here is an opaque placeholder: the call returns before using it."""
    import ctypes
    lib = qp.load_library()
    a = np.zeros((64, 64), np.uint8)
    table = (qp.Frame * 2)(qp.Frame(a.ctypes.data, a.ctypes.data, 64, 64, 64),
                           qp.Frame(a.ctypes.data, a.ctypes.data, 64, 64, 64))
    fi = np.array([0, 1, bad, 0], np.int32)
    org = np.zeros(4, np.int32)
    out = np.empty(4, qp.VECTOR_DTYPE)
    placeholder = ctypes.create_string_buffer(64)
    d = qp.Handle.desc(32)
    st = lib.qlpiv_pass_batch(ctypes.cast(placeholder, ctypes.c_void_p), ctypes.byref(d), qp.PIX_U8, 2, table, 4,
                              fi.ctypes.data, org.ctypes.data, org.ctypes.data, org.ctypes.data, org.ctypes.data,
                              out.ctypes.data)
    assert st == 1   # QLPIV_E_ARG
    assert b"frame_of_ia[2]" in lib.qlpiv_last_error()


def test_inherit_noalloc_checks_tensors_before_the_call(qp):
    """The Python wrapper of the allocation-free inheritance refuses host tensors and
    mis-sized or non-float32 tensors before anything reaches the library."""
    torch = pytest.importorskip("torch")
    t = torch.zeros(16, dtype=torch.float32)
    with pytest.raises(ValueError, match="CUDA tensor"):
        qp.inherit_noalloc(0, 0, t, t, t, t, t, t, t, t, 4, 4, 4, 4)


def _xpad(m, layout, pas, e):
    """Exchange-buffer index of qlpiv_fft.cuh's xpad<M, L, PASS>."""
    if layout == 1 and m >= 128:
        return e + (e >> 4) if pas == 0 else e + 4 * (e >> 5)
    return e + (e >> 3)


def _wavefronts8(addrs):
    """Shared-memory wavefronts of one warp's 8-byte accesses (complex indices; 16-lane halves)."""
    total = 0
    for half in (addrs[:16], addrs[16:]):
        banks = {}
        for a in half:
            for w in (2 * a, 2 * a + 1):
                banks.setdefault(w % 32, set()).add(w)
        total += max(len(v) for v in banks.values())
    return total


@pytest.mark.parametrize("m,g,pitch", [(128, 16, 140), (64, 8, 72), (256, 32, 289)])
def test_fft_exchange_layouts_conflict_free(m, g, pitch):
    """The K1 exchange layouts (layout 1, the group buffers `pitch` complex apart) give every
    8-byte store and load of the radix-8 Stockham passes one wavefront per half-warp."""
    passes = {64: [(8, 1)], 128: [(8, 1), (8, 8)], 256: [(8, 1), (8, 8)]}[m]
    for pas, (r, p) in enumerate(passes):
        for t in range(r):   # stores: lane g writes output t of its butterfly i = g
            addrs = []
            for lane in range(32):
                gg = lane % g
                k = gg & (p - 1)
                addrs.append((lane // g) * pitch + _xpad(m, 1, pas, (gg - k) * r + k + t * p))
            assert _wavefronts8(addrs) == 2, (m, pas, t)
        for mm in range(8):  # loads of the stride-G layout
            addrs = [(lane // g) * pitch + _xpad(m, 1, pas, lane % g + g * mm) for lane in range(32)]
            assert _wavefronts8(addrs) == 2, (m, pas, mm)
