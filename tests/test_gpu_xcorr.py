"""Parity of the CUDA FFT-PIV kernel (through the C ABI) with the CPU oracle.

Tolerances (see tests/parity.py): correlation planes within 1e-5 of the plane maximum
against the FP64 oracle; integer peaks identical to the FP64 oracle except exact ties;
sub-pixel displacement within 1e-3 px of the FP64 oracle.
"""
import numpy as np
import pytest

import parity
from conftest import GOLDEN, load_package

pytestmark = pytest.mark.gpu

PLANE_REL = 1e-5


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


def _random_tiles(rng, count, n, dtype):
    if dtype == np.uint8:
        return (rng.integers(0, 256, (count, n, n)).astype(np.uint8),
                rng.integers(0, 256, (count, n, n)).astype(np.uint8))
    if dtype == np.uint16:
        return (rng.integers(0, 4096, (count, n, n)).astype(np.uint16),
                rng.integers(0, 4096, (count, n, n)).astype(np.uint16))
    return (rng.uniform(0, 200, (count, n, n)).astype(np.float32),
            rng.uniform(0, 200, (count, n, n)).astype(np.float32))


@pytest.mark.parametrize("n", [16, 32, 64, 128])
@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.float32])
@pytest.mark.parametrize("norm", ["max_a", "own"])
def test_planes_match_fp64(qp, handle, oracle, n, dtype, norm):
    rng = np.random.default_rng(n * 7 + np.dtype(dtype).itemsize)
    count = 11
    ta, tb = _random_tiles(rng, count, n, dtype)
    mode = qp.NORM_MAX_A if norm == "max_a" else qp.NORM_OWN_MAX
    if dtype == np.float32:
        ma = ta.reshape(count, -1).max(1).astype(np.float32)
        mb = tb.reshape(count, -1).max(1).astype(np.float32)
        planes = handle.xcorr_planes(ta, tb, ma, mb, norm_mode=mode)
    else:
        ma = np.maximum(ta.reshape(count, -1).max(1), 16).astype(np.float32)
        mb = np.maximum(tb.reshape(count, -1).max(1), 16).astype(np.float32)
        planes = handle.xcorr_planes(ta, tb, norm_mode=mode)   # maxima computed on the GPU
    assert planes.shape == (count, 2 * n - 1, 2 * n - 1)
    for k in range(count):
        mbk = ma[k] if mode == qp.NORM_MAX_A else mb[k]
        ref = oracle.xcorr_fft(ta[k].astype(np.float32), tb[k].astype(np.float32), ma[k], mbk, precision=64)
        err = np.abs(planes[k] - ref).max() / np.abs(ref).max()
        assert err < PLANE_REL, (k, err)


def test_planes_raw_values(qp, handle, oracle):
    rng = np.random.default_rng(3)
    ta, tb = _random_tiles(rng, 4, 32, np.float32)
    planes = handle.xcorr_planes(ta, tb, norm_mode=qp.NORM_NONE)
    for k in range(4):
        ref = oracle.xcorr_direct(ta[k], tb[k], 1.0, 1.0, normalize=False)
        assert np.abs(planes[k] - ref).max() / np.abs(ref).max() < PLANE_REL


def test_gpu_fft_benchmark_golden(qp, handle, oracle, rankine_pair):
    """GpuFFTBenchmarkJob validation data: 16x16 IAs, own-max tiles, 1e-2 absolute."""
    a, b = rankine_pair
    g = np.load(GOLDEN / "gpu_fft_golden.npz")
    ta, tb = [], []
    for idx in g["index"]:
        ti, tj = divmod(int(idx), 32)
        ta.append(a[ti * 16:ti * 16 + 16, tj * 16:tj * 16 + 16])
        tb.append(b[ti * 16:ti * 16 + 16, tj * 16:tj * 16 + 16])
    planes = handle.xcorr_planes(np.stack(ta), np.stack(tb), norm_mode=qp.NORM_OWN_MAX)
    assert np.abs(planes - g["planes"]).max() <= 1e-2


@pytest.mark.parametrize("top,left,di,dj", [("320-n", "320-n", -10, -10), ("320", "320-n", 10, -10),
                                            ("320-n", "320", -10, 10), ("320", "320", 10, 10)])
def test_shift_kat(qp, handle, top, left, di, dj):
    d = np.load(GOLDEN / "shift_kat.npz")
    n = 64
    t0, l0 = eval(top, {"n": n}), eval(left, {"n": n})
    vec = handle.piv_pass(d["img1"], d["img2"], n, [t0], [l0], norm_mode=qp.NORM_OWN_MAX)
    dd = 2 * n - 1
    assert (int(vec["peak_i"][0]), int(vec["peak_j"][0])) == (dd // 2 + di, dd // 2 + dj)


def _pass_and_check(qp, handle, oracle, img_a, img_b, n, at, al, bt, bl, norm_mode, max_mode=0,
                    fixed=(255.0, 255.0)):
    qnorm = {oracle.NORM_MAX_A: qp.NORM_MAX_A, oracle.NORM_OWN_MAX: qp.NORM_OWN_MAX,
             oracle.NORM_FIXED: qp.NORM_OWN_MAX}[norm_mode]
    gpu = handle.piv_pass(img_a, img_b, n, at, al, bt, bl, norm_mode=qnorm, max_mode=max_mode, fixed_max=fixed)
    ref64 = oracle.piv_pass(img_a, img_b, n, at, al, bt, bl, norm_mode=norm_mode, fixed_max=fixed, precision=64)
    ref32 = oracle.piv_pass(img_a, img_b, n, at, al, bt, bl, norm_mode=norm_mode, fixed_max=fixed, precision=32)
    stats = parity.compare_vectors(oracle, gpu, ref64, img_a, img_b, n, at, al, bt, bl, norm_mode, fixed)
    # the reference's own FP32 path meets the same bar (sanity of the criterion)
    parity.compare_vectors(oracle, ref32, ref64, img_a, img_b, n, at, al, bt, bl, norm_mode, fixed)
    return gpu, ref32, stats


def test_rankine_reference_pair_parity(qp, handle, oracle, rankine_pair):
    """The reference's bundled 512x512 Rankine pair, 32x32 IAs at 50 % overlap (961 vectors)."""
    a, b = rankine_pair
    g = qp.grid.superposition(512, 512, 32, 0, 0.5)
    at, al = g.origins()
    assert len(at) == 961
    gpu, ref32, st = _pass_and_check(qp, handle, oracle, a, b, 32, at, al, at, al, oracle.NORM_MAX_A)
    same = (gpu["peak_i"] == ref32["peak_i"]) & (gpu["peak_j"] == ref32["peak_j"])
    assert same.mean() > 0.99, st


@pytest.mark.parametrize("n", [16, 32, 64, 128])
def test_synthetic_config1_parity(qp, handle, oracle, n):
    a, b = qp.synth.config1_pair(seed=11)
    g = qp.grid.superposition(512, 512, n, 0, 0.5)
    at, al = g.origins()
    _pass_and_check(qp, handle, oracle, a, b, n, at, al, at, al, oracle.NORM_MAX_A)


@pytest.mark.parametrize("n", [16, 32])
def test_synthetic_u16_own_and_fixed_max(qp, handle, oracle, n):
    a, b = qp.synth.particle_pair((256, 320), qp.synth.Flow(vmax=3.0, rc=40.0, shear=0.004), ppp=0.03, diam=2.5,
                                  diam_sd=0.0, bits=12, seed=5)
    g = qp.grid.superposition(256, 320, n, 0, 0.25)
    at, al = g.origins()
    _pass_and_check(qp, handle, oracle, a, b, n, at, al, at, al, oracle.NORM_OWN_MAX)
    _pass_and_check(qp, handle, oracle, a, b, n, at, al, at, al, oracle.NORM_FIXED, max_mode=qp.MAX_FIXED,
                    fixed=(65535.0, 65535.0))


def test_partial_clipping_parity(qp, handle, oracle):
    """B tiles displaced partly (or wholly) outside the image are zero-filled
    (Image.clipImageMatrix, partial clipping)."""
    a, b = qp.synth.config1_pair(seed=3)
    n = 32
    rng = np.random.default_rng(9)
    count = 300
    at = rng.integers(0, 512 - n, count).astype(np.int32)
    al = rng.integers(0, 512 - n, count).astype(np.int32)
    bt = (at + rng.integers(-n, n, count)).astype(np.int32)
    bl = (al + rng.integers(-n, n, count)).astype(np.int32)
    bt[:8] = [-40, 520, -5, 500, 0, -31, 511, 200]
    bl[:8] = [0, 3, -40, 600, -31, 511, 480, -32]
    _pass_and_check(qp, handle, oracle, a, b, n, at, al, bt, bl, oracle.NORM_MAX_A)


def test_empty_and_errors(qp, handle):
    a = np.zeros((64, 64), np.uint8)
    out = handle.piv_pass(a, a, 32, np.zeros(0, np.int32), np.zeros(0, np.int32))
    assert out.shape == (0,)
    with pytest.raises(qp.QlpivError) as ei:
        handle.piv_pass(a, a, 24, [0], [0])
    assert ei.value.status == qp.E_SHAPE
    with pytest.raises(qp.QlpivError) as ei:
        handle.xcorr_planes(np.zeros((2, 256, 256), np.uint8), np.zeros((2, 256, 256), np.uint8))
    assert ei.value.status == qp.E_SHAPE
    with pytest.raises(qp.QlpivError) as ei:   # IA 128 multi-peak: cell width 1 is invalid
        handle.piv_pass(np.zeros((256, 256), np.uint8), np.zeros((256, 256), np.uint8), 128, [0], [0], num_peaks=2,
                        peak_kernel=1)
    assert ei.value.status == qp.E_ARG
    with pytest.raises(ValueError):
        handle.piv_pass(a, a.astype(np.uint16), 32, [0], [0])


def test_ia128_shift_and_clipping(qp, handle, oracle):
    """IA 128 (two-CTA cluster kernel): known shifts, partly clipped B tiles, u8 and 12-bit,
    against the FP64 oracle; repeated runs are bit-identical."""
    rng = np.random.default_rng(128)
    for bits in (8, 12):
        a, b = qp.synth.particle_pair((400, 448), qp.synth.Flow(vmax=6.0, rc=90.0, shear=0.01), ppp=0.02, diam=2.6,
                                      diam_sd=0.3, bits=bits, seed=bits)
        count = 40
        at = rng.integers(0, 400 - 128, count).astype(np.int32)
        al = rng.integers(0, 448 - 128, count).astype(np.int32)
        bt = (at + rng.integers(-20, 21, count)).astype(np.int32)
        bl = (al + rng.integers(-20, 21, count)).astype(np.int32)
        bt[:3] = [-30, 300, 5]
        bl[:3] = [0, 330, -40]
        _pass_and_check(qp, handle, oracle, a, b, 128, at, al, bt, bl, oracle.NORM_MAX_A)
        r1 = handle.piv_pass(a, b, 128, at, al, bt, bl)
        r2 = handle.piv_pass(a, b, 128, at, al, bt, bl)
        assert r1.tobytes() == r2.tobytes()


def test_flat_tiles_and_determinism(qp, handle, oracle):
    # constant tiles: the plane is the pedestal tent; the peak is the zero shift
    n = 32
    t = np.full((3, n, n), 7, np.uint8)
    v1 = handle.xcorr_peaks(t, t)
    assert (v1["peak_i"] == n - 1).all() and (v1["peak_j"] == n - 1).all()
    a, b = qp.synth.config1_pair(seed=4)
    g = qp.grid.superposition(512, 512, 32, 0, 0.5)
    at, al = g.origins()
    r1 = handle.piv_pass(a, b, 32, at, al)
    r2 = handle.piv_pass(a, b, 32, at, al)
    assert r1.tobytes() == r2.tobytes()


def test_job_api(qp, handle, oracle, rankine_pair):
    a, b = rankine_pair
    tiles_a = [qp.jobs.Tile(a[i:i + 32, j:j + 32]) for i in range(0, 128, 32) for j in range(0, 128, 32)]
    tiles_b = [qp.jobs.Tile(b[i:i + 32, j:j + 32]) for i in range(0, 128, 32) for j in range(0, 128, 32)]
    job = qp.jobs.CrossCorrelationGpuJob(normalization="cpu", handle=handle)
    job.setInputParameters(qp.jobs.JobResultEnum.JOB_RESULT_CLIPPED_TILES_A, tiles_a)
    job.setInputParameters(qp.jobs.JobResultEnum.JOB_RESULT_CLIPPED_TILES_B, tiles_b)
    job.analyze()
    job.compute()
    res = job.getJobResult(qp.jobs.JobResultEnum.JOB_RESULT_CROSS_MATRICES)
    assert res.getNumberOfMatrices() == 16 and res.getDimI() == 63
    ta, ma = oracle.clip_tile(a, 32, 64, 32)
    tb, _ = oracle.clip_tile(b, 32, 64, 32)
    ref = oracle.xcorr_fft(ta, tb, ma, ma, precision=64)
    assert np.abs(res.getCrossMatrices()[6] - ref).max() / ref.max() < PLANE_REL
    stage = qp.jobs.GpuPivStageJob(normalization="cpu", handle=handle)
    stage.setInputParameters(qp.jobs.JobResultEnum.JOB_RESULT_CLIPPED_TILES_A, tiles_a)
    stage.setInputParameters(qp.jobs.JobResultEnum.JOB_RESULT_CLIPPED_TILES_B, tiles_b)
    stage.analyze()
    stage.compute()
    peaks = stage.getJobResult(qp.jobs.JobResultEnum.JOB_RESULT_CROSS_MAXIMUM)
    i, j, _, _ = oracle.find_max_from_center(ref)
    assert (peaks[6].peak_i, peaks[6].peak_j) == (i, j)


def test_device_resident_pass(qp, handle):
    torch = pytest.importorskip("torch")
    a, b = qp.synth.config1_pair(seed=8)
    g = qp.grid.superposition(512, 512, 32, 0, 0.5)
    at, al = g.origins()
    host = handle.piv_pass(a, b, 32, at, al)
    dev = torch.device("cuda:0")
    ta = torch.from_numpy(a).to(dev)
    tb = torch.from_numpy(b).to(dev)
    o = [torch.from_numpy(x).to(dev) for x in (at, al)]
    out = torch.empty(len(at) * 32, dtype=torch.uint8, device=dev)
    handle.piv_pass_device(ta, tb, 512, 512, qp.PIX_U8, 32, len(at), o[0], o[1], o[0], o[1], out)
    handle.synchronize()
    res = np.frombuffer(out.cpu().numpy().tobytes(), qp.VECTOR_DTYPE)
    assert res.tobytes() == host.tobytes()


def test_batched_frames_equal_single_passes(qp, handle):
    """A flattened work list over pairs of different sizes gives, IA by IA, exactly the
    vectors of the per-pair calls (deterministic per-IA computation)."""
    shapes = [(256, 256), (300, 200), (128, 512)]
    pairs = [qp.synth.particle_pair(s, qp.synth.Flow(vmax=3.0, rc=30.0), seed=20 + k) for k, s in enumerate(shapes)]
    fi, at, al, singles = [], [], [], []
    for k, (a, b) in enumerate(pairs):
        g = qp.grid.superposition(a.shape[0], a.shape[1], 32, 0, 0.5)
        t, l = g.origins()
        fi.append(np.full(len(t), k, np.int32))
        at.append(t)
        al.append(l)
        singles.append(handle.piv_pass(a, b, 32, t, l))
    fi, at, al = np.concatenate(fi), np.concatenate(at), np.concatenate(al)
    batch = handle.piv_pass_batch([p[0] for p in pairs], [p[1] for p in pairs], 32, fi, at, al)
    assert batch.tobytes() == np.concatenate(singles).tobytes()
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    keep = [(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)) for a, b in pairs]
    table = np.zeros(len(pairs), qp.FRAME_DTYPE)
    for k, (ta, tb) in enumerate(keep):
        table[k] = (ta.data_ptr(), tb.data_ptr(), ta.shape[0], ta.shape[1], ta.shape[1])
    ttab = torch.from_numpy(table.view(np.uint8)).to(dev)
    wl = [torch.from_numpy(x).to(dev) for x in (fi, at, al)]
    out = torch.empty(len(at) * 32, dtype=torch.uint8, device=dev)
    handle.piv_pass_batch_device(qp.PIX_U8, len(pairs), ttab, 32, len(at), wl[0], wl[1], wl[2], wl[1], wl[2], out)
    handle.synchronize()
    assert out.cpu().numpy().tobytes() == batch.tobytes()


def test_fit_logarithm_error_bound(qp):
    """The 3-point fit's float-pair logarithm stays within 1e-11 of CUDA's double log over the
    range of fit samples (plane values + 1e-8) and around every table and binade boundary."""
    rng = np.random.default_rng(17)
    x = np.exp(rng.uniform(np.log(1e-8), np.log(1e7), 200000)).astype(np.float32)
    k = np.arange(65, dtype=np.float64)
    edges = np.concatenate([(1.0 + (k + 0.5) / 64.0) * s for s in (1.0, 2.0 ** -20, 2.0 ** 10)])
    x = np.concatenate([x, edges.astype(np.float32), np.nextafter(edges.astype(np.float32), np.float32(0)),
                        np.float32([1e-8, 1.0, 2.0, 0.5, 16.0, 17.0, 255.0, 4095.0, 65535.0])])
    mine, ref = qp.probe_log(x)
    err = np.abs(mine - ref)
    assert err.max() < 1e-11, (float(err.max()), float(x[err.argmax()]))
