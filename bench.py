#!/usr/bin/env python3
"""FFT-PIV throughput benchmark (one JSON line on rank 0).

Workload ("adaptive-1024-u12"): 1024x1024 12-bit-in-uint16 synthetic particle pairs
(0.03 ppp, d = 2.5 px, shear 0.005 + Rankine vortex, max 6 px), adaptive PIV with
IA 64 -> 32 -> 16 at 75 % overlap (61^2 + 125^2 + 253^2 = 83,355 vectors per pair):
velocity inheritance, bicubic displacement field and BothImages bilinear warp between
passes, FP32, 3-point Gaussian sub-pixel fit of every peak, FindMaximumMultiPeaks (3 peaks,
3x3 cells) and the multi-peak normalised-median validation (threshold 2, epsilon0 0.1,
secondary-peak then bilinear replacement, at most 2 correction sweeps) after every level.
A step processes a batch of `pairs` pairs resident in HBM (inputs larger than L2)
through the whole level loop.

  value      frame-pairs/s with inputs resident in HBM (CUDA events on the library's
             stream, max over ranks);
  e2e        frame-pairs/s through the public host API (qlpiv_piv_adaptive): pinned host
             images copied to the device and the displacements copied back inside the
             timed region;
  roofline   dominant kernel (the stage with the largest device time, from CUDA events
             around every launch): for the correlation, algorithmic bytes
             2*N^2*bytes_per_px + 16 per IA against the measured HBM copy bandwidth, and
             (compute_roofline) formula flops 10*M^2*log2(M^2) + 8*M^2 (M = 2N) per IA
             against the live FP32 FMA peak;
  cpu_baseline  the oracle's FP32 restatement of the reference CPU path on one pair,
             all host threads.

--impl reference times that CPU restatement alone (the Java reference cannot run on
these machines).  Multi-GPU: independent replicas (no collective), weak scaling.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
LEVELS = (64, 32, 16)
OVERLAP_FACTOR = 0.25     # 75 % overlap
H = W = 1024


def load_pkg():
    import importlib.util
    name = "quicklabpiv_ng_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = ROOT / "quicklabpiv-ng_gb300"
    spec = importlib.util.spec_from_file_location(name, pkg_dir / "__init__.py",
                                                  submodule_search_locations=[str(pkg_dir)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def load_oracle():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    return oracle


def flops_per_ia(n):
    m = 2 * n
    return 10.0 * m * m * np.log2(m * m) + 8.0 * m * m


def bytes_per_ia(n, bpp):
    return 2.0 * n * n * bpp + 16.0


def level_grids(pkg):
    return [pkg.grid.superposition(H, W, LEVELS[0], lv, OVERLAP_FACTOR) for lv in range(len(LEVELS))]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 5 + k and r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_pairs(pkg, unique):
    return [pkg.synth.config2_pair(seed=2, pair_id=k) for k in range(unique)]


FULL_SCALE = 65535.0   # tiles copied from warped 16-bit images keep the full-scale max
# VelocityValidationOptionsMultiPeakNormalizedMedianModel settings of the workload
VALIDATION = dict(num_peaks=3, peak_kernel=3, threshold=2.0, epsilon0=0.1, max_iterations=2, iterate_until=False)


def oracle_validation(orc):
    v = VALIDATION
    return orc.valid_cfg(num_peaks=v["num_peaks"], kernel_width=v["peak_kernel"], threshold=v["threshold"],
                         epsilon0=v["epsilon0"], max_iterations=v["max_iterations"],
                         iterate_until_no_corrections=v["iterate_until"])


def c2_accuracy(pairs_host, u_host, v_host):
    """Last-level displacements of the timed workload against the FP64 oracle pipeline, per
    distinct pair: max and 99th-percentile |error| and the fraction within 1e-3 px."""
    orc = load_oracle()
    errs = []
    for k, (a, b) in enumerate(pairs_host):
        ou, ov = orc.piv_adaptive(a, b, LEVELS[0], LEVELS[-1], OVERLAP_FACTOR, norm_mode=orc.NORM_MAX_A,
                                  fixed_max=FULL_SCALE, precision=64, validation=oracle_validation(orc))
        errs.append(np.maximum(np.abs(u_host[k] - ou), np.abs(v_host[k] - ov)).ravel())
    e = np.concatenate(errs)
    return {"reference": "FP64 oracle pipeline (same algorithm in double)", "pairs": len(pairs_host),
            "vectors": int(e.size), "max_px": float(e.max()), "p99_px": float(np.quantile(e, 0.99)),
            "frac_within_1e-3": float(np.mean(e <= 1e-3))}


def cpu_baseline(pkg, pair, threads, reps=5, warmup=1):
    """Oracle FP32 restatement of the reference CPU path on one pair: the same adaptive
    loop (inheritance, bicubic field, bilinear warp, three correlation passes).  `warmup`
    untimed runs, then the median of `reps` timed repetitions (seconds per pair)."""
    orc = load_oracle()
    a, b = pair
    times = []
    for r in range(reps + warmup):
        t0 = time.perf_counter()
        orc.piv_adaptive(a, b, LEVELS[0], LEVELS[-1], OVERLAP_FACTOR, norm_mode=orc.NORM_MAX_A, fixed_max=FULL_SCALE,
                         precision=32, nthreads=threads, validation=oracle_validation(orc))
        if r >= warmup:
            times.append(time.perf_counter() - t0)
    return statistics.median(times)


WORKLOAD = ("adaptive-1024-u12: 1024x1024 12-bit pairs, IA 64 -> 32 -> 16 at 75 % overlap, BothImages bilinear "
            "warp between passes (velocity inheritance + bicubic displacement field), tile A max normalisation, "
            "FindMaximumMultiPeaks (3 peaks, 3x3 cells) + 3-point Gaussian sub-pixel of every peak, multi-peak "
            "normalised-median validation (threshold 2, eps0 0.1, secondary-peak then bilinear replacement, "
            "<= 2 sweeps) after every level")


# Hybrid PIV + dense optical flow (1024x1024 u8, one 32x32 pass at 50 % overlap, then dense
# Lucas-Kanade over a 2-level pyramid (prefilter sigma 2.0, 3 px; window 27; 5 iterations per
# level) and Liu-Shen (lambda 4, prefilter sigma 0.48, 5 px; 60 passes), dense field exported).
HYBRID_PAIRS = 8
HYBRID_WORKLOAD = ("hybrid-1024-u8: 1024x1024 u8 vortex pairs (0.05 ppp, max 3 px), one 32x32 PIV pass at 50 % "
                   "overlap, then dense Lucas-Kanade over a 2-level pyramid (sigma 2.0, window 27, 5 iterations per "
                   "level) and Liu-Shen (lambda 4, "
                   "sigma 0.48, 60 passes), FP32 dense field")


def hybrid_descs(pkg):
    piv = pkg.adaptive_desc(32, 32, 0.5, warp_mode=pkg.WARP_NONE, norm_mode=pkg.NORM_MAX_A, max_mode=pkg.MAX_COMPUTE)
    flow = pkg.flow_desc(mode=pkg.FLOW_LIU_SHEN, filter_sigma_lk=2.0, filter_px_lk=3, window_lk=27, iterations_lk=5,
                         filter_sigma_ls=0.48, filter_px_ls=5, lambda_ls=4.0, iterations_ls=60, dense_export=True,
                         pyramid_levels=2)
    return piv, flow


def hybrid_accuracy(pkg, h, pair, dense_u, dense_v):
    """Dense field of one hybrid pair against the FP64 twin of the flow stage, fed the GPU's own PIV
    tiles (RMS and max over every pixel, px)."""
    orc = load_oracle()
    piv, _ = hybrid_descs(pkg)
    a, b = pair
    pu, pv = h.piv_adaptive([a], [b], piv)
    _, tops, lefts = orc.grid(H, W, 32, 0, 0.5)
    _, _, du64, dv64 = orc.flow_after_piv(a, b, 32, tops, lefts, pu[0], pv[0], mode=2, sigma_lk=2.0, px_lk=3,
                                          sigma_ls=0.48, px_ls=5, window=27, iterations_lk=5, lam=4.0,
                                          iterations_ls=60, dense_export=True, pyramid_levels=2, precision=64)
    eu = dense_u.astype(np.float64) - du64
    ev = dense_v.astype(np.float64) - dv64
    return {"reference": "FP64 twin of the flow stage on the GPU's PIV tiles", "pairs": 1,
            "pixels": int(eu.size), "rms_px": float(np.sqrt(np.mean(eu * eu + ev * ev))),
            "max_px": float(max(np.abs(eu).max(), np.abs(ev).max()))}


def hybrid_cpu_baseline(pkg, pair):
    """The oracle's FP32 hybrid on one pair with all host threads: the 32 x 32 pass (FP32 single
    pass), then the flow stage (prefilters, LK over the 2-level pyramid, Liu-Shen, dense field)."""
    orc = load_oracle()
    threads = os.cpu_count() or 1
    a, b = pair
    _, tops, lefts = orc.grid(H, W, 32, 0, 0.5)
    t0 = time.perf_counter()
    vec = orc.piv_pass(a, b, 32, np.repeat(tops, len(lefts)), np.tile(lefts, len(tops)), precision=32,
                       nthreads=threads)
    tu = vec["u"].reshape(len(tops), len(lefts))
    tv = vec["v"].reshape(len(tops), len(lefts))
    orc.flow_after_piv(a, b, 32, tops, lefts, tu, tv, mode=2, sigma_lk=2.0, px_lk=3, sigma_ls=0.48, px_ls=5,
                       window=27, iterations_lk=5, lam=4.0, iterations_ls=60, dense_export=True, pyramid_levels=2,
                       precision=32)
    secs = time.perf_counter() - t0
    return {"value": 1.0 / secs, "unit": "frame-pairs/s", "cores": threads, "kind": "port",
            "sample": "one 1024x1024 pair: the oracle's FP32 32x32 pass and flow stage (LK pyramid, Liu-Shen, "
                      f"dense field), {secs:.1f} s"}


def run_hybrid(pkg, h, dev, stream, steps, warmup, accuracy=False):
    """Config-4 step: PIV + flow of HYBRID_PAIRS pairs resident in HBM, dense field out."""
    import torch
    piv, flow = hybrid_descs(pkg)
    hp = HYBRID_PAIRS
    pairs = [pkg.synth.config4_pair(pair_id=k) for k in range(4)]
    imgs = torch.empty((hp, 2, H, W), dtype=torch.uint8, device=dev)
    for k in range(hp):
        a, b = pairs[k % len(pairs)]
        imgs[k, 0].copy_(torch.from_numpy(a))
        imgs[k, 1].copy_(torch.from_numpy(b))
    table = np.zeros(hp, pkg.FRAME_DTYPE)
    for k in range(hp):
        table[k] = (imgs[k, 0].data_ptr(), imgs[k, 1].data_ptr(), H, W, W)
    dtable = torch.from_numpy(table.view(np.uint8)).to(dev)
    last = pkg.adaptive_levels(piv, H, W)[-1]
    tiles = last["tiles_i"] * last["tiles_j"]
    ou = torch.empty(hp * tiles, dtype=torch.float32, device=dev)
    ov = torch.empty_like(ou)
    du = torch.empty((hp, H, W), dtype=torch.float32, device=dev)
    dv = torch.empty_like(du)

    def step():
        h.piv_flow_device(piv, flow, pkg.PIX_U8, H, W, hp, dtable, ou, ov, du, dv)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    launches0 = h.launches
    t0.record(stream)
    for _ in range(steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1) / steps
    launches = (h.launches - launches0) // steps
    # per-kernel split from the library's stage events (flow = the whole flow stage of a pair)
    h.profile(True)
    h.profile_read()
    step()
    stages = h.profile_read()
    h.profile(False)
    # e2e: host frames in, tile vectors and dense field out
    fa = [pairs[k % len(pairs)][0] for k in range(hp)]
    fb = [pairs[k % len(pairs)][1] for k in range(hp)]
    res = h.piv_flow(fa, fb, piv, flow, dense=True)
    acc = hybrid_accuracy(pkg, h, pairs[0], res[2][0], res[3][0]) if accuracy else None
    cpu_line = hybrid_cpu_baseline(pkg, pairs[0]) if accuracy else None
    e2e_steps = 2
    tt = time.perf_counter()
    for _ in range(e2e_steps):
        h.piv_flow(fa, fb, piv, flow, dense=True)
    e2e_s = (time.perf_counter() - tt) / e2e_steps
    px = float(H * W)
    out = {
        "workload": HYBRID_WORKLOAD, "pairs_per_step": hp, "ms_per_step": ms, "frame_pairs_per_s": hp / (ms * 1e-3),
        "dense_mpx_per_s": hp * px / (ms * 1e-3) / 1e6, "gpu_launches_per_step": launches,
        "stages": [{"stage": st["stage"], "ia_side": st["ia_side"], "ms_per_step": st["ms"]} for st in stages],
        "e2e": {"value": hp / e2e_s, "unit": "frame-pairs/s", "h2d_bytes_per_step": hp * 2 * H * W,
                "d2h_bytes_per_step": hp * (2 * tiles + 2 * H * W) * 4},
    }
    if acc is not None:
        out["accuracy"] = acc
    if cpu_line is not None:
        out["cpu_baseline"] = cpu_line
    return out


C1_WORKLOAD = ("single-512-u8: 512x512 u8 Rankine pairs (0.02 ppp, d = 3 +- 0.5 px, max 4 px), one 32x32 pass at "
               "50 % overlap (961 vectors), FindMaximumFromCenter + 3-point Gaussian")


def run_config1(pkg, h, dev, stream, steps, warmup, cpu=True, pairs=256):
    """The plain single-pass workload three ways: a device-resident batch of `pairs` pairs through
    the fused adaptive entry point (one level), one synchronous qlpiv_pass per pair on host
    images, and the oracle's FP32 pass on the host cores; plus the error against the FP64 oracle."""
    import torch
    desc = pkg.adaptive_desc(32, 32, 0.5, warp_mode=pkg.WARP_NONE, norm_mode=pkg.NORM_MAX_A,
                             max_mode=pkg.MAX_COMPUTE)
    uniq = [pkg.synth.config1_pair(seed=1, pair_id=k) for k in range(8)]
    imgs = torch.empty((pairs, 2, 512, 512), dtype=torch.uint8, device=dev)
    table = np.zeros(pairs, pkg.FRAME_DTYPE)
    for k in range(pairs):
        imgs[k, 0].copy_(torch.from_numpy(uniq[k % 8][0]))
        imgs[k, 1].copy_(torch.from_numpy(uniq[k % 8][1]))
        table[k] = (imgs[k, 0].data_ptr(), imgs[k, 1].data_ptr(), 512, 512, 512)
    dtable = torch.from_numpy(table.view(np.uint8)).to(dev)
    ou = torch.empty(pairs * 961, dtype=torch.float32, device=dev)
    ov = torch.empty_like(ou)
    for _ in range(warmup):
        h.piv_adaptive_device(desc, pkg.PIX_U8, 512, 512, pairs, dtable, ou, ov)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        h.piv_adaptive_device(desc, pkg.PIX_U8, 512, 512, pairs, dtable, ou, ov)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    g = pkg.grid.superposition(512, 512, 32, 0, 0.5)
    at, al = g.origins()
    for k in range(3):
        vec = h.piv_pass(uniq[k][0], uniq[k][1], 32, at, al)
    reps = 32
    t0 = time.perf_counter()
    for k in range(reps):
        h.piv_pass(uniq[k % 8][0], uniq[k % 8][1], 32, at, al)
    per_call_s = (time.perf_counter() - t0) / reps
    out = {"workload": C1_WORKLOAD, "pairs_per_step": pairs, "ms_per_step": ms,
           "frame_pairs_per_s": pairs / (ms * 1e-3), "ia_vectors_per_s": pairs * 961 / (ms * 1e-3),
           "plain_per_call": {"frame_pairs_per_s": 1.0 / per_call_s,
                              "sample": f"{reps} pairs, one synchronous qlpiv_pass per pair (host images)"},
           "vs_per_call": (pairs / (ms * 1e-3)) * per_call_s}
    if cpu:
        orc = load_oracle()
        a, b = uniq[0]
        threads = os.cpu_count() or 1
        orc.piv_pass(a, b, 32, at, al, precision=32, nthreads=threads)
        times = []
        for _ in range(5):
            t0 = time.perf_counter()
            orc.piv_pass(a, b, 32, at, al, precision=32, nthreads=threads)
            times.append(time.perf_counter() - t0)
        out["cpu_baseline"] = {"value": 1.0 / statistics.median(times), "unit": "frame-pairs/s", "cores": threads,
                               "kind": "port", "sample": "one pair, median of 5 after 1 warm-up (FP32 oracle pass)"}
        gu = ou[:961].cpu().numpy()
        gv = ov[:961].cpu().numpy()
        o64 = orc.piv_pass(a, b, 32, at, al, precision=64, nthreads=threads)
        e = np.maximum(np.abs(gu - o64["u64"]), np.abs(gv - o64["v64"]))
        out["accuracy"] = {"reference": "FP64 oracle pass", "vectors": 961, "max_px": float(e.max()),
                           "p99_px": float(np.quantile(e, 0.99)), "frac_within_1e-3": float(np.mean(e <= 1e-3))}
    return out


def run_per_call(pkg, dev, desc, pairs_host, count):
    """The plain per-call GPU path: one pair at a time, one synchronous library call per stage
    (inheritance, warp, correlation pass, validation), host arrays in and out."""
    h2 = pkg.Handle(dev.index)
    try:
        a, b = pairs_host[0]
        pkg.per_call.piv_adaptive_per_call(h2, a, b, desc)
        t0 = time.perf_counter()
        for k in range(count):
            a, b = pairs_host[k % len(pairs_host)]
            pkg.per_call.piv_adaptive_per_call(h2, a, b, desc)
        per_call_s = (time.perf_counter() - t0) / count
        # one pair per call through the fused host API (no per-stage round trips)
        h2.piv_adaptive([a], [b], desc)
        t0 = time.perf_counter()
        for k in range(count):
            a, b = pairs_host[k % len(pairs_host)]
            h2.piv_adaptive([a], [b], desc)
        per_pair_s = (time.perf_counter() - t0) / count
    finally:
        h2.close()
    return 1.0 / per_call_s, 1.0 / per_pair_s


# Served stream: requests of log-uniform sizes 256^2..4096^2 (u8 / 12-bit u16 mixed), each with
# one of three schedules (single 32; 64 -> 32; 64 -> 32 -> 16 with BothImages warp), 50 % overlap.
SERVING_WORKLOAD = ("served-mixed: Poisson arrivals of frame pairs, sides log-uniform 256..4096 (multiples of 32), "
                    "u8 / 12-bit u16 mixed, schedules single 32 | 64->32 | 64->32->16 + BothImages warp, 50 % "
                    "overlap")


def serving_requests(pkg, count, seed=5):
    """Frames cropped from one synthetic 4096x4096 mosaic (a 2048x2048 vortex pair tiled 2 x 2)."""
    a0, b0 = pkg.synth.particle_pair((2048, 2048), pkg.synth.Flow(vmax=5.0, rc=200.0, shear=0.003), ppp=0.02,
                                     diam=2.8, bits=8, seed=seed)
    ma, mb = np.tile(a0, (2, 2)), np.tile(b0, (2, 2))
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        side = lambda: int(np.clip(round(np.exp(rng.uniform(np.log(256), np.log(4096))) / 32) * 32, 256, 4096))
        h, w = side(), side()
        y, x = int(rng.integers(0, 4096 - h + 1)), int(rng.integers(0, 4096 - w + 1))
        a, b = ma[y:y + h, x:x + w], mb[y:y + h, x:x + w]
        if rng.random() < 0.5:   # 12-bit in u16
            a, b = a.astype(np.uint16) * 16, b.astype(np.uint16) * 16
        out.append((np.ascontiguousarray(a), np.ascontiguousarray(b), int(rng.integers(3))))
    return out


def serving_schedules(pkg):
    return [pkg.adaptive_desc(32, 32, 0.5, warp_mode=pkg.WARP_NONE),
            pkg.adaptive_desc(64, 32, 0.5, warp_mode=pkg.WARP_NONE),
            pkg.adaptive_desc(64, 16, 0.5, warp_mode=pkg.WARP_BOTH_BILINEAR)]


def run_serving(pkg, dev, count=48, loads=(0.25, 0.5, 0.75, 0.9, 1.1), per_load=48, clients=4):
    """Saturation throughput of the request server (`clients` submitting threads, and one), the
    plain per-call paths on the same requests, and p50 / p99 latency (arrival -> results on the
    host) under Poisson arrivals at fractions of the saturation rate."""
    reqs = serving_requests(pkg, count)
    sch = serving_schedules(pkg)
    px = sum(a.size for a, _, _ in reqs)
    # plain per-call: one synchronous library call per request (fused adaptive loop), and one
    # synchronous call per stage (the reference's job pattern)
    h = pkg.Handle(dev.index)
    for a, b, k in reqs[:3]:
        h.piv_adaptive([a], [b], sch[k])
    t0 = time.perf_counter()
    for a, b, k in reqs:
        h.piv_adaptive([a], [b], sch[k])
    per_call = count / (time.perf_counter() - t0)
    for a, b, k in reqs[:3]:
        pkg.per_call.piv_adaptive_per_call(h, a, b, sch[k])
    t0 = time.perf_counter()
    for a, b, k in reqs:
        pkg.per_call.piv_adaptive_per_call(h, a, b, sch[k])
    per_stage = count / (time.perf_counter() - t0)
    h.close()

    from concurrent.futures import ThreadPoolExecutor
    srv = pkg.Server(dev.index, slots=16, staging_bytes=4 << 30)
    pool = ThreadPoolExecutor(clients)
    try:
        def closed_loop(nc):
            # nc client threads submit their share of the requests (each submit copies the pair into
            # pinned staging in the client's thread, the GIL released), then every result is polled
            t = time.perf_counter()
            futs = [pool.submit(lambda part: [srv.submit(a, b, sch[k]) for a, b, k in part], reqs[i::nc])
                    for i in range(nc)]
            tickets = [tk for f in futs for tk in f.result()]
            for tk in tickets:
                srv.poll(tk)
            return count / (time.perf_counter() - t)

        closed_loop(clients)                # warm-up: plans, pools
        saturation_one = closed_loop(1)
        saturation = closed_loop(clients)
        sweep = []
        rng = np.random.default_rng(9)

        def arrive(due, a, b, k):
            tk = srv.submit(a, b, sch[k])
            return tk, time.perf_counter() - due   # arrival -> request staged (s)

        for load in loads:
            rate = load * saturation
            gaps = rng.exponential(1.0 / rate, per_load)
            order = rng.integers(0, count, per_load)
            start = time.perf_counter()
            due = start
            futs = []
            for g, idx in zip(gaps, order):
                due += g
                while time.perf_counter() < due:
                    time.sleep(min(0.0005, max(0.0, due - time.perf_counter())))
                a, b, k = reqs[idx]
                futs.append(pool.submit(arrive, due, a, b, k))
            lat = []
            for f in futs:
                tk, staged = f.result()
                lat.append(staged * 1e3 + srv.poll(tk)[2]["total_ms"])
            elapsed = time.perf_counter() - start
            sweep.append({"offered_pairs_per_s": rate, "achieved_pairs_per_s": per_load / elapsed,
                          "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))})
    finally:
        pool.shutdown()
        srv.close()
    return {"workload": SERVING_WORKLOAD, "requests": count, "megapixels_per_request": px / count / 1e6,
            "clients": clients, "saturation_pairs_per_s": saturation, "saturation_one_client_pairs_per_s":
            saturation_one, "plain_per_call_pairs_per_s": per_call,
            "plain_per_stage_pairs_per_s": per_stage, "vs_per_call": saturation / per_call,
            "vs_per_stage": saturation / per_stage, "sweep": sweep,
            "latency": f"arrival -> displacements on the host: Poisson arrivals handed to {clients} client threads "
                       "(each submit copies the pair into pinned staging), plus the server's submit -> done time"}


# Batched launch: 256 pairs of sizes from {256^2, 512^2, 1024^2, 2048^2} u8, each with its own IA
# size from {16, 32, 64, 128} at 50 % overlap, one graph launch per batch.
BATCH_WORKLOAD = ("batched-mixed: 256 u8 pairs, sides from {256, 512, 1024, 2048} (uniform), IA size per pair from "
                  "{16, 32, 64, 128} (uniform), 50 % overlap, FindMaximumFromCenter + 3-point Gaussian; particles "
                  "(0.02 ppp, d = 3 px) cropped from a rendered 4096x4096 field, frame B resampled (bilinear) through "
                  "each pair's own random field: Rankine vortex (centre, core 5-15 % of the side, 2-6 px) plus "
                  "uniform shear, max 8 px; one captured graph per batch with autotuned launches")


def batch_field(rng, side):
    """A pair's random displacement field: Rankine vortex (random centre, core and strength) plus
    uniform shear, at most 8 px."""
    vmax = float(rng.uniform(2.0, 6.0))
    rc = float(rng.uniform(0.05, 0.15)) * side
    cy, cx = (float(x) for x in rng.uniform(0.2 * side, 0.8 * side, 2))
    shear = float(rng.uniform(-1.0, 1.0)) * (8.0 - vmax) / side      # |shear * dy| <= 8 - vmax
    return vmax, rc, (cy, cx), shear


def batch_pair(pkg, mosaic, rng, side):
    """A crop of the particle mosaic and its image resampled through the pair's own field
    (B(x) = A(x - d(x)))."""
    from scipy import ndimage
    y, x = (int(v) for v in rng.integers(0, mosaic.shape[0] - side + 1, 2))
    a = np.ascontiguousarray(mosaic[y:y + side, x:x + side])
    vmax, rc, centre, shear = batch_field(rng, side)
    flow = pkg.synth.Flow(vmax=vmax, rc=rc, shear=shear, centre=centre)
    rr, cc = np.meshgrid(np.arange(side, dtype=np.float64), np.arange(side, dtype=np.float64), indexing="ij")
    dr, dc = flow.displacement(rr, cc, (side, side))
    b = ndimage.map_coordinates(a.astype(np.float32), [rr - dr, cc - dc], order=1, mode="constant", cval=0.0)
    return a, np.clip(np.rint(b), 0, 255).astype(np.uint8)


def batch_accuracy(pkg, plan, vec, host, sizes, ofac, picks):
    """Batched vectors of sampled pairs against the FP64 oracle (the same single pass in double):
    integer peaks must agree except exact ties; sub-pixel |error| where they agree."""
    orc = load_oracle()
    errs, mism, n = [], 0, 0
    for q in picks:
        a, b = host[q]
        g = pkg.grid.superposition(a.shape[0], a.shape[1], int(sizes[q]), 0, float(ofac[q]))
        at, al = g.origins()
        ref = orc.piv_pass(a, b, int(sizes[q]), at, al, precision=64)
        got = plan.pair_vectors(vec, q).ravel()
        same = (got["peak_i"] == ref["peak_i"]) & (got["peak_j"] == ref["peak_j"])
        mism += int((~same).sum())
        n += got.size
        e = np.maximum(np.abs(got["u"].astype(np.float64) - ref["u64"]), np.abs(got["v"].astype(np.float64) - ref["v64"]))
        errs.append(e[same])
    e = np.concatenate(errs)
    return {"reference": "FP64 oracle single pass (same algorithm in double)", "pairs": len(picks),
            "sides": sorted({int(host[q][0].shape[0]) for q in picks}), "vectors": n,
            "peak_mismatches": mism, "max_px": float(e.max()), "p99_px": float(np.quantile(e, 0.99)),
            "frac_within_1e-3": float(np.mean(e <= 1e-3))}


def batch_cpu_baseline(pkg, host, sizes, ofac, picks, batch_flops, count):
    """The oracle's FP32 single pass on the sampled pairs with all host threads; the batch's time
    is extrapolated from the sample by the FFT-formula work (F(2N) per IA)."""
    orc = load_oracle()
    threads = os.cpu_count() or 1
    secs = work = 0.0
    for q in picks:
        a, b = host[q]
        n = int(sizes[q])
        g = pkg.grid.superposition(a.shape[0], a.shape[1], n, 0, float(ofac[q]))
        at, al = g.origins()
        t0 = time.perf_counter()
        orc.piv_pass(a, b, n, at, al, precision=32, nthreads=threads)
        secs += time.perf_counter() - t0
        work += flops_per_ia(n) * g.count
    batch_s = batch_flops / (work / secs)
    return {"value": count / batch_s, "unit": "frame-pairs/s", "cores": threads, "kind": "port",
            "sample": f"{len(picks)} pairs of the batch (every 8th: sides "
                      f"{sorted({int(host[q][0].shape[0]) for q in picks})}, IA sizes "
                      f"{sorted({int(sizes[q]) for q in picks})}) through the oracle's FP32 pass, {secs:.1f} s; the "
                      f"{count}-pair batch extrapolated by formula work"}


def run_batched(pkg, dev, stream, steps, warmup, count=256, ia_sizes=(16, 32, 64, 128), cpu=True):
    import torch
    rng = np.random.default_rng(3)
    a0, _ = pkg.synth.particle_pair((2048, 2048), pkg.synth.Flow(vmax=0.0), ppp=0.02, diam=3.0, bits=8, seed=33)
    mosaic = np.tile(a0, (2, 2))
    sides = rng.choice([256, 512, 1024, 2048], count)
    sizes = rng.choice(list(ia_sizes), count).astype(np.int32)
    ofac = np.full(count, 0.5, np.float32)
    keep, host, table = [], [], np.zeros(count, pkg.FRAME_DTYPE)
    for k in range(count):
        s_ = int(sides[k])
        a, b = batch_pair(pkg, mosaic, rng, s_)
        ta, tb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        keep.append((ta, tb))
        host.append((a, b))
        table[k] = (ta.data_ptr(), tb.data_ptr(), s_, s_, s_)
    h = pkg.Handle(dev.index)
    hs = torch.cuda.ExternalStream(h.stream, device=dev)
    def time_plan(pl):
        for _ in range(warmup):
            pl.run()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(hs)
        for _ in range(steps):
            pl.run()
        e1.record(hs)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    # the two schedules with default grids, then the autotuned plan (the reported one)
    schedules_ms = {}
    for name, mode in (("per_size_default_grids", pkg.AUTOTUNE_OFF), ("persistent", pkg.AUTOTUNE_PERSISTENT)):
        alt = pkg.MixedPlan(h, table, sizes, ofac, pkg.PIX_U8, autotune=mode)
        schedules_ms[name] = time_plan(alt)
        alt.close()
    t0 = time.perf_counter()
    plan = pkg.MixedPlan(h, table, sizes, ofac, pkg.PIX_U8, autotune=pkg.AUTOTUNE_ON)
    plan_s = time.perf_counter() - t0
    ms = time_plan(plan)
    schedules_ms["autotuned"] = ms
    total = plan.total
    ia_by_n = {n: int(sum(plan.tiles[q][0] * plan.tiles[q][1] for q in range(count) if sizes[q] == n))
               for n in (16, 32, 64, 128)}
    flops = sum(flops_per_ia(n) * c for n, c in ia_by_n.items())
    bytes_ = sum(bytes_per_ia(n, 1) * c for n, c in ia_by_n.items())
    vec = plan.vectors()
    # FP64 error on sampled pairs up to 1024^2, every IA size
    picks = []
    for n in ia_sizes:
        picks += [q for q in range(count) if sizes[q] == n and sides[q] <= 1024][:2]
    accuracy = batch_accuracy(pkg, plan, vec, host, sizes, ofac, picks)
    cpu_line = batch_cpu_baseline(pkg, host, sizes, ofac, list(range(0, count, 8)), flops, count) if cpu else None
    # adaptive batch: the same pairs, each with one of the served schedules (single 32 | 64->32 |
    # 64->32->16 + warp), groups of one size and schedule as graph branches; against one
    # synchronous qlpiv_piv_adaptive per pair with pinned frames
    sch = serving_schedules(pkg)
    sidx = np.random.default_rng(11).integers(0, len(sch), count)
    ab = pkg.AdaptiveBatch(h, table, pkg.PIX_U8, sch, sidx)
    ab_ms = time_plan(ab)
    ab_groups, ab_tiles = ab.groups, ab.total
    ab.close()
    # sorted by size and schedule, so that consecutive calls reuse the handle's plan
    ab_sample = sorted(range(0, count, 4), key=lambda q: (int(sides[q]), int(sidx[q])))
    ab_pinned = {q: tuple(torch.from_numpy(x).pin_memory().numpy() for x in host[q]) for q in ab_sample}
    for q in ab_sample[:2]:
        h.piv_adaptive([ab_pinned[q][0]], [ab_pinned[q][1]], sch[sidx[q]])
    tt = time.perf_counter()
    for q in ab_sample:
        h.piv_adaptive([ab_pinned[q][0]], [ab_pinned[q][1]], sch[sidx[q]])
    ab_per_call = len(ab_sample) / (time.perf_counter() - tt)
    adaptive = {"schedules": "single 32 | 64->32 | 64->32->16 + BothImages warp, 50 % overlap, one per pair "
                             "(seeded)", "groups": ab_groups, "tiles_per_step": ab_tiles, "ms_per_step": ab_ms,
                "frame_pairs_per_s": count / (ab_ms * 1e-3),
                "plain_per_call": {"frame_pairs_per_s": ab_per_call,
                                   "sample": f"{len(ab_sample)} pairs (every 4th, ordered by size and "
                                             "schedule), one synchronous qlpiv_piv_adaptive per pair, frames in "
                                             "pinned host memory"},
                "vs_per_call": count / (ab_ms * 1e-3) / ab_per_call}
    # plain per-call: one synchronous frame pass per pair through the host API, frames in pinned
    # host memory; three timed rounds over the sample give the spread
    sample = list(range(0, count, 8))
    pinned = {q: tuple(torch.from_numpy(x).pin_memory().numpy() for x in host[q]) for q in sample}
    origins = {}
    for q in sample:
        g = pkg.grid.superposition(int(sides[q]), int(sides[q]), int(sizes[q]), 0, 0.5)
        origins[q] = (g.origins(), g.count)
    for q in sample[:2]:
        h.piv_pass(*pinned[q], int(sizes[q]), *origins[q][0])
    rounds = []
    for _ in range(3):
        tt = time.perf_counter()
        for q in sample:
            h.piv_pass(*pinned[q], int(sizes[q]), *origins[q][0])
        rounds.append(len(sample) / (time.perf_counter() - tt))
    per_call_pairs = statistics.median(rounds)
    sample_ias = sum(origins[q][1] for q in sample)
    plan.close()
    h.close()
    fps = count / (ms * 1e-3)
    return {"workload": BATCH_WORKLOAD, "pairs_per_step": count, "ia_vectors_per_step": total,
            "ia_vectors_by_size": ia_by_n, "ms_per_step": ms, "frame_pairs_per_s": fps,
            "ia_vectors_per_s": total / (ms * 1e-3), "fp32_tflops": flops / (ms * 1e-3) / 1e12,
            "algorithmic_gbs": bytes_ / (ms * 1e-3) / 1e9, "plan_seconds": plan_s,
            "autotuned_waves": {str(n): int(plan.waves[k]) for k, n in enumerate((16, 32, 64, 128))},
            "autotuned_schedule": "persistent" if plan.schedule == pkg.SCHEDULE_PERSISTENT else "per_size",
            "schedules_ms_per_step": schedules_ms,
            "accuracy": accuracy,
            "plain_per_call": {"frame_pairs_per_s": per_call_pairs, "rounds_frame_pairs_per_s": rounds,
                               "ia_vectors_per_s": sample_ias * per_call_pairs / len(sample),
                               "sample": f"{len(sample)} pairs, one synchronous qlpiv_pass per pair, frames in "
                                         f"pinned host memory, median of 3 rounds"},
            "vs_per_call_pairs": fps / per_call_pairs,
            "vs_per_call_pairs_range": [fps / max(rounds), fps / min(rounds)],
            "cpu_baseline": cpu_line, "adaptive": adaptive}


def run_reference(args, rank):
    if rank != 0:
        return
    pkg = load_pkg()
    threads = os.cpu_count() or 1
    pair = make_pairs(pkg, 1)[0]
    for _ in range(args.warmup):
        cpu_baseline(pkg, pair, threads, reps=1, warmup=0)
    times = [cpu_baseline(pkg, pair, threads, reps=1, warmup=0) for _ in range(args.steps)]
    t = sum(times) / len(times)
    v = 1.0 / t
    line = {
        "impl": "reference", "metric": "frame-pairs/s", "value": v, "unit": "frame-pairs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD + "; one pair per step",
                   "pairs_per_step": 1, "ia_vectors_per_pair": sum(g.count for g in level_grids(pkg))},
        "cpu_baseline": {"value": v, "unit": "frame-pairs/s", "cores": threads, "kind": "port",
                         "sample": "one 1024x1024 pair through the whole adaptive loop (FP32 oracle)"},
        "e2e": {"value": v, "unit": "frame-pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def job_time_ms(ms_local, world, device=None):
    """Whole-job time of a replicated run: the slowest rank's time (MAX over the process group)."""
    if world <= 1:
        return float(ms_local)
    import torch
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, ms):
    """Units processed by all ranks per second (weak scaling: every rank runs the same work)."""
    return world * units_per_rank / (ms * 1e-3)


def run_gpu(args, rank, world):
    import torch
    pkg = load_pkg()
    pkg.build.build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    h = pkg.Handle(dev.index)
    stream = torch.cuda.ExternalStream(h.stream, device=dev)

    grids = level_grids(pkg)
    last = grids[-1]
    pairs_host = make_pairs(pkg, args.unique)
    P = args.pairs
    bpp = 2
    desc = pkg.adaptive_desc(LEVELS[0], LEVELS[-1], OVERLAP_FACTOR, warp_mode=pkg.WARP_BOTH_BILINEAR,
                             norm_mode=pkg.NORM_MAX_A, max_mode=pkg.MAX_FIXED, fixed_max=FULL_SCALE,
                             subpix_mode=pkg.SUBPIX_GAUSS3, validation=VALIDATION)
    # device-resident frames: P slots filled from `unique` distinct synthetic pairs
    imgs = torch.empty((P, 2, H, W), dtype=torch.int16, device=dev)
    for k in range(P):
        a, b = pairs_host[k % len(pairs_host)]
        imgs[k, 0].copy_(torch.from_numpy(a.view(np.int16)))
        imgs[k, 1].copy_(torch.from_numpy(b.view(np.int16)))
    table = np.zeros(P, pkg.FRAME_DTYPE)
    for k in range(P):
        table[k] = (imgs[k, 0].data_ptr(), imgs[k, 1].data_ptr(), H, W, W)
    dtable = torch.from_numpy(table.view(np.uint8)).to(dev)
    out_u = torch.empty(P * last.count, dtype=torch.float32, device=dev)
    out_v = torch.empty_like(out_u)
    ia_per_pair = sum(g.count for g in grids)

    def step():
        h.piv_adaptive_device(desc, pkg.PIX_U16, H, W, P, dtable, out_u, out_v)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    launches0 = h.launches
    sampler = ClockSampler(dev.index)
    torch.cuda.synchronize()
    with sampler:
        t_start.record(stream)
        for _ in range(args.steps):
            step()
        t_end.record(stream)
        torch.cuda.synchronize()
    launches = h.launches - launches0
    ms = job_time_ms(t_start.elapsed_time(t_end), world, dev)
    ms_per_step = ms / args.steps
    pairs_per_s = job_throughput(P * args.steps, world, ms)

    # ---- per-stage device time (events around every launch), two extra steps ----
    h.profile(True)
    h.profile_read()
    prof_steps = 2
    for _ in range(prof_steps):
        step()
    stages = h.profile_read()
    h.profile(False)
    for st in stages:
        st["ms_per_step"] = st["ms"] / prof_steps

    # ---- e2e through the host API: pinned host frames in, displacements out ----
    host_frames = [(torch.from_numpy(a).pin_memory(), torch.from_numpy(b).pin_memory()) for a, b in pairs_host]
    fa = [host_frames[k % len(host_frames)][0].numpy() for k in range(P)]
    fb = [host_frames[k % len(host_frames)][1].numpy() for k in range(P)]
    e2e_steps = max(1, min(args.steps, 5))
    for _ in range(2):
        h.piv_adaptive(fa, fb, desc)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        u_host, v_host = h.piv_adaptive(fa, fb, desc)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_val = world * P / e2e_s
    h2d = P * 2 * H * W * bpp
    d2h = 2 * P * last.count * 4

    # ---- accuracy of the timed workload: the e2e run's displacements against the FP64 oracle ----
    accuracy = None
    if rank == 0 and not args.no_cpu:
        accuracy = c2_accuracy(pairs_host, u_host, v_host)

    # ---- roofline of the dominant kernel ----
    dom = max(stages, key=lambda s_: s_["ms"])
    t_launch = dom["ms"] / dom["launches"] * 1e-3
    items_per_launch = dom["items"] / dom["launches"]
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    fp32_peak = pkg.measure_fp32_peak(dev.index)
    traffic = None
    if dom["stage"] == "xcorr":
        n_dom = dom["ia_side"]
        alg_bytes = bytes_per_ia(n_dom, bpp) * items_per_launch
        alg_flops = flops_per_ia(n_dom) * items_per_launch
        tfile = ROOT / "profiles" / "k1_traffic.json"
        if tfile.exists():
            per_ia = json.loads(tfile.read_text()).get("dram_bytes_per_ia", {}).get(str(n_dom))
            if per_ia is not None:
                traffic = per_ia * items_per_launch
        kernel = f"xcorr_kernel<{n_dom}>"
    else:
        alg_bytes = 4.0 * bpp * items_per_launch   # warp: read A, B; write A', B'
        alg_flops = 0.0
        kernel = dom["stage"]
    result = {
        "metric": "frame-pairs/s", "value": pairs_per_s, "unit": "frame-pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD,
                   "pairs_per_step": P, "unique_pairs": len(pairs_host), "ia_vectors_per_pair": ia_per_pair,
                   "inputs_exceed_l2": P * 2 * H * W * bpp > 129e6, "l2_flush": "inputs larger than L2",
                   "tile_max": "full scale 65535 (warped tiles, reference semantics)",
                   "parallelism": f"replicas x{world}"},
        "ia_vectors_per_s": world * ia_per_pair * P * args.steps / (ms * 1e-3),
        "stages": [{k: st[k] for k in ("stage", "level", "ia_side", "ms_per_step")} for st in stages],
        "e2e": {"value": e2e_val, "unit": "frame-pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": sampler.summary(),
    }
    hbm_view = {"bound": "hbm", "achieved": alg_bytes / t_launch / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": alg_bytes / t_launch / 1e9 / hbm_peak, "traffic": traffic, "kernel": kernel,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"}
    if alg_flops:
        # the correlation kernel is FP32 (CUDA-core) bound: its roofline is the FP32 FMA peak
        # measured live on this GPU; the HBM view is kept beside it
        result["roofline"] = {"bound": "fp32", "achieved": alg_flops / t_launch / 1e12, "peak": fp32_peak,
                              "unit": "TFLOP/s", "frac": alg_flops / t_launch / 1e12 / fp32_peak,
                              "traffic": traffic, "kernel": kernel,
                              "peak_source": "live FP32 FMA probe on this GPU (qlpiv_measure_fp32_peak, best of 3); "
                                             "nominal 152 SMs x 128 lanes x 2 flop x 2.07 GHz = 80.5 TFLOP/s",
                              "flops_per_ia": flops_per_ia(dom["ia_side"]),
                              "ias_per_launch": items_per_launch}
        result["roofline_hbm"] = hbm_view
    else:
        result["roofline"] = hbm_view
    if accuracy is not None:
        result["accuracy"] = {"adaptive-1024-u12": accuracy}
    # ---- the plain per-call GPU path on the same workload (denominator of the batching gain) ----
    pc_value, pp_value = run_per_call(pkg, dev, desc, pairs_host, 4)
    result["plain_per_call"] = {
        "value": world * pc_value, "unit": "frame-pairs/s",
        "sample": "4 pairs, one at a time, one synchronous library call per stage (host arrays in and out)",
        "value_vs": pairs_per_s / pc_value, "e2e_vs": e2e_val / (world * pc_value),
        "one_pair_per_call_fused": world * pp_value}
    result["single_pass"] = run_config1(pkg, h, dev, stream, max(3, min(args.steps, 10)), max(3, args.warmup),
                                        cpu=rank == 0 and not args.no_cpu)
    if not args.no_hybrid:
        result["hybrid"] = run_hybrid(pkg, h, dev, stream, max(2, min(args.steps, 5)), max(3, args.warmup),
                                      accuracy=rank == 0 and not args.no_cpu)
    if not args.no_batched:
        result["batched"] = run_batched(pkg, dev, stream, max(3, min(args.steps, 10)), max(3, args.warmup),
                                        cpu=rank == 0 and not args.no_cpu)
    if not args.no_serving and world == 1:
        result["serving"] = run_serving(pkg, dev)
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        t_cpu = cpu_baseline(pkg, pairs_host[0], threads)
        result["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "frame-pairs/s", "cores": threads, "kind": "port",
                                  "sample": "one 1024x1024 pair through the whole adaptive loop (FP32 oracle), "
                                            "median of 5 runs after 1 warm-up"}
    h.close()
    if rank == 0:
        print(json.dumps(result), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--pairs", type=int, default=48)
    ap.add_argument("--unique", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-hybrid", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    # profiling aid: only the batched mixed-size leg (its own JSON line), optionally with fewer
    # pairs and a subset of the IA sizes, so that one kernel can be captured on a small case
    ap.add_argument("--only-batched", action="store_true")
    ap.add_argument("--batched-pairs", type=int, default=256)
    ap.add_argument("--batched-sizes", default="16,32,64,128")
    # profiling aid: only the hybrid PIV + dense flow leg (its own JSON line)
    ap.add_argument("--only-hybrid", action="store_true")
    args = ap.parse_args()
    if args.only_hybrid:
        import torch
        pkg = load_pkg()
        pkg.build.build()
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        h = pkg.Handle(dev.index)
        try:
            stream = torch.cuda.ExternalStream(h.stream, device=dev)
            print(json.dumps(run_hybrid(pkg, h, dev, stream, max(1, args.steps), max(1, args.warmup))), flush=True)
        finally:
            h.close()
        return
    if args.only_batched:
        import torch
        pkg = load_pkg()
        pkg.build.build()
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        sizes = tuple(int(x) for x in args.batched_sizes.split(","))
        print(json.dumps(run_batched(pkg, dev, None, args.steps, args.warmup, args.batched_pairs, sizes)), flush=True)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    try:
        run_gpu(args, rank, world)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
