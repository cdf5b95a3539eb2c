#!/usr/bin/env python3
"""FFT-PIV throughput benchmark (one JSON line on rank 0).

Workload ("adaptive-1024-u12"): 1024x1024 12-bit-in-uint16 synthetic particle pairs
(0.03 ppp, d = 2.5 px, shear 0.005 + Rankine vortex, max 6 px), three correlation
passes with IA 64 -> 32 -> 16 at 75 % overlap (61^2 + 125^2 + 253^2 = 83,355 vectors
per pair), FP32, 3-point Gaussian sub-pixel fit.  A step processes a batch of `pairs`
pairs resident in HBM (inputs larger than L2), one batched launch per pass.

  value      frame-pairs/s with inputs resident in HBM (CUDA events on the library's
             stream, max over ranks);
  e2e        frame-pairs/s through the public host API (qlpiv_pass_batch): pinned host
             images copied to the device and vectors copied back inside the timed region;
  roofline   dominant kernel (the pass with the largest device time): algorithmic bytes
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


def cpu_baseline(pkg, pair, threads, reps=1):
    """Oracle FP32 restatement of the reference CPU path on one pair (all passes)."""
    orc = load_oracle()
    a, b = pair
    grids = level_grids(pkg)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        for g in grids:
            at, al = g.origins()
            orc.piv_pass(a, b, g.n, at, al, norm_mode=orc.NORM_MAX_A, precision=32, nthreads=threads)
        times.append(time.perf_counter() - t0)
    return min(times)


def run_reference(args, rank):
    if rank != 0:
        return
    pkg = load_pkg()
    threads = os.cpu_count() or 1
    pair = make_pairs(pkg, 1)[0]
    for _ in range(args.warmup):
        cpu_baseline(pkg, pair, threads)
    times = [cpu_baseline(pkg, pair, threads) for _ in range(args.steps)]
    t = sum(times) / len(times)
    v = 1.0 / t
    line = {
        "impl": "reference", "metric": "frame-pairs/s", "value": v, "unit": "frame-pairs/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "adaptive-1024-u12 (IA 64/32/16 at 75 %), one pair per step",
                   "pairs_per_step": 1, "ia_vectors_per_pair": sum(g.count for g in level_grids(pkg))},
        "cpu_baseline": {"value": v, "unit": "frame-pairs/s", "cores": threads, "kind": "port",
                         "sample": "one 1024x1024 pair, all three correlation passes"},
        "e2e": {"value": v, "unit": "frame-pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world):
    import torch
    pkg = load_pkg()
    pkg.build.build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    h = pkg.Handle(dev.index)
    stream = torch.cuda.ExternalStream(h.stream, device=dev)

    grids = level_grids(pkg)
    pairs_host = make_pairs(pkg, args.unique)
    P = args.pairs
    bpp = 2
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
    work = []
    for g in grids:
        at, al = g.origins()
        fi = np.repeat(np.arange(P, dtype=np.int32), len(at))
        wl = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (fi, np.tile(at, P), np.tile(al, P))]
        out = torch.empty(len(fi) * 32, dtype=torch.uint8, device=dev)
        work.append((g.n, len(fi), wl, out))
    total_ia = sum(c for _, c, _, _ in work)

    def step(evs=None):
        for lv, (n, count, wl, out) in enumerate(work):
            if evs is not None:
                evs[lv][0].record(stream)
            h.piv_pass_batch_device(pkg.PIX_U16, P, dtable, n, count, wl[0], wl[1], wl[2], wl[1], wl[2], out,
                                    norm_mode=pkg.NORM_MAX_A)
            if evs is not None:
                evs[lv][1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    lev_ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in work]
              for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    launches0 = h.launches
    sampler = ClockSampler(dev.index)
    torch.cuda.synchronize()
    with sampler:
        t_start.record(stream)
        for s in range(args.steps):
            step(lev_ev[s])
        t_end.record(stream)
        torch.cuda.synchronize()
    launches = h.launches - launches0
    ms = t_start.elapsed_time(t_end)
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    pairs_per_s = world * P * args.steps / (ms * 1e-3)
    lev_ms = [sum(lev_ev[s][lv][0].elapsed_time(lev_ev[s][lv][1]) for s in range(args.steps)) / args.steps
              for lv in range(len(work))]

    # ---- e2e through the host API: pinned host frames in, vectors out ----
    host_frames = [(torch.from_numpy(a).pin_memory(), torch.from_numpy(b).pin_memory()) for a, b in pairs_host]
    fa = [host_frames[k % len(host_frames)][0].numpy() for k in range(P)]
    fb = [host_frames[k % len(host_frames)][1].numpy() for k in range(P)]
    host_work = []
    for g in grids:
        at, al = g.origins()
        host_work.append((g.n, np.repeat(np.arange(P, dtype=np.int32), len(at)), np.tile(at, P), np.tile(al, P)))
    e2e_steps = max(1, min(args.steps, 5))
    for _ in range(2):
        for n, fi, at, al in host_work:
            h.piv_pass_batch(fa, fb, n, fi, at, al, norm_mode=pkg.NORM_MAX_A)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for n, fi, at, al in host_work:
            h.piv_pass_batch(fa, fb, n, fi, at, al, norm_mode=pkg.NORM_MAX_A)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_val = world * P / e2e_s
    h2d = len(host_work) * P * 2 * H * W * bpp + sum(len(fi) * 20 for _, fi, _, _ in host_work)
    d2h = total_ia * 32

    # ---- roofline of the dominant kernel ----
    dom = int(np.argmax(lev_ms))
    n_dom, cnt_dom = work[dom][0], work[dom][1]
    t_launch = lev_ms[dom] * 1e-3
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    fp32_peak = pkg.measure_fp32_peak(dev.index)
    alg_bytes = bytes_per_ia(n_dom, bpp) * cnt_dom
    alg_flops = flops_per_ia(n_dom) * cnt_dom
    traffic = None
    tfile = ROOT / "profiles" / "k1_traffic.json"
    if tfile.exists():
        tj = json.loads(tfile.read_text())
        per_ia = tj.get("dram_bytes_per_ia", {}).get(str(n_dom))
        if per_ia is not None:
            traffic = per_ia * cnt_dom

    result = {
        "metric": "frame-pairs/s", "value": pairs_per_s, "unit": "frame-pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "adaptive-1024-u12: 1024x1024 12-bit pairs, IA 64/32/16 at 75 % overlap, "
                               "3-point Gaussian; passes correlated at the grid origins (no warp/validation stage "
                               "between passes)",
                   "pairs_per_step": P, "unique_pairs": len(pairs_host), "ia_vectors_per_pair": total_ia // P,
                   "inputs_exceed_l2": P * 2 * H * W * bpp > 129e6, "l2_flush": "inputs larger than L2",
                   "norm": "tile A max (CPU path)", "parallelism": f"replicas x{world}"},
        "ia_vectors_per_s": world * total_ia * args.steps / (ms * 1e-3),
        "pass_ms": {str(work[k][0]): lev_ms[k] for k in range(len(work))},
        "e2e": {"value": e2e_val, "unit": "frame-pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": alg_bytes / t_launch / 1e9, "peak": hbm_peak, "unit": "GB/s",
                     "frac": alg_bytes / t_launch / 1e9 / hbm_peak, "traffic": traffic,
                     "kernel": f"xcorr_kernel<{n_dom}>", "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "compute_roofline": {"bound": "fp32", "achieved": alg_flops / t_launch / 1e12, "peak": fp32_peak,
                             "unit": "TFLOP/s", "frac": alg_flops / t_launch / 1e12 / fp32_peak,
                             "peak_source": "live FP32 FMA probe (qlpiv_measure_fp32_peak)"},
        "clocks": sampler.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        t_cpu = cpu_baseline(pkg, pairs_host[0], threads)
        result["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "frame-pairs/s", "cores": threads, "kind": "port",
                                  "sample": "one 1024x1024 pair, all three correlation passes (FP32 oracle)"}
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
    args = ap.parse_args()
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
