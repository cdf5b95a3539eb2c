"""The multi-rank bench path on CPU (gloo, world size 2): replicas run the same work, the job time
is the slowest rank's, throughput counts every rank's units, and the reference arm prints from
rank 0 only."""
import importlib.util
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b = _bench()
        ms = b.job_time_ms(10.0 + 5.0 * rank, world)     # rank 1 is slower
        q.put((rank, ms, b.job_throughput(48, world, ms)))
    finally:
        dist.destroy_process_group()


def test_job_time_is_max_over_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29650 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    assert out[0][2] == pytest.approx(2 * 48 / 0.015)


def test_single_rank_passthrough():
    b = _bench()
    assert b.job_time_ms(12.5, 1) == 12.5
    assert b.job_throughput(10, 1, 1000.0) == pytest.approx(10.0)


def test_reference_arm_prints_only_on_rank_0(tmp_path):
    """torchrun with 2 CPU ranks: the reference arm's JSON line comes from rank 0 alone and the
    other rank exits 0 without work."""
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(29750 + os.getpid() % 1000), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=tmp_path)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
