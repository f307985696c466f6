"""Multi-rank plumbing of bench.py on CPU: two gloo ranks (world size 2)
run the same helpers the benchmark uses under torchrun -- rendezvous from
the environment, barrier, max of the per-rank times, sum of the per-rank
ray counts -- and the reference arm's rank 1 exits without work."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import json, os, sys, argparse
sys.path.insert(0, sys.argv[1])
import bench
args = argparse.Namespace(gpus=2)
rank, world, local, dist = bench.dist_setup(args)
bench.barrier(dist)
t = bench.max_over_ranks(dist, 1.0 + rank)       # per-rank time: 1 s, 2 s
rays = bench.sum_over_ranks(dist, 100.0 * (rank + 1))
print(json.dumps({"rank": rank, "world": world, "local": local, "t": t, "rays": rays}))
dist.destroy_process_group()
"""


def _free_port():
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _run_ranks(code, world=2, timeout=120):
    port = _free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, WORLD_SIZE=str(world), RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", code, ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            o, e = p.communicate(timeout=timeout)
        except subprocess.TimeoutExpired:
            p.kill()
            raise
        assert p.returncode == 0, e
        outs.append(o)
    return outs


def test_two_gloo_ranks_max_time_and_sum_rays():
    pytest.importorskip("torch.distributed")
    outs = _run_ranks(WORKER)
    rows = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert sorted(r["rank"] for r in rows) == [0, 1]
    for r in rows:
        assert r["world"] == 2
        assert r["t"] == 2.0      # max over ranks
        assert r["rays"] == 300.0  # whole-job total


REF_WORKER = r"""
import sys, argparse
sys.path.insert(0, sys.argv[1])
import bench
args = argparse.Namespace(gpus=2, steps=1, warmup=0, ref_step_seconds=0.5)
wl = dict(bench.WORKLOADS["c1"], n=32, W=16, H=8)
bench.run_reference(args, wl)
"""


def test_reference_arm_runs_on_rank0_only():
    pytest.importorskip("torch.distributed")
    import oracle

    oracle.build()
    outs = _run_ranks(REF_WORKER)
    lines = [o.strip() for o in outs]
    printed = [l for l in lines if l]
    assert len(printed) == 1  # rank 0 prints the one JSON line, rank 1 exits without work
    d = json.loads(printed[0].splitlines()[-1])
    contract = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}
    assert contract <= set(d), contract - set(d)
    assert d["metric"].startswith("Grays/s") and d["unit"] == "Grays/s" and d["higher_is_better"] is True
    assert d["config"]["workload"].startswith("plain-32^3-16x8") and d["steps"] == 1 and d["warmup"] == 0
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
