"""bench.py's multi-rank path on the CPU: two gloo ranks (the replicas of a
torchrun launch) agree on the slowest rank's time, the job throughput counts
every rank's frames, and the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
rank, local, world = bench.dist_env()
dist.init_process_group("gloo", init_method="env://")
mine = 100.0 + 50.0 * rank
bench.barrier_sync(world)
total = bench.max_over_ranks(mine, world, device="cpu")
fps = bench.job_frames_per_s(1024, 20, world, total)
print(json.dumps({{"rank": rank, "total": total, "fps": fps}}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_ranks(code, world, extra_env=None):
    port = free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(world),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), **(extra_env or {}))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, cwd=ROOT,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        outs.append(out)
    return outs


def test_two_gloo_ranks_take_the_slowest_time():
    import json
    outs = run_ranks(WORKER.format(root=ROOT), 2)
    lines = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert {l["rank"] for l in lines} == {0, 1}
    assert all(l["total"] == 150.0 for l in lines)             # max over ranks
    assert all(abs(l["fps"] - 1024 * 20 * 2 / 0.150) < 1e-6 for l in lines)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2"], cwd=ROOT,
                       env=env, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0 and p.stdout.strip() == ""


def test_reference_arm_json_line():
    """The reference arm on rank 0 (a few envs of config1 through the CPU
    oracle) prints one JSON line with the contract's keys, its own e2e and a
    cpu_baseline describing the run."""
    import json
    env = dict(os.environ, RANK="0", LOCAL_RANK="0", WORLD_SIZE="1")
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                        "--envs", "8", "--cpu-seconds", "0.5"], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 1
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
