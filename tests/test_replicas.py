"""Multi-process path of bench.py on the CPU (gloo, world size 2).

The data path shards into replicas with no collective: each rank runs its own
domain, and the host synchronises only for the timed region (a barrier on
both sides) and the max over ranks of the elapsed time.  These tests run
that host logic in two gloo processes, and the reference arm under torchrun
(rank 0 alone measures and prints; the other rank exits 0 without work).
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ranks = bench.Ranks(dist)
    ranks.barrier()
    elapsed = [0.75, 1.25][rank]  # seconds each replica took
    slowest = ranks.max(elapsed)
    ranks.barrier()
    value = bench.aggregate_mlups(world, 1000, 10, slowest)
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as fh:
        json.dump({"slowest": slowest, "value": value}, fh)
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for rank in range(2):
        got = json.load(open(tmp_path / ("rank%d.json" % rank)))
        assert got["slowest"] == 1.25
        # two replicas of 1000 cells x 10 steps in 1.25 s
        assert got["value"] == pytest.approx(2 * 1000 * 10 / 1.25 / 1e6)


def test_single_process_ranks_are_noops():
    sys.path.insert(0, ROOT)
    import bench
    r = bench.Ranks(None)
    r.barrier()
    assert r.max(3.5) == 3.5
    assert bench.aggregate_mlups(1, 512 ** 3, 400, 2.0) == pytest.approx(512 ** 3 * 400 / 2.0 / 1e6)


def test_reference_arm_under_torchrun(tmp_path):
    port = _free_port()
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "3", "--size", "32"]
    p = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["n_gpus"] == 2 and line["steps"] == 1 and line["warmup"] == 3
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port"
    # the same workload description as the GPU arm's line
    assert line["config"] == bench_config(32, line["config"]["tau"], 2)


def bench_config(n, tau, world):
    sys.path.insert(0, ROOT)
    import bench
    return bench.roofline_config(n, tau, world)


def test_reference_arm_same_input_as_gpu_arm():
    """Both arms draw the roofline input from the same seed: tau is the
    seed's first draw, so every grid size of the recipe has the same tau."""
    sys.path.insert(0, ROOT)
    import bench
    t32 = bench.make_inputs(8)[0]
    t64 = bench.make_inputs(16)[0]
    assert t32 == t64 and 0.55 <= t32 <= 1.5
