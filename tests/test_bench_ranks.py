"""The multi-GPU path is replicas (queries shard by query, no collective on
the data path); its only cross-rank step is the timing reduction of
bench.py, checked here with two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t_dev, wall, n = bench.reduce_over_ranks(dist, torch, 1.0 + rank, 2.0 + 3 * rank,
                                             1000, "cpu")
    q.put((rank, t_dev, wall, n))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_reduction_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_dev, wall, n in out:
        assert t_dev == 2.0 and wall == 5.0 and n == 2000


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the CPU port on the host cores) prints one
    JSON line with the arm's keys; a small bounded sample keeps it short."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--batch", "4", "--ref-sample", "4",
                        "--node-budget", "300"],
                       cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "cpu_baseline", "e2e", "config"):
        assert k in line, k
    # value counts exact answers only; the sample ran under the same budget
    assert line["value"] >= 0 and line["config"]["all_answers_per_s"] > 0
    assert line["ms_per_step"] > 0 and line["config"]["sample_per_step"] == 4
    assert line["config"]["node_budget"] == 300 and line["config"]["wall_cap"] is None
    assert line["config"]["nproc"] >= 1
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
