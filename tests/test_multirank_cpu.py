"""Multi-rank paths of bench.py on CPU (gloo): the single case runs as replicas and the batched
sweep shards by case across ranks with no data-path collective; the only collectives are the
timing barrier and the max over ranks of the timed interval."""

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(REPO))
    import bench

    class A:
        pass

    world_, rank_, _, dist = bench.dist_setup(A())
    assert (world_, rank_) == (world, rank)
    bench.barrier(dist)
    mx = bench.reduce_max(dist, 10.0 + rank)
    pick, alphas, machs = bench.c4_draw(rank)
    out.put((rank, mx, pick.tolist(), float(alphas[0]), float(machs[0])))
    dist.destroy_process_group()


def test_gloo_two_ranks_max_reduction_and_case_sharding():
    import torch.multiprocessing as tmp

    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [11.0, 11.0]  # every rank sees the slowest rank's time
    assert got[0][2:] != got[1][2:]            # each rank draws its own share of the sweep
    sys.path.insert(0, str(REPO))
    import bench

    again = bench.c4_draw(1)
    assert again[0].tolist() == got[1][2] and float(again[1][0]) == got[1][3]  # seeded per rank


def test_reference_arm_under_torchrun_prints_one_line_from_rank0():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "3", "--mesh", "32", "8", "--cpu-procs", "2"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    res = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["cores"] == 2 and line["e2e"]["h2d_bytes_per_step"] == 0
