"""Host logic of the several-GPU bench path, on CPU with the gloo backend
(world size 2): every rank advances its own replica, the job time is the
slowest rank's and the job value counts all ranks' cells; the reference arm
under torchrun runs on rank 0 alone and prints exactly one line."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, loc = bench.dist_env()
        ms_local = 10.0 + 5.0 * rank  # rank 1 is the slow one
        ms = bench.replica_max(torch, ms_local, dist, "cpu")
        q.put((rank, (w, r, loc), ms, bench.job_value(w, 8192 * 4096, 10, ms)))
    finally:
        dist.barrier()
        dist.destroy_process_group()


def test_replica_timing_is_the_slowest_rank():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, env, ms, value in got:
        assert env == (world, rank, rank)
        assert ms == 15.0  # both ranks see the slowest rank's time
        assert value == pytest.approx(2 * 8192 * 4096 * 10 / 15e-3)



def test_job_value_is_weak_scaling():
    # per-GPU work fixed: N ranks at the same time give N times the value
    one = bench.job_value(1, 1000, 10, 5.0)
    assert bench.job_value(4, 1000, 10, 5.0) == pytest.approx(4 * one)
    assert bench.replica_max(torch, 3.0, None, "cpu") == 3.0


def test_reference_arm_under_torchrun_prints_one_line():
    """`torchrun --nproc-per-node 2 bench.py --impl reference`: rank 0 runs the
    CPU reference on a small sample and prints one JSON line; rank 1 exits 0
    without work."""
    pytest.importorskip("oracle.oracle")
    from oracle import oracle as O
    O.build()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference", "--gpus", "2",
           "--nx", "64", "--nz", "32", "--steps", "2", "--warmup", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
