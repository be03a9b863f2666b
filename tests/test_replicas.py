"""The multi-GPU path of bench.py on CPU: replicas only (each rank solves its
own field, no collective on the data path), with a barrier around the timed
region and the step time taken as the maximum over ranks.  Two gloo ranks on
127.0.0.1 stand in for two GPUs; the reference arm under torchrun prints one
line from rank 0 while the other rank exits 0 without work."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import argparse

    import bench
    import torch.distributed as dist

    args = argparse.Namespace(impl="reference")
    w, r, local = bench.dist_setup(args)
    bench.barrier(w)
    # each rank's own step time; the job's time is the slowest rank's
    t = bench.max_over_ranks(1.5 + r, w)
    bench.barrier(w)
    dist.destroy_process_group()
    q.put((r, w, local, t))


def test_two_gloo_ranks_take_the_max_step_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[3] == 2.5 for o in out)  # max(1.5, 2.5) on both ranks


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import argparse

    import bench

    w, r, local = bench.dist_setup(argparse.Namespace(impl="reference"))
    assert (w, r, local) == (1, 0, 0)
    assert bench.max_over_ranks(3.25, w) == 3.25
    bench.barrier(w)  # no-op


def test_reference_arm_under_torchrun_prints_one_line_from_rank_0():
    port = _free_port()
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0"]
    res = subprocess.run(cmd, cwd=ROOT, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0
