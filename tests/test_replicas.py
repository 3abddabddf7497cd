"""Multi-process paths of bench.py on CPU (gloo, world size 2).

The solve does not shard: with N GPUs bench.py runs N independent replicas
of the same workload, one process per GPU, with no collective on the data
path.  What the ranks share is the timing protocol -- a barrier on both
sides of the timed region and the maximum of the per-rank times -- and the
rule that rank 0 alone prints (and, for --impl reference, alone runs).
These tests exercise exactly that host logic with the gloo backend.
"""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    r, w, local = bench.dist_setup()
    assert (r, w, local) == (rank, world, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    # every rank reports its own time; all ranks agree on the slowest
    m = bench.max_over_ranks(0.25 * (rank + 1), w)
    bench.barrier(w)
    out.put((rank, m))
    dist.destroy_process_group()


def test_barrier_and_max_over_ranks_on_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert got == [(0, 0.5), (1, 0.5)]


def test_reference_arm_runs_on_rank_zero_only():
    """`bench.py --impl reference` under torchrun with two ranks: rank 0
    runs the oracle's CPU PCG+DIC sample and prints one JSON line; rank 1
    exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--size", "8", "--steps", "1", "--warmup", "0"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    # the iteration count the sample extrapolates to comes from a full solve
    # run first, and the config carries the same keys as the GPU arm's
    assert line["extrapolated"] is True and line["full_solve"]["converged"]
    assert line["full_solve"]["iterations"] > 1
    import argparse

    sys.path.insert(0, ROOT)
    import bench

    a = argparse.Namespace(n=8, rel_tol=1e-10)
    assert line["config"] == bench.headline_config(a, 512, 3 * 8 * 8 * 7, 2)


if __name__ == "__main__":
    pytest.main([__file__, "-q"])
