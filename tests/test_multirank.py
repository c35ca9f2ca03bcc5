"""The bench's multi-rank path on CPU (gloo, world size 2): the max-over-ranks
timing and the barrier, and the reference arm under torchrun (rank 0 alone
runs and prints one line, the other rank exits cleanly).  Multi-GPU runs are
independent replicas, so these host-side pieces are all the N > 1 path has."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      UNAP_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        pass

    world_, rank_, _, dist = bench.dist_setup(Args())
    assert (world_, rank_) == (world, rank)
    bench.barrier(dist)
    m = bench.max_over_ranks(0.5 + rank, dist)
    bench.barrier(dist)
    dist.destroy_process_group()
    out.put((rank, m))


def test_max_over_ranks_and_barrier_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 1.5, 1: 1.5}


def test_reference_arm_under_torchrun():
    pytest.importorskip("torch")
    env = dict(os.environ, UNAP_BENCH_BACKEND="gloo")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "3", "--scale", "0.08"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
