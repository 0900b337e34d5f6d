"""bench.py's multi-rank host logic on CPU with gloo ranks (world size 2):
the rank environment, the max-over-ranks time, the weak-scaling value, and
the reference arm under torchrun (rank 0 alone measures and prints)."""
import json
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


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        env = bench.dist_env()
        t = bench.max_over_ranks(10.0 + 3.0 * rank, world)
        v = bench.weak_value(world, 1000, 5, t)
        out.put((rank, env, t, v))
    finally:
        dist.destroy_process_group()


def test_two_ranks_max_time_and_weak_value():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [(0, 2, 0), (1, 2, 1)]
    assert all(r[2] == 13.0 for r in res)  # the slower rank's time on both
    assert all(r[3] == pytest.approx(2 * 1000 * 5 / 0.013) for r in res)


def test_single_rank_is_its_own_max():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.5, 1) == 7.5
    assert bench.weak_value(1, 10, 2, 1000.0) == pytest.approx(20.0)


def test_reference_arm_under_torchrun_two_ranks():
    """Rank 0 alone times the reference CPU path and prints one JSON line;
    rank 1 exits 0 without work."""
    import oracle
    try:
        oracle.Oracle("reference")
    except Exception as e:  # the reference-built oracle is absent
        pytest.skip("reference oracle not built: %s" % e)
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--size", "24",
           "--cpu-seconds", "0.05"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300,
                       env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0
