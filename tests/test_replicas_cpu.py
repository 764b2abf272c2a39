"""The N > 1 path of bench.py on CPU: two gloo ranks (replicas only, as the
path shards with no exchange step).  Checks the rendezvous, the max-over-
ranks timing every rank reports, and that the reference arm's non-zero
ranks leave without work."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class Args:
    impl = "reference"


def worker(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    r, w, local, pg = bench.dist_setup(Args())
    try:
        slowest = bench.max_over_ranks(pg, 1.0 + r, torch.device("cpu"))
        ran = bench.run_reference(Args(), r, w, pg) if r != 0 else None
        out.put((r, w, local, slowest, ran))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in results] == [0, 1]
    assert all(r[1] == world and r[0] == r[2] for r in results)
    assert all(r[3] == 2.0 for r in results)          # every rank reports the slowest rank's time
    assert results[1][4] is None                       # rank 1 of the reference arm does no work


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 3.5, "cpu") == 3.5
