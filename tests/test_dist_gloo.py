"""The replicas-only multi-GPU path of bench.py on CPU: two gloo ranks
rendezvous the way torchrun launches them (RANK / WORLD_SIZE / MASTER_*),
meet at the timing barriers and agree on the max over ranks of their
timings; the data path has no collective."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, REPO)
    import bench
    r, w, local, pg = bench.dist()
    assert (r, w, local) == (rank, world, rank) and pg is not None
    bench.barrier(pg)
    # each rank "measures" a different time; every rank gets the max
    m = bench.reduce_max(pg, 1.0 + rank * 0.5)
    bench.barrier(pg)
    pg.destroy_process_group()
    out.put((rank, m))


def test_two_gloo_ranks_agree_on_the_max_time():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 1.5, 1: 1.5}


def test_single_process_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    r, w, local, pg = bench.dist()
    assert (r, w, local, pg) == (0, 1, 0, None)
    assert bench.reduce_max(None, 2.5) == 2.5
