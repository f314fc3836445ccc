"""The bench's multi-process host logic on CPU: two ranks over gloo (127.0.0.1) join the
process group, meet at the barrier, and agree on the maximum of their timings (the job's
time is the slowest replica's)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank), NBKDT_DIST_BACKEND="gloo")
    import bench
    import torch.distributed as dist
    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank)
    bench.barrier(w)
    out[rank] = bench.max_over_ranks(1.5 + rank, w)
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        procs = [mp.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        assert dict(out) == {0: 2.5, 1: 2.5}
