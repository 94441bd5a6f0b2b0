"""bench.py's multi-GPU path is replicas only: each rank solves its own copy,
the only cross-rank step is the max of the timings.  Checked here with two
gloo ranks on the CPU (the GPU runs in this project have one GPU each)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(0.5 + rank, dist, "cpu")
    rate = bench.replica_rate(world, 1000, 4, 10, t)
    out.put((rank, t, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [1.5, 1.5]
    assert all(r[2] == pytest.approx(2 * 1000 * 4 * 10 / 1.5) for r in res)


def test_single_process_is_identity():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.25, None, "cpu") == 0.25
    assert bench.replica_rate(1, 100, 4, 5, 2.0) == 1000.0
