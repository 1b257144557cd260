"""The N>1 bench path on CPU: world_size-2 gloo ranks, each timing its own
replica; the whole-job time is the slowest rank's and the whole-job work is
the sum over ranks (weak scaling, no data-path collective)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, size, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(size), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from lbm2d.replicas import Replicas
    r = Replicas()
    r.barrier()
    slowest = r.max(1.0 + rank)  # rank-local "times"
    work = r.sum(100.0 * (rank + 1))
    out.put((rank, slowest, work))
    r.close()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(2))
    assert [x[1] for x in res] == [2.0, 2.0]
    assert [x[2] for x in res] == [300.0, 300.0]


def test_single_rank_is_identity():
    from lbm2d.replicas import Replicas
    r = Replicas()
    assert r.max(3.5) == 3.5 and r.sum(2.0) == 2.0
