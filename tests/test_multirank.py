"""The bench's multi-rank plumbing on the CPU: world_size-2 gloo ranks on 127.0.0.1 (the path the
GPU runs take under torchrun with one replica per GPU): the barrier and the max over ranks of the
timed region."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      LOCAL_RANK=str(rank))
    import bench
    r, w, td = bench.dist_init()
    try:
        bench.barrier(td)
        out.put((r, w, bench.allmax(td, 1.5 + r)))
    finally:
        td.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 2.5), (1, 2, 2.5)]

