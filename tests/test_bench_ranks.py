"""The replica path of bench.py (N>1 GPUs, one process per GPU) reduced on
CPU with the gloo backend, world size 2: the spans are the maximum over
ranks and the work the sum over ranks."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.combine_ranks(1.0 + rank, 2.0 * (1 + rank), 100, world, device="cpu")
    finally:
        dist.destroy_process_group()


def test_combine_ranks_gloo_world2():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        assert out[0] == (2.0, 4.0, 200) and out[1] == (2.0, 4.0, 200)


def test_combine_ranks_single():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.combine_ranks(1.5, 2.5, 7, 1) == (1.5, 2.5, 7)
