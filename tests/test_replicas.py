"""The N > 1 host path of bench.py on CPU: replicas only (every rank runs its
own shot; no data-path collective), with the timing reduced as the maximum
over ranks through torch.distributed (gloo here, NCCL on GPUs)."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench._dist()
    assert (ws, r, local) == (world, rank, rank)
    # each rank reports its own time; every rank gets the slowest
    out[rank] = bench._barrier_max(10.0 + rank, ws)
    bench._barrier(ws)
    dist.destroy_process_group()


def test_two_rank_timing_is_the_maximum():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        procs = [mp.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert dict(out) == {0: 11.0, 1: 11.0}


def test_single_rank_needs_no_process_group():
    import bench
    assert bench._barrier_max(3.5, 1) == 3.5
    bench._barrier(1)
