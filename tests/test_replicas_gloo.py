"""The multi-process path of bench.py ("replicas only": every rank advances
its own grid, no exchange on the data path) on CPU with the gloo backend at
world size 2: the reported time is the slowest rank's, and the whole-job
value counts every rank's cells."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    local_ms = [3.0, 5.0][rank]
    cells = 1000
    ms = bench.max_over_ranks(local_ms, dist, "cpu")
    value = world * cells / (ms * 1e-3)
    out.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_with_gloo_world_size_2():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in got:
        assert ms == 5.0
        assert value == 2 * 1000 / 5e-3


def test_single_process_is_unchanged():
    import bench

    assert bench.max_over_ranks(4.0, None) == 4.0
