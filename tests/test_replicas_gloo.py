"""Multi-GPU runs of the build are independent replicas (one tree per rank, no data-path
collective). The host-side pieces of that path run here as two gloo ranks on the CPU: the
max-over-ranks timing reduction, the barrier, and the whole-job throughput."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    import bench

    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(world)
    ms = bench.reduce_max([10.0 + rank, 5.0 - rank], world)
    value = bench.replica_throughput(16_000_000, ms[0], world)
    out[rank] = (ms, value)
    dist.destroy_process_group()


def test_two_replicas_reduce_to_the_slowest_rank():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        ms, value = out[r]
        assert ms == [11.0, 5.0]
        assert value == pytest.approx(2 * 16_000_000 / 0.011)
