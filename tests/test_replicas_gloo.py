"""The N-GPU replica path on CPU: two gloo ranks, max-over-ranks timing and
whole-job throughput (no GPU; the data path has no collective)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from thindb_gb300 import replicas

    local = 10.0 + 5.0 * rank  # rank 1 is the slowest
    slow = replicas.slowest_ms(local, dist)
    out[rank] = (slow, replicas.job_rows_per_s(1_000_000, world, slow))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        slow, value = res[r]
        assert slow == 15.0
        assert value == pytest.approx(2 * 1_000_000 / 0.015)


def test_single_rank_needs_no_process_group():
    from thindb_gb300 import replicas

    assert replicas.slowest_ms(3.5) == 3.5
    assert replicas.job_rows_per_s(100, 1, 1.0) == pytest.approx(100_000)
