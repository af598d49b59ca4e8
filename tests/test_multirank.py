"""The N > 1 path of bench.py on CPU: two gloo ranks (replicas, no data exchange) agree
on the slowest rank's time, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

sys.path.insert(0, str(ROOT))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.slowest_rank(dist, 1.0 + rank * 0.5)  # rank 1 is the slow one
    # value = units of all ranks over the slowest rank's time (weak scaling, replicas)
    units = 2_000_000
    rate = world * units / t
    ref = bench.run_reference(None, world, rank) if rank != 0 else "rank0"
    q.put((rank, t, rate, ref))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [1.5, 1.5]
    assert all(abs(o[2] - 2 * 2_000_000 / 1.5) < 1e-6 for o in out)
    assert out[1][3] is None  # the reference arm does no work off rank 0
