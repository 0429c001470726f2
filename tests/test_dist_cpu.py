"""Multi-process host logic of bench.py on CPU (gloo, world size 2).

The summators shard by points with no data-path collective; under torchrun
every rank runs its own workload (weak scaling), the ranks meet at barriers
and rank 0 reports the maximum step time over ranks.  This checks that logic
without a GPU.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    mx = bench.max_over_ranks(world, float(10 + rank))
    # shard helper: every rank gets a disjoint, covering slice of the points
    lo, hi = bench.shard_range(1001, rank, world)
    q.put((rank, mx, lo, hi))
    bench.barrier(world)
    dist.destroy_process_group()


def test_max_over_ranks_and_sharding_gloo():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [11.0, 11.0]
    spans = [(r[2], r[3]) for r in res]
    assert spans[0][0] == 0 and spans[-1][1] == 1001
    assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
