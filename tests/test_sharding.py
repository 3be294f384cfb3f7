"""Sharding an ensemble over ranks (fsibe_2d_gb300.sharding): the cost-balanced partition,
and the host-side gather in global run order over two gloo ranks on the CPU.  The runs'
GPU work is replaced by a stand-in (each rank evaluates a function of the run index): the
data path has no exchange, so the gather is the only multi-rank step."""
import os
import socket

import pytest

from fsibe_2d_gb300 import make_params
from fsibe_2d_gb300.sharding import partition, run_cost, gather_by_index


def _batched_configuration():
    return [make_params(nx=n, ny=n, ns=n // 4) for n, c in ((256, 48), (512, 12), (1024, 4)) for _ in range(c)]


def test_partition_covers_every_run_once_and_balances_cost():
    ps = _batched_configuration()
    for world in (1, 2, 3, 4, 8):
        share = partition(ps, world)
        assert sorted(i for s in share for i in s) == list(range(len(ps)))
        loads = [sum(run_cost(ps[i]) for i in s) for s in share]
        # the LPT bound: no rank above the mean by more than the largest single run
        assert max(loads) <= sum(loads) / world + max(run_cost(p) for p in ps) + 1e-6
        assert partition(ps, world) == share               # deterministic
    # four 1024^2 runs on four ranks: one each
    share = partition(ps, 4)
    big = [i for i, p in enumerate(ps) if p.nx == 1024]
    assert sorted(sum(i in s for i in big) for s in share) == [1, 1, 1, 1]


def test_partition_with_more_ranks_than_runs():
    ps = [make_params(nx=64, ny=64, ns=16) for _ in range(3)]
    share = partition(ps, 5)
    assert sum(len(s) for s in share) == 3 and sum(1 for s in share if not s) == 2


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ps = _batched_configuration()
        share = partition(ps, world)[rank]
        local = [float(i) * 10.0 + ps[i].nx for i in share]      # the stand-in of a run's result
        out = gather_by_index(local, share, world, len(ps))
        parts = [None] * world
        dist.all_gather_object(parts, partition(ps, world))
        q.put((rank, out, all(p == parts[0] for p in parts)))
    finally:
        dist.destroy_process_group()


def test_gather_in_global_order_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ps = _batched_configuration()
    want = [float(i) * 10.0 + ps[i].nx for i in range(len(ps))]
    for rank, out, same in res:
        assert same and out == want
