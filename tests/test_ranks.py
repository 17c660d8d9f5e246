"""The multi-rank path of bench.py on the host: two gloo ranks (world size 2,
CPU) agree on the slowest rank's step time and report the whole job's
throughput of independent replicas (every rank renders the full view)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    w, r, _ = bench.dist_setup()
    ms = bench.max_over_ranks(100.0 + 50.0 * rank)  # rank 1 is the slower replica
    value = bench.replica_value(1_000_000, w, ms)
    out.put((r, w, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[0] for g in got] == [0, 1]
    for r, w, ms, value in got:
        assert w == 2
        assert ms == 150.0  # both ranks see the slowest rank's time
        assert value == pytest.approx(2 * 1_000_000 / 0.150)


def test_single_rank_is_its_own_maximum():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.replica_value(10, 1, 1000.0) == pytest.approx(10.0)


def test_row_ranges_cover_the_view_once():
    sys.path.insert(0, ROOT)
    from newman_gb300.shard import row_range
    for nr in (1, 7, 1080, 4320):
        for world in (1, 2, 3, 8):
            spans = [row_range(nr, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == nr
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [r1 - r0 for r0, r1 in spans]
            assert max(sizes) - min(sizes) <= 1 and sizes[0] == max(sizes)


def _gather_rank(rank, world, port, nr, nc, out):
    import numpy as np
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from newman_gb300 import ESCAPE_DTYPE
    from newman_gb300.shard import gather_rows, row_range
    r0, r1 = row_range(nr, rank, world)
    part = np.zeros((r1 - r0, nc), ESCAPE_DTYPE)  # stands in for this rank's rendered rows
    part["iterations"] = np.arange(r0, r1)[:, None] * 1000 + np.arange(nc)[None, :]
    part["smoothing"] = rank + 0.5
    full = gather_rows(part, nr, nc, rank, world)
    if rank == 0:
        ok = bool((full["iterations"] == np.arange(nr)[:, None] * 1000 + np.arange(nc)).all())
        owner = np.concatenate([np.full(row_range(nr, k, world)[1] - row_range(nr, k, world)[0],
                                        k + 0.5) for k in range(world)])
        ok = ok and bool((full["smoothing"] == owner[:, None]).all())
        out.put(ok)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,nr", [(2, 7), (3, 10)])
def test_row_shards_gather_to_rank_zero(world, nr):
    """Row blocks of a view gathered from gloo ranks on the host land in the
    right rows of rank 0's grid (ragged blocks included)."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gather_rank, args=(r, world, port, nr, 5, q))
             for r in range(world)]
    for p in procs:
        p.start()
    assert q.get(timeout=120) is True
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
