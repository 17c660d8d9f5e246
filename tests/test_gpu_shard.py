"""One view's rows split across two processes on the same GPU (each a rank
of a gloo group; their kernels are independent), gathered to rank 0: the
gathered grid must equal one process's render of the whole view, bit for
bit.  Each rank precomputes the same view itself (the orbit and series are
replicated, not sent)."""
import os
import socket
import sys

import numpy as np
import pytest

from helpers import C2, step_for

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# deep: sample step 1e-14 / 960
VIEW = dict(C2, nr=270, nc=480, sc=2, step=step_for("1e-14", 480), N=20000)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _make(nm, path):
    m = nm.Mandelbrot(VIEW["nr"], VIEW["nc"])
    m.set_view(VIEW["cre"], VIEW["cim"], VIEW["step"], VIEW["step"], VIEW["N"], VIEW["tol"])
    m.scaleUp(VIEW["sc"])
    m.set_path(path)
    return m


def _rank(rank, world, port, path, out_file):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import newman_gb300 as nm
    from newman_gb300.shard import gather_rows, render_shard
    m = _make(nm, path)
    m.precompute()
    part = render_shard(m, rank, world)
    full = gather_rows(part, m.rows(), m.cols(), rank, world)
    if rank == 0:
        np.save(out_file, full)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("path_name", ["PATH_FE32", "PATH_MP"])
def test_row_shards_equal_whole_render(tmp_path, path_name):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import newman_gb300 as nm
    nm.load_library()
    path = getattr(nm, path_name)
    ctx = mp.get_context("spawn")  # never a fork of a process that holds CUDA
    out_file = str(tmp_path / "gathered.npy")
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, path, out_file)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=600)
        assert p.exitcode == 0
    m = _make(nm, path)
    m.precompute()
    m.render()
    assert np.array_equal(np.load(out_file), m.grid())
