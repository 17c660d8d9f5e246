"""One view's rows split across ranks, one GPU per rank.

The reference renders a view row by row (computeRow, mandelbrot.cpp:269-283,
called for every row by viewer.cpp:166-171); rows are independent, so a
view shards by rows with the reference orbit and series replicated -- every
rank precomputes the same view (the same bits) and renders its own block of
rows with nm_render_rows.  The only exchange is gathering the rows to one
rank at the end, on the host (torch.distributed, any backend: gloo here).
"""
import numpy as np

from . import ESCAPE_DTYPE


def row_range(nr, rank, world):
    """Rows [r0, r1) of rank `rank` of `world`: contiguous blocks, sizes
    differing by at most one row, the larger blocks first."""
    base, extra = divmod(nr, world)
    r0 = rank * base + min(rank, extra)
    return r0, r0 + base + (1 if rank < extra else 0)


def render_shard(m, rank, world, stream=None):
    """Renders this rank's rows of the handle's view (synchronously) and
    returns them as a (r1 - r0, cols) escape-value array."""
    r0, r1 = row_range(m.rows(), rank, world)
    m.render_rows(r0, r1, stream)
    m.synchronize()
    return m.grid()[r0:r1].copy()


def gather_rows(part, nr, nc, rank, world, dst=0, group=None):
    """The whole (nr, nc) grid on rank `dst` from every rank's row block
    (None on the other ranks).  Blocks travel as bytes, padded to the largest
    block."""
    import torch
    import torch.distributed as dist
    rows_max = row_range(nr, 0, world)[1]  # rank 0 holds a largest block
    buf = np.zeros((rows_max, nc), ESCAPE_DTYPE)
    buf[:part.shape[0]] = part
    t = torch.from_numpy(buf.view(np.uint8).reshape(-1).copy())
    bufs = [torch.empty_like(t) for _ in range(world)] if rank == dst else None
    dist.gather(t, bufs, dst=dst, group=group)
    if rank != dst:
        return None
    out = np.empty((nr, nc), ESCAPE_DTYPE)
    for k in range(world):
        r0, r1 = row_range(nr, k, world)
        block = bufs[k].numpy().view(ESCAPE_DTYPE).reshape(rows_max, nc)
        out[r0:r1] = block[:r1 - r0]
    return out
