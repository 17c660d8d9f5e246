"""The allocation-free render entry point, nm_render_fe32_noalloc.

Callers that cannot allocate device memory when they render -- code that
records its GPU work by stream capture, or a process whose device memory is
owned by another framework's allocator -- pass their own output buffer and
get the FP32-floatexp render of a prepared handle, with the kernels' scratch
taken from a static device array.  Its output must equal the allocating
entry point's (nm_render on the same handle): escape counts exactly, float
smoothing within 1e-6, on two calls in a row.

This file sorts last so that a run stopping at its first failure has already
run every other test.
"""
import ctypes

import numpy as np
import pytest

from helpers import C2, setup_gpu, shrink, step_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nm():
    import newman_gb300
    newman_gb300.load_library()
    return newman_gb300


def test_noalloc_matches_allocating_render(nm):
    torch = pytest.importorskip("torch")
    # 540 x 960 samples at width 1e-14: a view below the double loop's range
    view = dict(shrink(C2, 135, 240, N=20000), step=step_for("1e-14", 240))
    m = setup_gpu(nm, view, path=nm.PATH_FE32, keep64=False)
    m.precompute()
    m.upload()
    m.render()
    ref = m.grid().copy()
    rows, cols = m.rows(), m.cols()

    # caller-owned output: 8 bytes per sample
    out = torch.empty(rows * cols * 2, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):
        out.fill_(-7)
        m.render_noalloc(ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        stream.synchronize()
        got = out.cpu().numpy().view(nm.ESCAPE_DTYPE).reshape(rows, cols)
        assert np.array_equal(got["iterations"], ref["iterations"]), "call %d" % call
        assert np.abs(got["smoothing"] - ref["smoothing"]).max() <= 1e-6, "call %d" % call

    # a further call takes no device memory
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    m.render_noalloc(ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    stream.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before


def test_noalloc_refuses_oversize_and_unprepared(nm):
    big = nm.Mandelbrot(2048, 2049)  # 4,196,352 samples > 4,194,304
    with pytest.raises(nm.NewmanError) as e:
        big.render_noalloc(ctypes.c_void_p(1))
    assert e.value.code == nm.NM_ERR_ARG
    assert "4194304" in str(e.value)
    small = nm.Mandelbrot(8, 8)
    with pytest.raises(nm.NewmanError) as e:
        small.render_noalloc(ctypes.c_void_p(1))
    assert e.value.code == nm.NM_ERR_STATE


@pytest.mark.parametrize("width", ["1e-8", "6e-8"])
def test_noalloc_on_double_loop_views(nm, width):
    """Views where the reference takes its double loop: at a sample step below
    2^-33 (width 1e-8 on 240 columns) the FE32 path renders them with the
    double loop itself; above it (6e-8) with FE32 perturbation certified
    against the double loop, reworked by it.  Both through the allocation-free
    entry point must give nm_render's escape counts on the same handle."""
    torch = pytest.importorskip("torch")
    view = dict(shrink(C2, 90, 120, N=6000), step=step_for(width, 240), sc=2)
    m = setup_gpu(nm, view, path=nm.PATH_FE32, keep64=False)
    assert m.useHardware()
    m.precompute()
    m.upload()
    m.render()
    ref = m.grid().copy()
    rows, cols = m.rows(), m.cols()
    out = torch.empty(rows * cols * 2, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):
        out.fill_(-7)
        m.render_noalloc(ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        stream.synchronize()
        got = out.cpu().numpy().view(nm.ESCAPE_DTYPE).reshape(rows, cols)
        assert np.array_equal(got["iterations"], ref["iterations"]), "call %d" % call
        assert np.abs(got["smoothing"] - ref["smoothing"]).max() <= 1e-6, "call %d" % call
