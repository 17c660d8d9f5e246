"""FP32-floatexp path against the plain FP64 path on the same precomputed view.

Bar: at least 99.99% of samples with the identical escape count (every sample
whose error bound certified it, plus the uncertified ones re-rendered by the
FP64 kernel), on the full C2 frame and on small views.
"""
import numpy as np
import pytest

from helpers import C2, setup_gpu, shrink

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nm():
    import newman_gb300
    newman_gb300.load_library()
    return newman_gb300


def render_pair(nm, view):
    a = setup_gpu(nm, view, path=nm.PATH_FP64)
    a.precompute()
    a.render()
    b = setup_gpu(nm, view, path=nm.PATH_FE32)
    b.precompute()
    b.render()
    return a, b


def test_fe32_matches_fp64_on_c2(nm):
    a, b = render_pair(nm, C2)
    ga, gb = a.grid(), b.grid()
    exact = (ga["iterations"] == gb["iterations"]).mean()
    rework = b.stat(nm.STAT_FP64_REWORK) / ga.size
    print("exact %.6f rework %.4f" % (exact, rework))
    assert exact >= 0.9999, exact
    assert rework < 0.10, rework
    same = ga["iterations"] == gb["iterations"]
    d = np.abs(a.smoothing64()[same] - b.smoothing64()[same])
    assert np.median(d) < 1e-6


@pytest.mark.parametrize("shape,N", [((17, 23), 3000), ((64, 96), 20000)])
def test_fe32_matches_fp64_small(nm, shape, N):
    v = shrink(C2, shape[0], shape[1], N=N)
    a, b = render_pair(nm, v)
    ga, gb = a.grid(), b.grid()
    assert (ga["iterations"] == gb["iterations"]).mean() >= 0.999


def test_fe32_counts_every_sample(nm):
    v = shrink(C2, 48, 64, N=6000)
    a, b = render_pair(nm, v)
    n = b.rows() * b.cols()
    assert b.stat(nm.STAT_SAMPLES) == n
    assert 0 <= b.stat(nm.STAT_FP64_REWORK) <= n


def test_overlapped_rework_gives_the_same_grid(nm):
    """The FP64 rework inside the iteration pass (as uncertified samples
    appear) gives the grid that the rework after the pass gives."""
    v = shrink(C2, 96, 160, N=20000)
    out = []
    for overlap in (0, 1):
        m = setup_gpu(nm, v, path=nm.PATH_FE32)
        m.set_option(nm.OPT_FE32_OVERLAP, overlap)
        m.precompute()
        m.render()
        assert m.stat(nm.STAT_WAIT_TIMEOUTS) == 0
        assert m.stat(nm.STAT_SAMPLES) == m.rows() * m.cols()
        out.append((m.grid(), m.smoothing64(), m.stat(nm.STAT_FP64_REWORK)))
    (g0, s0, n0), (g1, s1, n1) = out
    assert n0 == n1 and n0 > 0
    assert np.array_equal(g0, g1)
    assert np.array_equal(s0, s1)
