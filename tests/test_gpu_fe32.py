"""FP32-floatexp path against the plain FP64 path on the same precomputed view.

Bar: at least 99.99% of samples with the identical escape count (every sample
whose error bound certified it, plus the uncertified ones re-rendered by the
FP64 kernel), on the full C2 frame and on small views.
"""
import numpy as np
import pytest

from helpers import C1, C2, setup_gpu, shrink, step_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nm():
    import newman_gb300
    newman_gb300.load_library()
    return newman_gb300


def render_pair(nm, view):
    """The FE32 path and its comparator: the plain FP64 path, or on a view the
    reference renders with its double loop, that loop."""
    a = setup_gpu(nm, view, path=nm.PATH_FP64)
    if a.useHardware():
        a.set_path(nm.PATH_REFERENCE)
    else:
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
    v = dict(shrink(C2, 96, 160, N=20000), step=step_for("1e-14", 160))  # below the double loop
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


@pytest.mark.parametrize("view", [
    dict(C1),  # 640x480, width 3, N 1024
    dict(nr=192, nc=256, sc=1, cre=C2["cre"], cim=C2["cim"], step="2e-10", N=20000, tol=1e-10),
    dict(nr=32, nc=48, sc=1, cre="-0.1225", cim="0.7449", step="0.004", N=100000, tol=1e-10),
], ids=["C1", "seahorse-5e-8", "period3-bulb"])
def test_fe32_on_double_loop_views_matches_the_double_loop(nm, view):
    """Views the reference renders with its double loop: the FE32 path
    (perturbation from a 256-bit view-center orbit, certified against the
    double loop's own rounding as well) gives the double loop's escape
    counts; uncertified samples are rendered by the double loop itself."""
    ref = setup_gpu(nm, view)
    assert ref.useHardware()
    ref.render()
    fe = setup_gpu(nm, view, path=nm.PATH_FE32)
    fe.precompute()
    fe.render()
    a, b = ref.grid(), fe.grid()
    same = a["iterations"] == b["iterations"]
    print("exact %.6f rework %d" % (same.mean(), fe.stat(nm.STAT_FP64_REWORK)))
    assert same.mean() >= 0.9999
    assert fe.stat(nm.STAT_SAMPLES) == fe.rows() * fe.cols()
    d = np.abs(ref.smoothing64()[same] - fe.smoothing64()[same])
    assert d.size == 0 or np.median(d) < 1e-6


def test_fe32_traps_interior_orbits_of_double_loop_views(nm):
    """A double-loop view inside the minibrot next to the C2 center (the C4
    zoom's frame 8, at its sample step): the FE32 path proves most interior
    orbits trapped long before N (a small disk that the double loop maps back
    into itself) and returns the double loop's escape counts on every sample."""
    view = dict(nr=128, nc=192, sc=1, cre="-0.743643899077151", cim="0.13182583196533",
                step="3.0e-10", N=17703, tol=1e-10)
    ref = setup_gpu(nm, view)
    assert ref.useHardware()
    ref.render()
    fe = setup_gpu(nm, view, path=nm.PATH_FE32)
    fe.precompute()
    fe.render()
    a, b = ref.grid()["iterations"], fe.grid()["iterations"]
    interior = a >= view["N"]
    print("interior %.3f, executed FE32 %d, double loop %d" % (
        interior.mean(), fe.stat(nm.STAT_EXECUTED_ITERS), ref.stat(nm.STAT_EXECUTED_ITERS)))
    assert interior.mean() > 0.5
    assert np.array_equal(a, b)
    assert fe.stat(nm.STAT_EXECUTED_ITERS) < 0.75 * ref.stat(nm.STAT_EXECUTED_ITERS)


@pytest.mark.parametrize("width", ["1e-14", "1e-330"])
def test_orbit_staging_changes_nothing(nm, width):
    """The FE32 iteration pass with the orbit's first entries staged in shared
    memory by the TMA unit (1024, and 3072 -- 96 KB a block), with the
    persisting L2 window, and with neither: identical grids, and every block's
    bulk copies arrived (no block copied the entries itself)."""
    view = dict(C2, nr=96, nc=160, sc=2, step=step_for(width, 160), N=40000)
    grids = []
    for stage, l2 in ((0, 0), (1024, 0), (3072, 1)):
        m = setup_gpu(nm, view, path=nm.PATH_FE32, keep64=False)
        m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
        m.set_option(nm.OPT_ORBIT_STAGE, stage)
        m.set_option(nm.OPT_L2_WINDOW, l2)
        m.precompute()
        m.render()
        assert m.stat(nm.STAT_STAGE_FALLBACKS) == 0
        grids.append(m.grid())
    for g in grids[1:]:
        assert np.array_equal(g, grids[0])
