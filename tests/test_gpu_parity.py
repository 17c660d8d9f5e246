"""GPU kernels against the oracle, through the C ABI (ctypes), on the same views.

Bar: escape counts bit-exact; unrounded smoothing within 1e-12 (CUDA's log /
log2 against glibc's); float smoothing within 1e-6.
"""
import numpy as np
import pytest

from helpers import C1, C2, sample_positions, setup_gpu, setup_oracle, shrink

pytestmark = pytest.mark.gpu

SMOOTH_TOL = 1e-12


@pytest.fixture(scope="module")
def nm():
    import newman_gb300
    newman_gb300.load_library()
    return newman_gb300


def _compare(it_gpu, sm_gpu, it_ref, sm_ref):
    mism = np.flatnonzero(it_gpu.ravel() != it_ref.ravel())
    assert mism.size == 0, "escape counts differ at %d samples, first %s: gpu %s ref %s" % (
        mism.size, mism[:5], it_gpu.ravel()[mism[:5]], it_ref.ravel()[mism[:5]])
    d = np.abs(sm_gpu.ravel() - sm_ref.ravel())
    assert d.max() <= SMOOTH_TOL, "max smoothing difference %g" % d.max()


def test_c1_full_frame_bit_exact(nm, oracle_mod):
    """640x480 at -0.75+0i, width 3, N 1024: the reference's double path."""
    m = setup_gpu(nm, C1)
    assert m.useHardware()
    m.precompute()
    m.render()
    g = m.grid()
    s64 = m.smoothing64()
    o = setup_oracle(oracle_mod, C1)
    it, sm = o.render_rows(0, C1["nr"])
    _compare(g["iterations"], s64, it, sm)
    assert np.abs(g["smoothing"] - sm.astype(np.float32)).max() <= 1e-6
    assert m.stat(nm.STAT_SAMPLES) == C1["nr"] * C1["nc"]
    assert (g["iterations"] == C1["N"]).mean() > 0.2  # cardioid + bulbs present


def test_c1_compute_row_matches_full_render(nm):
    m = setup_gpu(nm, C1)
    m.render()
    full = m.grid().copy()
    m2 = setup_gpu(nm, C1)
    for r in (0, 1, 239, 240, 479):
        m2.computeRow(r)
    g2 = m2.grid()
    for r in (0, 1, 239, 240, 479):
        assert np.array_equal(g2[r], full[r])
    assert np.all(g2[2]["iterations"] == 0)  # untouched rows stay zero


@pytest.mark.parametrize("tile", [(16, 16), (32, 4), (7, 5)])
def test_ragged_grids_and_tiles(nm, oracle_mod, tile):
    for nr, nc in [(1, 1), (7, 13), (33, 65)]:
        v = shrink(C1, nr, nc, N=300)
        m = setup_gpu(nm, v)
        m.set_option(nm.OPT_TILE_W, tile[0])
        m.set_option(nm.OPT_TILE_H, tile[1])
        m.render()
        o = setup_oracle(oracle_mod, v)
        it, sm = o.render_rows(0, nr)
        _compare(m.grid()["iterations"], m.smoothing64(), it, sm)


@pytest.mark.parametrize("N", [1, 2, 17])
def test_small_iteration_counts(nm, oracle_mod, N):
    v = shrink(C1, 40, 56, N=N)
    m = setup_gpu(nm, v)
    m.render()
    o = setup_oracle(oracle_mod, v)
    it, sm = o.render_rows(0, 40)
    _compare(m.grid()["iterations"], m.smoothing64(), it, sm)


def test_interior_view_all_N(nm):
    """A view inside the main cardioid: every sample returns N, smoothing 0."""
    v = dict(nr=24, nc=32, sc=1, cre="-0.1", cim="0.1", step="0.001", N=5000, tol=1e-10)
    m = setup_gpu(nm, v)
    m.render()
    g = m.grid()
    assert np.all(g["iterations"] == 5000) and np.all(g["smoothing"] == 0)


def test_period3_bulb_cycle_detection_bit_exact(nm, oracle_mod):
    """A view across the period-3 bulb (outside the cardioid test), N 100,000:
    the double loop's exact cycle detection ends the interior samples early and
    every escape count still equals the oracle's full-length loop."""
    v = dict(nr=32, nc=48, sc=1, cre="-0.1225", cim="0.7449", step="0.004", N=100000,
             tol=1e-10)
    m = setup_gpu(nm, v)
    assert m.useHardware()
    m.render()
    g = m.grid()
    o = setup_oracle(oracle_mod, v)
    it, sm = o.render_rows(0, v["nr"])
    _compare(g["iterations"], m.smoothing64(), it, sm)
    interior = (g["iterations"] == v["N"]).mean()
    assert interior > 0.3
    # most of the interior samples stopped well before N
    effective = int(g["iterations"].astype(np.int64).sum())
    assert m.stat(nm.STAT_EXECUTED_ITERS) < 0.2 * effective


def test_multisample_reduce_bit_exact(nm, oracle_mod):
    v = dict(C1, nr=60, nc=80, step="0.0375")
    v["sc"] = 3
    m = setup_gpu(nm, v)
    m.render()
    samples = m.grid()
    red = m.reduce(3)
    oi, osm = oracle_mod.reduce(samples["iterations"], samples["smoothing"], 3)
    assert np.array_equal(red["iterations"], oi)
    assert np.array_equal(red["smoothing"].view(np.int32), osm.view(np.int32))
    # scaleDown replaces the grid by the same values; at(r, c, sc) agrees too
    r, c = 17, 23
    assert m.at(r, c, 3) == (int(oi[r, c]), float(osm[r, c]))
    m.scaleDown(3)
    assert m.rows() == 60 and m.cols() == 80
    assert np.array_equal(m.grid(), red)
    m.scaleUp(2)
    up = m.grid()
    assert np.array_equal(up[::2, ::2], red) and np.array_equal(up[1::2, 1::2], red)


@pytest.fixture(scope="module")
def c2_pair(nm, oracle_mod):
    """The full 4320x7680-sample C2 frame on the FP64 perturbation path."""
    m = setup_gpu(nm, C2, path=nm.PATH_REFERENCE)
    assert not m.useHardware()
    m.precompute()
    o = setup_oracle(oracle_mod, C2)
    o.precompute()
    assert m.stat(nm.STAT_ORBIT_LENGTH) == o.orbit_length
    assert m.stat(nm.STAT_PROBE_INDEX) == o.probe_index
    m.render()
    return m, o


def test_c2_fp64_path_matches_fp64_oracle(nm, oracle_mod, c2_pair):
    m, o = c2_pair
    g = m.grid()
    s64 = m.smoothing64()
    rows, cols = sample_positions(m.rows(), m.cols(), 4000, seed=1)
    it, sm = o.render_pixels(rows, cols, oracle_mod.MODE_DELTA)
    _compare(g["iterations"][rows, cols], s64[rows, cols], it, sm)


def test_c2_fp64_path_vs_arbitrary_precision_reference(nm, oracle_mod, c2_pair):
    """FP64 perturbation against the reference's MP continuation.  The view is
    chaotic at the sample scale: a rounding change of 1 ulp (FP64 with or
    without FMA) already moves 0.14% of escape counts, and the MP
    continuation differs from any FP64 iteration on ~0.8% of samples.  So
    the bar here is agreement on >= 98.5% of samples, and the median
    smoothing difference is at perturbation accuracy."""
    m, o = c2_pair
    g = m.grid()
    rows, cols = sample_positions(m.rows(), m.cols(), 1500, seed=2)
    it, sm = o.render_pixels(rows, cols, oracle_mod.MODE_REF)
    agree = (g["iterations"][rows, cols] == it).mean()
    assert agree >= 0.985, agree
    d = np.abs(m.smoothing64()[rows, cols] - sm)
    assert np.median(d) < 1e-6


def test_c2_reduce_and_row_range(nm, oracle_mod, c2_pair):
    m, o = c2_pair
    g = m.grid()
    red = m.reduce(4)
    oi, osm = oracle_mod.reduce(g["iterations"], g["smoothing"], 4)
    assert np.array_equal(red["iterations"], oi)
    assert np.array_equal(red["smoothing"].view(np.int32), osm.view(np.int32))
    # a row range rendered alone equals the same rows of the full render
    m2 = setup_gpu(nm, C2)
    m2.precompute()
    m2.render_rows(1000, 1013)
    m2.synchronize()
    assert np.array_equal(m2.grid()[1000:1013], g[1000:1013])


def test_cancel_stops_render(nm):
    # 4M samples, many of them interior points that run all 100,000 iterations:
    # far more work than the lanes in flight, so the cancel lands mid-render.
    m = setup_gpu(nm, shrink(dict(C1, N=100000), 2048, 2048), keep64=False)
    m.render_rows(0, m.rows())
    m.cancel()
    with pytest.raises(nm.NewmanError) as e:
        m.synchronize()
    assert e.value.code == nm.NM_ERR_CANCELLED
    # the handle stays usable
    m.render_rows(0, 4)
    m.synchronize()
