"""The oracle against closed-form facts and against the independent pure-Python
/ mpmath restatement of the reference in tests/golden/ (make_golden.py)."""
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
BAILOUT2 = 1024.0 * 1024.0


def smoothing(r2):
    return 1.0 - math.log2(0.5 * math.log(r2) / math.log(1024.0))


def point_view(oracle_mod, cre, cim, N=1024, step="0.001"):
    """A 2x2 view whose sample (0, 1) is exactly the center."""
    o = oracle_mod.OracleView(2, 2)
    o.set_view(cre, cim, step, step, N)
    o.precompute()
    it, sm = o.render_pixels([0], [1])
    return int(it[0]), float(sm[0])


def escape_by_hand(c, N):
    """z -> z^2 + c on the real axis, counted like getIterationsHW."""
    z = c
    for it in range(N):
        z = z * z + c
        if z * z > BAILOUT2:
            return it, smoothing(z * z)
    return N, 0.0


# Binary fractions, so that the decimal string and the double are the same number.
@pytest.mark.parametrize("c", [2.0, 1.0, -2.125, 0.3125, 0.2578125])
def test_real_axis_escape_counts(oracle_mod, c):
    assert point_view(oracle_mod, repr(c), "0") == escape_by_hand(c, 1024)


def test_two_and_one_by_hand(oracle_mod):
    # c = 2: 2, 6, 38, 1446 -> escapes at the third step (iterations 2)
    assert point_view(oracle_mod, "2", "0") == (2, smoothing(1446.0 ** 2))
    # c = 1: 1, 2, 5, 26, 677, 458330 -> iterations 4
    assert point_view(oracle_mod, "1", "0") == (4, smoothing(458330.0 ** 2))


@pytest.mark.parametrize("c", [("0", "0"), ("-1", "0"), ("-0.1", "0.1"), ("-0.75", "0"),
                               ("-2", "0"), ("0.25", "0.5")])
def test_interior_and_boundary_points_reach_N(oracle_mod, c):
    # cardioid / period-2 disk interior; -0.75 and 0.25+0.5i lie exactly on the
    # boundaries (the strict '<' of mandelbrot.cpp:68,70 lets them iterate) and
    # never escape; -2 stays at 2 forever.
    assert point_view(oracle_mod, *c) == (1024, 0.0)


def test_precision_rule(oracle_mod):
    # mandelbrot.cpp:37-56: bits = max(64, (int)(64 - e + log2(1e-20)))
    for step, e in [("0.0046875", -7), ("1e-12", -39), ("1e-100", -332), ("1e-300", -996)]:
        o = oracle_mod.OracleView(4, 4)
        o.set_view("0", "0", step, step, 10)
        assert o.bits == max(64, int(64 - e + math.log2(1e-20)))


def test_hw_view_matches_golden(oracle_mod):
    g = np.load(os.path.join(HERE, "golden", "hw_view.npz"))
    o = oracle_mod.OracleView(int(g["nr"]), int(g["nc"]))
    o.set_view(str(g["center_re"]), str(g["center_im"]), str(g["step"]), str(g["step"]),
               int(g["N"]))
    assert o.use_hardware()
    R, C = np.meshgrid(g["rows"], g["cols"], indexing="ij")
    it, sm = o.render_pixels(R.ravel(), C.ravel())
    assert np.array_equal(it.reshape(R.shape), g["iterations"])
    assert np.array_equal(sm.reshape(R.shape), g["smoothing"])


def test_deep_view_matches_golden(oracle_mod):
    """Reference semantics with the arbitrary-precision continuation against
    the mpmath restatement (320 bits).  The probe search, the orbit length and
    the series skip of every sample are exact.  The continuation itself is not
    converged at the precision the reference's rule gives this view (64 bits,
    mandelbrot.cpp:37-56): GMP at that precision and mpmath at 320 bits agree
    on most escape counts but not all, so only that majority is asserted."""
    g = np.load(os.path.join(HERE, "golden", "deep_view.npz"))
    nr, nc = int(g["nr"]), int(g["nc"])
    o = oracle_mod.OracleView(nr, nc)
    o.set_view(str(g["center_re"]), str(g["center_im"]), str(g["step"]), str(g["step"]),
               int(g["N"]))
    assert not o.use_hardware()
    assert o.bits == 64
    o.precompute()
    assert o.probe_index == int(g["probe_index"])
    assert o.orbit_length == int(g["orbit_length"])
    R, C = np.meshgrid(np.arange(nr), np.arange(nc), indexing="ij")
    assert np.array_equal(o.series_skip(R.ravel(), C.ravel()).reshape(nr, nc),
                          g["series_skip"])
    it, sm = o.render_rows(0, nr, oracle_mod.MODE_REF)
    assert (it == g["iterations"]).mean() >= 0.8


def test_reduce_is_float_mean_in_reference_order(oracle_mod):
    rng = np.random.default_rng(3)
    sc = 3
    it = rng.integers(0, 5000, size=(6 * sc, 5 * sc)).astype(np.int32)
    sm = rng.random(size=it.shape).astype(np.float32)
    oi, osm = oracle_mod.reduce(it, sm, sc)
    for r in range(6):
        for c in range(5):
            s = np.float32(0.0)
            for r1 in range(sc):
                for c1 in range(sc):
                    k = (sc * r + r1, sc * c + c1)
                    s = np.float32(s + np.float32(np.float32(it[k]) + sm[k]))
            s = np.float32(s / np.float32(sc * sc))
            assert oi[r, c] == int(s) and osm[r, c] == np.float32(s - np.float32(int(s)))


def test_delta_mode_equals_reference_on_hw_free_front(oracle_mod):
    """MODE_DELTA shares the reference's series front: samples that escape
    before the skip point (binary search) get identical results."""
    g = np.load(os.path.join(HERE, "golden", "deep_view.npz"))
    nr, nc = int(g["nr"]), int(g["nc"])
    o = oracle_mod.OracleView(nr, nc)
    o.set_view(str(g["center_re"]), str(g["center_im"]), str(g["step"]), str(g["step"]),
               int(g["N"]))
    o.precompute()
    it_d, sm_d = o.render_rows(0, nr, oracle_mod.MODE_DELTA)
    it_r, sm_r = o.render_rows(0, nr, oracle_mod.MODE_REF)
    assert (it_d == it_r).mean() >= 0.95


def test_unbounded_exponent_delta_equals_plain_fp64_in_range(oracle_mod):
    """MODE_DELTA_FE (floatexp series front, FP64 deltas with an unbounded
    exponent) gives MODE_DELTA's results bit for bit on a view inside the
    double range: the floatexp front equals the FP64 front there, and the
    unbounded-exponent arithmetic equals double arithmetic on values that
    never leave the double range."""
    g = np.load(os.path.join(HERE, "golden", "deep_view.npz"))
    nr, nc = int(g["nr"]), int(g["nc"])
    o = oracle_mod.OracleView(nr, nc)
    o.set_view(str(g["center_re"]), str(g["center_im"]), str(g["step"]), str(g["step"]),
               int(g["N"]))
    o.precompute()
    it_d, sm_d = o.render_rows(0, nr, oracle_mod.MODE_DELTA)
    it_x, sm_x = o.render_rows(0, nr, oracle_mod.MODE_DELTA_FE)
    assert np.array_equal(it_d, it_x)
    assert np.array_equal(sm_d, sm_x)


def test_rebasing_removes_single_reference_glitches(oracle_mod):
    """On the seeded walk's view at width 1e-16 with the orbit at the view
    center, single-reference perturbation (MODE_DELTA_SINGLE, no rebase on
    |Y| < |delta|) misses the reference's escape counts in connected blobs
    (Pauldelbrot's glitches); the library's rebasing perturbation (MODE_DELTA)
    misses only isolated chaotic samples."""
    import json
    import os
    from decimal import Decimal, getcontext
    ndimage = pytest.importorskip("scipy.ndimage")
    walk = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                       "deep_centers.json")))["steps"]
    getcontext().prec = 200
    n = 48
    step = str(Decimal(walk[2]["width"]) / n)
    o = oracle_mod.OracleView(n, n)
    o.set_view(walk[1]["next_center_re"], walk[1]["next_center_im"], step, step, 60000)
    o.precompute(center=True)
    ref, _ = o.render_rows(0, n, oracle_mod.MODE_REF)

    def largest(mask):
        lab, k = ndimage.label(mask)
        return int(np.bincount(lab.ravel())[1:].max()) if k else 0

    single, _ = o.render_rows(0, n, oracle_mod.MODE_DELTA_SINGLE)
    rebased, _ = o.render_rows(0, n, oracle_mod.MODE_DELTA)
    assert (single != ref).mean() > 0.05 and largest(single != ref) >= 10
    assert (rebased != ref).mean() < 0.02 and largest(rebased != ref) <= 3
