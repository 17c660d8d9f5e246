"""Deep views (series terms outside the FP64 range): the views of the seeded
boundary-following in tests/golden/deep_centers.json, reference orbit at the
view center, from width 1e-48 down to 1e-360 (below the double range).

* FP64 path against the oracle's MODE_DELTA_FE (same algorithm restated on the
  CPU): escape counts bit-exact, smoothing within 1e-12.
* FE32 path against the FP64 path: >= 99.99 % identical escape counts.
* FP64 path against the arbitrary-precision continuation (MODE_REF_FE): most
  escape counts identical (the views are chaotic at the sample scale).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CENTERS = json.load(open(os.path.join(HERE, "golden", "deep_centers.json")))


def view_at(k, grid):
    """The view of step k: the center chosen at step k-1, width of step k."""
    from decimal import Decimal, getcontext
    getcontext().prec = 600
    s = CENTERS["steps"]
    cre, cim = s[k - 1]["next_center_re"], s[k - 1]["next_center_im"]
    step = str(Decimal(s[k]["width"]) / grid)
    return cre, cim, step


RESULTS = {}


def _record(key, value):
    """Keeps a measured fraction; written as JSON to the file named by the
    environment variable NM_TEST_RECORD (with a "deep" suffix) when set."""
    RESULTS[key] = value
    path = os.environ.get("NM_TEST_RECORD")
    if path:
        with open(path + ".deep.json", "w") as f:
            json.dump(RESULTS, f, indent=1)


@pytest.fixture(scope="module")
def nm():
    import newman_gb300
    newman_gb300.load_library()
    return newman_gb300


def gpu_render(nm, cre, cim, step, grid, N, path):
    m = nm.Mandelbrot(grid, grid)
    m.set_view(cre, cim, step, step, N)
    m.set_path(path)
    m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    m.set_option(nm.OPT_KEEP_SMOOTH64, 1)
    m.precompute()
    m.render()
    return m


# k = 80, 87: widths 1e-332 and 1e-360, below the double range (the FP64 path
# carries its deltas with an unbounded exponent there)
@pytest.mark.parametrize("k", [9, 30, 72, 80, 87])
def test_deep_fp64_matches_oracle(nm, oracle_mod, k):
    cre, cim, step = view_at(k, 64)
    N = 300000
    m = gpu_render(nm, cre, cim, step, 64, N, nm.PATH_FP64)
    o = oracle_mod.OracleView(64, 64)
    o.set_view(cre, cim, step, step, N)
    o.precompute(center=True)
    assert m.stat(nm.STAT_ORBIT_LENGTH) == o.orbit_length
    # every other row plus the center row, all columns (the center row and
    # column have an eps with a zero component): 2,112 samples
    rows, cols = np.meshgrid(np.union1d(np.arange(0, 64, 2), [31]), np.arange(64), indexing="ij")
    it, sm = o.render_pixels(rows.ravel(), cols.ravel(), oracle_mod.MODE_DELTA_FE)
    g = m.grid()["iterations"][rows.ravel(), cols.ravel()]
    assert np.array_equal(g, it)
    assert np.abs(m.smoothing64()[rows.ravel(), cols.ravel()] - sm).max() <= 1e-12
    # the arbitrary-precision continuation on all 2,112 compared samples:
    # measured 98.96 % to 100 % identical on 576 of them over the five views
    # (the FP64 orbit's own rounding, amplified where the views are chaotic)
    mp_it, _ = o.render_pixels(rows.ravel(), cols.ravel(), oracle_mod.MODE_REF_FE)
    frac = float((mp_it == it).mean())
    _record("deep_k%d_fp64_vs_mp_2112" % k, frac)
    assert frac >= 0.985


@pytest.mark.parametrize("k", [9, 30, 72, 80, 87])
def test_deep_fe32_matches_fp64(nm, k):
    cre, cim, step = view_at(k, 256)
    N = 300000
    a = gpu_render(nm, cre, cim, step, 256, N, nm.PATH_FP64)
    b = gpu_render(nm, cre, cim, step, 256, N, nm.PATH_FE32)
    same = (a.grid()["iterations"] == b.grid()["iterations"]).mean()
    assert same >= 0.9999, same
