"""The reference-exact path (NM_PATH_MP) against the oracle's MODE_REF -- the
reference's own semantics: its double loop where useHardware() holds, else
getIterations with its arbitrary-precision continuation (mandelbrot.cpp:144-
254), GMP mpf arithmetic throughout.

Bar: escape counts bit-exact on every compared sample; unrounded smoothing
within 1e-12 (CUDA's log / log2 against glibc's).
"""
import numpy as np
import pytest

from helpers import C1, C2, sample_positions, setup_gpu, setup_oracle, step_for

pytestmark = pytest.mark.gpu

SMOOTH_TOL = 1e-12


@pytest.fixture(scope="module")
def nm():
    import newman_gb300
    newman_gb300.load_library()
    return newman_gb300


def _exact(it_gpu, sm_gpu, it_ref, sm_ref):
    bad = np.flatnonzero(it_gpu != it_ref)
    assert bad.size == 0, "escape counts differ at %d of %d samples, e.g. gpu %s ref %s" % (
        bad.size, it_ref.size, it_gpu[bad[:5]], it_ref[bad[:5]])
    assert np.abs(sm_gpu - sm_ref).max() <= SMOOTH_TOL


def test_c2_view_bit_exact_with_reference(nm, oracle_mod):
    """1920x1080 x 4x4 at width 1e-12, N 50,000: the whole view on the GPU,
    20,000 seeded samples against the reference's MP continuation."""
    m = setup_gpu(nm, C2, path=nm.PATH_MP)
    m.precompute()
    m.render()
    assert m.stat(nm.STAT_CARDIOID_UNDECIDED) == 0
    g, s64 = m.grid(), m.smoothing64()
    o = setup_oracle(oracle_mod, C2)
    o.precompute()
    assert m.stat(nm.STAT_PROBE_INDEX) == o.probe_index
    assert m.stat(nm.STAT_ORBIT_LENGTH) == o.orbit_length
    rr, cc = sample_positions(m.rows(), m.cols(), 20000, seed=3)
    it, sm = o.render_pixels(rr, cc, oracle_mod.MODE_REF)
    _exact(g["iterations"][rr, cc], s64[rr, cc], it, sm)


@pytest.mark.parametrize("width,cols,min_bits", [
    ("1e-15", 96, 0),      # 64 bits: 3 limbs a value
    ("1e-25", 96, 0),      # 87 bits: 4 limbs
    ("1e-38", 128, 0),     # 130 bits: 5 limbs
    ("1e-15", 96, 300),    # 300 bits: 7 limbs
    ("1e-20", 96, 448),    # 448 bits: 9 limbs, the widest built
])
def test_precisions_bit_exact(nm, oracle_mod, width, cols, min_bits):
    v = dict(C2, nr=72, nc=cols, sc=1, step=step_for(width, cols), N=20000, min_bits=min_bits)
    m = setup_gpu(nm, v, path=nm.PATH_MP)
    m.precompute()
    m.render()
    o = setup_oracle(oracle_mod, v)
    o.precompute()
    assert m.stat(nm.STAT_PRECISION_BITS) == o.bits
    it, sm = o.render_rows(0, v["nr"], oracle_mod.MODE_REF)
    _exact(m.grid()["iterations"], m.smoothing64(), it, sm)


def test_c1_double_loop_with_exact_cardioid(nm, oracle_mod):
    """640x480 at -0.75+0i, width 3: the double loop, the cardioid test in the
    view's precision."""
    m = setup_gpu(nm, C1, path=nm.PATH_MP)
    assert m.useHardware()
    m.precompute()
    m.render()
    o = setup_oracle(oracle_mod, C1)
    it, sm = o.render_rows(0, C1["nr"], oracle_mod.MODE_REF)
    _exact(m.grid()["iterations"].ravel(), m.smoothing64().ravel(), it.ravel(), sm.ravel())


@pytest.mark.parametrize("tile", [(16, 16), (7, 5)])
def test_ragged_grids_and_row_ranges(nm, oracle_mod, tile):
    v = dict(C2, nr=33, nc=65, sc=1, step=step_for("1e-15", 65), N=5000)
    m = setup_gpu(nm, v, path=nm.PATH_MP)
    m.set_option(nm.OPT_TILE_W, tile[0])
    m.set_option(nm.OPT_TILE_H, tile[1])
    m.precompute()
    for r0, r1 in ((0, 5), (5, 33)):
        m.render_rows(r0, r1)
        m.synchronize()
    o = setup_oracle(oracle_mod, v)
    o.precompute()
    it, sm = o.render_rows(0, 33, oracle_mod.MODE_REF)
    _exact(m.grid()["iterations"], m.smoothing64(), it, sm)


def test_refusals(nm):
    # below the double range of the series: the reference renders nothing there
    deep = dict(C2, nr=16, nc=16, sc=1, step="1e-320", N=1000)
    m = setup_gpu(nm, deep, path=nm.PATH_MP)
    with pytest.raises(nm.NewmanError) as e:
        m.render()
    assert e.value.code == nm.NM_ERR_UNSUPPORTED
    # precision above the widest kernel
    wide = dict(C2, nr=16, nc=16, sc=1, step=step_for("1e-15", 16), N=1000, min_bits=600)
    m = setup_gpu(nm, wide, path=nm.PATH_MP)
    with pytest.raises(nm.NewmanError) as e:
        m.render()
    assert e.value.code == nm.NM_ERR_UNSUPPORTED
    # precomputed for another path, then switched to this one
    v = dict(C2, nr=16, nc=16, sc=1, step=step_for("1e-15", 16), N=1000)
    m = setup_gpu(nm, v, path=nm.PATH_FP64)
    m.precompute()
    m.set_path(nm.PATH_MP)
    with pytest.raises(nm.NewmanError) as e:
        m.render()
    assert e.value.code == nm.NM_ERR_STATE
    m.precompute()
    m.render()
