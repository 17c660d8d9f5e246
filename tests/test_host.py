"""Host-side tests (no GPU): the C ABI's exports, the view arithmetic and the
arbitrary-precision precompute against the oracle."""
import os
import re
from decimal import Decimal

import numpy as np
import pytest

import newman_gb300 as nm
from helpers import step_for, C2, setup_oracle, shrink

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "newman_gb300.h")).read()
    return sorted(set(re.findall(r"\b(nm_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = nm.load_library()
    declared = header_symbols()
    assert declared == sorted(nm.EXPORTS)
    for name in declared:
        assert hasattr(L, name), name


def test_view_fields_round_trip():
    m = nm.Mandelbrot(480, 640)
    # constructor defaults of mandelbrot.cpp:8-17
    assert m.N == 256 and m.rows() == 480 and m.cols() == 640
    assert Decimal(m.center[0]) == Decimal("-0.5")
    m.set_view("-0.743643887037151", "0.131825904205330", "1.3e-16", "1.3e-16", 50000)
    assert m.N == 50000
    assert abs(Decimal(m.center[0]) - Decimal("-0.743643887037151")) < Decimal("1e-30")
    assert abs(Decimal(m.sz[1]) - Decimal("1.3e-16")) < Decimal("1e-45")
    assert not m.useHardware()
    m.scaleUp(4)
    assert m.rows() == 1920 and m.cols() == 2560


def test_bad_arguments_raise():
    with pytest.raises(nm.NewmanError) as e:
        nm.Mandelbrot(0, 10)
    m = nm.Mandelbrot(4, 4)
    with pytest.raises(nm.NewmanError) as e:
        m.set_view("x", "0", "1", "1", 10)
    assert e.value.code == nm.NM_ERR_PARSE
    with pytest.raises(nm.NewmanError) as e:
        m.N = 0
    assert e.value.code == nm.NM_ERR_ARG
    with pytest.raises(nm.NewmanError) as e:
        m.set_view("0", "0", "1e-20", "1e-20", 100)
        m.render_rows(0, 4)  # deep view without precompute
    assert e.value.code == nm.NM_ERR_STATE
    # FE32 chunk length: 0 picks the default, 1..256 explicit, anything else an error
    for ok in (0, 1, 64, 256):
        m.set_option(nm.OPT_RENORM, ok)
    for bad in (-1, 257):
        with pytest.raises(nm.NewmanError) as e:
            m.set_option(nm.OPT_RENORM, bad)
        assert e.value.code == nm.NM_ERR_ARG


@pytest.mark.parametrize("shape,N", [((48, 64), 3000), ((27, 31), 8000)])
def test_precompute_matches_oracle(oracle_mod, shape, N):
    v = shrink(C2, shape[0], shape[1], N=N)
    v["sc"] = 2
    m = nm.Mandelbrot(v["nr"], v["nc"])
    m.set_view(v["cre"], v["cim"], v["step"], v["step"], v["N"], v["tol"])
    m.scaleUp(2)
    m.precompute()
    o = setup_oracle(oracle_mod, v)
    o.precompute()
    assert m.stat(nm.STAT_ORBIT_LENGTH) == o.orbit_length
    assert m.stat(nm.STAT_PROBE_INDEX) == o.probe_index
    assert m.stat(nm.STAT_PRECISION_BITS) == o.bits


# Deep views at increasing precision: 64, 86 and 130 bits, 300 bits by the
# precision floor, and the 1100-bit view at width 1e-300 (seeded boundary
# walk) with its orbit at the view center.
DEEP_CASES = [("1e-15", 96, 0, 30000, False), ("1e-25", 96, 0, 30000, False),
              ("1e-38", 128, 0, 30000, False), ("1e-15", 96, 300, 20000, False),
              ("c3", 64, 1100, 200000, True)]


@pytest.mark.parametrize("width,cols,min_bits,N,center", DEEP_CASES)
def test_precompute_tables_match_oracle(oracle_mod, width, cols, min_bits, N, center):
    """The probe search, the winner's orbit and its series computed by the
    library (fixed-precision limbs, GMP's results reproduced) against the
    oracle's GMP calls: every exported double identical."""
    import json, os
    from decimal import Decimal, getcontext
    cre, cim = C2["cre"], C2["cim"]
    if width == "c3":
        walk = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                           "deep_centers.json")))["steps"]
        getcontext().prec = 400
        cre, cim = walk[71]["next_center_re"], walk[71]["next_center_im"]
        step = str(Decimal(walk[72]["width"]) / cols)
    else:
        step = step_for(width, cols)
    m = nm.Mandelbrot(48, cols)
    m.set_view(cre, cim, step, step, N, 1e-10, min_bits)
    m.set_path(nm.PATH_FP64)
    if center:
        m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    m.precompute()
    o = oracle_mod.OracleView(48, cols)
    o.set_view(cre, cim, step, step, N, 1e-10, min_bits)
    o.precompute(center=center)
    assert m.stat(nm.STAT_PRECISION_BITS) == o.bits
    assert m.stat(nm.STAT_ORBIT_LENGTH) == o.orbit_length > 100
    if not center:
        assert m.stat(nm.STAT_PROBE_INDEX) == o.probe_index
    got = m.orbit()
    ref = o.export_orbit()
    for name, g in zip(("x", "xlo", "a", "b", "c"), got):
        r = ref[name]
        same = (g.view(np.uint64) == r.view(np.uint64)) | (np.isnan(g) & np.isnan(r))
        assert same.all(), "%s differs at %d entries" % (name, (~same).sum())


def test_point_at_and_view_edits(oracle_mod):
    m = nm.Mandelbrot(480, 640)
    m.set_view("-0.75", "0", "0.0046875", "0.0046875", 1024)
    o = oracle_mod.OracleView(480, 640)
    o.set_view("-0.75", "0", "0.0046875", "0.0046875", 1024)
    re_, im_ = o.coords()
    for r, c in [(0, 0), (239, 320), (479, 639)]:
        pr, pi = m.pointAt(r, c)
        assert abs(float(Decimal(pr)) - re_[c]) <= 1e-15 and abs(float(Decimal(pi)) - im_[r]) <= 1e-15
    # zoomAt keeps the zoom point fixed (mandelbrot.cpp:304-316)
    before = [Decimal(x) for x in m.pointAt(100, 200)]
    m.zoomAt(2.0, 100, 200)
    after = [Decimal(x) for x in m.pointAt(100, 200)]
    assert all(abs(a - b) < Decimal("1e-18") for a, b in zip(before, after))
    assert abs(Decimal(m.sz[0]) - Decimal("0.00234375")) < Decimal("1e-20")
    # translate moves the center by whole samples (mandelbrot.cpp:292-295)
    c0 = Decimal(m.center[0])
    m.translate(0, 10)
    assert abs(Decimal(m.center[0]) - (c0 - 10 * Decimal(m.sz[0]))) < Decimal("1e-18")


def test_save_and_load_legacy(tmp_path):
    m = nm.Mandelbrot(600, 800)
    m.set_view("-0.743643887037151", "0.131825904205330", "1e-10", "1e-10", 4096)
    p = str(tmp_path / "view.txt")
    m.save(p)
    lines = open(p).read().split()
    assert lines[0] == "4096" and len(lines) == 5
    # loadLegacy rescales the step from an 800x600 window to the grid
    m2 = nm.Mandelbrot(300, 400)
    m2.loadLegacy(p)
    assert m2.N == 4096
    assert abs(Decimal(m2.sz[0]) - Decimal("2e-10")) < Decimal("1e-25")
    with pytest.raises(nm.NewmanError) as e:
        m2.loadLegacy(str(tmp_path / "missing.txt"))
    assert e.value.code == nm.NM_ERR_IO


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU failure mode")
def test_render_without_gpu_fails_loudly():
    m = nm.Mandelbrot(8, 8)
    with pytest.raises(nm.NewmanError) as e:
        m.render()
    assert e.value.code == nm.NM_ERR_CUDA


def test_batch_refuses_reference_exact_frames():
    """A batch groups its frames by the FE32, FP64 and double-loop kernels;
    a frame on the reference-exact path is refused, not rendered by another
    path's arithmetic (host check: the refusal comes before any GPU work)."""
    m = nm.Mandelbrot(8, 8)
    m.set_path(nm.PATH_MP)
    b = nm.Batch(sc=1)
    with pytest.raises(nm.NewmanError) as e:
        b.add(m)
    assert e.value.code == nm.NM_ERR_UNSUPPORTED
