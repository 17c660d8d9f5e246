"""The colouring step (multiwave.cpp, viewer.cpp:89-124): palette files, the
cached palette against the oracle's independent restatement (host only), and
the GPU colouring of rendered grids against the oracle (byte for byte)."""
import os

import numpy as np
import pytest

from helpers import C1, setup_gpu

# A palette in the reference's text format (two hue cycles, a saturation
# cycle, two luminance waves); the values are this test's own.
PALETTE = """2
3 10.0 130.5 250.25 90
2 300.0 45.0 60
70

3
0.9 0.4 0.7
33

2
1.5 40
0.75 13
"""


@pytest.fixture
def pal_path(tmp_path):
    p = tmp_path / "test.pal"
    p.write_text(PALETTE)
    return str(p)


def test_palette_cache_matches_oracle_and_roundtrips(pal_path, tmp_path, oracle_mod):
    import newman_gb300 as nm
    pal = nm.Palette(pal_path)
    got = pal.cache(5000)
    ref = oracle_mod.palette_cache(pal_path, 5000)
    assert np.array_equal(got, ref)
    assert got.std() > 10  # a real gradient, not a constant
    out = str(tmp_path / "again.pal")
    pal.save(out)
    assert np.array_equal(nm.Palette(out).cache(5000), got)


def test_bad_palette_file_is_an_error(tmp_path):
    import newman_gb300 as nm
    p = tmp_path / "bad.pal"
    p.write_text("2\n3 1.0 2.0\n")
    with pytest.raises(nm.NewmanError):
        nm.Palette(str(p))


def test_oracle_colorize_rules(pal_path, oracle_mod):
    pal = oracle_mod.palette_cache(pal_path, 64)
    iters = np.array([[64, 5], [10, 0]], np.int32)
    smooth = np.array([[0.0, 0.25], [0.0, 0.5]], np.float32)
    img = oracle_mod.colorize(iters, smooth, 64, pal, 1, smooth_flag=False)
    assert (img[0, 0] == 0).all()  # reached N: black
    assert (img[0, 1] == pal[5]).all() and (img[1, 0] == pal[10]).all()
    mean = oracle_mod.colorize(iters, smooth, 64, pal, 2, smooth_flag=False)[0, 0]
    expect = (pal[5].astype(np.float32) + pal[10] + pal[0]) / np.float32(4)
    assert (np.abs(mean.astype(int) - np.floor(expect + 0.5)) <= 0).all()


@pytest.mark.gpu
@pytest.mark.parametrize("sc,smooth", [(1, True), (1, False), (2, True)])
def test_gpu_colorize_matches_oracle(pal_path, oracle_mod, sc, smooth):
    import newman_gb300 as nm
    nm.load_library()
    view = dict(C1)
    m = setup_gpu(nm, view)
    if sc > 1:
        m.scaleUp(sc)
    m.render()
    g = m.grid()
    pal = nm.Palette(pal_path)
    img = m.colorize(pal, sc=sc, smooth=smooth)
    ref = oracle_mod.colorize(g["iterations"], g["smoothing"], m.N, pal.cache(m.N), sc, smooth)
    assert img.shape == (C1["nr"], C1["nc"], 3)
    assert np.array_equal(img, ref)
    path = os.path.join(os.path.dirname(pal_path), "c1.ppm")
    nm.write_ppm(path, img)
    assert os.path.getsize(path) == len("P6\n640 480\n255\n") + img.size
