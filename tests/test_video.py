"""Keyframe interpolation of the zoom video (VideoZoom::nextFrame,
video.cpp:14-34): the oracle's restatement on its own properties (host only),
argument errors of the C ABI, and the GPU frames against the oracle byte for
byte on seeded keyframes, ragged sizes and rendered, coloured keyframes."""
import numpy as np
import pytest

from helpers import setup_gpu


def keyframes(seed, kh, kw):
    rng = np.random.default_rng(seed)
    prev = rng.integers(0, 256, (kh, kw, 3), dtype=np.uint8)
    cur = rng.integers(0, 256, (kh, kw, 3), dtype=np.uint8)
    return prev, cur


def test_oracle_first_frame_is_the_previous_keyframe_cropped(oracle_mod):
    prev, cur = keyframes(1, 45, 60)
    frames = oracle_mod.video_interpolate(prev, cur, 30, 40, 6)
    assert frames.shape == (6, 30, 40, 3)
    # frame 0: the previous keyframe at scale 1, centered; the new one has weight 0
    assert np.array_equal(frames[0], prev[7:37, 10:50])


def test_oracle_constant_keyframes_give_constant_frames(oracle_mod):
    prev = np.full((36, 48, 3), 17, np.uint8)
    cur = np.full((36, 48, 3), 201, np.uint8)
    frames = oracle_mod.video_interpolate(prev, cur, 24, 32, 8)
    for i in range(8):
        t = np.float32(i) / np.float32(8)
        blended = int(np.floor((np.float32(1) - t) * np.float32(17) + t * np.float32(201) + 0.5))
        vals = set(np.unique(frames[i]).tolist())
        assert vals <= {17, blended}
        if i:
            # the new keyframe at scale (2/3) v^i covers the center of the frame
            assert (frames[i][12, 16] == blended).all()


def test_video_argument_errors():
    import newman_gb300 as nm
    prev, cur = keyframes(2, 20, 20)
    with pytest.raises(nm.NewmanError):
        nm.video_interpolate(prev, cur, 30, 30, 4)  # keyframes smaller than the frames
    with pytest.raises(nm.NewmanError):
        nm.video_interpolate(prev, cur, 10, 10, 0)  # no frames
    with pytest.raises(ValueError):
        nm.video_interpolate(prev, cur[:10], 10, 10, 4)


@pytest.mark.gpu
@pytest.mark.parametrize("kh,kw,rows,cols,rate", [
    (45, 60, 30, 40, 1),
    (45, 60, 30, 40, 30),
    (97, 131, 64, 87, 7),   # ragged sizes, odd offsets
    (64, 64, 64, 64, 5),    # keyframes the size of the frames
    (1080, 1920, 720, 1280, 4),
])
def test_gpu_video_matches_oracle(oracle_mod, kh, kw, rows, cols, rate):
    import newman_gb300 as nm
    nm.load_library()
    prev, cur = keyframes(kh * 7 + rate, kh, kw)
    got = nm.video_interpolate(prev, cur, rows, cols, rate)
    ref = oracle_mod.video_interpolate(prev, cur, rows, cols, rate)
    assert np.array_equal(got, ref)


@pytest.mark.gpu
def test_gpu_video_of_rendered_keyframes(oracle_mod, tmp_path):
    """Two keyframes of a zoom (the second 1.5x deeper), rendered and coloured
    on the GPU at 1.5 times the frame size, interpolated as the viewer's
    auto-zoom does."""
    import newman_gb300 as nm
    nm.load_library()
    pal_path = tmp_path / "p.pal"
    pal_path.write_text("1\n3 0.0 120.0 240.0 50\n50\n1\n0.8\n1\n1\n1.0 30\n")
    pal = nm.Palette(str(pal_path))
    keys = []
    for width in (0.012, 0.008):
        view = dict(nr=180, nc=240, sc=1, cre="-0.7453", cim="0.1127", step=str(width / 240),
                    N=600, tol=1e-10)
        m = setup_gpu(nm, view)
        m.render()
        keys.append(m.colorize(pal))
    got = nm.video_interpolate(keys[0], keys[1], 120, 160, 12)
    ref = oracle_mod.video_interpolate(keys[0], keys[1], 120, 160, 12)
    assert np.array_equal(got, ref)
    assert got.std() > 10
