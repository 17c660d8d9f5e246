"""Batched frames (nm_batch_*): one CUDA graph over the frames of a zoom video
must give every frame exactly what rendering it alone gives."""
import numpy as np
import pytest

from helpers import make_frame, zoom_frames

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nm():
    import newman_gb300
    newman_gb300.load_library()
    return newman_gb300


@pytest.fixture(scope="module")
def video(nm):
    views = zoom_frames(12, 64, 96, "4.0", "1e-60", 500, 20000)
    frames = [make_frame(nm, v, 2, nm.PATH_FE32) for v in views]
    for f in frames:
        f.precompute()
    return views, frames


def test_batch_equals_frame_at_a_time(nm, video):
    views, frames = video
    kinds = [f.useHardware() for f in frames]
    assert any(kinds) and not all(kinds)  # both the double path and FE32 frames
    batch = nm.Batch(sc=2)
    for f in frames:
        batch.add(f)
    batch.render()
    got = batch.frames_out()
    assert batch.stat(nm.STAT_SAMPLES) == sum(f.rows() * f.cols() for f in frames)
    for v, g in zip(views, got):
        alone = make_frame(nm, v, 2, nm.PATH_FE32)
        alone.precompute()
        alone.render()
        ref = alone.reduce(2)
        assert np.array_equal(g["iterations"], ref["iterations"])
        assert np.array_equal(g["smoothing"], ref["smoothing"])
    # replaying the graph gives the same frames again
    batch.render()
    again = batch.frames_out()
    for a, b in zip(got, again):
        assert np.array_equal(a, b)


def test_batch_graph_and_direct_launches_agree(nm, video):
    views, frames = video
    out = []
    for graph in (1, 0):
        batch = nm.Batch(sc=2)
        for f in frames:
            batch.add(f)
        batch.set_option(nm.OPT_BATCH_GRAPH, graph)
        batch.render()
        out.append(batch.frames_out())
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_batch_autotune_keeps_results(nm, video):
    views, frames = video
    batch = nm.Batch(sc=2)
    for f in frames:
        batch.add(f)
    batch.render()
    before = batch.frames_out()
    tw, th, rn = batch.autotune(stride=3)
    assert tw in (8, 16, 32, 64) and th in (8, 16, 32, 64) and 8 <= rn <= 256
    batch.render()
    after = batch.frames_out()
    for a, b in zip(before, after):
        assert np.array_equal(a["iterations"], b["iterations"])


def test_batch_overlap_matches_separate_launches(nm, video):
    """The double-path frames and the FP64 rework inside the FE32 iteration
    pass give the frames that separate launches give."""
    views, frames = video
    out = []
    for overlap in (1, 0):
        batch = nm.Batch(sc=2)
        for f in frames:
            batch.add(f)
        batch.set_option(nm.OPT_FE32_OVERLAP, overlap)
        batch.render()
        assert batch.stat(nm.STAT_WAIT_TIMEOUTS) == 0
        out.append(batch.frames_out())
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_batch_with_fe32_double_loop_frames(nm):
    """All frames on the FE32 path, the double-loop frames included: the batch
    gives what rendering each frame alone gives, and the double-loop frames'
    escape counts are the double loop's."""
    views = zoom_frames(8, 48, 64, "4.0", "1e-40", 500, 8000)
    frames = [make_frame(nm, v, 2, nm.PATH_FE32, nm.PATH_FE32) for v in views]
    for f in frames:
        f.precompute()
    assert any(f.useHardware() for f in frames)
    batch = nm.Batch(sc=2)
    for f in frames:
        batch.add(f)
    batch.render()
    got = batch.frames_out()
    assert batch.stat(nm.STAT_WAIT_TIMEOUTS) == 0
    for v, f, g in zip(views, frames, got):
        alone = make_frame(nm, v, 2, nm.PATH_FE32, nm.PATH_FE32)
        alone.precompute()
        alone.render()
        assert np.array_equal(g["iterations"], alone.reduce(2)["iterations"])
        if f.useHardware():
            dl = make_frame(nm, v, 2, nm.PATH_FE32)
            dl.render()
            assert (dl.grid()["iterations"] == alone.grid()["iterations"]).mean() >= 0.9999


def test_batch_rebuilds_after_a_frame_changes(nm):
    """A frame whose view changes after the batch captured its graph (N here,
    re-precomputed and re-uploaded into buffers of the same size, so that no
    device pointer moves) must be rendered with its new tables, not replayed
    from the old graph."""
    views = zoom_frames(4, 64, 96, "1e-3", "1e-40", 2000, 8000)
    frames = [make_frame(nm, v, 2, nm.PATH_FE32) for v in views]
    for f in frames:
        f.precompute()
        f.upload()
    batch = nm.Batch(sc=2)
    for f in frames:
        batch.add(f)
    batch.render()
    k = len(frames) - 1
    grid_before = frames[k].device_grid()
    frames[k].N = 3000
    frames[k].precompute()
    frames[k].upload()
    assert frames[k].device_grid() == grid_before  # same buffers: pointers cannot tell
    batch.render()
    got = batch.frames_out()
    for j, v in enumerate(views):
        alone = make_frame(nm, v, 2, nm.PATH_FE32)
        if j == k:
            alone.N = 3000
        alone.precompute()
        alone.render()
        ref = alone.reduce(2)
        assert np.array_equal(got[j]["iterations"], ref["iterations"]), "frame %d" % j
    assert int(got[k]["iterations"].max()) <= 3000
