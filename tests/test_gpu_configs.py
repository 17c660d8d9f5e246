"""The measured workloads at their full sizes.

* 3840x2160 at width 1e-300 (N 1,000,000, 1100-bit orbit at the seeded deep
  center): the FE32 frame against the plain FP64 frame (>= 99.99 % identical
  escape counts), the FP64 frame against the oracle's restatement of its own
  algorithm (MODE_DELTA_FE, bit-exact) and against the arbitrary-precision
  continuation (MODE_REF_FE) on seeded samples.
* The 240-frame zoom video (1280x720, 2x2 samples, widths 4 -> 1e-200, N
  1,000 -> 500,000): the batched graph launch against every frame rendered
  alone, bit-identical.
* One learned-scheduling view (3840x2160, 2x2 samples, N 2,000,000): the
  render in the cost model's longest-first tile order against the static
  order, bit-identical.
* The 1e-300 view in the order the cost model predicts from a capped preview
  (computed on the GPU): bit-identical to the static order and a shorter
  render; the times with and without the preview are recorded.

Measured fractions are written as JSON when NM_TEST_RECORD names a file
prefix.
"""
import json
import os

import numpy as np
import pytest

from helpers import make_frame, sample_positions, zoom_frames

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
WALK = json.load(open(os.path.join(HERE, "golden", "deep_centers.json")))["steps"]
RESULTS = {}


def _record(key, value):
    """Keeps a measured fraction; written as JSON to the file named by the
    environment variable NM_TEST_RECORD (with a "configs" suffix) when set."""
    RESULTS[key] = value
    path = os.environ.get("NM_TEST_RECORD")
    if path:
        with open(path + ".configs.json", "w") as f:
            json.dump(RESULTS, f, indent=1)


@pytest.fixture(scope="module")
def nm():
    import newman_gb300
    newman_gb300.load_library()
    return newman_gb300


def deep_view(k, cols):
    from decimal import Decimal, getcontext
    getcontext().prec = 700
    return (WALK[k - 1]["next_center_re"], WALK[k - 1]["next_center_im"],
            str(Decimal(WALK[k]["width"]) / cols))


def test_c3_full_frame(nm, oracle_mod):
    nr, nc, N, bits = 2160, 3840, 1000000, 1100
    cre, cim, step = deep_view(72, nc)  # width 1e-300
    fe = nm.Mandelbrot(nr, nc)
    fe.set_view(cre, cim, step, step, N, 1e-10, bits)
    fe.set_path(nm.PATH_FE32)
    fe.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    fe.precompute()
    fe.render()
    assert fe.stat(nm.STAT_WAIT_TIMEOUTS) == 0
    assert fe.stat(nm.STAT_CARDIOID_UNDECIDED) == 0
    fp = fe.copy()
    fp.set_path(nm.PATH_FP64)
    fp.set_option(nm.OPT_KEEP_SMOOTH64, 1)
    fp.upload()
    fp.render()
    g_fe = fe.grid()["iterations"]
    g_fp = fp.grid()["iterations"]
    exact = float((g_fe == g_fp).mean())
    _record("c3_fe32_vs_fp64", exact)
    assert exact >= 0.9999

    o = oracle_mod.OracleView(nr, nc)
    o.set_view(cre, cim, step, step, N, 1e-10, bits)
    o.precompute(center=True)
    assert o.orbit_length == fe.stat(nm.STAT_ORBIT_LENGTH)
    rr, cc = sample_positions(nr, nc, 4096, seed=72)
    it, sm = o.render_pixels(rr, cc, oracle_mod.MODE_DELTA_FE)
    bad = np.flatnonzero(g_fp[rr, cc] != it)
    assert bad.size == 0, "FP64 frame vs MODE_DELTA_FE: %d of 4096 differ" % bad.size
    assert np.abs(fp.smoothing64()[rr, cc] - sm).max() <= 1e-12
    # the arbitrary-precision continuation (the reference's algorithm with a
    # floatexp series front): the view is chaotic at the sample scale and the
    # perturbation's FP64 orbit (2^-53 of |X| absolute) differs from it by a
    # few sample steps; measured 2047 of the 2048 seeded samples identical
    mp_it, _ = o.render_pixels(rr[:2048], cc[:2048], oracle_mod.MODE_REF_FE)
    frac_fp = float((g_fp[rr[:2048], cc[:2048]] == mp_it).mean())
    frac_fe = float((g_fe[rr[:2048], cc[:2048]] == mp_it).mean())
    _record("c3_fp64_vs_mp_2048", frac_fp)
    _record("c3_fe32_vs_mp_2048", frac_fe)
    assert frac_fp >= 0.999 and frac_fe >= 0.999


def test_c4_240_frame_batch_equals_frames_alone(nm):
    views = zoom_frames(240, 720, 1280, "4.0", "1e-200", 1000, 500000)
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 8) as ex:
        def one(v):
            f = make_frame(nm, v, 2, nm.PATH_FE32, nm.PATH_FE32)
            f.precompute()
            return f
        frames = list(ex.map(one, views))
    batch = nm.Batch(sc=2)
    for f in frames:
        batch.add(f)
    batch.render()
    got = batch.frames_out()
    assert batch.stat(nm.STAT_SAMPLES) == sum(f.rows() * f.cols() for f in frames)
    same = 0
    for f, g in zip(frames, got):
        alone = f.copy()
        alone.upload()
        alone.render()
        ref = alone.reduce(2)
        same += int(np.array_equal(g, ref))
        del alone
    _record("c4_frames_identical", same)
    assert same == len(frames)


def test_c5_learned_order_bit_identical(nm):
    from decimal import Decimal, getcontext
    getcontext().prec = 700
    # the first view of the walk at width 1e-413 or below (the learned-
    # scheduling workload's deepest stopping widths lie there)
    k = next(i for i, s in enumerate(WALK) if Decimal(s["width"]) <= Decimal("1e-413"))
    cre, cim = WALK[k - 1]["next_center_re"], WALK[k - 1]["next_center_im"]
    step = str(Decimal(WALK[k]["width"]) / 3840)
    m = nm.Mandelbrot(2160, 3840)
    m.set_view(cre, cim, step, step, 2000000, 1e-10)
    m.scaleUp(2)
    m.set_path(nm.PATH_FE32)
    m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    m.precompute()
    tile = 64  # 32x32 pixels of 2x2 samples
    m.set_option(nm.OPT_TILE_W, tile)
    m.set_option(nm.OPT_TILE_H, tile)
    m.set_option(nm.OPT_LOG_TILE_COSTS, 1)
    m.render()
    static = m.grid().copy()
    costs = m.tile_costs().astype(np.float64).ravel()
    m.set_option(nm.OPT_LOG_TILE_COSTS, 0)
    p = m.preview(16)
    p.render()
    feats = p.tile_features(tile // 16, tile // 16)
    model = nm.CostModel(seed=7)
    y = np.log2(1.0 + costs)
    model.train(feats, (y - y.mean()).astype(np.float32), epochs=50, lr=2e-3)
    order = np.argsort(-model.predict(feats), kind="stable").astype(np.int32)
    m.set_tile_order(order)
    m.render()
    learned = m.grid()
    assert np.array_equal(static, learned)


def _tile_log(nm, m, tile, f, extra=512):
    """Tile costs of one whole render of m (tiles of tile x tile samples) and
    the features of a preview one sample per f x f, its iterations capped at
    the orbit length + extra (where the view has an orbit)."""
    m.set_option(nm.OPT_TILE_W, tile)
    m.set_option(nm.OPT_TILE_H, tile)
    m.set_option(nm.OPT_LOG_TILE_COSTS, 1)
    m.render()
    costs = m.tile_costs().astype(np.float64).ravel()
    m.set_option(nm.OPT_LOG_TILE_COSTS, 0)
    p = m.preview(f)
    if not p.useHardware():
        p.set_option(nm.OPT_ITER_CAP, m.stat(nm.STAT_ORBIT_LENGTH) + extra)
    p.render()
    return p.tile_features(tile // f, tile // f), costs


def test_c3_learned_order_gain(nm):
    """What the trained network gains on the 1e-300 view, whose frame time is
    set by its longest samples: the model is trained on the tile costs its
    own renders logged on C1, C2 and C3 (32x32-pixel tiles), then orders C3's
    tiles from a capped preview on the GPU (nm_order_tiles).  The render in
    that order is bit-identical to the static order's, and in this test's runs
    shorter; the recorded times give the gain with and without the preview (measured:
    render 34.0 -> 29.9, 30.6 -> 27.8 and 28.4 -> 25.3 ms, order by the true
    costs 28.8, 28.0 and 24.7 ms, preview and ordering ~3 ms)."""
    import time
    import torch
    from decimal import Decimal, getcontext
    getcontext().prec = 700
    nr, nc, N, bits = 2160, 3840, 1000000, 1100
    cre, cim, step = deep_view(72, nc)

    def view(nr, nc, sc, cre, cim, step, N, bits=0):
        m = nm.Mandelbrot(nr, nc)
        m.set_view(cre, cim, step, step, N, 1e-10, bits)
        if sc > 1:
            m.scaleUp(sc)
        if not m.useHardware():
            m.set_path(nm.PATH_FE32)
            m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
            m.precompute()
        return m

    c1 = view(480, 640, 1, "-0.75", "0", "0.0046875", 1024)
    c2 = view(1080, 1920, 4, "-0.743643887037151", "0.131825904205330",
              str(Decimal("1e-12") / 1920), 50000)
    c3 = view(nr, nc, 1, cre, cim, step, N, bits)
    logs = [_tile_log(nm, c1, 32, 8), _tile_log(nm, c2, 128, 32), _tile_log(nm, c3, 32, 8)]
    X = np.concatenate([x for x, _ in logs])
    Y = np.concatenate([np.log2(1.0 + c) - np.log2(1.0 + c).mean() for _, c in logs])
    model = nm.CostModel(seed=2026)
    model.train(X, Y.astype(np.float32), epochs=300, lr=2e-3)
    costs = logs[2][1]

    def kernel_ms(n=5):
        c3.render()
        ts = []
        for _ in range(n):
            c3.render()
            ts.append(c3.stat(nm.STAT_KERNEL_NS) * 1e-6)
        return float(np.median(ts))

    def wall_ms(fn, n=5):
        ts = []
        for _ in range(n):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append((time.perf_counter() - t0) * 1e3)
        return float(np.median(ts))

    c3.set_tile_order(None)
    static_ms = kernel_ms()
    static = c3.grid().copy()
    static_wall = wall_ms(c3.render)

    def learned():
        p = c3.preview(8)
        p.set_option(nm.OPT_ITER_CAP, c3.stat(nm.STAT_ORBIT_LENGTH) + 512)
        p.render()
        c3.order_tiles(p, model)
        c3.render()

    learned_wall = wall_ms(learned)
    order = c3.tile_order()
    learned_ms = kernel_ms()
    assert np.array_equal(c3.grid(), static)
    c3.set_tile_order(np.argsort(-costs, kind="stable").astype(np.int32))
    cost_order_ms = kernel_ms()
    assert np.array_equal(c3.grid(), static)
    rank = lambda a: np.argsort(np.argsort(a))
    position = np.empty_like(order)
    position[order] = np.arange(len(order))
    _record("c3_learned_order", {
        "render_ms_static": static_ms, "render_ms_learned": learned_ms,
        "render_ms_true_cost_order": cost_order_ms, "wall_ms_static": static_wall,
        "wall_ms_learned_with_preview": learned_wall,
        "spearman_order_vs_costs": float(np.corrcoef(rank(-position), rank(costs))[0, 1])})
    # measured 10-14 % shorter in this test's runs (and from 12 % longer to
    # 14 % shorter with the benchmark's model): the frame time of this view
    # follows the order in which its longest samples are claimed, so the bar
    # only rules out an order that wrecks the frame; the times are recorded
    assert learned_ms <= 1.15 * static_ms
