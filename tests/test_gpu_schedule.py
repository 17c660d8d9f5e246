"""Learned tile scheduling on the GPU: the cost model's kernels against the
CPU restatement (forward pass and gradient), training, and the image's
independence of the tile order (bit for bit)."""
import numpy as np
import pytest

from helpers import C1, C2, setup_gpu, shrink

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nm():
    import newman_gb300
    newman_gb300.load_library()
    return newman_gb300


def data(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.random((n, 18)).astype(np.float32)
    X[:, :16] /= X[:, :16].sum(1, keepdims=True)
    T = (3.0 * X[:, 16] - 2.0 * X[:, 17] + X[:, :16] @ np.linspace(-1, 1, 16)).astype(np.float32)
    return X, T


def test_forward_matches_cpu(nm):
    from oracle import cost_model as cm
    m = nm.CostModel(seed=11)
    X, _ = data(777, 1)
    y = m.predict(X)
    ref, _ = cm.forward(cm.unpack(m.params()), X)
    assert np.abs(y - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


def test_gradient_matches_cpu(nm):
    from oracle import cost_model as cm
    m = nm.CostModel(seed=12)
    X, T = data(1500, 2)
    g, loss = m.gradient(X, T)
    ref_loss, ref_g = cm.loss_and_grad(cm.unpack(m.params()), X, T)
    ref = cm.pack(ref_g)
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    assert np.abs(g - ref).max() <= 1e-4 * np.abs(ref).max(), np.abs(g - ref).max()


def test_training_reduces_loss(nm):
    m = nm.CostModel(seed=13)
    X, T = data(4000, 3)
    _, before = m.gradient(X, T)
    after = m.train(X, T, epochs=300, lr=3e-3)
    assert after < 0.1 * before, (before, after)
    y = m.predict(X)
    assert np.corrcoef(y, T)[0, 1] > 0.9


@pytest.mark.parametrize("view,path", [(C1, 0), (shrink(C2, 96, 160, N=20000), 2)])
def test_tile_order_does_not_change_the_image(nm, view, path):
    m = setup_gpu(nm, view, path=path)
    if path:
        m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
        m.precompute()
    m.render()
    ref, ref64 = m.grid(), m.smoothing64()
    tx, ty = m.tiles()
    rng = np.random.default_rng(4)
    for order in (rng.permutation(tx * ty), np.arange(tx * ty)[::-1]):
        m.set_tile_order(order)
        m.set_option(nm.OPT_LOG_TILE_COSTS, 1)
        m.render()
        assert np.array_equal(m.grid(), ref)
        assert np.array_equal(m.smoothing64(), ref64)
        costs = m.tile_costs()
        assert costs.shape == (ty, tx) and costs.sum() > 0
    with pytest.raises(nm.NewmanError):
        m.set_tile_order(np.zeros(tx * ty, np.int32))  # not a permutation


def test_preview_shares_the_orbit(nm):
    """Preview sample (pr, pc) is full-grid sample (f pr + f - 1, f pc):
    same coordinates, same orbit, same result."""
    v = shrink(C2, 96, 160, N=20000)
    m = setup_gpu(nm, v, path=nm.PATH_FE32)
    m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    m.precompute()
    m.render()
    f = 8
    p = m.preview(f)
    assert (p.rows(), p.cols()) == (m.rows() // f, m.cols() // f)
    p.render()
    full = m.grid()
    assert np.array_equal(p.grid(), full[f - 1::f, ::f])
    feats = p.tile_features(4, 4)
    assert feats.shape == ((p.cols() // 4) * (p.rows() // 4), 18)
    assert np.allclose(feats[:, :16].sum(1), 1.0)
    assert (feats[:, 16] <= feats[:, 17] + 1e-7).all()
    # an iteration cap renders as if N were the cap: min(full count, cap)
    sub = full["iterations"][f - 1::f, ::f]
    cap = int(np.median(sub))
    p.set_option(nm.OPT_ITER_CAP, cap)
    p.render()
    assert np.array_equal(p.grid()["iterations"], np.minimum(sub, cap))


def test_preview_reads_the_orbit_in_place(nm):
    """On a view past the double loop (a crop of C2 at its own sample
    spacing, 64 bits) the preview reads the view's orbit and series in place:
    it renders the view's samples, and once the view is precomputed again it
    refuses to render rather than read tables that were replaced."""
    v = dict(C2, nr=48, nc=80, N=20000)
    m = setup_gpu(nm, v, path=nm.PATH_FE32)
    m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    m.precompute()
    assert not m.useHardware()
    m.render()
    f = 4
    p = m.preview(f)
    p.render()
    assert np.array_equal(p.grid(), m.grid()[f - 1::f, ::f])
    q = p.copy()  # a copy of the preview shares the same orbit
    q.render()
    assert np.array_equal(q.grid(), p.grid())
    m.precompute()
    for h in (p, q):
        with pytest.raises(nm.NewmanError):
            h.render()


def test_order_tiles_on_the_gpu(nm):
    """nm_order_tiles: features, forward pass and sort on the GPU give the
    permutation of a stable host sort of -prediction, and the render under it
    is the static order's image bit for bit."""
    v = dict(C2, nr=64, nc=96, N=20000)
    m = setup_gpu(nm, v, path=nm.PATH_FE32)
    m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    m.precompute()
    m.set_option(nm.OPT_TILE_W, 16)
    m.set_option(nm.OPT_TILE_H, 16)
    m.render()
    ref = m.grid()
    assert m.tile_order() is None
    f = 4
    p = m.preview(f)
    p.render()
    model = nm.CostModel(seed=5)
    X = p.tile_features(16 // f, 16 // f)
    model.train(X, np.linspace(-1, 1, len(X)).astype(np.float32), epochs=50, lr=3e-3)
    pred = model.predict(X)
    m.order_tiles(p, model)
    order = m.tile_order()
    assert np.array_equal(order, np.argsort(-pred, kind="stable"))
    assert np.array_equal(model.predict(X), pred)  # the model's inputs were not disturbed
    m.render()
    assert np.array_equal(m.grid(), ref)
    c = m.copy()  # a copy carries the order (read back to the host)
    assert np.array_equal(c.tile_order(), order)
    m.set_tile_order(None)
    assert m.tile_order() is None
