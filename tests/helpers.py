"""Views and small helpers shared by the tests."""
from decimal import Decimal, getcontext

import numpy as np


def step_for(width, cols, digits=40):
    """Pixel step width/cols as a decimal string (exact decimal division)."""
    getcontext().prec = digits
    return str(Decimal(str(width)) / Decimal(cols))


# 640x480, center -0.75+0i, width 3.0, N 1024: the reference's double path.
C1 = dict(nr=480, nc=640, sc=1, cre="-0.75", cim="0", step="0.0046875", N=1024, tol=1e-10)
# 1920x1080 with 4x4 samples, width 1e-12, N 50,000: the arbitrary-precision path.
C2 = dict(nr=1080, nc=1920, sc=4, cre="-0.743643887037151", cim="0.131825904205330",
          step=step_for("1e-12", 1920), N=50000, tol=1e-10)


def shrink(view, nr, nc, N=None):
    """Same center and width at a smaller grid (for fast tests)."""
    v = dict(view)
    width = Decimal(view["step"]) * view["nc"]
    v["nr"], v["nc"] = nr, nc
    v["step"] = step_for(width, nc)
    if N is not None:
        v["N"] = N
    return v


def setup_oracle(oracle_mod, view):
    o = oracle_mod.OracleView(view["nr"], view["nc"])
    o.set_view(view["cre"], view["cim"], view["step"], view["step"], view["N"], view["tol"],
               view.get("min_bits", 0))
    if view["sc"] > 1:
        o.scale_up(view["sc"])
    return o


def setup_gpu(nm, view, path=0, keep64=True):
    m = nm.Mandelbrot(view["nr"], view["nc"])
    m.set_view(view["cre"], view["cim"], view["step"], view["step"], view["N"], view["tol"],
               view.get("min_bits", 0))
    if view["sc"] > 1:
        m.scaleUp(view["sc"])
    m.set_path(path)
    if keep64:
        m.set_option(nm.OPT_KEEP_SMOOTH64, 1)
    return m


def zoom_frames(nframes, nr, nc, width0, width1, N0, N1, center=None):
    """The frames of a zoom video: widths geometric from width0 to width1,
    N linear from N0 to N1, all into one center (the C2 center by default)."""
    getcontext().prec = 60
    cre, cim = center or (C2["cre"], C2["cim"])
    w0, w1 = Decimal(str(width0)), Decimal(str(width1))
    out = []
    for k in range(nframes):
        t = Decimal(k) / Decimal(max(1, nframes - 1))
        w = w0 * (w1 / w0) ** t
        N = int(round(N0 + (N1 - N0) * float(t)))
        out.append(dict(nr=nr, nc=nc, cre=cre, cim=cim, step=str(w / nc), N=N, tol=1e-10))
    return out


def make_frame(nm, view, sc, deep_path, double_loop_path=None):
    """A frame handle: the reference's double path where it applies (or
    `double_loop_path` there, when given), else `deep_path` with the reference
    orbit at the view center."""
    m = nm.Mandelbrot(view["nr"], view["nc"])
    m.set_view(view["cre"], view["cim"], view["step"], view["step"], view["N"], view["tol"])
    if sc > 1:
        m.scaleUp(sc)
    if not m.useHardware():
        m.set_path(deep_path)
        m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    elif double_loop_path is not None:
        m.set_path(double_loop_path)
    return m


def sample_positions(nr, nc, n, seed):
    rng = np.random.default_rng(seed)
    k = rng.choice(nr * nc, size=min(n, nr * nc), replace=False)
    return (k // nc).astype(np.int32), (k % nc).astype(np.int32)
