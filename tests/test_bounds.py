"""Host checks of the rounding bounds the GPU certificates rest on, on seeded
random inputs with exact rational arithmetic as the yardstick:

* the double loop's step F (mandelbrot.cpp:242-246, doubles in the reference's
  order) against f(z) = z^2 + c:  |F(z) - f(z)| <= 2^-53 (3|z|^2 + |F(z)|_1)(1 + 2^-52),
  and |F(z)|_1 <= 1.5 (|z|^2 + |c|_1) -- the interior trapping of double-loop
  views (fe_core.cuh) propagates a disk with these;
* the float-float sum t = 2Z + delta of the FE32 step (ff32.cuh):
  |t.h|_1 <= (2|Z.h|_1 + |delta.h|_1)(1 + 2^-22.9), which lets the step's two local
  rounding terms share one product (kFeUT).
"""
from fractions import Fraction as Q

import numpy as np


def _double_loop_step(zr, zi, cr, ci):
    # the reference's order: squares of the current z, then the new z
    sr, si = zr * zr, zi * zi
    nr = (sr - si) + cr
    ni = 2.0 * (zr * zi) + ci  # (2 zr) zi == 2 (zr zi) exactly
    return nr, ni


def test_double_loop_rounding_bound():
    rng = np.random.default_rng(11)
    worst = 0.0
    for _ in range(20000):
        # |z| up to 2 (interior orbits), |c| up to 2.5; some tiny and some
        # cancelling components
        zr, zi = rng.uniform(-1.5, 1.5, 2) * 10.0 ** rng.integers(-6, 1, 2)
        cr, ci = rng.uniform(-2.0, 0.5), rng.uniform(-1.2, 1.2)
        fr, fi = _double_loop_step(float(zr), float(zi), float(cr), float(ci))
        er = Q(zr) * Q(zr) - Q(zi) * Q(zi) + Q(cr)
        ei = 2 * Q(zr) * Q(zi) + Q(ci)
        err = abs(Q(fr) - er) + abs(Q(fi) - ei)  # 1-norm >= Euclidean
        z2 = Q(zr) * Q(zr) + Q(zi) * Q(zi)
        bound = Q(1, 2 ** 53) * (3 * z2 + abs(Q(fr)) + abs(Q(fi))) * (1 + Q(1, 2 ** 52))
        assert err <= bound
        worst = max(worst, float(err / bound) if bound else 0.0)
        assert abs(fr) + abs(fi) <= 1.5 * (float(z2) + abs(cr) + abs(ci)) * (1 + 2.0 ** -50)
    assert worst > 0.01  # the bound is not vacuous on these inputs


def _ff_add(ah, al, bh, bl):
    f = np.float32
    ah, al, bh, bl = f(ah), f(al), f(bh), f(bl)
    s = f(ah + bh)
    bb = f(s - ah)
    e = f(f(ah - f(s - bb)) + f(bh - bb))
    lo = f(e + f(al + bl))
    h = f(s + lo)
    return h, f(lo - f(h - s))


def _ff_of(x):
    h = np.float32(x)
    return h, np.float32(x - float(h))


def test_float_float_t_bound():
    rng = np.random.default_rng(12)
    limit = 1.0 + 2.0 ** -22.9
    for _ in range(50000):
        z = rng.uniform(-2.0, 2.0) * 10.0 ** rng.integers(-3, 1)
        d = rng.uniform(-2.0, 2.0) * 10.0 ** rng.integers(-12, 1)
        if rng.random() < 0.2:
            d = -2.0 * z * (1.0 + rng.uniform(-1e-6, 1e-6))  # cancellation near a rebase
        zh, zl = _ff_of(z)
        dh, dl = _ff_of(d)
        th, _ = _ff_add(2.0 * zh, 2.0 * zl, dh, dl)
        assert abs(float(th)) <= (2.0 * abs(float(zh)) + abs(float(dh))) * limit
