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


# ---- the float-float complex multiply-add of the FE32 step ----------------------

def _rn32(q):
    """q (a Fraction) rounded to the nearest float32, ties to even (normal range)."""
    if q == 0:
        return Q(0)
    sign = -1 if q < 0 else 1
    a = abs(q)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Q(2) ** e > a:
        e -= 1
    scale = Q(2) ** (23 - e)  # a * scale in [2^23, 2^24)
    m = a * scale
    fl = m.numerator // m.denominator
    rem = m - fl
    if rem > Q(1, 2) or (rem == Q(1, 2) and fl % 2 == 1):
        fl += 1
    return sign * Q(fl) / scale


def _add(a, b):
    return _rn32(a + b)


def _mul(a, b):
    return _rn32(a * b)


def _fma(a, b, c):
    return _rn32(a * b + c)


def _two_sum(a, b):
    s = _add(a, b)
    bb = _add(s, -a)
    return s, _add(_add(a, -_add(s, -bb)), _add(b, -bb))


def _fast_two_sum(a, b):
    s = _add(a, b)
    return s, _add(b, -_add(s, -a))


def _cmul_add(ar, ai, br, bi, c, d):
    """ff32.cuh's ff_cmul_add, step for step, on (hi, lo) pairs of Fractions."""
    p1 = _mul(ar[0], br[0]); e1 = _fma(ar[0], br[0], -p1)
    p2 = _mul(ai[0], bi[0]); e2 = _fma(ai[0], bi[0], -p2)
    s = _two_sum(p1, -p2)
    s2 = _two_sum(s[0], c[0])
    lo = _add(_add(s[1], s2[1]), _add(e1, -e2))
    lo = _fma(ar[0], br[1], lo)
    lo = _fma(ar[1], br[0], lo)
    lo = _fma(-ai[0], bi[1], lo)
    lo = _fma(-ai[1], bi[0], lo)
    lo = _add(lo, c[1])
    outr = _fast_two_sum(s2[0], lo)
    p1 = _mul(ar[0], bi[0]); e1 = _fma(ar[0], bi[0], -p1)
    p2 = _mul(ai[0], br[0]); e2 = _fma(ai[0], br[0], -p2)
    s = _two_sum(p1, p2)
    s2 = _two_sum(s[0], d[0])
    lo = _add(_add(s[1], s2[1]), _add(e1, e2))
    lo = _fma(ar[0], bi[1], lo)
    lo = _fma(ar[1], bi[0], lo)
    lo = _fma(ai[0], br[1], lo)
    lo = _fma(ai[1], br[0], lo)
    lo = _add(lo, d[1])
    outi = _fast_two_sum(s2[0], lo)
    return outr, outi


def _ffq(x):
    h = _rn32(Q(x))
    return h, _rn32(Q(x) - h)


def test_float_float_multiply_add_rounding_bound():
    """|delta' - (t delta + eps)| <= u (|t.h|_1 |delta.h|_1 + |eps|_1), u = 0x1.2p-43
    (the FE32 certificate's kFeU; its derivation takes every low-word term at
    its worst)."""
    rng = np.random.default_rng(13)
    u = Q(9, 8) * Q(1, 2 ** 43)
    worst = Q(0)
    for _ in range(4000):
        t = [_ffq(rng.uniform(-4, 4) * 10.0 ** rng.integers(-2, 1)) for _ in range(2)]
        dl = [_ffq(rng.uniform(-1, 1) * 10.0 ** rng.integers(-8, 0)) for _ in range(2)]
        ep = [_ffq(rng.uniform(-1, 1) * 10.0 ** rng.integers(-10, -2)) for _ in range(2)]
        (nr, ni) = _cmul_add(t[0], t[1], dl[0], dl[1], ep[0], ep[1])
        T = [a[0] + a[1] for a in t]
        D = [a[0] + a[1] for a in dl]
        E = [a[0] + a[1] for a in ep]
        xr = T[0] * D[0] - T[1] * D[1] + E[0]
        xi = T[0] * D[1] + T[1] * D[0] + E[1]
        err = abs(nr[0] + nr[1] - xr) + abs(ni[0] + ni[1] - xi)
        bound = u * ((abs(t[0][0]) + abs(t[1][0])) * (abs(dl[0][0]) + abs(dl[1][0]))
                     + abs(ep[0][0]) + abs(ep[1][0]))
        assert err <= bound
        worst = max(worst, err / bound)
    assert worst > Q(1, 1000)  # not vacuous


def _add_twice_raw(zh, zl, dh, dl):
    """ff32.cuh's ff_add_twice_raw (t = 2Z + delta, not renormalised)."""
    s = _fma(Q(2), zh, dh)
    bb = _fma(Q(-2), zh, s)
    e = _add(_fma(Q(2), zh, -_add(s, -bb)), _add(dh, -bb))
    return s, _add(e, _fma(Q(2), zl, dl))


def test_fe32_step_local_error_bound():
    """One FE32 step's arithmetic, t = 2Z + delta unnormalised then the
    float-float multiply-add, against (2Z + delta) delta + eps in exact
    arithmetic: within (kFeUT - u_z) P' + u |eps|_1, P' = (2|Z.h|_1 + |delta.h|_1)
    |delta.h|_1 (fe_core.cuh's derivation), also where 2Z + delta cancels."""
    rng = np.random.default_rng(21)
    k_t = Q(0x194, 256) * Q(1, 2 ** 43) - Q(1, 2 ** 45)  # kFeUT - u_z = 1.328125 * 2^-43
    u = Q(9, 8) * Q(1, 2 ** 43)
    worst = Q(0)
    for _ in range(3000):
        z = [_ffq(rng.uniform(-2, 2) * 10.0 ** rng.integers(-3, 1)) for _ in range(2)]
        d = [_ffq(rng.uniform(-1, 1) * 10.0 ** rng.integers(-8, 1)) for _ in range(2)]
        if rng.random() < 0.3:  # Y near -Z: t = 2Z + delta cancels
            k = int(rng.integers(0, 2))
            d[k] = _ffq(float(-2 * (z[k][0] + z[k][1])) * (1 + rng.uniform(-1e-6, 1e-6)))
        ep = [_ffq(rng.uniform(-1, 1) * 10.0 ** rng.integers(-12, -2)) for _ in range(2)]
        t = [_add_twice_raw(z[k][0], z[k][1], d[k][0], d[k][1]) for k in range(2)]
        for k in range(2):  # |t.h| <= (2|Z.h| + |delta.h|)(1 + 2^-24)
            assert abs(t[k][0]) <= (2 * abs(z[k][0]) + abs(d[k][0])) * (1 + Q(1, 2 ** 24))
        (nr, ni) = _cmul_add(t[0], t[1], d[0], d[1], ep[0], ep[1])
        T = [2 * (z[k][0] + z[k][1]) + d[k][0] + d[k][1] for k in range(2)]
        D = [a[0] + a[1] for a in d]
        E = [a[0] + a[1] for a in ep]
        xr = T[0] * D[0] - T[1] * D[1] + E[0]
        xi = T[0] * D[1] + T[1] * D[0] + E[1]
        err = abs(nr[0] + nr[1] - xr) + abs(ni[0] + ni[1] - xi)
        p = (2 * (abs(z[0][0]) + abs(z[1][0])) + abs(d[0][0]) + abs(d[1][0])) * (abs(d[0][0]) + abs(d[1][0]))
        bound = k_t * p + u * (abs(ep[0][0]) + abs(ep[1][0]))
        assert err <= bound
        worst = max(worst, err / bound)
    assert worst > Q(1, 1000)  # not vacuous


def test_eps_below_the_double_range_is_below_half_an_ulp():
    """The plain FP64 step on floatexp views leaves out an eps component below
    2^-1022 (pixel_xd.cuh: plain_eps): exact because every sum it would be
    added to is nonzero and at least 2^-400 in magnitude (the guard), so the
    correctly rounded sum is the sum itself."""
    rng = np.random.default_rng(14)
    for _ in range(20000):
        q = float(rng.uniform(1.0, 2.0) * 2.0 ** int(rng.integers(-400, 60)) * rng.choice([-1, 1]))
        eps = Q(int(rng.integers(1, 2 ** 53)), 2 ** int(rng.integers(1075, 1700)))  # < 2^-1022
        eps = eps if rng.random() < 0.5 else -eps
        assert float(Q(q) + eps) == q  # float(Fraction) rounds to nearest


def test_quick_bailout_decision_is_implied():
    """fe_core.cuh decides the bailout test without evaluating it while
    |Y|^2 <= 2^20 (1 - 2^-10), Z is not the orbit's escaped last point and the
    bound e < 0.2: then |Z.h|_1 < 1449 and |delta.h|_1 < 2900, and the full test's
    band 2 (2^-20 (|Z| + |delta|) + yerr) stays below 1024 - |Y|.  Checked at the
    extremes of those ranges, in exact arithmetic."""
    kfeu, kfeuz = Q(9, 8) * Q(1, 2 ** 43), Q(1, 2 ** 45)
    lo_band = Q(2 ** 20) * (1 - Q(1, 2 ** 10))
    ym_max = Q(1024) * (1 - Q(1, 2 ** 11)) * (1 + Q(1, 2 ** 21))  # sqrt(lo_band) and rsqrt's error
    assert ym_max ** 2 >= lo_band
    zn1, dn1, err = Q(1449), Q(2900), Q(1, 5)
    yerr = err + kfeuz * zn1 + kfeu * (zn1 + dn1)
    band = 2 * (Q(1, 2 ** 20) * (zn1 + dn1) + yerr)
    assert band < 1024 - ym_max
    # and the ranges themselves: a non-escaped orbit point and |Y| <= 1024
    assert Q(1448) ** 2 < 2 * Q(2 ** 20) < Q(1449) ** 2  # |Z|_1 <= sqrt(2) * 1024
    assert 2 * Q(1449) < 2900
