"""Generates the golden fixtures in this directory from an independent
restatement of the reference's per-pixel path in pure Python (Python floats
for the `double` code, which Python evaluates one rounding per operation like
the reference's x86-64 build; exact fractions or mpmath for the arbitrary
precision parts).  It shares no code with the oracle or the GPU library.

    python tests/golden/make_golden.py

Views use centers and steps whose decimal strings are exact binary fractions,
so that every arbitrary-precision library converts them to the same value.

hw_view.npz   : mandelbrot.cpp:231-254 (getIterationsHW) on a 480x640 view,
                center -0.75+0i, step 2^-8, N 1024, every 8th row and column.
deep_view.npz : mandelbrot.cpp:73-229 (findProbe, computeOrbit, computeSeries,
                getIterations with its arbitrary-precision continuation) on a
                16x16 view 3e-13 / 2e-13 off the C2 center, step 2^-53, N 3000,
                computed with mpmath at 320 bits.
"""
import math
import os
from decimal import Decimal
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BAILOUT = 1024.0
BAILOUT2 = BAILOUT * BAILOUT


def smoothing(r2):  # mandelbrot.cpp:133-136
    return 1.0 - math.log2(0.5 * math.log(r2) / math.log(BAILOUT))


def to_fraction(x):
    """An mpmath mpf as an exact Fraction."""
    import mpmath
    sign, man, exp, _ = mpmath.mpf(x)._mpf_  # value = (-1)^sign * man * 2^exp
    man, exp = (-1) ** sign * int(man), int(exp)
    return Fraction(man * 2 ** exp) if exp >= 0 else Fraction(man, 2 ** (-exp))


def trunc_double(q):
    """A rational (Fraction) or mpmath mpf as a double, truncated toward zero
    (mpf_get_d)."""
    if not isinstance(q, Fraction):
        q = to_fraction(q)
    if q == 0:
        return 0.0
    neg = q < 0
    a = -q if neg else q
    e = math.floor(math.log2(a.numerator) - math.log2(a.denominator))
    while Fraction(2) ** e > a:
        e -= 1
    while Fraction(2) ** (e + 1) <= a:
        e += 1
    scale = Fraction(2) ** (52 - e)
    m = math.floor(a * scale)
    v = math.ldexp(m, -(52 - e))
    return -v if neg else v


def in_cardioid(x, y):  # mandelbrot.cpp:63-71, exact
    xmf = x - Fraction(1, 4)
    y2 = y * y
    q = xmf * xmf + y2
    if q * (q + xmf) < Fraction(1, 4) * y2:
        return True
    q = x + 1
    return q * q + y2 < Fraction(1, 16)


def hw_pixel(x, y, N):  # mandelbrot.cpp:231-254
    if in_cardioid(x, y):
        return N, 0.0
    z0r, z0i = trunc_double(x), trunc_double(y)
    zr, zi = z0r, z0i
    it = 0
    while it < N:
        zr, zi = (zr * zr - zi * zi) + z0r, (2.0 * zr) * zi + z0i
        if zr * zr + zi * zi > BAILOUT2:
            break
        it += 1
    if it < N:
        return it, smoothing(zr * zr + zi * zi)
    return it, 0.0


def make_hw():
    nr, nc, N = 480, 640, 1024
    cre, cim, step = Fraction(-3, 4), Fraction(0), Fraction(1, 256)
    rows = list(range(0, nr, 8))
    cols = list(range(0, nc, 8))
    it = np.zeros((len(rows), len(cols)), np.int32)
    sm = np.zeros((len(rows), len(cols)), np.float64)
    for a, r in enumerate(rows):
        y = cim + (nr // 2 - r - 1) * step
        for b, c in enumerate(cols):
            x = cre + (c - nc // 2) * step
            it[a, b], sm[a, b] = hw_pixel(x, y, N)
    np.savez_compressed(os.path.join(HERE, "hw_view.npz"), rows=np.array(rows, np.int32),
                        cols=np.array(cols, np.int32), iterations=it, smoothing=sm,
                        nr=nr, nc=nc, N=N, center_re="-0.75", center_im="0",
                        step="0.00390625")


def make_deep():
    import mpmath
    mpmath.mp.prec = 320
    mpf = mpmath.mpf
    nr, nc, N = 16, 16, 3000
    # doubles 3e-13 and 2e-13 off the C2 center: exact binary fractions
    cre_s = str(Decimal(-0.743643887037151 + 3e-13))
    cim_s = str(Decimal(0.131825904205330 + 2e-13))
    step_s = str(Decimal(2.0 ** -53))
    cre, cim, step = mpf(cre_s), mpf(cim_s), mpf(step_s)

    def point(r, c):
        return cre + (c - nc // 2) * step, cim + (nr // 2 - r - 1) * step

    def bailed(zr, zi):
        a, b = trunc_double(zr), trunc_double(zi)
        return a * a + b * b > BAILOUT2

    def orbit(x0, y0, store):  # mandelbrot.cpp:97-110
        X = [(x0, y0)]
        xr, xi = x0, y0
        for i in range(1, N):
            xr, xi = xr * xr - xi * xi + x0, 2 * (xr * xi) + y0
            if bailed(xr, xi):
                return X if store else i
            if store:
                X.append((xr, xi))
        return X if store else N

    # findProbe, mandelbrot.cpp:73-95: longest orbit, first on ties
    pts = []
    for c in range(0, nc, 2):
        pts += [(nr // 4, c), (nr // 2, c), (3 * nr // 4, c)]
    pts += [(r, nc // 2) for r in range(0, nr, 2)]
    lens = [orbit(*point(r, c), store=False) for r, c in pts]
    best = max(range(len(pts)), key=lambda k: (lens[k], -k))
    X = orbit(*point(*pts[best]), store=True)

    # computeSeries, mandelbrot.cpp:112-131
    A, B, C = [(mpf(1), mpf(0))], [(mpf(0), mpf(0))], [(mpf(0), mpf(0))]
    for i in range(1, len(X)):
        xr, xi = X[i - 1]
        ar, ai = A[-1]
        br, bi = B[-1]
        cr, ci = C[-1]
        nar = 2 * (xr * ar - xi * ai) + 1
        nai = 2 * (xr * ai + xi * ar)
        nbr = 2 * (xr * br - xi * bi) + nar * nar - nai * nai
        nbi = 2 * (xr * bi + xi * br + nar * nai)
        ncr = 2 * (xr * cr - xi * ci + nar * nbr - nai * nbi)
        nci = 2 * (xr * ci + xi * cr + nar * nbi + nai * nbr)
        A.append((nar, nai))
        B.append((nbr, nbi))
        C.append((ncr, nci))
    Ad = [(trunc_double(a), trunc_double(b)) for a, b in A]
    Bd = [(trunc_double(a), trunc_double(b)) for a, b in B]
    Cd = [(trunc_double(a), trunc_double(b)) for a, b in C]

    def cmul(a, b):
        return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])

    skips = []

    def pixel(y0r, y0i):  # getIterations, mandelbrot.cpp:144-229
        if in_cardioid(to_fraction(y0r), to_fraction(y0i)):
            skips.append(-1)
            return N, 0.0
        eps = (trunc_double(y0r - X[0][0]), trunc_double(y0i - X[0][1]))
        eps2 = (eps[0] * eps[0] - eps[1] * eps[1], (2.0 * eps[0]) * eps[1])
        eps3 = cmul(eps, eps2)
        d = [eps]
        for i in range(1, len(X)):
            a = cmul(Ad[i], eps)
            b = cmul(Bd[i], eps2)
            c = cmul(Cd[i], eps3)
            if (b[0] * b[0] + b[1] * b[1]) * 1e-10 < c[0] * c[0] + c[1] * c[1]:
                d = d[:max(i - 3, 1)]
                break
            d.append(((a[0] + b[0]) + c[0], (a[1] + b[1]) + c[1]))
        skips.append(len(d))
        found = len(d) - 1

        def y_at(k):
            return X[k][0] + d[k][0], X[k][1] + d[k][1]

        if bailed(*y_at(found)):
            low, high, mid = 0, len(d) - 1, len(d) // 2
            while low <= high:
                if not bailed(*y_at(mid)):
                    low = mid + 1
                else:
                    high, found = mid - 1, mid
                mid = (low + high) // 2
            yr, yi = y_at(found)
            a, b = trunc_double(yr), trunc_double(yi)
            return found, smoothing(a * a + b * b)
        yr, yi = y_at(found)
        for i in range(len(d), N):
            yr, yi = yr * yr - yi * yi + y0r, 2 * (yr * yi) + y0i
            if bailed(yr, yi):
                a, b = trunc_double(yr), trunc_double(yi)
                return i, smoothing(a * a + b * b)
        return N, 0.0

    it = np.zeros((nr, nc), np.int32)
    sm = np.zeros((nr, nc), np.float64)
    for r in range(nr):
        for c in range(nc):
            it[r, c], sm[r, c] = pixel(*point(r, c))
    np.savez_compressed(os.path.join(HERE, "deep_view.npz"), iterations=it, smoothing=sm,
                        series_skip=np.array(skips, np.int32).reshape(nr, nc),
                        nr=nr, nc=nc, N=N, center_re=cre_s, center_im=cim_s, step=step_s,
                        probe_index=best, orbit_length=len(X))


if __name__ == "__main__":
    make_hw()
    make_deep()
    print("written", os.listdir(HERE))
