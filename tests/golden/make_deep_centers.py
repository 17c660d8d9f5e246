"""Seeded boundary-following from the C2 center down to width 1e-500 (the
procedure that defines the deep C3 view at 1e-300 and the deep centers of the
learned-scheduling workload), written to deep_centers.json.

    python tests/golden/make_deep_centers.py [--steps K] [--to 1e-500] [--gpu]

Start at center -0.743643887037151+0.131825904205330i, width 1e-12.  Repeat:
render 64x64 samples (N = 1,000,000, series tolerance 1e-10, reference orbit
at the view center), recenter on the sample with the highest escape count
below N (ties broken by a seeded RNG), divide the width by 1e4 -- until the
width is at most 1e-500.  The center is carried as a 560-digit decimal
(every recentering is exact at that precision down to 1e-500).

The renders use the plain FP64 perturbation semantics (series front in
floatexp, deltas in FP64 with an unbounded exponent below the FP64 range): on
the CPU through the oracle's MODE_DELTA_FE, or with --gpu through the
library's FP64 path, which computes the same escape counts bit for bit, so
both backends follow the same trajectory.
"""
import argparse
import json
import os
import sys
from decimal import Decimal, getcontext

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

DIGITS = 560
SEED = 2026
N = 1000000
GRID = 64


def render_cpu(cre, cim, step, n):
    from oracle import oracle as om
    o = om.OracleView(GRID, GRID)
    o.set_view(cre, cim, step, step, n)
    o.precompute(center=True)
    mode = om.MODE_REF if o.use_hardware() else om.MODE_DELTA_FE
    it, _ = o.render_rows(0, GRID, mode)
    return it, o.bits


def render_gpu(cre, cim, step, n):
    import newman_gb300 as nm
    m = nm.Mandelbrot(GRID, GRID)
    m.set_view(cre, cim, step, step, n)
    # the reference's choice: its double loop while useHardware(), else FP64
    # perturbation -- what MODE_REF / MODE_DELTA_FE compute on the CPU
    m.set_path(nm.PATH_REFERENCE)
    m.set_option(nm.OPT_REFERENCE, nm.REFERENCE_CENTER)
    m.precompute()
    m.render()
    return m.grid()["iterations"].copy(), m.stat(nm.STAT_PRECISION_BITS)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--to", default="1e-500", help="stop once the width is at most this")
    ap.add_argument("--gpu", action="store_true")
    ap.add_argument("--out", default=os.path.join(HERE, "deep_centers.json"))
    args = ap.parse_args()
    getcontext().prec = DIGITS + 20
    rng = np.random.default_rng(SEED)
    cre, cim = Decimal("-0.743643887037151"), Decimal("0.131825904205330")
    width = Decimal("1e-12")
    render = render_gpu if args.gpu else render_cpu
    steps = []
    for k in range(args.steps):
        if width < Decimal(args.to) * Decimal("0.999999"):
            break
        step = width / GRID
        it, bits = render(str(cre), str(cim), str(step), N)
        below = it[it < N]
        if below.size == 0:
            raise SystemExit("every sample reached N at width %s" % width)
        best = int(below.max())
        cand = np.argwhere(it == best)
        r, c = cand[rng.integers(len(cand))]
        # pointAt(r, c): center + (c - nc/2) step, center + (nr/2 - r - 1) step
        cre = cre + (int(c) - GRID // 2) * step
        cim = cim + (GRID // 2 - int(r) - 1) * step
        getcontext().prec = DIGITS
        cre, cim = +cre, +cim
        getcontext().prec = DIGITS + 20
        steps.append({"width": str(width), "bits": int(bits), "best": best,
                      "row": int(r), "col": int(c), "candidates": int(len(cand)),
                      "next_center_re": str(cre), "next_center_im": str(cim)})
        print("width %s bits %d best %d" % (width, bits, best), flush=True)
        width = width / Decimal(10000)
    with open(args.out, "w") as f:
        json.dump({"seed": SEED, "N": N, "grid": GRID, "digits": DIGITS,
                   "start": ["-0.743643887037151", "0.131825904205330", "1e-12"],
                   "steps": steps}, f, indent=1)


if __name__ == "__main__":
    main()
