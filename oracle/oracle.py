"""ctypes binding of the oracle (test infrastructure only).

`OracleView` mirrors the reference's `Mandelbrot` object (mandelbrot.h:7-53)
closely enough for the tests to drive both sides with the same calls.  Only
tests/, the smoke check and bench.py's CPU-baseline leg import this module.
"""
import ctypes
import os

import numpy as np

from . import build as _build

MODE_REF = 0
MODE_DELTA = 1
MODE_REF_FE = 2
MODE_DELTA_FE = 3
MODE_DELTA_SINGLE = 4  # planted mistake: no rebase on |Y| < |delta|

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, i32, dbl, cp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_char_p
        P = ctypes.POINTER
        L.nmo_create.restype = vp
        L.nmo_create.argtypes = [i32, i32]
        L.nmo_destroy.argtypes = [vp]
        L.nmo_set_view.argtypes = [vp, cp, cp, cp, cp, i32, dbl, i32]
        L.nmo_set_iterations.argtypes = [vp, i32]
        for f in ("nmo_rows", "nmo_cols", "nmo_bits", "nmo_use_hardware", "nmo_probe_index",
                  "nmo_orbit_length"):
            getattr(L, f).argtypes = [vp]
        L.nmo_scale_up.argtypes = [vp, i32]
        L.nmo_scale_down.argtypes = [vp, i32]
        L.nmo_precompute.argtypes = [vp, i32]
        L.nmo_precompute_center.argtypes = [vp]
        L.nmo_export_orbit.argtypes = [vp] + [P(dbl)] * 5
        L.nmo_coords.argtypes = [vp, P(dbl), P(dbl)]
        L.nmo_render_pixels.argtypes = [vp, i32, ctypes.c_long, P(ctypes.c_int32),
                                        P(ctypes.c_int32), P(ctypes.c_int32), P(dbl), i32]
        L.nmo_render_rows.argtypes = [vp, i32, i32, i32, P(ctypes.c_int32), P(dbl), i32]
        L.nmo_reduce.argtypes = [i32, i32, i32, P(ctypes.c_int32), P(ctypes.c_float),
                                 P(ctypes.c_int32), P(ctypes.c_float)]
        L.nmo_series_skip.argtypes = [vp, ctypes.c_long, P(ctypes.c_int32), P(ctypes.c_int32),
                                      P(ctypes.c_int32)]
        L.nmo_get_view.argtypes = [vp, i32, ctypes.c_char_p, i32]
        L.nmo_palette_cache.argtypes = [ctypes.c_char_p, i32, vp]
        L.nmo_colorize.argtypes = [vp, vp, i32, i32, i32, vp, i32, i32, vp]
        L.nmo_video_interpolate.argtypes = [vp, vp, i32, i32, i32, i32, i32, vp]
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def default_threads():
    return max(1, os.cpu_count() or 1)


class OracleView:
    """CPU restatement of one `Mandelbrot` object."""

    def __init__(self, nr, nc):
        self._h = lib().nmo_create(nr, nc)
        if not self._h:
            raise ValueError("bad grid size")

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h and _lib is not None:
            _lib.nmo_destroy(h)

    def set_view(self, cre, cim, sre, sim, N, tol=1e-10, min_bits=0):
        rc = lib().nmo_set_view(self._h, str(cre).encode(), str(cim).encode(), str(sre).encode(),
                                str(sim).encode(), int(N), float(tol), int(min_bits))
        if rc:
            raise ValueError("nmo_set_view failed: %d" % rc)

    def set_iterations(self, N):
        if lib().nmo_set_iterations(self._h, int(N)):
            raise ValueError("bad N")

    rows = property(lambda self: lib().nmo_rows(self._h))
    cols = property(lambda self: lib().nmo_cols(self._h))
    bits = property(lambda self: lib().nmo_bits(self._h))
    probe_index = property(lambda self: lib().nmo_probe_index(self._h))
    orbit_length = property(lambda self: lib().nmo_orbit_length(self._h))

    def use_hardware(self):
        return bool(lib().nmo_use_hardware(self._h))

    def scale_up(self, sc):
        assert lib().nmo_scale_up(self._h, sc) == 0

    def scale_down(self, sc):
        assert lib().nmo_scale_down(self._h, sc) == 0

    def precompute(self, threads=None, center=False):
        if center:
            assert lib().nmo_precompute_center(self._h) == 0
        else:
            assert lib().nmo_precompute(self._h, threads or default_threads()) == 0

    def export_orbit(self):
        n = self.orbit_length
        arrs = [np.zeros(2 * n, np.float64) for _ in range(5)]
        lib().nmo_export_orbit(self._h, *[_p(a, ctypes.c_double) for a in arrs])
        x, xlo, a, b, c = [a.reshape(n, 2) for a in arrs]
        return dict(x=x, xlo=xlo, a=a, b=b, c=c)

    def coords(self):
        re = np.zeros(self.cols, np.float64)
        im = np.zeros(self.rows, np.float64)
        lib().nmo_coords(self._h, _p(re, ctypes.c_double), _p(im, ctypes.c_double))
        return re, im

    def render_pixels(self, rows, cols, mode=MODE_REF, threads=None):
        rows = np.ascontiguousarray(rows, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        it = np.zeros(rows.shape, np.int32)
        sm = np.zeros(rows.shape, np.float64)
        rc = lib().nmo_render_pixels(self._h, mode, rows.size, _p(rows, ctypes.c_int32),
                                     _p(cols, ctypes.c_int32), _p(it, ctypes.c_int32),
                                     _p(sm, ctypes.c_double), threads or default_threads())
        if rc:
            raise RuntimeError("nmo_render_pixels failed: %d" % rc)
        return it, sm

    def render_rows(self, r0, r1, mode=MODE_REF, threads=None):
        n = (r1 - r0) * self.cols
        it = np.zeros(n, np.int32)
        sm = np.zeros(n, np.float64)
        rc = lib().nmo_render_rows(self._h, mode, r0, r1, _p(it, ctypes.c_int32),
                                   _p(sm, ctypes.c_double), threads or default_threads())
        if rc:
            raise RuntimeError("nmo_render_rows failed: %d" % rc)
        return it.reshape(r1 - r0, self.cols), sm.reshape(r1 - r0, self.cols)

    def series_skip(self, rows, cols):
        """d.size() after the series loop for each sample (-1: cardioid)."""
        rows = np.ascontiguousarray(rows, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        out = np.zeros(rows.shape, np.int32)
        rc = lib().nmo_series_skip(self._h, rows.size, _p(rows, ctypes.c_int32),
                                   _p(cols, ctypes.c_int32), _p(out, ctypes.c_int32))
        if rc:
            raise RuntimeError("nmo_series_skip failed: %d" % rc)
        return out

    def get_view(self):
        out = []
        for w in range(4):
            buf = ctypes.create_string_buffer(8192)
            assert lib().nmo_get_view(self._h, w, buf, 8192) == 0
            out.append(buf.value.decode())
        return out


def reduce(iters, smooth, sc):
    """mandelbrot.cpp:320-332 over a (nr*sc, nc*sc) sample grid."""
    iters = np.ascontiguousarray(iters, np.int32)
    smooth = np.ascontiguousarray(smooth, np.float32)
    NR, NC = iters.shape
    nr, nc = NR // sc, NC // sc
    oi = np.zeros((nr, nc), np.int32)
    os_ = np.zeros((nr, nc), np.float32)
    lib().nmo_reduce(nr, nc, sc, _p(iters, ctypes.c_int32), _p(smooth, ctypes.c_float),
                     _p(oi, ctypes.c_int32), _p(os_, ctypes.c_float))
    return oi, os_


def palette_cache(path, n):
    """MultiWaveGenerator::cache(n) of the palette file at `path`: (n, 3) uint8."""
    out = np.empty((n, 3), np.uint8)
    if lib().nmo_palette_cache(str(path).encode(), int(n), out.ctypes.data):
        raise IOError("cannot read palette %s" % path)
    return out


def colorize(iters, smooth, N, pal, sc, smooth_flag=True):
    """colorLine over every row: (rows/sc, cols/sc, 3) uint8."""
    iters = np.ascontiguousarray(iters, dtype=np.int32)
    smooth = np.ascontiguousarray(smooth, dtype=np.float32)
    pal = np.ascontiguousarray(pal, dtype=np.uint8)
    nr, nc = iters.shape
    out = np.empty((nr // sc, nc // sc, 3), np.uint8)
    lib().nmo_colorize(iters.ctypes.data, smooth.ctypes.data, nr, nc, int(N), pal.ctypes.data,
                       int(sc), 1 if smooth_flag else 0, out.ctypes.data)
    return out


def video_interpolate(prev, cur, rows, cols, rate):
    """VideoZoom::nextFrame's `rate` frames between keyframes prev and cur
    ((kh, kw, 3) uint8 each): (rate, rows, cols, 3) uint8."""
    prev = np.ascontiguousarray(prev, dtype=np.uint8)
    cur = np.ascontiguousarray(cur, dtype=np.uint8)
    out = np.empty((rate, rows, cols, 3), np.uint8)
    lib().nmo_video_interpolate(prev.ctypes.data, cur.ctypes.data, prev.shape[0], prev.shape[1],
                                rows, cols, rate, out.ctypes.data)
    return out
