"""newman_gb300: GPU per-pixel Mandelbrot path with the reference's interface.

`Mandelbrot` mirrors the C++ class of axnjaxn/newman (mandelbrot.h:7-53) over
the C ABI of include/newman_gb300.h: the same fields (N, error_tolerance,
center, sz), the same calls (precompute, computeRow, at, scaleUp, scaleDown,
pointAt, translate, zoom, zoomAt, loadLegacy) and the same grid of
{int32 iterations, float smoothing} samples.  The per-sample work always runs
in the CUDA library; if the library is missing, importing this module fails.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libnewman_gb300.so")

# include/newman_gb300.h
NM_OK, NM_ERR_ARG, NM_ERR_PARSE, NM_ERR_STATE, NM_ERR_CUDA, NM_ERR_CANCELLED, NM_ERR_IO, \
    NM_ERR_UNSUPPORTED = range(8)
PATH_REFERENCE, PATH_FP64, PATH_FE32, PATH_MP = 0, 1, 2, 3
OPT_TILE_W, OPT_TILE_H, OPT_CHUNK, OPT_KEEP_SMOOTH64, OPT_THREADS, OPT_BLOCKS, OPT_RENORM, \
    OPT_FE32_SINGLE_PASS, OPT_REFERENCE, OPT_BATCH_GRAPH, OPT_FE32_OVERLAP, \
    OPT_LOG_TILE_COSTS, OPT_BATCH_FP64_WARPS, OPT_ORBIT_STAGE, OPT_L2_WINDOW, OPT_ITER_CAP = range(16)
REFERENCE_PROBES, REFERENCE_CENTER = 0, 1
STAT_CARDIOID_UNDECIDED, STAT_EXECUTED_ITERS, STAT_SAMPLES, STAT_REBASES, STAT_FP64_REWORK, \
    STAT_WAIT_TIMEOUTS, STAT_FRONT_FP64, STAT_STAGE_FALLBACKS = range(8)
STAT_ORBIT_LENGTH, STAT_PROBE_INDEX, STAT_PRECISION_BITS, STAT_PRECOMPUTE_US = 16, 17, 18, 19
STAT_KERNEL_NS, STAT_REWORK_KERNEL_NS, STAT_ITER_KERNEL_NS, STAT_KERNEL_LAUNCHES = 20, 21, 22, 23

COST_FEATURES, COST_PARAMS = 18, 9601

ESCAPE_DTYPE = np.dtype([("iterations", "<i4"), ("smoothing", "<f4")])

# Every symbol include/newman_gb300.h declares.
EXPORTS = (
    "nm_create", "nm_copy", "nm_destroy", "nm_last_error", "nm_set_view", "nm_get_view",
    "nm_set_iterations", "nm_get_iterations", "nm_set_tolerance", "nm_rows", "nm_cols",
    "nm_use_hardware", "nm_set_path", "nm_set_option", "nm_get_stat", "nm_precompute",
    "nm_upload", "nm_get_orbit", "nm_compute_row", "nm_render_rows", "nm_render", "nm_synchronize", "nm_cancel",
    "nm_at", "nm_at_sc", "nm_scale_up", "nm_scale_down", "nm_reduce", "nm_get_grid",
    "nm_get_smoothing64", "nm_device_grid", "nm_point_at", "nm_translate", "nm_zoom",
    "nm_zoom_at", "nm_load_legacy", "nm_save", "nm_render_fe32_noalloc",
    "nm_batch_create", "nm_batch_destroy", "nm_batch_add", "nm_batch_set_option",
    "nm_batch_render", "nm_batch_get_stat", "nm_batch_frames", "nm_batch_autotune",
    "nm_preview", "nm_tiles", "nm_set_tile_order", "nm_get_tile_costs", "nm_tile_features",
    "nm_order_tiles", "nm_get_tile_order", "nm_cost_model_create", "nm_cost_model_destroy", "nm_cost_model_params",
    "nm_cost_model_set_params", "nm_cost_model_predict", "nm_cost_model_gradient",
    "nm_cost_model_train", "nm_palette_load", "nm_palette_save", "nm_palette_destroy",
    "nm_palette_cache", "nm_colorize", "nm_write_ppm", "nm_video_interpolate",
)


class NewmanError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


class EscapeValue(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("smoothing", ctypes.c_float)]


_lib = None


def load_library(path=LIB_PATH):
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("newman_gb300 CUDA library not built (%s); run "
                          "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    L = ctypes.CDLL(path)
    vp, i32, dbl, cp, ll = (ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_char_p,
                            ctypes.c_longlong)
    P = ctypes.POINTER
    sig = {
        "nm_create": (vp, [i32, i32]),
        "nm_copy": (vp, [vp]),
        "nm_destroy": (None, [vp]),
        "nm_last_error": (cp, []),
        "nm_set_view": (i32, [vp, cp, cp, cp, cp, i32, dbl, i32]),
        "nm_get_view": (i32, [vp, i32, cp, i32]),
        "nm_set_iterations": (i32, [vp, i32]),
        "nm_get_iterations": (i32, [vp]),
        "nm_set_tolerance": (i32, [vp, dbl]),
        "nm_rows": (i32, [vp]),
        "nm_cols": (i32, [vp]),
        "nm_use_hardware": (i32, [vp]),
        "nm_set_path": (i32, [vp, i32]),
        "nm_set_option": (i32, [vp, i32, ll]),
        "nm_get_stat": (i32, [vp, i32, P(ll)]),
        "nm_precompute": (i32, [vp]),
        "nm_upload": (i32, [vp]),
        "nm_get_orbit": (i32, [vp, vp, vp, vp, vp, vp, i32]),
        "nm_compute_row": (i32, [vp, i32]),
        "nm_render_rows": (i32, [vp, i32, i32, vp]),
        "nm_render": (i32, [vp]),
        "nm_synchronize": (i32, [vp]),
        "nm_cancel": (i32, [vp]),
        "nm_at": (i32, [vp, i32, i32, P(EscapeValue)]),
        "nm_at_sc": (i32, [vp, i32, i32, i32, P(EscapeValue)]),
        "nm_scale_up": (i32, [vp, i32]),
        "nm_scale_down": (i32, [vp, i32]),
        "nm_reduce": (i32, [vp, i32, vp]),
        "nm_get_grid": (i32, [vp, vp]),
        "nm_get_smoothing64": (i32, [vp, vp]),
        "nm_device_grid": (i32, [vp, P(vp), P(vp)]),
        "nm_point_at": (i32, [vp, i32, i32, i32, cp, cp, i32]),
        "nm_translate": (i32, [vp, i32, i32, i32]),
        "nm_zoom": (i32, [vp, ctypes.c_float]),
        "nm_zoom_at": (i32, [vp, ctypes.c_float, i32, i32, i32]),
        "nm_load_legacy": (i32, [vp, cp]),
        "nm_save": (i32, [vp, cp]),
        "nm_render_fe32_noalloc": (i32, [vp, vp, vp]),
        "nm_batch_create": (vp, [i32]),
        "nm_batch_destroy": (None, [vp]),
        "nm_batch_add": (i32, [vp, vp]),
        "nm_batch_set_option": (i32, [vp, i32, ll]),
        "nm_batch_render": (i32, [vp]),
        "nm_batch_get_stat": (i32, [vp, i32, P(ll)]),
        "nm_batch_frames": (i32, [vp, vp]),
        "nm_batch_autotune": (i32, [vp, i32, P(i32), P(i32), P(i32)]),
        "nm_preview": (vp, [vp, i32]),
        "nm_tiles": (i32, [vp, P(i32), P(i32)]),
        "nm_set_tile_order": (i32, [vp, vp, i32]),
        "nm_get_tile_costs": (i32, [vp, vp, i32]),
        "nm_tile_features": (i32, [vp, i32, i32, vp, i32]),
        "nm_order_tiles": (i32, [vp, vp, vp]),
        "nm_get_tile_order": (i32, [vp, vp, i32]),
        "nm_cost_model_create": (vp, [ctypes.c_ulonglong]),
        "nm_cost_model_destroy": (None, [vp]),
        "nm_cost_model_params": (i32, [vp, vp, i32]),
        "nm_cost_model_set_params": (i32, [vp, vp, i32]),
        "nm_cost_model_predict": (i32, [vp, vp, i32, vp]),
        "nm_cost_model_gradient": (i32, [vp, vp, vp, i32, vp, vp]),
        "nm_cost_model_train": (i32, [vp, vp, vp, i32, i32, ctypes.c_float, vp]),
        "nm_palette_load": (vp, [cp]),
        "nm_palette_save": (i32, [vp, cp]),
        "nm_palette_destroy": (None, [vp]),
        "nm_palette_cache": (i32, [vp, i32, vp]),
        "nm_colorize": (i32, [vp, vp, i32, i32, vp]),
        "nm_write_ppm": (i32, [cp, vp, i32, i32]),
        "nm_video_interpolate": (i32, [vp, vp, i32, i32, i32, i32, i32, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != NM_OK:
        raise NewmanError(rc, _lib.nm_last_error().decode(errors="replace"))


def _s(x):
    return str(x).encode()


class Batch:
    """Frames rendered together by one CUDA graph (nm_batch_*).  Keeps the
    Mandelbrot objects it was given alive."""

    def __init__(self, sc=1):
        L = load_library()
        self._b = L.nm_batch_create(int(sc))
        if not self._b:
            raise NewmanError(NM_ERR_ARG, L.nm_last_error().decode())
        self.sc = int(sc)
        self.frames = []

    def __del__(self):
        b, self._b = getattr(self, "_b", None), None
        if b and _lib is not None:
            _lib.nm_batch_destroy(b)

    def add(self, frame):
        _check(_lib.nm_batch_add(self._b, frame._h))
        self.frames.append(frame)

    def set_option(self, option, value):
        _check(_lib.nm_batch_set_option(self._b, int(option), int(value)))

    def render(self):
        _check(_lib.nm_batch_render(self._b))

    def stat(self, which):
        v = ctypes.c_longlong(0)
        _check(_lib.nm_batch_get_stat(self._b, int(which), ctypes.byref(v)))
        return v.value

    def frames_out(self):
        """The reduced frames as a list of (rows/sc, cols/sc) structured arrays."""
        shapes = [(f.rows() // self.sc, f.cols() // self.sc) for f in self.frames]
        flat = np.empty(sum(r * c for r, c in shapes), ESCAPE_DTYPE)
        _check(_lib.nm_batch_frames(self._b, flat.ctypes.data))
        out, at = [], 0
        for r, c in shapes:
            out.append(flat[at:at + r * c].reshape(r, c))
            at += r * c
        return out

    def autotune(self, stride=1):
        w, h, rn = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(_lib.nm_batch_autotune(self._b, int(stride), ctypes.byref(w), ctypes.byref(h),
                                      ctypes.byref(rn)))
        return w.value, h.value, rn.value


class Palette:
    """MultiWaveGenerator (multiwave.h:8-37) read from its text format."""

    def __init__(self, path):
        L = load_library()
        self._p = L.nm_palette_load(_s(path))
        if not self._p:
            raise NewmanError(NM_ERR_IO, L.nm_last_error().decode())

    def __del__(self):
        p, self._p = getattr(self, "_p", None), None
        if p and _lib is not None:
            _lib.nm_palette_destroy(p)

    def save(self, path):
        _check(_lib.nm_palette_save(self._p, _s(path)))

    def cache(self, n):
        """cache(n) (multiwave.cpp:75-116) as an (n, 3) uint8 array."""
        out = np.empty((n, 3), np.uint8)
        _check(_lib.nm_palette_cache(self._p, int(n), out.ctypes.data))
        return out


def write_ppm(path, rgb):
    """A binary PPM of an (rows, cols, 3) uint8 image."""
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    _check(load_library().nm_write_ppm(_s(path), rgb.ctypes.data, rgb.shape[0], rgb.shape[1]))


def video_interpolate(prev, cur, rows, cols, rate):
    """VideoZoom::nextFrame (video.cpp:14-34): the `rate` frames between two
    keyframes ((kh, kw, 3) uint8, kh >= rows, kw >= cols) as
    (rate, rows, cols, 3) uint8."""
    prev = np.ascontiguousarray(prev, dtype=np.uint8)
    cur = np.ascontiguousarray(cur, dtype=np.uint8)
    if prev.shape != cur.shape or prev.ndim != 3 or prev.shape[2] != 3:
        raise ValueError("keyframes must be two (rows, cols, 3) images of one size")
    out = np.empty((rate, rows, cols, 3), np.uint8)
    _check(load_library().nm_video_interpolate(prev.ctypes.data, cur.ctypes.data, prev.shape[0],
                                               prev.shape[1], int(rows), int(cols), int(rate),
                                               out.ctypes.data))
    return out


class CostModel:
    """The tile cost model (nm_cost_model_*): MLP 18 -> 64 -> 64 -> 64 -> 1 with
    FP16 weights and FP32 accumulation, trained with Adam on the GPU."""

    def __init__(self, seed=0):
        L = load_library()
        self._m = L.nm_cost_model_create(int(seed))
        if not self._m:
            raise NewmanError(NM_ERR_CUDA, L.nm_last_error().decode())

    def __del__(self):
        m, self._m = getattr(self, "_m", None), None
        if m and _lib is not None:
            _lib.nm_cost_model_destroy(m)

    def params(self):
        out = np.empty(COST_PARAMS, np.float32)
        _check(_lib.nm_cost_model_params(self._m, out.ctypes.data, out.size))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(_lib.nm_cost_model_set_params(self._m, p.ctypes.data, p.size))

    def predict(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, COST_FEATURES)
        out = np.empty(len(x), np.float32)
        _check(_lib.nm_cost_model_predict(self._m, x.ctypes.data, len(x), out.ctypes.data))
        return out

    def gradient(self, x, t):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, COST_FEATURES)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.empty(COST_PARAMS, np.float32)
        loss = ctypes.c_float()
        _check(_lib.nm_cost_model_gradient(self._m, x.ctypes.data, t.ctypes.data, len(x),
                                           g.ctypes.data, ctypes.byref(loss)))
        return g, loss.value

    def train(self, x, t, epochs, lr=1e-3):
        x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, COST_FEATURES)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = ctypes.c_float()
        _check(_lib.nm_cost_model_train(self._m, x.ctypes.data, t.ctypes.data, len(x),
                                        int(epochs), float(lr), ctypes.byref(loss)))
        return loss.value


class Mandelbrot:
    """One reference `Mandelbrot` object (mandelbrot.h:7-53) on the GPU."""

    def __init__(self, nr=1, nc=1, _handle=None):
        L = load_library()
        self._h = _handle if _handle is not None else L.nm_create(int(nr), int(nc))
        if not self._h:
            raise NewmanError(NM_ERR_ARG, L.nm_last_error().decode())

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h and _lib is not None:
            _lib.nm_destroy(h)

    def copy(self):
        """Value copy (the reference assigns Mandelbrot objects, viewer.cpp:193)."""
        h = _lib.nm_copy(self._h)
        if not h:
            raise NewmanError(NM_ERR_CUDA, _lib.nm_last_error().decode())
        c = Mandelbrot(_handle=h)
        c._source = getattr(self, "_source", None)  # a preview's copy reads the same orbit
        return c

    # ---- learned tile scheduling (no reference counterpart) -----------------
    def preview(self, factor):
        """The same view on a grid `factor` times coarser (nm_preview); reads a
        precomputed view-center orbit and series in place, so it renders only
        while this view keeps them (a new precompute or view makes it refuse)."""
        h = _lib.nm_preview(self._h, int(factor))
        if not h:
            raise NewmanError(NM_ERR_ARG, _lib.nm_last_error().decode())
        p = Mandelbrot(_handle=h)
        p._source = self  # the preview may read this view's orbit in place
        return p

    def tiles(self):
        """(tiles_x, tiles_y) of the whole grid at the current tile size."""
        tx, ty = ctypes.c_int(), ctypes.c_int()
        _check(_lib.nm_tiles(self._h, ctypes.byref(tx), ctypes.byref(ty)))
        return tx.value, ty.value

    def set_tile_order(self, order=None):
        """Hand-out order of the tiles (a permutation of row-major tile ids);
        None restores row-major."""
        if order is None:
            _check(_lib.nm_set_tile_order(self._h, None, 0))
            return
        o = np.ascontiguousarray(order, dtype=np.int32)
        _check(_lib.nm_set_tile_order(self._h, o.ctypes.data, o.size))

    def order_tiles(self, preview, model):
        """The cost model's longest-first order from a rendered preview, computed
        on the GPU after the preview's render (nm_order_tiles); no host round trip."""
        _check(_lib.nm_order_tiles(self._h, preview._h, model._m))

    def tile_order(self):
        """The tile order in effect, or None under the static order."""
        tx, ty = self.tiles()
        out = np.empty(tx * ty, np.int32)
        rc = _lib.nm_get_tile_order(self._h, out.ctypes.data, out.size)
        if rc == NM_ERR_STATE:
            return None
        _check(rc)
        return out

    def tile_costs(self):
        """Per-tile work of the last whole-grid render (NM_OPT_LOG_TILE_COSTS),
        shaped (tiles_y, tiles_x)."""
        tx, ty = self.tiles()
        out = np.empty(tx * ty, np.uint64)
        _check(_lib.nm_get_tile_costs(self._h, out.ctypes.data, out.size))
        return out.reshape(ty, tx)

    def colorize(self, palette, sc=1, smooth=True):
        """FractalViewer::colorLine over every row (viewer.cpp:98-124): the
        image as (rows/sc, cols/sc, 3) uint8."""
        out = np.empty((self.rows() // sc, self.cols() // sc, 3), np.uint8)
        _check(_lib.nm_colorize(self._h, palette._p, int(sc), 1 if smooth else 0,
                                out.ctypes.data))
        return out

    def tile_features(self, tile_w, tile_h):
        """Features of this (rendered preview) grid's tiles of tile_w x tile_h
        samples: (tiles, COST_FEATURES) float32, row-major tiles."""
        tx = (self.cols() + tile_w - 1) // tile_w
        ty = (self.rows() + tile_h - 1) // tile_h
        out = np.empty((tx * ty, COST_FEATURES), np.float32)
        _check(_lib.nm_tile_features(self._h, int(tile_w), int(tile_h), out.ctypes.data,
                                     tx * ty))
        return out

    # ---- fields -----------------------------------------------------------
    @property
    def N(self):
        return _lib.nm_get_iterations(self._h)

    @N.setter
    def N(self, value):
        _check(_lib.nm_set_iterations(self._h, int(value)))

    @property
    def error_tolerance(self):
        return self._tol if hasattr(self, "_tol") else 1e-10

    @error_tolerance.setter
    def error_tolerance(self, value):
        _check(_lib.nm_set_tolerance(self._h, float(value)))
        self._tol = float(value)

    def _view(self, which):
        buf = ctypes.create_string_buffer(1 << 16)
        _check(_lib.nm_get_view(self._h, which, buf, len(buf)))
        return buf.value.decode()

    @property
    def center(self):
        return self._view(0), self._view(1)

    @property
    def sz(self):
        return self._view(2), self._view(3)

    def set_view(self, center_re, center_im, step_re, step_im=None, N=None, tolerance=None,
                 min_bits=0):
        """Sets center, pixel step (decimal strings), N and tolerance at once."""
        step_im = step_re if step_im is None else step_im
        N = self.N if N is None else N
        tol = self.error_tolerance if tolerance is None else tolerance
        _check(_lib.nm_set_view(self._h, _s(center_re), _s(center_im), _s(step_re), _s(step_im),
                                int(N), float(tol), int(min_bits)))
        self._tol = float(tol)

    def rows(self):
        return _lib.nm_rows(self._h)

    def cols(self):
        return _lib.nm_cols(self._h)

    def useHardware(self):
        return bool(_lib.nm_use_hardware(self._h))

    def set_path(self, path):
        _check(_lib.nm_set_path(self._h, int(path)))

    def set_option(self, option, value):
        _check(_lib.nm_set_option(self._h, int(option), int(value)))

    def stat(self, which):
        v = ctypes.c_longlong(0)
        _check(_lib.nm_get_stat(self._h, int(which), ctypes.byref(v)))
        return v.value

    # ---- rendering ----------------------------------------------------------
    def precompute(self):
        _check(_lib.nm_precompute(self._h))

    def upload(self):
        _check(_lib.nm_upload(self._h))

    def orbit(self):
        """(X, X - get_d(X), A, B, C) of the last precompute as (n, 2) double
        arrays of get_d values."""
        n = self.stat(STAT_ORBIT_LENGTH)
        out = [np.empty((n, 2), np.float64) for _ in range(5)]
        _check(_lib.nm_get_orbit(self._h, *[o.ctypes.data for o in out], n))
        return tuple(out)

    def computeRow(self, r):
        _check(_lib.nm_compute_row(self._h, int(r)))

    def render_rows(self, r0, r1, stream=None):
        _check(_lib.nm_render_rows(self._h, int(r0), int(r1), stream))

    def render(self):
        _check(_lib.nm_render(self._h))

    def synchronize(self):
        _check(_lib.nm_synchronize(self._h))

    def cancel(self):
        _check(_lib.nm_cancel(self._h))

    # ---- grid ----------------------------------------------------------------
    def at(self, r, c, sc=None):
        e = EscapeValue()
        if sc is None:
            _check(_lib.nm_at(self._h, int(r), int(c), ctypes.byref(e)))
        else:
            _check(_lib.nm_at_sc(self._h, int(r), int(c), int(sc), ctypes.byref(e)))
        return e.iterations, e.smoothing

    def grid(self, out=None):
        """The grid as a (rows, cols) structured array {iterations, smoothing}."""
        shape = (self.rows(), self.cols())
        if out is None:
            out = np.empty(shape, ESCAPE_DTYPE)
        assert out.dtype == ESCAPE_DTYPE and out.shape == shape and out.flags.c_contiguous
        _check(_lib.nm_get_grid(self._h, out.ctypes.data))
        return out

    def smoothing64(self):
        out = np.empty((self.rows(), self.cols()), np.float64)
        _check(_lib.nm_get_smoothing64(self._h, out.ctypes.data))
        return out

    def render_noalloc(self, out_ptr, stream=None):
        """FP32-floatexp render into caller-owned device memory (rows*cols
        escape values at `out_ptr`), allocating nothing; asynchronous on
        `stream`.  Needs precompute() and upload() first."""
        _check(_lib.nm_render_fe32_noalloc(self._h, out_ptr, stream))

    def reduce(self, sc, out=None):
        """scaleDown(sc)'s averaged grid, returned without changing the object."""
        shape = (self.rows() // sc, self.cols() // sc)
        if out is None:
            out = np.empty(shape, ESCAPE_DTYPE)
        assert out.dtype == ESCAPE_DTYPE and out.shape == shape and out.flags.c_contiguous
        _check(_lib.nm_reduce(self._h, int(sc), out.ctypes.data))
        return out

    def device_grid(self):
        g, s = ctypes.c_void_p(), ctypes.c_void_p()
        _check(_lib.nm_device_grid(self._h, ctypes.byref(g), ctypes.byref(s)))
        return g.value, s.value

    def scaleUp(self, sc):
        _check(_lib.nm_scale_up(self._h, int(sc)))

    def scaleDown(self, sc):
        _check(_lib.nm_scale_down(self._h, int(sc)))

    # ---- view edits ------------------------------------------------------------
    def pointAt(self, r, c, sc=1):
        a = ctypes.create_string_buffer(1 << 16)
        b = ctypes.create_string_buffer(1 << 16)
        _check(_lib.nm_point_at(self._h, int(r), int(c), int(sc), a, b, len(a)))
        return a.value.decode(), b.value.decode()

    def translate(self, dr, dc, sc=1):
        _check(_lib.nm_translate(self._h, int(dr), int(dc), int(sc)))

    def zoom(self, scale):
        _check(_lib.nm_zoom(self._h, float(scale)))

    def zoomAt(self, scale, r, c, sc=1):
        _check(_lib.nm_zoom_at(self._h, float(scale), int(r), int(c), int(sc)))

    def loadLegacy(self, path):
        _check(_lib.nm_load_legacy(self._h, _s(path)))

    def save(self, path):
        _check(_lib.nm_save(self._h, _s(path)))
