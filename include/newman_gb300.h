/*
 * newman_gb300 -- C ABI of the GPU per-pixel Mandelbrot path.
 *
 * One `nm_handle` stands in for one object of the reference's C++ class
 * `Mandelbrot` (mandelbrot.h:7-53 of axnjaxn/newman): it owns the view (center,
 * pixel step, iteration count, series tolerance, arbitrary precision), the
 * precomputed reference orbit and series, and the output grid -- a row-major
 * array of {int32 iterations, float smoothing} samples, index r*nc + c, the
 * layout of the reference's RenderGrid (grid.h:6-25).  The grid lives in GPU
 * memory and is copied out on request.
 *
 * Every call returns an int status (NM_OK = 0) unless stated otherwise; the
 * message of the last failure on the calling thread is nm_last_error().  A
 * handle is used by one thread at a time (nm_cancel excepted); separate
 * handles are independent.  Views are exchanged as decimal strings, the
 * format of the reference's save files (viewer.cpp:12-23).
 */
#ifndef NEWMAN_GB300_H
#define NEWMAN_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nm_handle nm_handle;

/* grid.h:8-14, RenderGrid::EscapeValue -- 8 bytes, same layout. */
typedef struct {
  int32_t iterations;
  float smoothing;
} nm_escape_value;

enum nm_status {
  NM_OK = 0,
  NM_ERR_ARG = 1,        /* bad argument (size, index, N < 1, null pointer) */
  NM_ERR_PARSE = 2,      /* a decimal string did not parse */
  NM_ERR_STATE = 3,      /* call out of order, e.g. a deep render before nm_precompute */
  NM_ERR_CUDA = 4,       /* CUDA runtime error (message in nm_last_error) */
  NM_ERR_CANCELLED = 5,  /* nm_cancel stopped the render; the grid is partial */
  NM_ERR_IO = 6,         /* file could not be opened / read */
  NM_ERR_UNSUPPORTED = 7 /* option or path not available for this view */
};

/* Arithmetic of the per-sample work (nm_set_path). */
enum nm_path {
  /* The reference's choice: its double loop when useHardware() holds
     (mandelbrot.cpp:231-259), else the plain FP64 perturbation path. */
  NM_PATH_REFERENCE = 0,
  /* Plain FP64 perturbation: series skip, then FP64 delta iteration. */
  NM_PATH_FP64 = 1,
  /* FP32 mantissa + int exponent delta iteration (floatexp). */
  NM_PATH_FE32 = 2,
  /* The reference's own arithmetic, bit for bit: where useHardware() holds
     its double loop, else its series front in doubles followed by the
     arbitrary-precision continuation of getIterations (mandelbrot.cpp:209-224)
     with GMP mpf's truncations reproduced on the GPU; the cardioid test in
     the view's precision in both.  Views of 64 to 448 bits of precision
     whose series stays in the double range (where the reference renders at
     all); others are refused with NM_ERR_UNSUPPORTED.  Choose it before
     nm_precompute, which then keeps the orbit in arbitrary precision. */
  NM_PATH_MP = 3
};

enum nm_option {
  NM_OPT_TILE_W = 0,      /* sample order: tile width (default 16) */
  NM_OPT_TILE_H = 1,      /* tile height (default 16) */
  NM_OPT_CHUNK = 2,       /* iterations between lane refills (default 32) */
  NM_OPT_KEEP_SMOOTH64 = 3, /* 1: also keep the unrounded double smoothing */
  NM_OPT_THREADS = 4,     /* host threads for the probe search (0 = all) */
  NM_OPT_BLOCKS = 5,      /* persistent blocks (0 = fill the GPU) */
  NM_OPT_RENORM = 6,      /* FE32: steps between exponent renormalisations (0: 64,
                             32 on views below the double range) */
  NM_OPT_FE32_SINGLE_PASS = 7, /* FE32 in one persistent kernel (default: three passes) */
  NM_OPT_REFERENCE = 8,   /* reference orbit: 0 the reference's probe search
                             (findProbe, mandelbrot.cpp:73-95), 1 the view center */
  NM_OPT_BATCH_GRAPH = 9, /* batches: 1 replay one captured CUDA graph (default), 0 launch */
  NM_OPT_FE32_OVERLAP = 10, /* FE32 passes: 1 render the uncertified samples in FP64 inside
                              the iteration pass, as they appear (default); 0 after it */
  NM_OPT_LOG_TILE_COSTS = 11, /* 1: whole-grid renders log every tile's work (nm_get_tile_costs) */
  NM_OPT_BATCH_FP64_WARPS = 12, /* batches: warps of 8 a block on the FP64 side of the FE32 pass
                                  (2, 4 or 6; 0 = 4 with double-loop frames, else 2) */
  NM_OPT_ORBIT_STAGE = 13,  /* FE32 iteration pass: the first n (0..3072) reference-orbit entries
                               copied into each block's shared memory by the TMA unit, where
                               every rebased sample restarts (0: none; -1, the default: 1024 on
                               views whose series leaves the double range, else none) */
  NM_OPT_L2_WINDOW = 14,    /* FE32 iteration pass: 1 runs it with a persisting L2 access-policy
                               window over the reference orbit (the process's L2 set-aside is
                               raised to the orbit's size, within the device's limit) */
  NM_OPT_ITER_CAP = 15      /* renders stop every sample at min(N, cap) iterations (0: N), as
                               if N were the cap: for previews that show where a view's work
                               lies without running its longest samples to the end */
};

enum nm_stat {
  NM_STAT_CARDIOID_UNDECIDED = 0, /* cardioid tests within 2^-96 of the boundary */
  NM_STAT_EXECUTED_ITERS = 1,     /* z^2 + c steps run on the GPU in the last render */
  NM_STAT_SAMPLES = 2,            /* samples finished in the last render */
  NM_STAT_REBASES = 3,            /* perturbation rebases in the last render */
  NM_STAT_FP64_REWORK = 4,        /* FE32 samples not certified, re-rendered in FP64 */
  NM_STAT_WAIT_TIMEOUTS = 5,      /* overlapped FP64 rework: bounded waits that ran out (0) */
  NM_STAT_FRONT_FP64 = 6,         /* FE32 samples whose series front fell back to FP64 */
  NM_STAT_STAGE_FALLBACKS = 7,    /* blocks that copied the staged orbit themselves (0) */
  NM_STAT_ORBIT_LENGTH = 16,      /* X.size() of the last precompute */
  NM_STAT_PROBE_INDEX = 17,       /* winning probe of findProbe */
  NM_STAT_PRECISION_BITS = 18,    /* arbitrary precision of the view */
  NM_STAT_PRECOMPUTE_US = 19,     /* host time of the last nm_precompute */
  NM_STAT_KERNEL_NS = 20,         /* GPU time of the last render's main kernel */
  NM_STAT_REWORK_KERNEL_NS = 21,  /* GPU time of the last FE32 render's FP64 rework */
  NM_STAT_ITER_KERNEL_NS = 22,    /* GPU time of the last FE32 render's iteration pass */
  NM_STAT_KERNEL_LAUNCHES = 23    /* kernels this library launched in this process, over all
                                     handles (a batch's graph replay adds its kernels) */
};

/* Mandelbrot::Mandelbrot(int nr, int nc), mandelbrot.cpp:8-17: center -0.5,
   step 4/nc x 3/nr, N 256, tolerance 1e-10.  Binds to the current CUDA
   device.  Returns NULL on failure (nm_last_error). */
nm_handle* nm_create(int nr, int nc);
/* Value copy (the reference copies Mandelbrot objects, viewer.cpp:193,251). */
nm_handle* nm_copy(const nm_handle* src);
/* No reference counterpart: the same view on a grid `factor` times coarser in
   each direction (rows and columns must be multiples of it).  A precomputed
   view with its reference orbit at the view center shares that orbit and its
   series: the preview is ready to render without nm_precompute, and reads the
   source's orbit and series tables in place (host and GPU; the first render
   of either uploads them) -- destroy the preview before its source. */
nm_handle* nm_preview(const nm_handle* src, int factor);
void nm_destroy(nm_handle* h);
const char* nm_last_error(void);

/* Public fields N, error_tolerance, center, sz (mandelbrot.h:23-25).  The
   step string fixes the precision (setPrecision, mandelbrot.cpp:37-56);
   min_bits > 0 raises it.  Decimal strings as mpf_set_str reads them. */
int nm_set_view(nm_handle* h, const char* center_re, const char* center_im, const char* step_re,
                const char* step_im, int N, double tolerance, int min_bits);
/* which: 0 center.re, 1 center.im, 2 sz.re, 3 sz.im.  Writes a decimal string. */
int nm_get_view(const nm_handle* h, int which, char* buf, int buflen);
int nm_set_iterations(nm_handle* h, int N);          /* Mandelbrot::N */
int nm_get_iterations(const nm_handle* h);
int nm_set_tolerance(nm_handle* h, double tolerance); /* Mandelbrot::error_tolerance */
int nm_rows(const nm_handle* h);                       /* rows(), mandelbrot.h:33 */
int nm_cols(const nm_handle* h);                       /* cols(), mandelbrot.h:34 */
int nm_use_hardware(const nm_handle* h);               /* useHardware(), mandelbrot.cpp:256 */

int nm_set_path(nm_handle* h, int path);               /* enum nm_path */
int nm_set_option(nm_handle* h, int option, long long value);
int nm_get_stat(nm_handle* h, int stat, long long* value);

/* precompute(), mandelbrot.cpp:261-267: for deep views the probe search,
   reference orbit and series coefficients, on host threads, and their upload. */
int nm_precompute(nm_handle* h);
/* Re-issue the host-to-device copy of the precomputed tables on the handle's
   stream (asynchronous). */
int nm_upload(nm_handle* h);
/* No reference counterpart (the reference keeps X, A, B, C private,
   mandelbrot.h:45-50): the last precompute's orbit and series as doubles,
   get_d of each (mandelbrot.cpp:166-168), n = X.size() entries of (re, im)
   pairs in each non-null array; xlo holds get_d(X - get_d(X)).  n must be
   NM_STAT_ORBIT_LENGTH. */
int nm_get_orbit(nm_handle* h, double* x, double* xlo, double* a, double* b, double* c, int n);

/* computeRow(r), mandelbrot.cpp:269-283: render one row, synchronously. */
int nm_compute_row(nm_handle* h, int r);
/* Render rows [r0, r1) asynchronously on `stream` (a cudaStream_t; NULL =
   the handle's own stream).  nm_synchronize waits and reports cancellation. */
int nm_render_rows(nm_handle* h, int r0, int r1, void* stream);
/* All rows, synchronously: the row loop of viewer.cpp:166-171. */
int nm_render(nm_handle* h);
int nm_synchronize(nm_handle* h);
/* Stop the render in flight at the next sample hand-out (any thread); the
   reference polls ESC between rows (viewer.cpp:126-155). */
int nm_cancel(nm_handle* h);

/* at(r, c), mandelbrot.cpp:318 */
int nm_at(nm_handle* h, int r, int c, nm_escape_value* out);
/* at(r, c, sc), mandelbrot.cpp:320-332: float mean of sc x sc samples */
int nm_at_sc(nm_handle* h, int r, int c, int sc, nm_escape_value* out);
/* scaleUp(sc) / scaleDown(sc), mandelbrot.cpp:334-360, on the GPU grid. */
int nm_scale_up(nm_handle* h, int sc);
int nm_scale_down(nm_handle* h, int sc);
/* The whole scaleDown(sc) grid written to host memory, handle unchanged:
   (rows/sc) x (cols/sc) values. */
int nm_reduce(nm_handle* h, int sc, nm_escape_value* host_out);
/* Copy the grid (rows x cols) to host memory. */
int nm_get_grid(nm_handle* h, nm_escape_value* host_out);
/* Copy the unrounded double smoothing (needs NM_OPT_KEEP_SMOOTH64). */
int nm_get_smoothing64(nm_handle* h, double* host_out);
/* Device pointers of the grid (valid until the next resize). */
int nm_device_grid(nm_handle* h, nm_escape_value** grid, double** smooth64);

/* pointAt(r, c, sc), mandelbrot.cpp:285-290, as two decimal strings. */
int nm_point_at(const nm_handle* h, int r, int c, int sc, char* re, char* im, int buflen);
int nm_translate(nm_handle* h, int dr, int dc, int sc);            /* mandelbrot.cpp:292-295 */
int nm_zoom(nm_handle* h, float scale);                            /* mandelbrot.cpp:297-302 */
int nm_zoom_at(nm_handle* h, float scale, int r, int c, int sc);   /* mandelbrot.cpp:304-316 */
int nm_load_legacy(nm_handle* h, const char* path);                /* mandelbrot.cpp:19-35 */
int nm_save(const nm_handle* h, const char* path);                 /* viewer.cpp:12-23 */

/* ---- colouring (multiwave.cpp, viewer.cpp:89-124) ---------------------------
   nm_palette is MultiWaveGenerator: nm_palette_load reads its text format
   (load_filename, multiwave.cpp:19-50; NULL on failure), nm_palette_save
   writes it (save_filename, :52-73), nm_palette_cache is cache(n) (:75-116)
   as n RGB triples.  nm_colorize is FractalViewer::colorLine over every row
   (viewer.cpp:98-124) on the GPU: per pixel the palette colour of each of its
   sc x sc samples (getColor, :89-94: black at N, the blend of the entries on
   either side of the smoothed count when `smooth`), their float mean, into
   rgb_out as (rows/sc) x (cols/sc) RGB bytes.  The reference takes HSL
   conversion, blending and clipping from libbyteimage (not in the reference
   tree); they are the standard definitions here (round half up). */
typedef struct nm_palette nm_palette;
nm_palette* nm_palette_load(const char* path);
int nm_palette_save(const nm_palette* p, const char* path);
void nm_palette_destroy(nm_palette* p);
int nm_palette_cache(nm_palette* p, int n, unsigned char* rgb_out);
int nm_colorize(nm_handle* h, nm_palette* p, int sc, int smooth, unsigned char* rgb_out);
/* VideoZoom::nextFrame (video.cpp:14-34) on the GPU: the `rate` frames between
   keyframes prev and cur (key_rows x key_cols RGB, rendered at 1.5 times the
   frame size as the viewer's auto-zoom does, viewer.cpp:270-286), as
   rate x rows x cols RGB bytes in frames_out.  The reference writes them to
   an AVI; here they are returned (headless).  libbyteimage's scaled / blend
   are restated as bilinear resampling and a per-channel blend. */
int nm_video_interpolate(const unsigned char* prev_rgb, const unsigned char* cur_rgb,
                         int key_rows, int key_cols, int rows, int cols, int rate,
                         unsigned char* frames_out);
/* A binary PPM (P6) of rows x cols RGB bytes: headless image output. */
int nm_write_ppm(const char* path, const unsigned char* rgb, int rows, int cols);

/* ---- learned tile scheduling (no reference counterpart) ---------------------
   Tiles are the render's tiles of NM_OPT_TILE_W x NM_OPT_TILE_H samples,
   row-major ids over the whole grid.  nm_set_tile_order sets the order in
   which whole-grid renders hand them out (a permutation; NULL restores
   row-major); the image does not depend on it.  With NM_OPT_LOG_TILE_COSTS a
   whole-grid render logs each tile's work: the iteration steps its samples
   ran, FP64 steps counted 8 (FP32-step equivalents). */
int nm_tiles(nm_handle* h, int* tiles_x, int* tiles_y);
int nm_set_tile_order(nm_handle* h, const int* order, int n);
int nm_get_tile_costs(nm_handle* h, unsigned long long* out, int n);

/* Features of the tiles of a rendered preview (nm_preview), tile_w x tile_h
   preview samples each, NM_COST_FEATURES floats per tile, row-major tiles:
   a 16-bin histogram of x = (log2(1 + it) - lo) / (hi - lo) over the tile's
   samples (lo, hi: the preview's escaping samples' range; x = 1 at N), then
   the mean and the max of x. */
#define NM_COST_FEATURES 18
#define NM_COST_PARAMS 9601
int nm_tile_features(nm_handle* preview, int tile_w, int tile_h, float* out, int ntiles);

/* Cost model: MLP 18 -> 64 -> 64 -> 64 -> 1 (ReLU), FP16 weights with FP32
   accumulation in hand-written kernels; FP32 master parameters (NM_COST_PARAMS,
   layout W1[64][18] b1 W2[64][64] b2 W3[64][64] b3 W4[64] b4) trained with
   Adam on the mean squared error.  Inputs / outputs are host arrays. */
typedef struct nm_costmodel nm_costmodel;
nm_costmodel* nm_cost_model_create(unsigned long long seed);
void nm_cost_model_destroy(nm_costmodel* m);
int nm_cost_model_params(nm_costmodel* m, float* out, int n);
int nm_cost_model_set_params(nm_costmodel* m, const float* in, int n);
int nm_cost_model_predict(nm_costmodel* m, const float* features, int n, float* out);
/* Gradient of mean((y - target)^2) over the n rows, FP32, parameter layout. */
int nm_cost_model_gradient(nm_costmodel* m, const float* features, const float* targets, int n,
                           float* grad, float* loss);
int nm_cost_model_train(nm_costmodel* m, const float* features, const float* targets, int n,
                        int epochs, float lr, float* loss);

/* The learned longest-first order, all on the GPU and asynchronous on h's
   stream: the tile features of `preview` (a rendered nm_preview of h, or any
   view whose grid divides h's by the same factor in both directions), the
   model's forward pass and a sort by decreasing prediction (ties by tile id:
   the order of a stable sort of -prediction) are enqueued after the
   preview's render, and the result becomes h's tile order for its next
   whole-grid renders, as nm_set_tile_order would make it.  h's tile size
   must be a multiple of the preview factor; at most 16,384 tiles.  The
   model's later calls wait for the order to be computed. */
int nm_order_tiles(nm_handle* h, nm_handle* preview, nm_costmodel* m);
/* The order in effect (nm_set_tile_order's or nm_order_tiles'), n entries;
   NM_ERR_STATE under the static order. */
int nm_get_tile_order(nm_handle* h, int* out, int n);

/* Batches: many frames rendered together, e.g. every frame of a zoom video,
   each frame a handle with its own view, orbit, series skip and N (no
   reference counterpart; the reference renders one view at a time).  The
   first nm_batch_render captures all of the batch's kernels -- the FE32
   passes over every FE32 frame at once, the double-path and FP64 frames, and
   the multisample reduce of every frame -- into one CUDA graph, and every
   render replays it.  Frames must be precomputed first and stay alive while
   in the batch; a frame whose tables or grid change is noticed and the graph
   rebuilt.  sc: the frames' multisample factor (their rows and columns are
   multiples of it); nm_batch_frames returns the reduced frames, frame-major.
   Frames on NM_PATH_MP are refused (NM_ERR_UNSUPPORTED): render them alone. */
typedef struct nm_batch nm_batch;
nm_batch* nm_batch_create(int sc);
void nm_batch_destroy(nm_batch* b);
int nm_batch_add(nm_batch* b, nm_handle* frame);
/* NM_OPT_TILE_W, NM_OPT_TILE_H, NM_OPT_CHUNK, NM_OPT_RENORM, NM_OPT_BATCH_GRAPH,
   NM_OPT_FE32_OVERLAP, NM_OPT_BATCH_FP64_WARPS */
int nm_batch_set_option(nm_batch* b, int option, long long value);
int nm_batch_render(nm_batch* b);
/* NM_STAT_EXECUTED_ITERS, NM_STAT_SAMPLES, NM_STAT_FP64_REWORK, NM_STAT_KERNEL_NS */
int nm_batch_get_stat(nm_batch* b, int stat, long long* value);
int nm_batch_frames(nm_batch* b, nm_escape_value* host_out);
/* Times every tile shape (8x8 .. 64x64) and FE32 renormalisation interval
   (8 .. 256) on every stride-th frame and keeps the fastest, then the FP64
   side's share of the FE32 pass (NM_OPT_BATCH_FP64_WARPS 2, 4, 6); last, the
   result against the batch's own settings on the whole batch, keeping the
   faster (a sub-batch can miss the few frames that dominate the batch). */
int nm_batch_autotune(nm_batch* b, int stride, int* tile_w, int* tile_h, int* renorm);

/* Render the handle's view on the FP32-floatexp path into device memory the
   caller owns, allocating nothing (no cudaMalloc, cudaFree or allocating
   library call).  No counterpart in the reference.  It is for callers that
   cannot allocate device memory when they render: code recording its GPU
   work into a CUDA graph by stream capture, or a process whose device memory
   belongs to another framework's allocator or to a fixed budget.
   The handle's tables must already be on the GPU (nm_precompute, then
   nm_upload -- those two calls do allocate).  `out` is a device array of
   rows*cols nm_escape_value; `stream` a cudaStream_t (NULL: the legacy
   default stream); the call is asynchronous.  The scratch the kernels need
   (work counters, statistics, the list of samples re-rendered in FP64) is
   one static device array of NM_NOALLOC_MAX_SAMPLES * 4 + 256 bytes per GPU,
   held by every GPU that loads the library until the process exits; views
   of more than NM_NOALLOC_MAX_SAMPLES samples are refused with NM_ERR_ARG.
   The first call on a device looks the array up (cudaGetSymbolAddress):
   make that first call before any stream capture.  The handle's device must
   be the current device (else NM_ERR_STATE).  All calls share the one
   array, so calls whose kernels overlap on the GPU (other streams or
   threads) race: serialise them.  The escape counts are those of nm_render
   on the FE32 path; on views where the reference takes its double loop the
   interior-orbit trapping is off here (it needs a per-sample record), so
   such views render the same counts more slowly.  The call's statistics
   (executed steps, reworked samples) stay in the scratch array: nm_get_stat
   reports the handle's own renders only. */
#define NM_NOALLOC_MAX_SAMPLES 4194304
int nm_render_fe32_noalloc(nm_handle* h, nm_escape_value* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NEWMAN_GB300_H */
