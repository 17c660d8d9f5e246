// Device-side description of one render: the sample grid, the per-row and
// per-column tables the host computed in arbitrary precision, the FP64 copy
// of the reference orbit and series, and the output grid.  Passed to every
// kernel by value.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define NM_HD __host__ __device__ __forceinline__
#else
#define NM_HD inline
#endif

namespace nmg {

// grid.h:8-14 -- one sample of the output grid, 8 bytes, row-major r*nc+c.
struct EscapeValue {
  int32_t iterations;
  float smoothing;
};

struct Dbl2 {
  double x, y;
};

struct alignas(16) Flt4 {
  float x, y, z, w;
};

// Per-sample record of the interior-orbit trapping on double-loop views
// (fe_core.cuh): the center P of the trapping disk in float-float, its radius
// R, and the radius rho of its image around the exact orbit (0: none).
struct alignas(16) FeTrap {
  float pxh, pxl, pyh, pyl;
  float rho, R;
  int32_t pad_[2];
};

// Floatexp values: FP64 mantissas with an int exponent.
struct CFE {  // (re + i im) * 2^e
  double re, im;
  int32_t e;
};
struct RFE {  // m * 2^e
  double m;
  int32_t e;
};

// Tables of the FP32 series front (fe_front32.cuh), all normalised so that the
// larger high word lies in [1, 2) (or is 0):
struct alignas(16) FFE {   // (h + l) * 2^e: a real in float-float with an exponent
  float h, l;
  int32_t e, pad_;
};
struct alignas(16) CFFE {  // ((rh + rl) + i (ih + il)) * 2^e
  float rh, rl, ih, il;
  int32_t e, pad_[3];
};
struct TFE {               // m * 2^e, m in [1, 2); e = kTfeInf: +inf, kTfeZero: 0
  float m;
  int32_t e;
};
constexpr int32_t kTfeInf = 0x7fffffff, kTfeZero = -0x7fffffff;

enum CardioidMode : int32_t {
  CARDIOID_PER_SAMPLE = 0,  // evaluate the test for each sample (double-double)
  CARDIOID_NONE = 1,        // the view box is provably outside both regions
};

struct DeviceView {
  int32_t nr, nc;          // sample grid
  int32_t N;               // iteration count
  int32_t cardioid_mode;
  double tol;              // series error tolerance
  double bailout2;         // 1024^2 (mandelbrot.cpp:58-59)
  double log_bailout;      // log(1024), rounded on the host
  int32_t tile_w, tile_h;  // sample order: tiles of tile_w x tile_h, row-major inside
  int32_t tiles_x, tiles_y;
  int32_t row0, row1;      // rows [row0, row1) of the grid take part in this launch
  int64_t total;           // tiles_x * tiles_y * tile_w * tile_h (padded)

  const Dbl2* coord_re;    // [nc] per column: pt.re = hi + lo
  const Dbl2* coord_im;    // [nr] per row:    pt.im = hi + lo

  // deep path (not the reference's hardware path)
  const double* eps_re;    // [nc] get_d(pt.re - X[0].re)
  const double* eps_im;    // [nr] get_d(pt.im - X[0].im)
  const Dbl2* z;           // [zlen] 0, get_d(X[k]), escaped element
  const Flt4* zf;          // [zlen] the same as float-float {hi.re, hi.im, lo.re, lo.im}
  int32_t zlen;
  int32_t z_stage;         // entries [0, z_stage) of zf and z are also in the launch's
                           // dynamic shared memory (orbit_stage.cuh); 0: none
  int32_t xlen;            // X.size()
  const Dbl2* xhi;         // [xlen] get_d(X[k])
  const Dbl2* xlo;         // [xlen] get_d(X[k] - xhi)
  const Dbl2* sa_a;        // [xlen] get_d(A[k])
  const Dbl2* sa_b;
  const Dbl2* sa_c;
  const double* sa_min;    // [xlen] prefix min of tol |B_i|^2/|C_i|^2
  int32_t sa_scan;         // 1: walk the series term by term (no threshold shortcut)
  int32_t sa_fe;           // 1: eps, series and thresholds in floatexp (tables below)
  int32_t double_loop;     // 1: FE32 path certified against the double loop (no series;
                           //    eps = get_d(get_d(pt) - X[0]), orbit at the view center)
  float c_abs;             // |c|_1 <= c_abs for every sample c (as the double loop takes it)
  FeTrap* trap;            // double-loop views: one record per sample (tile order), or null
  const RFE* eps_re_fe;    // [nc]
  const RFE* eps_im_fe;    // [nr]
  const CFE* sa_a_fe;      // [xlen]
  const CFE* sa_b_fe;
  const CFE* sa_c_fe;
  const RFE* sa_min_fe;    // [xlen]
  // the same for the FP32 series front (null: that front is not used)
  const FFE* eps32_re;     // [nc]
  const FFE* eps32_im;     // [nr]
  const CFFE* sa_a32;      // [xlen]
  const CFFE* sa_b32;
  const CFFE* sa_c32;
  const TFE* sa_min32;     // [xlen]

  // the reference-exact path: values in the view's arbitrary precision as
  // records of mp_limbs limbs (mpf_fixed.cuh; word 0: exponent << 32 | sign)
  int32_t mp_limbs;        // limbs of a value (GMP's P + 1)
  const uint64_t* coord_re_mp;  // [nc] pt.re
  const uint64_t* coord_im_mp;  // [nr] pt.im
  const uint64_t* x_mp;         // [xlen] X[k].re, X[k].im

  EscapeValue* grid;       // [nr*nc]
  double* smooth64;        // optional [nr*nc] unrounded smoothing

  // Scheduling (whole-grid launches only; both may be null).
  const int32_t* tile_order;     // [tiles_x*tiles_y] hand-out position -> tile (row-major id)
  unsigned long long* tile_cost; // [tiles_x*tiles_y] work of each tile's samples, in
                                 // FP32-step equivalents (kCostFp64Step per FP64 step)
};

// An FP64 step counted in FP32-step equivalents for the tile cost log: GB300
// issues FP64 at about 1/64 of the FP32 rate, and an FP64 step has 7-14 FP64
// operations against about 140 FP32 instructions for an FE32 step.
constexpr int kCostFp64Step = 8;

// ---- the reference orbit, from shared memory where it is staged -------------
// A launch with z_stage > 0 holds zf[0, z_stage) and then z[0, z_stage) at the
// start of its dynamic shared memory (orbit_stage.cuh).
#if defined(__CUDACC__)
extern __shared__ __align__(16) unsigned char nm_orbit_smem[];
#endif

// kStaged: the calling kernel staged the prefix (a compile-time choice, so
// that the loads of every other kernel carry no test).
template <bool kStaged = false>
NM_HD Dbl2 orbit_z(const DeviceView& v, int j) {
#if defined(__CUDA_ARCH__)
  if (kStaged && j < v.z_stage)
    return reinterpret_cast<const Dbl2*>(nm_orbit_smem + 16 * v.z_stage)[j];
#endif
  return v.z[j];
}

template <bool kStaged = false>
NM_HD Flt4 orbit_zf(const DeviceView& v, int j) {
#if defined(__CUDA_ARCH__)
  if (kStaged && j < v.z_stage) return reinterpret_cast<const Flt4*>(nm_orbit_smem)[j];
#endif
  return v.zf[j];
}

// Sample index in tile order -> (r, c); false for padding past the grid edge.
// With a tile order, the k-th tile handed out is tile_order[k].
NM_HD bool sample_rc(const DeviceView& v, int64_t s, int& r, int& c) {
  const int64_t per_tile = (int64_t)v.tile_w * v.tile_h;
  const int64_t tile = s / per_tile;
  const int t = (int)(s - tile * per_tile);
  const int64_t id = v.tile_order ? (int64_t)v.tile_order[tile] : tile;
  const int ty = (int)(id / v.tiles_x);
  const int tx = (int)(id - (int64_t)ty * v.tiles_x);
  r = v.row0 + ty * v.tile_h + t / v.tile_w;
  c = tx * v.tile_w + t % v.tile_w;
  return r < v.row1 && c < v.nc;
}

// Row-major id of the tile holding sample (r, c).
NM_HD int64_t tile_at(const DeviceView& v, int r, int c) {
  return (int64_t)((r - v.row0) / v.tile_h) * v.tiles_x + c / v.tile_w;
}

}  // namespace nmg
