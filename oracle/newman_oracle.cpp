// newman oracle -- TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of newman's per-pixel Mandelbrot path (mandelbrot.cpp,
// complex.h, grid.h of axnjaxn/newman), used by the tests and the smoke check
// to compare the GPU results against, and timed as the benchmark's CPU
// baseline.  Nothing in the product (newman_gb300/) links, loads or calls this
// file.
//
// Parity status: PARITY UNPINNED.  The reference ships no tests, golden
// vectors or fixtures, and it cannot be compiled here (gmpxx.h / gmp.h,
// libbyteimage, SDL2 and Magick++ are absent), so this restatement is checked
// against closed-form facts and an independent mpmath evaluation instead
// (tests/test_oracle.py), not against the reference's own outputs.
//
// Arbitrary precision: the reference uses GMP's C++ wrapper (mpf_class).  Here
// every gmpxx expression is written out as the mpf_* calls it evaluates to,
// against the runtime libgmp.so.10, with every temporary at the precision of
// the expression's destination (the documented gmpxx rule).  `double`
// constants that gmpxx lifts into temporaries are exact (0.25, 1.0, 2.0).
//
// Floating point: compiled with -ffp-contract=off so that a*b+c*d is two
// roundings, as on x86-64 where the reference's -O3 build has no FMA.
//
// Two per-pixel modes:
//   MODE_REF   : the reference semantics -- getIterationsHW when useHardware()
//                holds, else getIterations with its arbitrary-precision
//                continuation (mandelbrot.cpp:144-254).
//   MODE_DELTA : the plain FP64 perturbation path of the GPU library, restated
//                sequentially: the reference's cardioid test, eps, series
//                approximation and binary search verbatim, then the FP64
//                delta iteration with rebasing instead of the MP loop.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "gmp_abi.h"

namespace {

constexpr double kBailout = 1024.0;                 // mandelbrot.cpp:58
constexpr double kBailout2 = kBailout * kBailout;   // mandelbrot.cpp:59
constexpr double kMinPreview = 1.5e-16;             // mandelbrot.cpp:257

// MODE_REF_FE / MODE_DELTA_FE: the same with the floatexp series front, for
// views whose series terms leave the FP64 range.
// MODE_DELTA_SINGLE: MODE_DELTA without the rebase on |Y| < |delta| -- plain
// single-reference perturbation, which loses precision where a sample's orbit
// passes far closer to 0 than the reference's (Pauldelbrot's glitches).  A
// planted mistake for the tests to show what the rebase catches; the orbit's
// end still rebases, so that every sample can go on.
enum { MODE_REF = 0, MODE_DELTA = 1, MODE_REF_FE = 2, MODE_DELTA_FE = 3, MODE_DELTA_SINGLE = 4 };

// RAII holder for one mpf_t at a fixed precision.
struct MP {
  mpf_t v;
  explicit MP(unsigned long bits) { mpf_init2(v, bits); }
  ~MP() { mpf_clear(v); }
  MP(const MP&) = delete;
  MP& operator=(const MP&) = delete;
  operator mpf_ptr() { return v; }
  operator mpf_srcptr() const { return v; }
};

// A complex array of mpf values at one precision (std::vector<HPComplex>).
struct MPArray {
  std::vector<__mpf_struct> re, im;
  unsigned long bits = 64;
  MPArray() = default;
  MPArray(const MPArray&) = delete;
  MPArray& operator=(const MPArray&) = delete;
  ~MPArray() { clear(); }
  void clear() {
    for (auto& x : re) mpf_clear(&x);
    for (auto& x : im) mpf_clear(&x);
    re.clear();
    im.clear();
  }
  void resize(size_t n, unsigned long b) {
    clear();
    bits = b;
    re.resize(n);
    im.resize(n);
    for (size_t i = 0; i < n; i++) {
      mpf_init2(&re[i], b);
      mpf_init2(&im[i], b);
    }
  }
  size_t size() const { return re.size(); }
  void swap(MPArray& o) {
    re.swap(o.re);
    im.swap(o.im);
    std::swap(bits, o.bits);
  }
};

struct LP {  // LPComplex, complex.h:6-11
  double re, im;
};
// complex.h:19-31, in the reference's operation order (no contraction).
inline LP sq(LP a) { return {a.re * a.re - a.im * a.im, 2.0 * a.re * a.im}; }
inline double sqMag(LP a) { return a.re * a.re + a.im * a.im; }
inline LP add(LP a, LP b) { return {a.re + b.re, a.im + b.im}; }
inline LP mul(LP a, LP b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }

// mandelbrot.cpp:133-136.  log(bailout) is evaluated the way the compiler
// folds the constant expression: correctly rounded.
inline double smoothing_magnitude(double r2) {
  static const double log_bailout = std::log(kBailout);
  return 1.0 - std::log2(0.5 * std::log(r2) / log_bailout);
}

// Per-thread scratch for the arbitrary-precision per-pixel work.
struct Scratch {
  MP t1, t2, t3, t4, fourth, y2, q, xmf, yr, yi, ynr, yni, dtmp, two, one;
  explicit Scratch(unsigned long bits)
      : t1(bits), t2(bits), t3(bits), t4(bits), fourth(bits), y2(bits), q(bits), xmf(bits),
        yr(bits), yi(bits), ynr(bits), yni(bits), dtmp(64), two(64), one(64) {
    mpf_set_d(fourth, 0.25);
    mpf_set_d(two, 2.0);
    mpf_set_d(one, 1.0);
  }
};

struct Pixel {
  int32_t iterations;
  double smoothing;  // before the float cast of grid.h:11
};

struct View {
  int nr = 1, nc = 1;
  int N = 256;
  double tol = 1e-10;
  unsigned long bits = 64;
  unsigned long min_bits = 0;
  std::unique_ptr<MP> cre, cim, sre, sim;
  // precompute results
  MPArray X, A, B, C;
  bool precomputed = false;
  int probe_index = -1;
  std::string err;

  // mandelbrot.cpp:37-56, setPrecision(): bits = max(64, (int)(64 - e + log2(1e-20)))
  // where sz.re = m * 2^e with 0.5 <= |m| < 1.  `min_bits` raises it.
  void set_precision() {
    const double log_alpha = std::log2(1.0e-20);
    const int beta = 64;
    long e = 0;
    mpf_get_d_2exp(&e, *sre);
    int b = (int)(beta - e + log_alpha);
    if (b < 64) b = 64;
    if ((unsigned long)b < min_bits) b = (int)min_bits;
    bits = (unsigned long)b;
    mpf_set_prec(*cre, bits);
    mpf_set_prec(*cim, bits);
    mpf_set_prec(*sre, bits);
    mpf_set_prec(*sim, bits);
    X.clear();
    A.clear();
    B.clear();
    C.clear();
    precomputed = false;
  }

  bool use_hardware() const {  // mandelbrot.cpp:256-259
    return mpf_get_d(*sre) >= kMinPreview && mpf_get_d(*sim) >= kMinPreview;
  }

  // pt.re = center.re + (c - cols()/2) * sz.re   (mandelbrot.cpp:275, :286-287)
  void point_re(int c, mpf_ptr out, mpf_ptr tmp) const {
    long k = (long)c - nc / 2;
    mpf_mul_ui(tmp, *sre, (unsigned long)(k < 0 ? -k : k));
    if (k < 0) mpf_neg(tmp, tmp);
    mpf_add(out, *cre, tmp);
  }
  // pt.im = center.im + (rows()/2 - r - 1) * sz.im   (mandelbrot.cpp:271, :288)
  void point_im(int r, mpf_ptr out, mpf_ptr tmp) const {
    long k = (long)(nr / 2) - r - 1;
    mpf_mul_ui(tmp, *sim, (unsigned long)(k < 0 ? -k : k));
    if (k < 0) mpf_neg(tmp, tmp);
    mpf_add(out, *cim, tmp);
  }
};

// mandelbrot.cpp:58-61: bailedOut(z) = sqMag(descend(z)) > bailout^2, with
// descend = mpf_get_d (truncation toward zero).
inline bool bailed_out(mpf_srcptr re, mpf_srcptr im) {
  LP z{mpf_get_d(re), mpf_get_d(im)};
  return sqMag(z) > kBailout2;
}

// mandelbrot.cpp:63-71
bool in_cardioid(mpf_srcptr zre, mpf_srcptr zim, Scratch& s) {
  mpf_sub(s.xmf, zre, s.fourth);          // xmf = Z.re - fourth
  mpf_mul(s.y2, zim, zim);                // y2 = Z.im * Z.im
  mpf_mul(s.q, s.xmf, s.xmf);             // q = xmf * xmf + y2
  mpf_add(s.q, s.q, s.y2);
  mpf_add(s.t1, s.q, s.xmf);              // q * (q + xmf)
  mpf_mul(s.t1, s.q, s.t1);
  mpf_mul(s.t2, s.fourth, s.y2);          // fourth * y2
  if (mpf_cmp(s.t1, s.t2) < 0) return true;
  mpf_add(s.q, zre, s.one);               // q = Z.re + 1.0
  mpf_mul(s.t1, s.q, s.q);                // q * q + y2
  mpf_add(s.t1, s.t1, s.y2);
  mpf_mul(s.t2, s.fourth, s.fourth);      // fourth * fourth
  return mpf_cmp(s.t1, s.t2) < 0;
}

// One step of computeOrbit (mandelbrot.cpp:102-103):
//   X[i].re = X[i-1].re * X[i-1].re - X[i-1].im * X[i-1].im + X0.re;
//   X[i].im = 2.0 * (X[i-1].re * X[i-1].im) + X0.im;
inline void orbit_step(mpf_ptr nre, mpf_ptr nim, mpf_srcptr xr, mpf_srcptr xi, mpf_srcptr x0r,
                       mpf_srcptr x0i, Scratch& s) {
  mpf_mul(s.t1, xr, xr);
  mpf_mul(s.t2, xi, xi);
  mpf_sub(s.t1, s.t1, s.t2);
  mpf_mul(s.t3, xr, xi);
  mpf_mul(s.t3, s.two, s.t3);
  mpf_add(nre, s.t1, x0r);
  mpf_add(nim, s.t3, x0i);
}

// Length of the orbit computeOrbit(X0) leaves in X (mandelbrot.cpp:97-110),
// without storing it.
int orbit_length(mpf_srcptr x0r, mpf_srcptr x0i, int N, unsigned long bits) {
  Scratch s(bits);
  MP ar(bits), ai(bits), br(bits), bi(bits);
  mpf_set(ar, x0r);
  mpf_set(ai, x0i);
  for (int i = 1; i < N; i++) {
    orbit_step(br, bi, ar, ai, x0r, x0i, s);
    if (bailed_out(br, bi)) return i;
    mpf_set(ar, br);
    mpf_set(ai, bi);
  }
  return N;
}

// mandelbrot.cpp:97-110
void compute_orbit(View& v, mpf_srcptr x0r, mpf_srcptr x0i, MPArray& X) {
  Scratch s(v.bits);
  X.resize(v.N, v.bits);
  mpf_set(&X.re[0], x0r);
  mpf_set(&X.im[0], x0i);
  for (int i = 1; i < v.N; i++) {
    orbit_step(&X.re[i], &X.im[i], &X.re[i - 1], &X.im[i - 1], x0r, x0i, s);
    if (bailed_out(&X.re[i], &X.im[i])) {
      // X.resize(i)
      for (size_t j = i; j < X.size(); j++) {
        mpf_clear(&X.re[j]);
        mpf_clear(&X.im[j]);
      }
      X.re.resize(i);
      X.im.resize(i);
      return;
    }
  }
}

// mandelbrot.cpp:73-95.  The probe orbits are independent, so their lengths
// are found on `threads` threads; the winner is the longest, the first probe
// in the reference's order winning ties (the strict `>` at :90).
int find_probe(View& v, int threads) {
  struct Pt { int r, c; };
  std::vector<Pt> pts;
  for (int c = 0; c < v.nc; c += 2) {
    pts.push_back({v.nr / 4, c});
    pts.push_back({v.nr / 2, c});
    pts.push_back({3 * v.nr / 4, c});
  }
  for (int r = 0; r < v.nr; r += 2) pts.push_back({r, v.nc / 2});

  std::vector<int> len(pts.size(), 0);
  std::atomic<size_t> next{0};
  auto worker = [&]() {
    MP pr(v.bits), pi(v.bits), tmp(v.bits);
    for (;;) {
      size_t k = next.fetch_add(1);
      if (k >= pts.size()) break;
      v.point_re(pts[k].c, pr, tmp);
      v.point_im(pts[k].r, pi, tmp);
      len[k] = orbit_length(pr, pi, v.N, v.bits);
    }
  };
  int T = std::max(1, threads);
  std::vector<std::thread> pool;
  for (int t = 0; t < T; t++) pool.emplace_back(worker);
  for (auto& t : pool) t.join();

  int best = 0;
  for (size_t k = 1; k < pts.size(); k++)
    if (len[k] > len[best]) best = (int)k;

  MP pr(v.bits), pi(v.bits), tmp(v.bits);
  v.point_re(pts[best].c, pr, tmp);
  v.point_im(pts[best].r, pi, tmp);
  compute_orbit(v, pr, pi, v.X);
  return best;
}

// mandelbrot.cpp:112-131
void compute_series(View& v) {
  Scratch s(v.bits);
  size_t n = v.X.size();
  v.A.resize(n, v.bits);
  v.B.resize(n, v.bits);
  v.C.resize(n, v.bits);
  mpf_set_d(&v.A.re[0], 1.0);
  mpf_set_d(&v.A.im[0], 0.0);
  mpf_set_d(&v.B.re[0], 0.0);
  mpf_set_d(&v.B.im[0], 0.0);
  mpf_set_d(&v.C.re[0], 0.0);
  mpf_set_d(&v.C.im[0], 0.0);
  MP u(v.bits);
  for (size_t i = 1; i < n; i++) {
    mpf_srcptr xr = &v.X.re[i - 1], xi = &v.X.im[i - 1];
    mpf_srcptr ar = &v.A.re[i - 1], ai = &v.A.im[i - 1];
    mpf_srcptr br = &v.B.re[i - 1], bi = &v.B.im[i - 1];
    mpf_srcptr cr = &v.C.re[i - 1], ci = &v.C.im[i - 1];
    mpf_ptr Ar = &v.A.re[i], Ai = &v.A.im[i];
    mpf_ptr Br = &v.B.re[i], Bi = &v.B.im[i];
    mpf_ptr Cr = &v.C.re[i], Ci = &v.C.im[i];
    // A[i].re = 2.0 * (X.re * A.re - X.im * A.im) + 1.0;
    mpf_mul(s.t1, xr, ar); mpf_mul(s.t2, xi, ai); mpf_sub(s.t1, s.t1, s.t2);
    mpf_mul(s.t1, s.two, s.t1); mpf_add(Ar, s.t1, s.one);
    // A[i].im = 2.0 * (X.re * A.im + X.im * A.re);
    mpf_mul(s.t1, xr, ai); mpf_mul(s.t2, xi, ar); mpf_add(s.t1, s.t1, s.t2);
    mpf_mul(Ai, s.two, s.t1);
    // B[i].re = 2.0 * (X.re * B.re - X.im * B.im) + A[i].re * A[i].re - A[i].im * A[i].im;
    mpf_mul(s.t1, xr, br); mpf_mul(s.t2, xi, bi); mpf_sub(s.t1, s.t1, s.t2);
    mpf_mul(s.t1, s.two, s.t1);
    mpf_mul(s.t2, Ar, Ar); mpf_add(s.t1, s.t1, s.t2);
    mpf_mul(s.t2, Ai, Ai); mpf_sub(Br, s.t1, s.t2);
    // B[i].im = 2.0 * (X.re * B.im + X.im * B.re + A[i].re * A[i].im);
    mpf_mul(s.t1, xr, bi); mpf_mul(s.t2, xi, br); mpf_add(s.t1, s.t1, s.t2);
    mpf_mul(s.t2, Ar, Ai); mpf_add(s.t1, s.t1, s.t2);
    mpf_mul(Bi, s.two, s.t1);
    // C[i].re = 2.0 * (X.re * C.re - X.im * C.im + A[i].re * B[i].re - A[i].im * B[i].im);
    mpf_mul(s.t1, xr, cr); mpf_mul(s.t2, xi, ci); mpf_sub(s.t1, s.t1, s.t2);
    mpf_mul(s.t2, Ar, Br); mpf_add(s.t1, s.t1, s.t2);
    mpf_mul(s.t2, Ai, Bi); mpf_sub(s.t1, s.t1, s.t2);
    mpf_mul(Cr, s.two, s.t1);
    // C[i].im = 2.0 * (X.re * C.im + X.im * C.re + A[i].re * B[i].im + A[i].im * B[i].re);
    mpf_mul(s.t1, xr, ci); mpf_mul(s.t2, xi, cr); mpf_add(s.t1, s.t1, s.t2);
    mpf_mul(s.t2, Ar, Bi); mpf_add(s.t1, s.t1, s.t2);
    mpf_mul(s.t2, Ai, Br); mpf_add(s.t1, s.t1, s.t2);
    mpf_mul(Ci, s.two, s.t1);
  }
}

// mandelbrot.cpp:231-254
Pixel get_iterations_hw(View& v, mpf_srcptr y0r, mpf_srcptr y0i, Scratch& s) {
  LP z0{mpf_get_d(y0r), mpf_get_d(y0i)};
  if (in_cardioid(y0r, y0i, s)) return {v.N, 0.0};
  LP z = z0;
  int it;
  for (it = 0; it < v.N; it++) {
    z = add(sq(z), z0);
    if (sqMag(z) > kBailout2) break;
  }
  if (it < v.N) return {it, smoothing_magnitude(sqMag(z))};
  return {it, 0.0};
}

// Series-approximation term d[i] = a + b + c (mandelbrot.cpp:166-180) and the
// instability test (:138-142, :173).
struct SATerm {
  LP d;
  bool unstable;
};
inline SATerm sa_term(const View& v, size_t i, LP eps, LP eps2, LP eps3) {
  LP a{mpf_get_d(&v.A.re[i]), mpf_get_d(&v.A.im[i])};
  LP b{mpf_get_d(&v.B.re[i]), mpf_get_d(&v.B.im[i])};
  LP c{mpf_get_d(&v.C.re[i]), mpf_get_d(&v.C.im[i])};
  a = mul(a, eps);
  b = mul(b, eps2);
  c = mul(c, eps3);
  double bmag = b.re * b.re + b.im * b.im;
  double cmag = c.re * c.re + c.im * c.im;
  SATerm t;
  t.unstable = bmag * v.tol < cmag;
  t.d = add(add(a, b), c);
  return t;
}

// Shared front half of getIterations (mandelbrot.cpp:144-207): cardioid test,
// eps, the series skip, and the binary search when the skipped point has
// already escaped.  Returns true when the pixel is finished; otherwise leaves
// the continuation start in (found, dfound, Y).
struct SAState {
  LP eps;
  size_t dsize;
  LP dfound;
};
bool series_front(View& v, mpf_srcptr y0r, mpf_srcptr y0i, Scratch& s, Pixel& out, SAState& st) {
  if (in_cardioid(y0r, y0i, s)) {
    out = {v.N, 0.0};
    return true;
  }
  mpf_sub(s.yr, y0r, &v.X.re[0]);
  mpf_sub(s.yi, y0i, &v.X.im[0]);
  LP eps{mpf_get_d(s.yr), mpf_get_d(s.yi)};
  LP eps2 = sq(eps);
  LP eps3 = mul(eps, eps2);

  const size_t n = v.X.size();
  std::vector<LP> d(n);
  d[0] = eps;
  size_t dsize = n;
  for (size_t i = 1; i < n; i++) {
    SATerm t = sa_term(v, i, eps, eps2, eps3);
    if (t.unstable) {
      long good = (long)i - 3;
      if (good < 1) good = 1;
      dsize = (size_t)good;
      break;
    }
    d[i] = t.d;
  }

  size_t found = dsize - 1;
  auto xplusd = [&](size_t k) {  // Y = X[k] + d[k]   (mpf + double)
    mpf_set_d(s.dtmp, d[k].re);
    mpf_add(s.yr, &v.X.re[k], s.dtmp);
    mpf_set_d(s.dtmp, d[k].im);
    mpf_add(s.yi, &v.X.im[k], s.dtmp);
  };
  xplusd(found);
  if (bailed_out(s.yr, s.yi)) {
    long low = 0, high = (long)dsize - 1, mid = (long)dsize / 2;
    while (low <= high) {
      xplusd((size_t)mid);
      if (!bailed_out(s.yr, s.yi))
        low = mid + 1;
      else {
        high = mid - 1;
        found = (size_t)mid;
      }
      mid = (low + high) / 2;
    }
    xplusd(found);
    LP y{mpf_get_d(s.yr), mpf_get_d(s.yi)};
    out = {(int32_t)found, smoothing_magnitude(sqMag(y))};
    return true;
  }
  st.eps = eps;
  st.dsize = dsize;
  st.dfound = d[found];
  return false;
}

// mandelbrot.cpp:144-229 (MODE_REF, deep path)
Pixel get_iterations(View& v, mpf_srcptr y0r, mpf_srcptr y0i, Scratch& s) {
  Pixel out;
  SAState st;
  if (series_front(v, y0r, y0i, s, out, st)) return out;
  // s.yr/s.yi hold Y = X[found] + d[found]
  for (int i = (int)st.dsize; i < v.N; i++) {
    orbit_step(s.ynr, s.yni, s.yr, s.yi, y0r, y0i, s);
    if (bailed_out(s.ynr, s.yni)) {
      LP y{mpf_get_d(s.ynr), mpf_get_d(s.yni)};
      return {i, smoothing_magnitude(sqMag(y))};
    }
    mpf_set(s.yr, s.ynr);
    mpf_set(s.yi, s.yni);
  }
  return {v.N, 0.0};
}

// MODE_DELTA: the GPU library's plain FP64 perturbation path.  Identical to
// getIterations up to the continuation; the continuation iterates the FP64
// delta against the reference orbit Z (Z[0] = 0, Z[k+1] = get_d(X[k]), plus
// the escaped element) with rebasing to Z[0] (Zhuoran) whenever |Y| < |delta|
// or the orbit is exhausted:
//   t = 2 Z[j] + delta;  delta = t * delta + eps;  j += 1;  Y = Z[j] + delta
Pixel get_iterations_delta(View& v, mpf_srcptr y0r, mpf_srcptr y0i, Scratch& s,
                           const std::vector<LP>& Z, bool rebase_small = true) {
  Pixel out;
  SAState st;
  if (series_front(v, y0r, y0i, s, out, st)) return out;
  LP dl = st.dfound;
  const LP eps = st.eps;
  size_t j = st.dsize;  // Y = Z[found + 1] + delta, found = dsize - 1
  const size_t zlast = Z.size() - 1;
  for (int i = (int)st.dsize; i < v.N; i++) {
    LP z = Z[j];
    double tr = 2.0 * z.re + dl.re;
    double ti = 2.0 * z.im + dl.im;
    double nre = (tr * dl.re - ti * dl.im) + eps.re;
    double nim = (tr * dl.im + ti * dl.re) + eps.im;
    dl = {nre, nim};
    j++;
    LP y{Z[j].re + dl.re, Z[j].im + dl.im};
    double r2 = y.re * y.re + y.im * y.im;
    if (r2 > kBailout2) return {i, smoothing_magnitude(r2)};
    double d2 = dl.re * dl.re + dl.im * dl.im;
    if ((rebase_small && r2 < d2) || j == zlast) {
      dl = y;
      j = 0;
    }
  }
  return {v.N, 0.0};
}

// ---- floatexp series front (views outside the FP64 range) -------------------
// The reference's series arithmetic on FP64 mantissas with a separate
// exponent, each result rescaled exactly so that its larger component lies in
// [0.5, 1).  In the FP64 range it gives the FP64 results; below it, the same
// operations without overflow (the reference itself turns to NaN there).
struct FX {
  double re, im;
  long e;
};
inline FX fx_norm(FX a) {
  double m = std::max(std::fabs(a.re), std::fabs(a.im));
  if (m == 0.0) return {a.re, a.im, 0};
  int k;
  std::frexp(m, &k);
  return {std::ldexp(a.re, -k), std::ldexp(a.im, -k), a.e + k};
}
inline FX fx_of(mpf_srcptr re, mpf_srcptr im) {
  long er, ei;
  double dr = mpf_get_d_2exp(&er, re), di = mpf_get_d_2exp(&ei, im);
  if (dr == 0.0 && di == 0.0) return {0.0, 0.0, 0};
  long e = dr == 0.0 ? ei : di == 0.0 ? er : std::max(er, ei);
  return fx_norm({std::ldexp(dr, (int)(er - e)), std::ldexp(di, (int)(ei - e)), e});
}
inline FX fx_mul(FX a, FX b) {
  LP p = mul({a.re, a.im}, {b.re, b.im});
  return fx_norm({p.re, p.im, a.e + b.e});
}
inline FX fx_sq(FX a) {
  LP p = sq({a.re, a.im});
  return fx_norm({p.re, p.im, 2 * a.e});
}
inline FX fx_add(FX a, FX b) {
  if (a.e < b.e) std::swap(a, b);
  int d = (int)std::max<long>(b.e - a.e, -2000);
  return fx_norm({a.re + std::ldexp(b.re, d), a.im + std::ldexp(b.im, d), a.e});
}
// |a|^2 as (mantissa, exponent)
inline std::pair<double, long> fx_mag2(FX a) { return {a.re * a.re + a.im * a.im, 2 * a.e}; }
inline bool fx_less(std::pair<double, long> x, std::pair<double, long> y) {
  if (!(x.first > 0.0)) return y.first > 0.0;
  if (!(y.first > 0.0)) return false;
  int ex, ey;
  double mx = std::frexp(x.first, &ex), my = std::frexp(y.first, &ey);
  long tx = ex + x.second, ty = ey + y.second;
  if (tx != ty) return tx < ty;
  return mx < my;
}
inline double fx_re(FX a) { return std::ldexp(a.re, (int)std::max<long>(a.e, -2000)); }
inline double fx_im(FX a) { return std::ldexp(a.im, (int)std::max<long>(a.e, -2000)); }

struct SAStateFX {
  FX eps;
  size_t dsize;
  FX dfound;
};

// series_front with the floatexp series arithmetic (mandelbrot.cpp:144-207).
bool series_front_fx(View& v, mpf_srcptr y0r, mpf_srcptr y0i, Scratch& s, Pixel& out,
                     SAStateFX& st) {
  if (in_cardioid(y0r, y0i, s)) {
    out = {v.N, 0.0};
    return true;
  }
  mpf_sub(s.yr, y0r, &v.X.re[0]);
  mpf_sub(s.yi, y0i, &v.X.im[0]);
  FX eps = fx_of(s.yr, s.yi);
  FX eps2 = fx_sq(eps);
  FX eps3 = fx_mul(eps, eps2);
  const size_t n = v.X.size();
  auto term = [&](size_t i, bool& unstable) {
    FX a = fx_mul(fx_of(&v.A.re[i], &v.A.im[i]), eps);
    FX b = fx_mul(fx_of(&v.B.re[i], &v.B.im[i]), eps2);
    FX c = fx_mul(fx_of(&v.C.re[i], &v.C.im[i]), eps3);
    auto bm = fx_mag2(b), cm = fx_mag2(c);
    bm.first *= v.tol;
    unstable = fx_less(bm, cm);  // bmag * tol < cmag
    return fx_add(fx_add(a, b), c);
  };
  size_t dsize = n;
  for (size_t i = 1; i < n; i++) {
    bool u;
    term(i, u);
    if (u) {
      long good = (long)i - 3;
      dsize = (size_t)(good < 1 ? 1 : good);
      break;
    }
  }
  auto dval = [&](size_t k) {
    if (k == 0) return eps;
    bool u;
    return term(k, u);
  };
  auto xplusd = [&](size_t k) {
    FX d = dval(k);
    mpf_set_d(s.dtmp, fx_re(d));
    mpf_add(s.yr, &v.X.re[k], s.dtmp);
    mpf_set_d(s.dtmp, fx_im(d));
    mpf_add(s.yi, &v.X.im[k], s.dtmp);
  };
  size_t found = dsize - 1;
  xplusd(found);
  if (bailed_out(s.yr, s.yi)) {
    long low = 0, high = (long)dsize - 1, mid = (long)dsize / 2;
    while (low <= high) {
      xplusd((size_t)mid);
      if (!bailed_out(s.yr, s.yi))
        low = mid + 1;
      else {
        high = mid - 1;
        found = (size_t)mid;
      }
      mid = (low + high) / 2;
    }
    xplusd(found);
    LP y{mpf_get_d(s.yr), mpf_get_d(s.yi)};
    out = {(int32_t)found, smoothing_magnitude(sqMag(y))};
    return true;
  }
  st.eps = eps;
  st.dsize = dsize;
  st.dfound = dval(found);
  return false;
}

// MODE_REF_FE: getIterations with the floatexp series front and the
// reference's arbitrary-precision continuation.
Pixel get_iterations_fx(View& v, mpf_srcptr y0r, mpf_srcptr y0i, Scratch& s) {
  Pixel out;
  SAStateFX st;
  if (series_front_fx(v, y0r, y0i, s, out, st)) return out;
  for (int i = (int)st.dsize; i < v.N; i++) {
    orbit_step(s.ynr, s.yni, s.yr, s.yi, y0r, y0i, s);
    if (bailed_out(s.ynr, s.yni)) {
      LP y{mpf_get_d(s.ynr), mpf_get_d(s.yni)};
      return {i, smoothing_magnitude(sqMag(y))};
    }
    mpf_set(s.yr, s.ynr);
    mpf_set(s.yi, s.yni);
  }
  return {v.N, 0.0};
}

// FP64 with an unbounded exponent: a real m * 2^e with m = 0 or 0.5 <= |m| < 1
// (frexp's convention).  Each operation rounds its exact result to 53 bits,
// round-to-nearest-even, as a double operation would without exponent
// limits: a sum aligns the smaller operand by ldexp (exact for shifts up to
// 60 bits; beyond that it lies below half an ulp of the larger and the sum
// is the larger), a product multiplies mantissas in [0.5, 1).  On values in
// the double range this is the double arithmetic itself.
struct XR {
  double m;
  long e;
};
constexpr long kXrZeroExp = -(1L << 40);
inline XR xr_norm(double x, long e) {
  if (x == 0.0) return {0.0, kXrZeroExp};
  int k;
  double m = std::frexp(x, &k);
  return {m, e + k};
}
inline XR xr_add(XR a, XR b) {
  if (b.m == 0.0) return a;
  if (a.m == 0.0) return b;
  if (a.e < b.e) std::swap(a, b);
  long d = a.e - b.e;
  if (d > 60) return a;
  return xr_norm(a.m + std::ldexp(b.m, (int)-d), a.e);
}
inline XR xr_neg(XR a) { return {-a.m, a.e}; }
inline XR xr_mul(XR a, XR b) { return xr_norm(a.m * b.m, a.e + b.e); }
inline bool xr_gt(XR a, XR b) {  // a > b for a, b >= 0
  if (a.m == 0.0) return false;
  if (b.m == 0.0) return true;
  return a.e > b.e || (a.e == b.e && a.m > b.m);
}

// MODE_DELTA_FE: the GPU library's FP64 perturbation path on a floatexp
// view: delta_steps' operations in FP64 with an unbounded exponent.
Pixel get_iterations_delta_fx(View& v, mpf_srcptr y0r, mpf_srcptr y0i, Scratch& s,
                              const std::vector<LP>& Z) {
  Pixel out;
  SAStateFX st;
  if (series_front_fx(v, y0r, y0i, s, out, st)) return out;
  XR dr = xr_norm(st.dfound.re, st.dfound.e), di = xr_norm(st.dfound.im, st.dfound.e);
  const XR er = xr_norm(st.eps.re, st.eps.e), ei = xr_norm(st.eps.im, st.eps.e);
  const XR bail2 = xr_norm(kBailout2, 0);
  size_t j = st.dsize;
  const size_t zlast = Z.size() - 1;
  for (int i = (int)st.dsize; i < v.N; i++) {
    const LP z = Z[j];
    XR zr = xr_norm(z.re, 0), zi = xr_norm(z.im, 0);
    XR tr = xr_add(xr_add(zr, zr), dr);  // 2 z exactly
    XR ti = xr_add(xr_add(zi, zi), di);
    XR nre = xr_add(xr_add(xr_mul(tr, dr), xr_neg(xr_mul(ti, di))), er);
    XR nim = xr_add(xr_add(xr_mul(tr, di), xr_mul(ti, dr)), ei);
    dr = nre;
    di = nim;
    j++;
    XR yr = xr_add(xr_norm(Z[j].re, 0), dr), yi = xr_add(xr_norm(Z[j].im, 0), di);
    XR r2 = xr_add(xr_mul(yr, yr), xr_mul(yi, yi));
    if (xr_gt(r2, bail2)) return {i, smoothing_magnitude(std::ldexp(r2.m, (int)r2.e))};
    XR d2 = xr_add(xr_mul(dr, dr), xr_mul(di, di));
    if (xr_gt(d2, r2) || j == zlast) {
      dr = yr;
      di = yi;
      j = 0;
    }
  }
  return {v.N, 0.0};
}

// The FP64 copy of the orbit the delta path iterates against.
std::vector<LP> delta_orbit(View& v) {
  std::vector<LP> Z;
  Z.reserve(v.X.size() + 2);
  Z.push_back({0.0, 0.0});
  for (size_t k = 0; k < v.X.size(); k++) Z.push_back({mpf_get_d(&v.X.re[k]), mpf_get_d(&v.X.im[k])});
  if ((int)v.X.size() < v.N) {  // keep the element that escaped
    Scratch s(v.bits);
    MP er(v.bits), ei(v.bits);
    size_t m = v.X.size() - 1;
    orbit_step(er, ei, &v.X.re[m], &v.X.im[m], &v.X.re[0], &v.X.im[0], s);
    Z.push_back({mpf_get_d(er), mpf_get_d(ei)});
  }
  return Z;
}

template <typename F>
void parallel_for(size_t n, int threads, F f) {
  int T = std::max(1, std::min<int>(threads, (int)std::max<size_t>(n, 1)));
  std::atomic<size_t> next{0};
  auto worker = [&]() {
    for (;;) {
      size_t k = next.fetch_add(1);
      if (k >= n) break;
      f(k);
    }
  };
  if (T == 1) {
    worker();
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < T; t++) pool.emplace_back(worker);
  for (auto& t : pool) t.join();
}

}  // namespace

extern "C" {

struct nmo_view;

nmo_view* nmo_create(int nr, int nc) {
  if (nr < 1 || nc < 1) return nullptr;
  View* v = new View();
  v->nr = nr;
  v->nc = nc;
  // mandelbrot.cpp:8-17 defaults
  v->cre.reset(new MP(64));
  v->cim.reset(new MP(64));
  v->sre.reset(new MP(64));
  v->sim.reset(new MP(64));
  mpf_set_d(*v->cre, -0.5);
  mpf_set_d(*v->cim, 0.0);
  mpf_set_d(*v->sre, 4.0 / nc);
  mpf_set_d(*v->sim, 3.0 / nr);
  v->set_precision();
  return reinterpret_cast<nmo_view*>(v);
}

void nmo_destroy(nmo_view* h) { delete reinterpret_cast<View*>(h); }

// The view a reference save file holds (viewer.cpp:14-22): center and pixel
// step as decimal strings.  The step is parsed first to fix the precision,
// then every string is parsed at that precision.
int nmo_set_view(nmo_view* h, const char* cre, const char* cim, const char* sre, const char* sim,
                 int N, double tol, int min_bits) {
  View* v = reinterpret_cast<View*>(h);
  if (!v || N < 1) return 1;
  v->N = N;
  v->tol = tol;
  v->min_bits = min_bits > 0 ? (unsigned long)min_bits : 0;
  MP probe(4096);
  if (mpf_set_str(probe, sre, 10) != 0) return 2;
  mpf_set_prec(*v->sre, 4096);
  mpf_set(*v->sre, probe);
  v->set_precision();
  if (mpf_set_str(*v->cre, cre, 10) || mpf_set_str(*v->cim, cim, 10) ||
      mpf_set_str(*v->sre, sre, 10) || mpf_set_str(*v->sim, sim, 10))
    return 2;
  return 0;
}

int nmo_set_iterations(nmo_view* h, int N) {
  View* v = reinterpret_cast<View*>(h);
  if (N < 1) return 1;
  v->N = N;
  v->X.clear(); v->A.clear(); v->B.clear(); v->C.clear();
  v->precomputed = false;
  return 0;
}

int nmo_rows(nmo_view* h) { return reinterpret_cast<View*>(h)->nr; }
int nmo_cols(nmo_view* h) { return reinterpret_cast<View*>(h)->nc; }
int nmo_bits(nmo_view* h) { return (int)reinterpret_cast<View*>(h)->bits; }
int nmo_use_hardware(nmo_view* h) { return reinterpret_cast<View*>(h)->use_hardware() ? 1 : 0; }

// mandelbrot.cpp:334-346 / :348-360 (geometry; the grid values are reduced by
// nmo_reduce).
int nmo_scale_up(nmo_view* h, int sc) {
  View* v = reinterpret_cast<View*>(h);
  if (sc < 1) return 1;
  v->nr *= sc;
  v->nc *= sc;
  mpf_div_ui(*v->sre, *v->sre, (unsigned long)sc);
  mpf_div_ui(*v->sim, *v->sim, (unsigned long)sc);
  v->set_precision();
  return 0;
}
int nmo_scale_down(nmo_view* h, int sc) {
  View* v = reinterpret_cast<View*>(h);
  if (sc < 1) return 1;
  v->nr /= sc;
  v->nc /= sc;
  mpf_mul_ui(*v->sre, *v->sre, (unsigned long)sc);
  mpf_mul_ui(*v->sim, *v->sim, (unsigned long)sc);
  v->set_precision();
  return 0;
}

// mandelbrot.cpp:261-267
int nmo_precompute(nmo_view* h, int threads) {
  View* v = reinterpret_cast<View*>(h);
  if (v->use_hardware()) {
    v->precomputed = true;
    v->probe_index = -1;
    return 0;
  }
  v->X.clear(); v->A.clear(); v->B.clear(); v->C.clear();
  v->probe_index = find_probe(*v, threads);
  compute_series(*v);
  v->precomputed = true;
  return 0;
}

// precompute with the view center as the only probe (pointAt(nr/2 - 1, nc/2)
// is exactly the center): the reference orbit of the library's
// REFERENCE_CENTER mode.
int nmo_precompute_center(nmo_view* h) {
  View* v = reinterpret_cast<View*>(h);
  v->X.clear(); v->A.clear(); v->B.clear(); v->C.clear();
  MP pr(v->bits), pi(v->bits), tmp(v->bits);
  v->point_re(v->nc / 2, pr, tmp);
  v->point_im(v->nr / 2 - 1, pi, tmp);
  compute_orbit(*v, pr, pi, v->X);
  compute_series(*v);
  v->probe_index = 0;
  v->precomputed = true;
  return 0;
}

int nmo_probe_index(nmo_view* h) { return reinterpret_cast<View*>(h)->probe_index; }
int nmo_orbit_length(nmo_view* h) { return (int)reinterpret_cast<View*>(h)->X.size(); }

// get_d of X, A, B, C (each 2*len doubles: re, im interleaved), plus the
// remainder X - get_d(X) as a second double (xlo).
int nmo_export_orbit(nmo_view* h, double* x, double* xlo, double* a, double* b, double* c) {
  View* v = reinterpret_cast<View*>(h);
  MP t(v->bits), hi(v->bits);
  for (size_t i = 0; i < v->X.size(); i++) {
    if (x) { x[2 * i] = mpf_get_d(&v->X.re[i]); x[2 * i + 1] = mpf_get_d(&v->X.im[i]); }
    if (xlo) {
      mpf_set_d(hi, mpf_get_d(&v->X.re[i])); mpf_sub(t, &v->X.re[i], hi); xlo[2 * i] = mpf_get_d(t);
      mpf_set_d(hi, mpf_get_d(&v->X.im[i])); mpf_sub(t, &v->X.im[i], hi); xlo[2 * i + 1] = mpf_get_d(t);
    }
    if (a) { a[2 * i] = mpf_get_d(&v->A.re[i]); a[2 * i + 1] = mpf_get_d(&v->A.im[i]); }
    if (b) { b[2 * i] = mpf_get_d(&v->B.re[i]); b[2 * i + 1] = mpf_get_d(&v->B.im[i]); }
    if (c) { c[2 * i] = mpf_get_d(&v->C.re[i]); c[2 * i + 1] = mpf_get_d(&v->C.im[i]); }
  }
  return 0;
}

// get_d of the pixel coordinates (pt.re per column, pt.im per row).
int nmo_coords(nmo_view* h, double* re, double* im) {
  View* v = reinterpret_cast<View*>(h);
  MP p(v->bits), t(v->bits);
  for (int c = 0; c < v->nc; c++) { v->point_re(c, p, t); re[c] = mpf_get_d(p); }
  for (int r = 0; r < v->nr; r++) { v->point_im(r, p, t); im[r] = mpf_get_d(p); }
  return 0;
}

// Render an explicit list of sample positions.  mode: MODE_REF or MODE_DELTA.
int nmo_render_pixels(nmo_view* h, int mode, long npix, const int32_t* rows, const int32_t* cols,
                      int32_t* iters, double* smooth, int threads) {
  View* v = reinterpret_cast<View*>(h);
  const bool hw = v->use_hardware();
  if (!hw && !v->precomputed) return 3;
  if (mode != MODE_REF && hw) return 4;
  std::vector<LP> Z;
  if (mode == MODE_DELTA || mode == MODE_DELTA_FE || mode == MODE_DELTA_SINGLE)
    Z = delta_orbit(*v);
  for (long k = 0; k < npix; k++)
    if (rows[k] < 0 || rows[k] >= v->nr || cols[k] < 0 || cols[k] >= v->nc) return 5;
  parallel_for((size_t)npix, threads, [&](size_t k) {
    thread_local std::unique_ptr<Scratch> s;
    thread_local unsigned long sbits = 0;
    if (!s || sbits != v->bits) { s.reset(new Scratch(v->bits)); sbits = v->bits; }
    MP pr(v->bits), pi(v->bits), tmp(v->bits);
    v->point_im(rows[k], pi, tmp);
    v->point_re(cols[k], pr, tmp);
    Pixel p;
    if (hw) p = get_iterations_hw(*v, pr, pi, *s);
    else if (mode == MODE_REF) p = get_iterations(*v, pr, pi, *s);
    else if (mode == MODE_DELTA) p = get_iterations_delta(*v, pr, pi, *s, Z);
    else if (mode == MODE_DELTA_SINGLE) p = get_iterations_delta(*v, pr, pi, *s, Z, false);
    else if (mode == MODE_REF_FE) p = get_iterations_fx(*v, pr, pi, *s);
    else p = get_iterations_delta_fx(*v, pr, pi, *s, Z);
    iters[k] = p.iterations;
    smooth[k] = p.smoothing;
  });
  return 0;
}

// d.size() after the series loop of getIterations (mandelbrot.cpp:163-181)
// for each listed sample: the number of iterations the series skips.  -1 for
// samples inside the cardioid / period-2 disk.
int nmo_series_skip(nmo_view* h, long npix, const int32_t* rows, const int32_t* cols,
                    int32_t* dsize) {
  View* v = reinterpret_cast<View*>(h);
  if (v->use_hardware() || !v->precomputed) return 3;
  Scratch s(v->bits);
  MP pr(v->bits), pi(v->bits), tmp(v->bits);
  for (long k = 0; k < npix; k++) {
    v->point_im(rows[k], pi, tmp);
    v->point_re(cols[k], pr, tmp);
    if (in_cardioid(pr, pi, s)) {
      dsize[k] = -1;
      continue;
    }
    mpf_sub(s.yr, pr, &v->X.re[0]);
    mpf_sub(s.yi, pi, &v->X.im[0]);
    LP eps{mpf_get_d(s.yr), mpf_get_d(s.yi)};
    LP eps2 = sq(eps), eps3 = mul(eps, eps2);
    size_t n = v->X.size(), ds = n;
    for (size_t i = 1; i < n; i++)
      if (sa_term(*v, i, eps, eps2, eps3).unstable) {
        long good = (long)i - 3;
        ds = (size_t)(good < 1 ? 1 : good);
        break;
      }
    dsize[k] = (int32_t)ds;
  }
  return 0;
}

// Render rows [r0, r1) of the sample grid, row-major (computeRow, :269-283).
int nmo_render_rows(nmo_view* h, int mode, int r0, int r1, int32_t* iters, double* smooth,
                    int threads) {
  View* v = reinterpret_cast<View*>(h);
  if (r0 < 0 || r1 > v->nr || r0 > r1) return 5;
  long n = (long)(r1 - r0) * v->nc;
  std::vector<int32_t> rr(n), cc(n);
  for (long k = 0; k < n; k++) {
    rr[k] = r0 + (int32_t)(k / v->nc);
    cc[k] = (int32_t)(k % v->nc);
  }
  return nmo_render_pixels(h, mode, n, rr.data(), cc.data(), iters, smooth, threads);
}

// Multisample average, mandelbrot.cpp:320-332 (at(r, c, sc)), over a
// row-major (nr*sc) x (nc*sc) grid of {iterations, float smoothing}.
int nmo_reduce(int nr, int nc, int sc, const int32_t* iters, const float* smooth,
               int32_t* out_iters, float* out_smooth) {
  if (sc < 1) return 1;
  const int NC = nc * sc;
  for (int r = 0; r < nr; r++)
    for (int c = 0; c < nc; c++) {
      float sum = 0.0f;
      for (int r1 = 0; r1 < sc; r1++)
        for (int c1 = 0; c1 < sc; c1++) {
          long k = (long)(sc * r + r1) * NC + (sc * c + c1);
          sum += iters[k] + smooth[k];
        }
      sum /= sc * sc;
      int it = (int)sum;
      out_iters[(long)r * nc + c] = it;
      out_smooth[(long)r * nc + c] = sum - it;
    }
  return 0;
}

// ---- colouring: multiwave.cpp:5-116 and viewer.cpp:89-124 --------------------
// libbyteimage's helpers (absent from the reference tree) as their standard
// definitions: clip rounds half up into [0, 255]; interp blends per channel;
// hsl2rgb is the usual six-sector map.
namespace colour {
unsigned char clip(float x) {
  if (x > 0.0f) return x >= 255.0f ? 255 : (unsigned char)(x + 0.5f);
  return 0;
}
struct C3 {
  unsigned char c[3];
};
C3 blend(C3 a, C3 b, float t) {
  C3 o;
  for (int k = 0; k < 3; k++) o.c[k] = clip((1.0f - t) * a.c[k] + t * b.c[k]);
  return o;
}
C3 hsl(float h, float s, float l) {
  float hue = std::fmod(h, 360.0f);
  if (hue < 0.0f) hue += 360.0f;
  const float chroma = (1.0f - std::fabs(2.0f * l - 1.0f)) * s;
  const float sector = hue / 60.0f;
  const float mid = chroma * (1.0f - std::fabs(std::fmod(sector, 2.0f) - 1.0f));
  const float tab[6][3] = {{chroma, mid, 0.0f}, {mid, chroma, 0.0f}, {0.0f, chroma, mid},
                           {0.0f, mid, chroma}, {mid, 0.0f, chroma}, {chroma, 0.0f, mid}};
  const float* t = tab[(int)sector % 6];
  const float base = l - 0.5f * chroma;
  C3 o;
  for (int k = 0; k < 3; k++) o.c[k] = clip(255.0f * (t[k] + base));
  return o;
}
struct Cycle {
  std::vector<float> v;
  int period = 1;
  // (1.0 - t) promotes the blend to double (multiwave.cpp:11)
  float at(int step) const {
    float t = (int)v.size() * (step % period) / (float)period;
    int i0 = (int)t;
    t -= i0;
    return (float)((1.0 - t) * v[i0] + t * v[(i0 + 1) % v.size()]);
  }
};
struct Palette {
  std::vector<Cycle> hue;
  int hue_period = 1;
  Cycle sat;
  std::vector<std::pair<float, int>> waves;  // amplitude, period
};
bool read_palette(const char* path, Palette& p) {
  std::FILE* fp = std::fopen(path, "r");
  if (!fp) return false;
  auto cycle = [&](Cycle& c) {
    int n = 0;
    if (std::fscanf(fp, "%d", &n) != 1 || n < 1) return false;
    c.v.assign(n, 0.0f);
    for (float& x : c.v)
      if (std::fscanf(fp, "%f", &x) != 1) return false;
    return std::fscanf(fp, "%d", &c.period) == 1 && c.period > 0;
  };
  int n = 0;
  bool ok = std::fscanf(fp, "%d", &n) == 1 && n > 0;
  if (ok) p.hue.resize(n);
  for (Cycle& c : p.hue) ok = ok && cycle(c);
  ok = ok && std::fscanf(fp, "%d", &p.hue_period) == 1 && p.hue_period > 0;
  ok = ok && cycle(p.sat);
  ok = ok && std::fscanf(fp, "%d", &n) == 1 && n >= 0;
  if (ok) p.waves.resize(n);
  for (auto& w : p.waves) ok = ok && std::fscanf(fp, "%f %d", &w.first, &w.second) == 2 && w.second > 0;
  std::fclose(fp);
  return ok;
}
std::vector<C3> cache(const Palette& p, int n) {
  constexpr float tau = 2.0 * 3.14159265358979;  // multiwave.cpp:15
  std::vector<C3> out(n);
  for (int i = 0; i < n; i++) {
    const float sat = p.sat.at(i);
    float lum = 0.0f;
    for (auto& w : p.waves) lum += w.first * std::sin(i * tau / w.second);
    lum = 1.0 / (1.0 + std::exp(-lum));
    auto along = [&](const Cycle& c) {
      float tx = (int)c.v.size() * (i % c.period) / (float)c.period;
      int x0 = (int)tx;
      tx -= x0;
      return blend(hsl(c.v[x0], sat, lum), hsl(c.v[(x0 + 1) % c.v.size()], sat, lum), tx);
    };
    float ty = (int)p.hue.size() * (i % p.hue_period) / (float)p.hue_period;
    int y0 = (int)ty;
    ty -= y0;
    out[i] = blend(along(p.hue[y0]), along(p.hue[(y0 + 1) % p.hue.size()]), ty);
  }
  return out;
}
}  // namespace colour

int nmo_palette_cache(const char* path, int n, unsigned char* out) {
  colour::Palette p;
  if (!colour::read_palette(path, p)) return 1;
  auto pal = colour::cache(p, n);
  for (int i = 0; i < n; i++)
    for (int k = 0; k < 3; k++) out[3 * i + k] = pal[i].c[k];
  return 0;
}

// getColor + colorLine (viewer.cpp:89-124) over a sample grid; pal is the
// cached palette as RGB triples (npal >= N).
int nmo_colorize(const int32_t* iters, const float* smooth, int nr, int nc, int N,
                 const unsigned char* pal, int sc, int smooth_flag, unsigned char* out) {
  auto entry = [&](int k) {
    colour::C3 c;
    for (int q = 0; q < 3; q++) c.c[q] = pal[3 * k + q];
    return c;
  };
  for (int r = 0; r < nr / sc; r++)
    for (int c = 0; c < nc / sc; c++) {
      float acc[3] = {0.0f, 0.0f, 0.0f};
      for (int r1 = r * sc; r1 < (r + 1) * sc; r1++)
        for (int c1 = c * sc; c1 < (c + 1) * sc; c1++) {
          const long k = (long)r1 * nc + c1;
          colour::C3 col = {{0, 0, 0}};
          if (iters[k] < N) {
            col = smooth_flag ? colour::blend(entry(iters[k] > 0 ? iters[k] - 1 : 0),
                                              entry(iters[k]), smooth[k])
                              : entry(iters[k]);
          }
          for (int q = 0; q < 3; q++) acc[q] += col.c[q];
        }
      unsigned char* o = out + 3 * ((long)r * (nc / sc) + c);
      for (int q = 0; q < 3; q++)
        o[q] = sc == 1 ? (unsigned char)acc[q] : colour::clip(acc[q] / (float)(sc * sc));
    }
  return 0;
}

// VideoZoom::nextFrame (video.cpp:14-34): `rate` frames between two keyframes.
// ByteImage::scaled restated as bilinear resampling (pixel centres aligned),
// blend as (1 - t) a + t b, both rounded half up (libbyteimage is absent).
int nmo_video_interpolate(const unsigned char* prev, const unsigned char* cur, int kh, int kw,
                          int nr, int nc, int rate, unsigned char* out) {
  auto scaled = [](const unsigned char* src, int sh, int sw, int dh, int dw) {
    std::vector<unsigned char> dst((size_t)dh * dw * 3);
    const float ry = (float)sh / (float)dh, rx = (float)sw / (float)dw;
    for (int y = 0; y < dh; y++)
      for (int x = 0; x < dw; x++) {
        float fy = ((float)y + 0.5f) * ry - 0.5f, fx = ((float)x + 0.5f) * rx - 0.5f;
        fy = std::min(std::max(fy, 0.0f), (float)(sh - 1));
        fx = std::min(std::max(fx, 0.0f), (float)(sw - 1));
        const int y0 = (int)fy, x0 = (int)fx;
        const int y1 = std::min(y0 + 1, sh - 1), x1 = std::min(x0 + 1, sw - 1);
        const float wy = fy - (float)y0, wx = fx - (float)x0;
        for (int k = 0; k < 3; k++) {
          const float a = src[((long)y0 * sw + x0) * 3 + k], b = src[((long)y0 * sw + x1) * 3 + k];
          const float c = src[((long)y1 * sw + x0) * 3 + k], d = src[((long)y1 * sw + x1) * 3 + k];
          const float top = (1.0f - wx) * a + wx * b, bot = (1.0f - wx) * c + wx * d;
          dst[((size_t)y * dw + x) * 3 + k] = colour::clip((1.0f - wy) * top + wy * bot);
        }
      }
    return dst;
  };
  std::vector<unsigned char> canvas((size_t)nr * nc * 3, 0);
  float v = std::pow(1.5, 1.0 / rate), sm = 2.0 / 3.0, lg = 1.0;
  for (int i = 0; i < rate; i++) {
    const float t = (float)i / rate;
    const int sh = (int)(kh * sm), sw = (int)(kw * sm), lh = (int)(kh * lg), lw = (int)(kw * lg);
    const auto small = scaled(cur, kh, kw, sh, sw);
    const auto large = scaled(prev, kh, kw, lh, lw);
    const int lr = (nr - lh) / 2, lc = (nc - lw) / 2, sr = (nr - sh) / 2, sc = (nc - sw) / 2;
    for (int r = 0; r < nr; r++)
      for (int c = 0; c < nc; c++) {
        unsigned char* px = &canvas[((size_t)r * nc + c) * 3];
        if (r - lr >= 0 && r - lr < lh && c - lc >= 0 && c - lc < lw)
          for (int k = 0; k < 3; k++) px[k] = large[((size_t)(r - lr) * lw + (c - lc)) * 3 + k];
        if (r - sr >= 0 && r - sr < sh && c - sc >= 0 && c - sc < sw)
          for (int k = 0; k < 3; k++)
            px[k] = colour::clip((1.0f - t) * px[k] + t * small[((size_t)(r - sr) * sw + (c - sc)) * 3 + k]);
      }
    std::memcpy(out + (size_t)i * nr * nc * 3, canvas.data(), canvas.size());
    sm *= v;
    lg *= v;
  }
  return 0;
}

// Decimal string of the center / step (for carrying views between handles).
int nmo_get_view(nmo_view* h, int which, char* buf, int buflen) {
  View* v = reinterpret_cast<View*>(h);
  mpf_srcptr f = which == 0 ? (mpf_srcptr)*v->cre : which == 1 ? (mpf_srcptr)*v->cim
               : which == 2 ? (mpf_srcptr)*v->sre : (mpf_srcptr)*v->sim;
  mp_exp_t e;
  char* s = mpf_get_str(nullptr, &e, 10, 0, f);
  std::string out;
  if (s[0] == '-') out = std::string("-0.") + (s + 1);
  else if (s[0] == 0) out = "0";
  else out = std::string("0.") + s;
  if (s[0] != 0) out += "e" + std::to_string((long)e);
  free(s);
  if ((int)out.size() + 1 > buflen) return 1;
  std::memcpy(buf, out.c_str(), out.size() + 1);
  return 0;
}

}  // extern "C"
