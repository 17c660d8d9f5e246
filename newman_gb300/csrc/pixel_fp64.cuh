// Per-sample FP64 arithmetic of the reference's per-pixel path.
//
// Every multiply and add of the reference's `double` code is written with a
// round-to-nearest intrinsic (never contracted into an FMA), in the grouping
// of complex.h:19-31 and mandelbrot.cpp, so that the results are the
// reference's bit for bit.  FMAs appear only inside the double-double helpers
// used for the cardioid test and the truncating sum X[k] + d.
#pragma once

#include <cmath>
#include <cstring>

#include "view_device.cuh"

namespace nmg {

#if defined(__CUDA_ARCH__)
NM_HD double mul_(double a, double b) { return __dmul_rn(a, b); }
NM_HD double add_(double a, double b) { return __dadd_rn(a, b); }
NM_HD double sub_(double a, double b) { return __dsub_rn(a, b); }
NM_HD double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
NM_HD double add_rz_(double a, double b) { return __dadd_rz(a, b); }
NM_HD double log_(double x) { return log(x); }
NM_HD double log2_(double x) { return log2(x); }
#else
inline double mul_(double a, double b) { return a * b; }
inline double add_(double a, double b) { return a + b; }
inline double sub_(double a, double b) { return a - b; }
inline double fma_(double a, double b, double c) { return std::fma(a, b, c); }
inline double add_rz_(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double err = (a - (s - bb)) + (b - bb);
  if (err != 0.0 && ((err < 0.0) != (s < 0.0))) s = std::nextafter(s, 0.0);
  return s;
}
inline double log_(double x) { return std::log(x); }
inline double log2_(double x) { return std::log2(x); }
#endif

// ---- complex.h in the reference's order -----------------------------------
struct C64 {
  double re, im;
};
NM_HD C64 c_sq(C64 a) {  // complex.h:19-21
  return {sub_(mul_(a.re, a.re), mul_(a.im, a.im)), mul_(mul_(2.0, a.re), a.im)};
}
NM_HD C64 c_add(C64 a, C64 b) { return {add_(a.re, b.re), add_(a.im, b.im)}; }
NM_HD C64 c_mul(C64 a, C64 b) {  // complex.h:29-31
  return {sub_(mul_(a.re, b.re), mul_(a.im, b.im)), add_(mul_(a.re, b.im), mul_(a.im, b.re))};
}
NM_HD double c_mag2(C64 a) { return add_(mul_(a.re, a.re), mul_(a.im, a.im)); }

// mandelbrot.cpp:133-136
NM_HD double smoothing_of(double r2, double log_bailout) {
  return 1.0 - log2_(0.5 * log_(r2) / log_bailout);
}

// ---- double-double helpers -------------------------------------------------
struct DD {
  double hi, lo;
};
NM_HD DD two_sum(double a, double b) {
  double s = add_(a, b);
  double bb = sub_(s, a);
  double err = add_(sub_(a, sub_(s, bb)), sub_(b, bb));
  return {s, err};
}
NM_HD DD quick_two_sum(double a, double b) {
  double s = add_(a, b);
  return {s, sub_(b, sub_(s, a))};
}
NM_HD DD dd_add(DD a, DD b) {
  DD s = two_sum(a.hi, b.hi);
  DD t = two_sum(a.lo, b.lo);
  s.lo = add_(s.lo, t.hi);
  s = quick_two_sum(s.hi, s.lo);
  s.lo = add_(s.lo, t.lo);
  return quick_two_sum(s.hi, s.lo);
}
NM_HD DD dd_mul(DD a, DD b) {
  double p = mul_(a.hi, b.hi);
  double e = fma_(a.hi, b.hi, -p);
  e = add_(e, add_(mul_(a.hi, b.lo), mul_(a.lo, b.hi)));
  return quick_two_sum(p, e);
}
NM_HD double dd_abs_hi(DD a) { return a.hi < 0 ? -a.hi : a.hi; }

// mandelbrot.cpp:63-71 on the sample's coordinates held as hi + lo (106
// bits).  The reference evaluates in >= 128-bit mpf; the two can disagree
// only when a polynomial lies within ~2^-100 of zero, which `undecided`
// reports.
NM_HD bool in_cardioid_dd(Dbl2 px, Dbl2 py, bool& undecided) {
  const DD x{px.x, px.y}, y{py.x, py.y};
  const DD fourth{0.25, 0.0};
  DD xmf = dd_add(x, DD{-0.25, 0.0});
  DD y2 = dd_mul(y, y);
  DD q = dd_add(dd_mul(xmf, xmf), y2);
  DD lhs = dd_mul(q, dd_add(q, xmf));
  DD rhs = dd_mul(fourth, y2);
  DD g = dd_add(lhs, DD{-rhs.hi, -rhs.lo});
  const double tiny = 0x1p-96;
  double bound = tiny * (dd_abs_hi(lhs) + dd_abs_hi(rhs)) + 1e-300;
  undecided = false;
  if (dd_abs_hi(g) <= bound) undecided = true;
  if (g.hi < 0.0) return true;
  DD q2 = dd_add(x, DD{1.0, 0.0});
  DD lhs2 = dd_add(dd_mul(q2, q2), y2);
  DD g2 = dd_add(lhs2, DD{-0.0625, 0.0});
  if (dd_abs_hi(g2) <= tiny * (dd_abs_hi(lhs2) + 0.0625)) undecided = true;
  return g2.hi < 0.0;
}

// get_d(X[k] + d): the arbitrary-precision sum of mandelbrot.cpp:184-185,
// truncated toward zero like mpf_get_d, from X[k] = hi + lo.
NM_HD double trunc_sum(double hi, double lo, double d) {
  DD s = two_sum(hi, d);
  return add_rz_(s.hi, add_(s.lo, lo));
}

// ---- the reference's double path (mandelbrot.cpp:231-254) ------------------
//
// The loop keeps zr^2 and zi^2 of the bailout test for the next step's
// squaring (the same products of the same operands), forms 2 zr zi as
// 2 * round(zr zi) by an exponent increment where that equals the reference's
// round((2 zr) zi), and compares |Z|^2 with the bailout on its bit pattern
// (non-negative doubles order like their bits): 7 FP64 operations a step
// instead of 11, with the reference's results bit for bit.
//
// Exact cycle detection (Brent): the loop state (zr, zi) is saved at every
// power-of-two step; when the state equals the saved one bit for bit, the
// deterministic double loop repeats forever without escaping, so the sample's
// result is N, exactly what running to N gives.
struct HwState {
  double z0r, z0i, zr, zi;
  double sr, si;      // zr * zr, zi * zi of the current state
  double cr, ci;      // state saved for cycle detection
  int32_t it;
  int32_t save_at;    // next step at which the state is saved
};

// 2 (a b) rounded as the reference's (2 a) b: equal when round(a b) is a
// normal double at least 2^-1021 (rounding scales with powers of two there).
NM_HD double twice_product(double a, double b) {
  const double p = mul_(a, b);
#if defined(__CUDA_ARCH__)
  const int hi = __double2hiint(p);
  const int e = (hi >> 20) & 0x7ff;
  if (e >= 2 && e <= 0x7fd) return __hiloint2double(hi + 0x00100000, __double2loint(p));
#else
  const int e = std::ilogb(p);
  if (p != 0.0 && e >= -1021 && e <= 1022) return p + p;
#endif
  return mul_(mul_(2.0, a), b);
}

NM_HD bool same_bits(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(a) == __double_as_longlong(b);
#else
  long long x, y;
  std::memcpy(&x, &a, 8);
  std::memcpy(&y, &b, 8);
  return x == y;
#endif
}

// 2 x exactly (the reference's mul(2.0, x)): an exponent increment for a
// normal x whose double stays finite, else the multiply.
NM_HD double twice_(double x) {
#if defined(__CUDA_ARCH__)
  const int hi = __double2hiint(x);
  const int e = (hi >> 20) & 0x7ff;
  if (e >= 1 && e <= 0x7fd) return __hiloint2double(hi + 0x00100000, __double2loint(x));
#endif
  return mul_(2.0, x);
}

// Biased exponent field of x (0 for zero and subnormals).
NM_HD int exp_field(double x) {
#if defined(__CUDA_ARCH__)
  return (__double2hiint(x) >> 20) & 0x7ff;
#else
  long long b;
  std::memcpy(&b, &x, 8);
  return (int)((b >> 52) & 0x7ff);
#endif
}

// True when |(yr, yi)| exceeds |(dr, di)| by so much that the FP64 values of
// yr^2 + yi^2 and dr^2 + di^2 compare greater, whatever their rounding: the
// larger component of Y is at least 4 times the larger of delta's (|Y|^2 >=
// 16 max^2 > 2 |delta|^2, far beyond 2^-52).
NM_HD bool clearly_larger(double yr, double yi, double dr, double di) {
  const int ay = exp_field(yr), by = exp_field(yi), ad = exp_field(dr), bd = exp_field(di);
  const int ey = ay > by ? ay : by, ed = ad > bd ? ad : bd;
  return ey >= ed + 2 && ey > 0;
}

// r2 > bailout2 for r2 >= 0 and bailout2 > 0, on the bit patterns.
NM_HD bool above_bits(double r2, double bailout2) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(r2) > __double_as_longlong(bailout2);
#else
  return r2 > bailout2;
#endif
}

// |yr|, |yi| < 2^8 (biased exponents below 1031): yr^2 + yi^2 then rounds to
// at most 2^17, below the bailout radius squared (always 2^20 here), so the
// bailout test is decided without forming it.
NM_HD bool inside_bailout(double yr, double yi) {
  return exp_field(yr) < 1031 && exp_field(yi) < 1031;
}

// Both tests decided before Y = Z + delta is formed: every component of Z and
// of delta below 2^7 (so |Y|'s components stay below 2^8: no bailout), and Z's
// larger component at least 8 times delta's (so Y's larger component is at
// least 4 times delta's: clearly_larger, no rebase).  Not at the orbit's end.
NM_HD bool no_event_before_y(Dbl2 zn, double dr, double di) {
  const int zr = exp_field(zn.x), zi = exp_field(zn.y), ar = exp_field(dr), ai = exp_field(di);
  const int ez = zr > zi ? zr : zi, ed = ar > ai ? ar : ai;
  return ez < 1030 && ed < 1030 && ez >= ed + 3;
}

// |x| as a float from the double's high word: its exponent rebiased and the
// top 20 of its 52 mantissa bits, so within 2^-20 below |x|.  For biased
// exponents in [963, 1083] (|x| in [2^-60, 2^61)), where the float and the
// squares below stay normal.
NM_HD float abs_hi_float(double x) {
#if defined(__CUDA_ARCH__)
  const unsigned hi = (unsigned)__double2hiint(x) & 0x7fffffffu;
  return __uint_as_float((hi - ((1023u - 127u) << 20)) << 3);
#else
  unsigned long long b;
  std::memcpy(&b, &x, 8);
  const unsigned hi = (unsigned)(b >> 32) & 0x7fffffffu;
  const unsigned f = (hi - ((1023u - 127u) << 20)) << 3;
  float r;
  std::memcpy(&r, &f, 4);
  return r;
#endif
}

// The rebase test (FP64 d2 > r2) decided on FP32 estimates where they lie far
// apart, else -1.  Each estimate is within 2^-18 of its exact value (operands
// within 2^-20 below, two FP32 roundings) and each FP64 sum within 2^-51, so a
// ratio beyond 1 + 2^-15 between the estimates orders the FP64 values too.
NM_HD int rebase_by_estimate(double yr, double yi, double dr, double di) {
  const int a = exp_field(yr), b = exp_field(yi), c = exp_field(dr), d = exp_field(di);
  const int lo1 = a < b ? a : b, lo2 = c < d ? c : d, hi1 = a > b ? a : b, hi2 = c > d ? c : d;
  if ((lo1 < lo2 ? lo1 : lo2) < 963 || (hi1 > hi2 ? hi1 : hi2) > 1083) return -1;
  const float yrf = abs_hi_float(yr), yif = abs_hi_float(yi);
  const float drf = abs_hi_float(dr), dif = abs_hi_float(di);
  const float r2f = fmaf(yrf, yrf, yif * yif), d2f = fmaf(drf, drf, dif * dif);
  if (d2f > r2f * (1.0f + 0x1p-15f)) return 1;
  if (r2f > d2f * (1.0f + 0x1p-15f)) return 0;
  return -1;
}

// The step's bailout and rebase tests in delta_steps' order and rounding, with
// the FP64 operations of r2 = yr^2 + yi^2 and d2 = dr^2 + di^2 spent only where
// the exponents leave the outcome open: 0 go on, 1 rebase, 2 escape (r2 set).
NM_HD int bailout_and_rebase(double yr, double yi, double dr, double di, bool last,
                             double bailout2, double& r2) {
  const bool inside = inside_bailout(yr, yi);
  if (!inside) {
    r2 = add_(mul_(yr, yr), mul_(yi, yi));
    if (above_bits(r2, bailout2)) return 2;
  }
  if (last) return 1;
  if (clearly_larger(yr, yi, dr, di)) return 0;
  // delta clearly larger (and of at least 2^-500, so that d2 is no underflow)
  if (clearly_larger(dr, di, yr, yi) && (exp_field(dr) >= 523 || exp_field(di) >= 523)) return 1;
  const int q = rebase_by_estimate(yr, yi, dr, di);
  if (q >= 0) return q;
  if (inside) r2 = add_(mul_(yr, yr), mul_(yi, yi));
  return above_bits(add_(mul_(dr, dr), mul_(di, di)), r2) ? 1 : 0;
}


// The double loop's start at Z0 = descend(pt) (mandelbrot.cpp:234, 242).
NM_HD void hw_start(Dbl2 px, Dbl2 py, HwState& st) {
  st.z0r = px.x;
  st.z0i = py.x;
  st.zr = px.x;
  st.zi = py.x;
  st.sr = mul_(px.x, px.x);
  st.si = mul_(py.x, py.x);
  st.cr = px.x;
  st.ci = py.x;
  st.it = 0;
  st.save_at = 1;
}

// Returns true when the sample is already decided (cardioid).
NM_HD bool hw_init(const DeviceView& v, int r, int c, HwState& st, EscapeValue& out, double& sm,
                   bool& undecided) {
  const Dbl2 px = v.coord_re[c], py = v.coord_im[r];
  undecided = false;
  if (v.cardioid_mode == CARDIOID_PER_SAMPLE && in_cardioid_dd(px, py, undecided)) {
    out = {v.N, 0.0f};
    sm = 0.0;
    return true;
  }
  hw_start(px, py, st);
  return false;
}

// Up to `steps` iterations of Z = sq(Z) + Z0; true when the sample is done.
NM_HD bool hw_steps(const DeviceView& v, HwState& st, int steps, EscapeValue& out, double& sm) {
  double zr = st.zr, zi = st.zi, sr = st.sr, si = st.si, cr = st.cr, ci = st.ci;
  int it = st.it, save_at = st.save_at;
  const int stop = (v.N - it < steps) ? v.N : it + steps;
  bool cycle = false;
  for (; it < stop; it++) {
    const double nre = add_(sub_(sr, si), st.z0r);
    const double nim = add_(twice_product(zr, zi), st.z0i);
    zr = nre;
    zi = nim;
    sr = mul_(zr, zr);
    si = mul_(zi, zi);
    // both squares below 2^19 (biased exponents under 1042): their sum rounds
    // to at most 2^20, which does not bail out (bailout2 = 2^20); the sum is
    // formed only where it can
    if (exp_field(sr) >= 1042 || exp_field(si) >= 1042) {
      const double r2 = add_(sr, si);
      if (above_bits(r2, v.bailout2)) {
        sm = smoothing_of(r2, v.log_bailout);
        out = {it, (float)sm};
        return true;
      }
    }
    if (same_bits(zr, cr) && same_bits(zi, ci)) {
      cycle = true;
      break;
    }
    if (it == save_at) {
      cr = zr;
      ci = zi;
      save_at = save_at < (1 << 29) ? 2 * save_at : save_at;
    }
  }
  st.zr = zr;
  st.zi = zi;
  st.sr = sr;
  st.si = si;
  st.cr = cr;
  st.ci = ci;
  st.save_at = save_at;
  st.it = cycle ? it + 1 : it;  // steps actually run
  if (cycle || it >= v.N) {
    out = {v.N, 0.0f};
    sm = 0.0;
    return true;
  }
  return false;
}

// ---- the series front of getIterations (mandelbrot.cpp:144-207) -------------
struct SeriesFront {
  C64 eps;       // Y0 - X[0]  (times 2^eps_e)
  C64 dfound;    // d[found]   (times 2^d_e)
  int32_t dsize; // d.size() after the skip
  int32_t eps_e, d_e;  // exponents of the floatexp front (0 in the FP64 range)
};

NM_HD C64 sa_term(const DeviceView& v, int i, C64 eps, C64 eps2, C64 eps3, bool& unstable) {
  const Dbl2 A = v.sa_a[i], B = v.sa_b[i], Cc = v.sa_c[i];
  C64 a = c_mul(C64{A.x, A.y}, eps);
  C64 b = c_mul(C64{B.x, B.y}, eps2);
  C64 c = c_mul(C64{Cc.x, Cc.y}, eps3);
  double bmag = add_(mul_(b.re, b.re), mul_(b.im, b.im));
  double cmag = add_(mul_(c.re, c.re), mul_(c.im, c.im));
  unstable = mul_(bmag, v.tol) < cmag;  // mandelbrot.cpp:138-142
  return c_add(c_add(a, b), c);
}

NM_HD C64 sa_value(const DeviceView& v, int i, C64 eps, C64 eps2, C64 eps3) {
  if (i == 0) return eps;
  bool u;
  return sa_term(v, i, eps, eps2, eps3, u);
}

// First index i in [lo, hi) with sa_min[i] < t (sa_min is non-increasing), or hi.
NM_HD int first_below(const double* m, int lo, int hi, double t) {
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (m[mid] < t)
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}

// The index at which the reference's loop (mandelbrot.cpp:165-181) first sees
// an unstable term, or xlen when none.  The test tol|B_i eps2|^2 < |C_i eps3|^2
// is, in exact arithmetic, T_i < u with T_i = tol|B_i|^2/|C_i|^2 and
// u = |eps3|^2/|eps2|^2; the FP64 evaluation differs from exact by far less
// than 2^-40 relative.  So the prefix minimum of T_i locates the first firing
// term by binary search, and only terms whose ratio lies within 2^-40 of 1
// are re-evaluated exactly as the reference does.
NM_HD int sa_first_unstable(const DeviceView& v, C64 eps, C64 eps2, C64 eps3) {
  const int n = v.xlen;
  if (v.sa_scan) {
    for (int i = 1; i < n; i++) {
      bool u;
      sa_term(v, i, eps, eps2, eps3, u);
      if (u) return i;
    }
    return n;
  }
  const double m2 = c_mag2(eps2), m3 = c_mag2(eps3);
  if (!(m2 > 0.0) || !(m3 > 0.0)) return n;  // b = c = 0 or c = 0: never unstable
  const double u = m3 / m2;
  const double hi_u = u * (1.0 + 0x1p-40), lo_u = u * (1.0 - 0x1p-40);
  const int i_fp = first_below(v.sa_min, 1, n, hi_u);
  if (i_fp >= n) return n;
  const int i_c = first_below(v.sa_min, i_fp, n, lo_u);
  for (int i = i_fp; i < i_c; i++) {
    bool un;
    sa_term(v, i, eps, eps2, eps3, un);
    if (un) return i;
  }
  return i_c;  // fires for certain, or n
}

// Returns true when the sample is finished in the front half (cardioid, or
// escaped before the skip point -- the binary search of :186-207).
NM_HD bool series_front(const DeviceView& v, int r, int c, SeriesFront& f, EscapeValue& out,
                        double& sm, bool& undecided) {
  undecided = false;
  if (v.cardioid_mode == CARDIOID_PER_SAMPLE &&
      in_cardioid_dd(v.coord_re[c], v.coord_im[r], undecided)) {
    out = {v.N, 0.0f};
    sm = 0.0;
    return true;
  }
  const C64 eps{v.eps_re[c], v.eps_im[r]};
  const C64 eps2 = c_sq(eps);
  const C64 eps3 = c_mul(eps, eps2);
  const int fire = sa_first_unstable(v, eps, eps2, eps3);
  int dsize = v.xlen;
  if (fire < v.xlen) dsize = fire - 3 < 1 ? 1 : fire - 3;
  int found = dsize - 1;
  C64 d = sa_value(v, found, eps, eps2, eps3);
  double yr = trunc_sum(v.xhi[found].x, v.xlo[found].x, d.re);
  double yi = trunc_sum(v.xhi[found].y, v.xlo[found].y, d.im);
  double r2 = add_(mul_(yr, yr), mul_(yi, yi));
  if (r2 > v.bailout2) {
    int low = 0, high = dsize - 1, mid = dsize / 2;
    while (low <= high) {
      C64 dm = sa_value(v, mid, eps, eps2, eps3);
      double mr = trunc_sum(v.xhi[mid].x, v.xlo[mid].x, dm.re);
      double mi = trunc_sum(v.xhi[mid].y, v.xlo[mid].y, dm.im);
      if (!(add_(mul_(mr, mr), mul_(mi, mi)) > v.bailout2))
        low = mid + 1;
      else {
        high = mid - 1;
        found = mid;
      }
      mid = (low + high) / 2;
    }
    d = sa_value(v, found, eps, eps2, eps3);
    yr = trunc_sum(v.xhi[found].x, v.xlo[found].x, d.re);
    yi = trunc_sum(v.xhi[found].y, v.xlo[found].y, d.im);
    sm = smoothing_of(add_(mul_(yr, yr), mul_(yi, yi)), v.log_bailout);
    out = {found, (float)sm};
    return true;
  }
  f.eps = eps;
  f.dfound = d;
  f.dsize = dsize;
  f.eps_e = 0;
  f.d_e = 0;
  return false;
}

// ---- plain FP64 perturbation continuation ---------------------------------
// The pixel is Y = Z[j] + delta against the FP64 reference orbit Z (Z[0] = 0,
// Z[k+1] = X[k]); one step is
//     t = 2 Z[j] + delta;  delta = t * delta + eps;  j += 1;  Y = Z[j] + delta
// and the pixel rebases to Z[0] (delta = Y, j = 0) when |Y| < |delta| or the
// orbit is exhausted.  `i` counts like getIterations' continuation (:212).
// The doubling is an exponent increment, the comparisons work on bit
// patterns, and |delta|^2 is formed only when |Y| is not clearly larger: 13
// FP64 operations a step instead of 20, with the same results.
struct DeltaState {
  double dr, di, er, ei;  // er, ei: eps as the plain step adds it
  int32_t j, i;
  // eps exactly, xr 2^xre + i xi 2^xie (floatexp views, where the plain step
  // adds 0 for a component below the double range: eps_tiny)
  double xr, xi;
  int32_t xre, xie, eps_tiny;
};

NM_HD double scalbn_d(double x, int n) {
#if defined(__CUDA_ARCH__)
  return n == 0 ? x : scalbn(x, n);
#else
  return n == 0 ? x : std::scalbn(x, n);
#endif
}

NM_HD void delta_start(const SeriesFront& f, DeltaState& st) {
  st.dr = scalbn_d(f.dfound.re, f.d_e);
  st.di = scalbn_d(f.dfound.im, f.d_e);
  st.er = scalbn_d(f.eps.re, f.eps_e);
  st.ei = scalbn_d(f.eps.im, f.eps_e);
  st.j = f.dsize;  // found + 1
  st.i = f.dsize;
  st.xr = st.er;
  st.xi = st.ei;
  st.xre = st.xie = 0;
  st.eps_tiny = 0;
}

template <bool kStaged = false>
NM_HD bool delta_steps(const DeviceView& v, DeltaState& st, int steps, EscapeValue& out,
                       double& sm) {
  double dr = st.dr, di = st.di;
  int j = st.j, i = st.i;
  const int zlast = v.zlen - 1;
  const int stop = (v.N - i < steps) ? v.N : i + steps;
  Dbl2 z = orbit_z<kStaged>(v, j);
  for (; i < stop; i++) {
    // the next orbit element, loaded before the step's arithmetic
    const Dbl2 zn = orbit_z<kStaged>(v, j < zlast ? j + 1 : zlast);
    double tr = add_(twice_(z.x), dr);
    double ti = add_(twice_(z.y), di);
    double nre = add_(sub_(mul_(tr, dr), mul_(ti, di)), st.er);
    double nim = add_(add_(mul_(tr, di), mul_(ti, dr)), st.ei);
    dr = nre;
    di = nim;
    j++;
    z = zn;
    // the bailout test r2 > 2^20, then the rebase test r2 < d2 (or the
    // orbit's end), with Y and the FP64 sums formed only where exponents do
    // not decide
    double yr = 0.0, yi = 0.0, r2 = 0.0;
    int event = 0;
    if (j == zlast || !no_event_before_y(zn, dr, di)) {
      yr = add_(zn.x, dr);
      yi = add_(zn.y, di);
      event = bailout_and_rebase(yr, yi, dr, di, j == zlast, v.bailout2, r2);
    }
    if (event == 2) {
      sm = smoothing_of(r2, v.log_bailout);
      out = {i, (float)sm};
      return true;
    }
    if (event == 1) {
      dr = yr;
      di = yi;
      j = 0;
      z = orbit_z<kStaged>(v, 0);
    }
  }
  st.dr = dr;
  st.di = di;
  st.j = j;
  st.i = i;
  if (i >= v.N) {
    out = {v.N, 0.0f};
    sm = 0.0;
    return true;
  }
  return false;
}

}  // namespace nmg
