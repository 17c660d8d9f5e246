// The series front of getIterations (mandelbrot.cpp:144-207) for views whose
// series coefficients or eps leave the FP64 range (widths below ~1e-100, where
// the reference's own get_d conversions overflow to inf and its series test
// turns to NaN).  Every complex value is a pair of FP64 mantissas sharing one
// int exponent, (re + i im) * 2^e.  The arithmetic is the reference's FP64
// arithmetic on the mantissas: a product multiplies mantissas and adds
// exponents, a sum scales the smaller operand by an exact power of two first,
// and a value is renormalised (exactly) only when its mantissa leaves
// [2^-400, 2^400].  So in the FP64 range this computes exactly what the FP64
// front computes; outside it, the same operations without overflow.
#pragma once

#include "pixel_fp64.cuh"

namespace nmg {

#if defined(__CUDA_ARCH__)
NM_HD int ilogb_(double x) { return ilogb(x); }
NM_HD double scalbn_(double x, int n) { return scalbn(x, n); }
#else
inline int ilogb_(double x) { return std::ilogb(x); }
inline double scalbn_(double x, int n) { return std::scalbn(x, n); }
#endif

NM_HD CFE cfe_norm(CFE a) {
  const double m = fmax(fabs(a.re), fabs(a.im));
  if (m == 0.0) return {a.re, a.im, 0};
  const int k = ilogb_(m);
  if (k > 400 || k < -400) return {scalbn_(a.re, -k), scalbn_(a.im, -k), a.e + k};
  return a;
}
NM_HD CFE cfe_mul(CFE a, CFE b) {  // complex.h:29-31 on the mantissas
  return cfe_norm({sub_(mul_(a.re, b.re), mul_(a.im, b.im)),
                   add_(mul_(a.re, b.im), mul_(a.im, b.re)), a.e + b.e});
}
NM_HD CFE cfe_sq(CFE a) {  // complex.h:19-21 on the mantissas
  return cfe_norm({sub_(mul_(a.re, a.re), mul_(a.im, a.im)), mul_(mul_(2.0, a.re), a.im),
                   a.e + a.e});
}
NM_HD CFE cfe_add(CFE a, CFE b) {
  if (a.e >= b.e) {
    const int d = b.e - a.e;
    return cfe_norm({add_(a.re, scalbn_(b.re, d)), add_(a.im, scalbn_(b.im, d)), a.e});
  }
  const int d = a.e - b.e;
  return cfe_norm({add_(scalbn_(a.re, d), b.re), add_(scalbn_(a.im, d), b.im), b.e});
}
// |a|^2 as a real floatexp (the reference's re*re + im*im on the mantissas)
NM_HD RFE cfe_mag2(CFE a) { return {add_(mul_(a.re, a.re), mul_(a.im, a.im)), 2 * a.e}; }
NM_HD double cfe_re(CFE a) { return scalbn_(a.re, a.e); }
NM_HD double cfe_im(CFE a) { return scalbn_(a.im, a.e); }

// x < y for real floatexp values (any sign of mantissa allowed for x, y >= 0).
NM_HD bool rfe_less(RFE x, RFE y) {
  if (!(x.m > 0.0)) return y.m > 0.0 || (x.m < y.m);
  if (!(y.m > 0.0)) return false;
  const int ex = ilogb_(x.m) + x.e, ey = ilogb_(y.m) + y.e;
  if (ex != ey) return ex < ey;
  return scalbn_(x.m, x.e - ex) < scalbn_(y.m, y.e - ey);
}
NM_HD RFE rfe_scale(RFE x, double s) {  // x * s, s near 1
  return {mul_(x.m, s), x.e};
}

// First index i in [lo, hi) with m[i] < t (m non-increasing), or hi.
NM_HD int first_below_fe(const RFE* m, int lo, int hi, RFE t) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (rfe_less(m[mid], t))
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}

// Series term of index i in floatexp, and the reference's instability test.
NM_HD CFE sa_term_fe(const DeviceView& v, int i, CFE eps, CFE eps2, CFE eps3, bool& unstable) {
  const CFE a = cfe_mul(v.sa_a_fe[i], eps);
  const CFE b = cfe_mul(v.sa_b_fe[i], eps2);
  const CFE c = cfe_mul(v.sa_c_fe[i], eps3);
  const RFE bm = cfe_mag2(b), cm = cfe_mag2(c);
  unstable = rfe_less(rfe_scale(bm, v.tol), cm);  // bmag * tol < cmag
  return cfe_add(cfe_add(a, b), c);
}
NM_HD CFE sa_value_fe(const DeviceView& v, int i, CFE eps, CFE eps2, CFE eps3) {
  if (i == 0) return eps;
  bool u;
  return sa_term_fe(v, i, eps, eps2, eps3, u);
}

// As sa_first_unstable, in floatexp: the thresholds T_i = tol|B_i|^2/|C_i|^2
// (prefix minima) against u = |eps3|^2/|eps2|^2.
NM_HD int sa_first_unstable_fe(const DeviceView& v, CFE eps, CFE eps2, CFE eps3) {
  const int n = v.xlen;
  const RFE m2 = cfe_mag2(eps2), m3 = cfe_mag2(eps3);
  if (!(m2.m > 0.0) || !(m3.m > 0.0)) return n;
  const RFE u = {m3.m / m2.m, m3.e - m2.e};
  const RFE hi_u = rfe_scale(u, 1.0 + 0x1p-40), lo_u = rfe_scale(u, 1.0 - 0x1p-40);
  const int i_fp = first_below_fe(v.sa_min_fe, 1, n, hi_u);
  if (i_fp >= n) return n;
  const int i_c = first_below_fe(v.sa_min_fe, i_fp, n, lo_u);
  for (int i = i_fp; i < i_c; i++) {
    bool un;
    sa_term_fe(v, i, eps, eps2, eps3, un);
    if (un) return i;
  }
  return i_c;
}

// series_front for floatexp views; the result's eps and d[found] carry
// exponents (SeriesFront::eps_e, ::d_e).
NM_HD bool series_front_fe(const DeviceView& v, int r, int c, SeriesFront& f, EscapeValue& out,
                           double& sm, bool& undecided) {
  undecided = false;
  if (v.cardioid_mode == CARDIOID_PER_SAMPLE &&
      in_cardioid_dd(v.coord_re[c], v.coord_im[r], undecided)) {
    out = {v.N, 0.0f};
    sm = 0.0;
    return true;
  }
  const RFE er = v.eps_re_fe[c], ei = v.eps_im_fe[r];
  // the shared exponent is the larger of the nonzero components' (a zero
  // component -- the center row or column -- carries no exponent)
  const int e = er.m == 0.0 ? ei.e : ei.m == 0.0 ? er.e : (er.e > ei.e ? er.e : ei.e);
  const CFE eps = cfe_norm({scalbn_(er.m, er.e - e), scalbn_(ei.m, ei.e - e), e});
  const CFE eps2 = cfe_sq(eps);
  const CFE eps3 = cfe_mul(eps, eps2);
  const int fire = sa_first_unstable_fe(v, eps, eps2, eps3);
  int dsize = v.xlen;
  if (fire < v.xlen) dsize = fire - 3 < 1 ? 1 : fire - 3;
  int found = dsize - 1;
  CFE d = sa_value_fe(v, found, eps, eps2, eps3);
  double yr = trunc_sum(v.xhi[found].x, v.xlo[found].x, cfe_re(d));
  double yi = trunc_sum(v.xhi[found].y, v.xlo[found].y, cfe_im(d));
  if (add_(mul_(yr, yr), mul_(yi, yi)) > v.bailout2) {
    int low = 0, high = dsize - 1, mid = dsize / 2;
    while (low <= high) {
      const CFE dm = sa_value_fe(v, mid, eps, eps2, eps3);
      const double mr = trunc_sum(v.xhi[mid].x, v.xlo[mid].x, cfe_re(dm));
      const double mi = trunc_sum(v.xhi[mid].y, v.xlo[mid].y, cfe_im(dm));
      if (!(add_(mul_(mr, mr), mul_(mi, mi)) > v.bailout2))
        low = mid + 1;
      else {
        high = mid - 1;
        found = mid;
      }
      mid = (low + high) / 2;
    }
    d = sa_value_fe(v, found, eps, eps2, eps3);
    yr = trunc_sum(v.xhi[found].x, v.xlo[found].x, cfe_re(d));
    yi = trunc_sum(v.xhi[found].y, v.xlo[found].y, cfe_im(d));
    sm = smoothing_of(add_(mul_(yr, yr), mul_(yi, yi)), v.log_bailout);
    out = {found, (float)sm};
    return true;
  }
  f.eps = {eps.re, eps.im};
  f.eps_e = eps.e;
  f.dfound = {d.re, d.im};
  f.d_e = d.e;
  f.dsize = dsize;
  return false;
}

// The series front a view calls for.
NM_HD bool series_front_any(const DeviceView& v, int r, int c, SeriesFront& f, EscapeValue& out,
                            double& sm, bool& undecided) {
  if (v.sa_fe) return series_front_fe(v, r, c, f, out, sm, undecided);
  f.eps_e = 0;
  f.d_e = 0;
  return series_front(v, r, c, f, out, sm, undecided);
}

}  // namespace nmg
