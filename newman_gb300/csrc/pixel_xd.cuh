// The plain FP64 perturbation continuation (pixel_fp64.cuh: delta_steps) in
// FP64 with an unbounded exponent (xd64.cuh), for views whose series front is
// floatexp: there the pixel offsets eps, and the deltas right after the
// series skip, lie below the double range (widths under ~1e-300).  The
// operations, their order and their rounding are delta_steps' own; on values
// inside the double range the results are the plain path's bit for bit.
#pragma once

#include "pixel_fp64.cuh"
#include "xd64.cuh"

namespace nmg {

struct DeltaXDState {
  XD dr, di, er, ei;
  int32_t j, i;
};

NM_HD void delta_xd_start(const SeriesFront& f, DeltaXDState& st) {
  st.dr = xd_of(f.dfound.re, f.d_e);
  st.di = xd_of(f.dfound.im, f.d_e);
  st.er = xd_of(f.eps.re, f.eps_e);
  st.ei = xd_of(f.eps.im, f.eps_e);
  st.j = f.dsize;
  st.i = f.dsize;
}

template <bool kStaged = false>
NM_HD bool delta_xd_steps(const DeviceView& v, DeltaXDState& st, int steps, EscapeValue& out,
                          double& sm) {
  XD dr = st.dr, di = st.di;
  int j = st.j, i = st.i;
  const int zlast = v.zlen - 1;
  const int stop = (v.N - i < steps) ? v.N : i + steps;
  const XD bail2 = xd_of(v.bailout2);
  Dbl2 z = orbit_z<kStaged>(v, j);
  for (; i < stop; i++) {
    const Dbl2 zn = orbit_z<kStaged>(v, j < zlast ? j + 1 : zlast);  // loaded before the step's arithmetic
    const XD tr = xd_add(xd_twice(xd_of(z.x)), dr);
    const XD ti = xd_add(xd_twice(xd_of(z.y)), di);
    const XD nre = xd_add(xd_sub(xd_mul(tr, dr), xd_mul(ti, di)), st.er);
    const XD nim = xd_add(xd_add(xd_mul(tr, di), xd_mul(ti, dr)), st.ei);
    dr = nre;
    di = nim;
    j++;
    z = zn;
    const XD yr = xd_add(xd_of(zn.x), dr), yi = xd_add(xd_of(zn.y), di);
    // components of Y below 2^8: r2 < 2^17 does not bail out (bail2 = 2^20);
    // r2 is formed only where a test needs it (delta_steps' bailout_and_rebase)
    const int32_t ey = yr.e > yi.e ? yr.e : yi.e, ed = dr.e > di.e ? dr.e : di.e;
    const bool inside = ey < 8;
    XD r2 = XD{0.0, kXdZeroExp};
    if (!inside) {
      r2 = xd_add(xd_mul(yr, yr), xd_mul(yi, yi));
      if (xd_gt(r2, bail2)) {
        sm = smoothing_of(xd_to_double(r2), v.log_bailout);
        out = {i, (float)sm};
        return true;
      }
    }
    // the rebase test r2 < d2, decided by exponents where one of Y and delta
    // is at least 4 times the other (|Y|^2 > 2 |delta|^2 or the reverse)
    bool rebase = j == zlast;
    if (!rebase && !(ey >= ed + 2 && (yr.m != 0.0 || yi.m != 0.0))) {
      if (ed >= ey + 2 && (dr.m != 0.0 || di.m != 0.0)) {
        rebase = true;
      } else {
        if (inside) r2 = xd_add(xd_mul(yr, yr), xd_mul(yi, yi));
        rebase = xd_gt(xd_add(xd_mul(dr, dr), xd_mul(di, di)), r2);
      }
    }
    if (rebase) {
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

// ---- plain doubles while nothing comes near the underflow range ------------
//
// On a floatexp view most samples never bring a value of the delta step near
// 2^-1022: then the plain double operations round exactly as the unbounded-
// exponent ones (a double operation rounds like unbounded arithmetic whenever
// its result is normal).  delta_guarded_steps runs the plain step and checks
// its operands and results; a step that has a nonzero value below 2^-400
// (where a product could underflow) is not taken -- the state before it,
// exact in both forms, moves to DeltaXDState and the step runs there.

// Nonzero and below 2^-400 (biased exponent field under 623).
NM_HD bool near_underflow(double x) {
  const int64_t b = xd_bits_(x);
  return ((b >> 52) & 0x7ff) < 623 && (b & 0x7fffffffffffffffll) != 0;
}

// An eps component m 2^e for the plain step: the double itself when it is
// zero or normal (exactly), else 0 with `tiny` set when it lies below the
// double range -- it is then below half an ulp of every sum it is added to
// while those sums are nonzero and at least 2^-400, which the guarded steps
// check.  False beyond the double range.
NM_HD bool plain_eps(double m, int32_t e, double& out, int32_t& tiny) {
  const XD x = xd_of(m, e);
  out = 0.0;
  if (x.m == 0.0) return true;
  if (x.e < -1022) {
    tiny = 1;
    return true;
  }
  if (x.e > 1000) return false;
  out = xd_to_double(x);  // normal: exact
  return true;
}

// eps and d[found] of an FE front as plain doubles, when delta is exactly
// representable with room to spare (zero, or a normal double of at least
// 2^-400) and eps by plain_eps.
NM_HD bool delta_plain_start(const SeriesFront& f, DeltaState& st) {
  const double dr = scalbn_d(f.dfound.re, f.d_e), di = scalbn_d(f.dfound.im, f.d_e);
  auto normal_or_zero = [](double x) {
    const int e = exp_field(x);
    return x == 0.0 || (e >= 1 && e <= 2045);
  };
  if (near_underflow(dr) || near_underflow(di) || !normal_or_zero(dr) || !normal_or_zero(di))
    return false;
  // the scalbn results are exact here: the FE mantissas carry 53 bits
  if (scalbn_d(dr, -f.d_e) != f.dfound.re || scalbn_d(di, -f.d_e) != f.dfound.im) return false;
  double er, ei;
  int32_t tiny = 0;
  if (!plain_eps(f.eps.re, f.eps_e, er, tiny) || !plain_eps(f.eps.im, f.eps_e, ei, tiny))
    return false;
  st.dr = dr;
  st.di = di;
  st.er = er;
  st.ei = ei;
  st.j = f.dsize;
  st.i = f.dsize;
  st.xr = f.eps.re;
  st.xi = f.eps.im;
  st.xre = st.xie = f.eps_e;
  st.eps_tiny = tiny;
  return true;
}

// delta_steps with the guard; `handover` is set when a step was left to the
// unbounded-exponent form (st is the exact state before it).
template <bool kStaged = false>
NM_HD bool delta_guarded_steps(const DeviceView& v, DeltaState& st, int steps, EscapeValue& out,
                               double& sm, bool& handover) {
  double dr = st.dr, di = st.di;
  int j = st.j, i = st.i;
  const int zlast = v.zlen - 1;
  const int stop = (v.N - i < steps) ? v.N : i + steps;
  const bool eps_tiny = st.eps_tiny != 0;
  handover = false;
  Dbl2 z = orbit_z<kStaged>(v, j);
  for (; i < stop; i++) {
    const Dbl2 zn = orbit_z<kStaged>(v, j < zlast ? j + 1 : zlast);  // loaded before the step's arithmetic
    const double tr = add_(twice_(z.x), dr);
    const double ti = add_(twice_(z.y), di);
    const double nre = add_(sub_(mul_(tr, dr), mul_(ti, di)), st.er);
    const double nim = add_(add_(mul_(tr, di), mul_(ti, dr)), st.ei);
    // Y = Z + delta only where the tests need it (delta_steps); a Y that is
    // not formed feeds nothing, so only the formed values are guarded
    const bool need_y = j + 1 == zlast || !no_event_before_y(zn, nre, nim);
    double yr = 0.0, yi = 0.0;
    if (need_y) {
      yr = add_(zn.x, nre);
      yi = add_(zn.y, nim);
    }
    // (with eps below the double range its components were not added: exact
    // unless a sum came out 0)
    if (near_underflow(tr) || near_underflow(ti) || near_underflow(nre) || near_underflow(nim) ||
        (need_y && (near_underflow(yr) || near_underflow(yi))) ||
        (eps_tiny && ((xd_bits_(nre) << 1) == 0 || (xd_bits_(nim) << 1) == 0))) {
      handover = true;  // state (dr, di, j, i) is before this step
      break;
    }
    dr = nre;
    di = nim;
    j++;
    z = zn;
    double r2 = 0.0;
    const int event =
        need_y ? bailout_and_rebase(yr, yi, dr, di, j == zlast, v.bailout2, r2) : 0;
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
  if (handover) return false;
  if (i >= v.N) {
    out = {v.N, 0.0f};
    sm = 0.0;
    return true;
  }
  return false;
}

// The unbounded-exponent state back in plain doubles, when each value is
// exactly a double that the guarded steps accept: delta's components zero or
// in [2^-400, 2^1000), eps's zero or normal.  (After a rebase delta is of the
// order of the orbit again: the rest of a long sample runs in plain doubles.)
NM_HD bool delta_xd_to_plain(const DeltaXDState& x, DeltaState& d) {
  const DeltaXDState c = x;  // x and d may share storage
  auto fits = [](const XD& a) { return a.m == 0.0 || (a.e >= -400 && a.e < 1000); };
  double er, ei;
  int32_t tiny = 0;
  if (!fits(c.dr) || !fits(c.di) || !plain_eps(c.er.m, c.er.e, er, tiny) ||
      !plain_eps(c.ei.m, c.ei.e, ei, tiny))
    return false;
  d.dr = xd_to_double(c.dr);
  d.di = xd_to_double(c.di);
  d.er = er;
  d.ei = ei;
  d.j = c.j;
  d.i = c.i;
  d.xr = c.er.m;
  d.xi = c.ei.m;
  d.xre = c.er.e;
  d.xie = c.ei.e;
  d.eps_tiny = tiny;
  return true;
}

NM_HD void delta_to_xd(const DeltaState& d, DeltaXDState& x) {
  const DeltaState c = d;  // d and x may share storage
  x.dr = xd_of(c.dr);
  x.di = xd_of(c.di);
  x.er = xd_of(c.xr, c.xre);
  x.ei = xd_of(c.xi, c.xie);
  x.j = c.j;
  x.i = c.i;
}

}  // namespace nmg
