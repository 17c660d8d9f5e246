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

NM_HD bool delta_xd_steps(const DeviceView& v, DeltaXDState& st, int steps, EscapeValue& out,
                          double& sm) {
  XD dr = st.dr, di = st.di;
  int j = st.j, i = st.i;
  const int zlast = v.zlen - 1;
  const int stop = (v.N - i < steps) ? v.N : i + steps;
  const XD bail2 = xd_of(v.bailout2);
  for (; i < stop; i++) {
    const Dbl2 z = v.z[j];
    const XD tr = xd_add(xd_twice(xd_of(z.x)), dr);
    const XD ti = xd_add(xd_twice(xd_of(z.y)), di);
    const XD nre = xd_add(xd_sub(xd_mul(tr, dr), xd_mul(ti, di)), st.er);
    const XD nim = xd_add(xd_add(xd_mul(tr, di), xd_mul(ti, dr)), st.ei);
    dr = nre;
    di = nim;
    j++;
    const Dbl2 zn = v.z[j];
    const XD yr = xd_add(xd_of(zn.x), dr), yi = xd_add(xd_of(zn.y), di);
    const XD r2 = xd_add(xd_mul(yr, yr), xd_mul(yi, yi));
    if (xd_gt(r2, bail2)) {
      sm = smoothing_of(xd_to_double(r2), v.log_bailout);
      out = {i, (float)sm};
      return true;
    }
    // the rebase test r2 < d2, evaluated only when |Y| is not clearly larger
    // (larger component of Y at least 4 times delta's: |Y|^2 > 2 |delta|^2)
    bool rebase = j == zlast;
    const int32_t ey = yr.e > yi.e ? yr.e : yi.e, ed = dr.e > di.e ? dr.e : di.e;
    if (!rebase && !(ey >= ed + 2 && (yr.m != 0.0 || yi.m != 0.0)))
      rebase = xd_gt(xd_add(xd_mul(dr, dr), xd_mul(di, di)), r2);
    if (rebase) {
      dr = yr;
      di = yi;
      j = 0;
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
