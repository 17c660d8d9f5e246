// The FP32 floatexp delta iteration with its error bound, shared by the
// single-pass FE32 kernel and the multi-pass FE32 pipeline (render_fe32.cu).
//
//     t = 2 Z[j] + delta;  delta = t * delta + eps;  j += 1;  Y = Z[j] + delta
//
// delta, eps and the reference orbit Z are float-float pairs (two FP32 words)
// and, while |delta| < 2^-60, delta and eps share one int exponent E per
// sample (delta = mantissa * 2^E), renormalised at the end of every chunk of
// steps and whenever the mantissa passes 2^60.
//
// Certification.  Alongside delta the iteration propagates a bound on the
// absolute error of delta against exact arithmetic from the same start,
//     e' = 2|Y| e + e^2 + u (|t||delta| + |eps|) + u_z 2|Z||delta|,
// u the float-float rounding, u_z the float-float representation of the FP64
// orbit.  u: one component of the float-float multiply-add (ff32.cuh) rounds
// 8 times into its low word; with unit roundoff 2^-24 and every low-word term
// at most 2^-24 of the products P = |a.h b.h| + |a'.h b'.h|, the worst case
// (terms aligned, partial sums at their largest) is 30 * 2^-48 P +
// 8 * 2^-48 |eps|, plus 2^-48 P for the dropped lo*lo products; the two
// components' P add up to |t.h|_1 |delta.h|_1, so u = 1.125 * 2^-43.  u_z:
// Z in float-float is within (2^-48 + 2^-52) |Z| of the exact orbit (the
// FP64 orbit is mpf_get_d's truncation), and t = 2Z + delta rounds by at
// most 2^-46 (2|Z| + |delta|); the bound carries u_z (2|Z| + |delta|)|delta|
// with u_z = 2^-45.  Every operation on the bound rounds upward, so over
// millions of steps it never falls below the exact recurrence.
// The FP64 path's own rounding is below 2^-6 of that bound, so when every
// bailout test of a sample is decided by more than twice the bound, both paths
// take the same branch at every test and return the same escape count.  A
// sample with a test inside the band ends "uncertified".  The escape test
// itself is float-float (|Y|^2 compared with 2^20), so the iteration uses no
// FP64 at all.
#pragma once

#include "engine.hpp"
#include "ff32.cuh"
#include "pixel_fe64.cuh"

namespace nmg {

constexpr int kFeScaledBelow = -60;   // delta kept as mantissa * 2^E below 2^-60
constexpr float kFeU = 0x1.2p-43f;    // float-float multiply-add rounding per step (worst case)
constexpr float kFeUZ = 0x1p-45f;     // Z's representation and the rounding of t = 2Z + delta
// u (1 + 2^-22) + u_z, rounded up: the two local terms on one product.  The
// float-float t = 2Z + delta has |t.h|_1 <= (2|Z.h|_1 + |delta.h|_1)(1 + 2^-22.9)
// (both inputs' low words are within 2^-24 of their high words, and t.h is
// their sum rounded once more), so
//   u |t.h|_1 |delta| + u_z (2|Z| + |delta|) |delta| <= kFeUT (2|Z| + |delta|) |delta|.
// (u in units of 2^-48 and of A = the sum of a component's two |t.h||delta.h|
// products, C = |eps.h|: the eight roundings into the low word 30 A + 8 C, the
// final fast two-sum -- not exact when the high part cancels below the low
// word -- at most 2^-24 of the low word, 5 A + 2 C, the dropped t.l delta.l
// products A: 36 A + 10 C.)
constexpr float kFeUT = 0x1.61p-43f;
// The same two terms when t enters the multiply-add unnormalised
// (ff_add_twice_raw, 6 FP32 additions a step fewer): t.h = RN(2 Z.h + delta.h),
// |t.l| <= 2^-23 T with T = 2|Z.h| + |delta.h| per component, so a cross term
// t.l delta.h reaches 2^-23 T |delta.h| instead of 2^-24 |t.h||delta.h|.  With
// B = the sum of a component's T |delta.h| (A <= B (1 + 2^-24)): roundings
// 26 A + 8 B + 8 C, final fast two-sum 4 A + 2 B + 2 C, dropped products 2 B,
// 42.5 B + 10 C with the (1 + 2^-24) factors.  The components' B add up to
// P' = (2|Z.h|_1 + |delta.h|_1) |delta.h|_1, so the step rounds by at most
// 1.33 * 2^-43 P' + u |eps|_1, and with u_z kFeUTRaw = 1.578125 * 2^-43.
// Both assume the delta a step reads is normalised, which the final fast
// two-sum gives unless the new delta cancels below its own low word; what the
// next step then rounds or drops beyond the derivation is below 2^-60 of
// (|Z| + |delta|) times the carried bound's own local term, inside the 2^-20
// margin on |Y| in the amplification.
constexpr float kFeUTRaw = 0x1.94p-43f;
// Which t a view's FE32 steps take, the same in every kernel (a frame of a
// batch and the frame rendered alone give the same bits): unnormalised on
// views inside the FP64 range; floatexp views keep the renormalised t, whose
// smaller bound reworks fewer samples, and their frame time follows the
// reworked ones.
NM_HD bool fe_raw_t(const DeviceView& v) { return !v.sa_fe; }
// t = 2Z + delta for the step's multiply-add, renormalised or not.
template <bool kRawT>
__device__ __forceinline__ FF fe_twice_plus(float ah, float al, FF b) {
  return kRawT ? ff_add_twice_raw(ah, al, b) : ff_add_twice(ah, al, b);
}
// A bound below which the bailout test of a state with |Y|^2 <= 2^20 (1 - 2^-10)
// and Z not the orbit's escaped last point is decided without evaluating it:
// |Z.h|_1 < 1449, |delta.h|_1 < 2900, so the band of the full test,
// 2 (2^-20 (|Z| + |delta|) + e + u_z |Z| + u (|Z| + |delta|)), stays below
// 2 (0.0043 + e + 2^-30) < 0.49 <= 1024 - |Y| whenever e < 0.2.
constexpr float kFeQuickErr = 0.2f;

// Interior orbits on double-loop views.  The reference's double loop F (one
// step z -> z^2 + c in doubles, mandelbrot.cpp:242-246) rounds by at most
//   |F(z) - f(z)| <= 2^-53 (3|z|^2 + |F(z)|_1) (1 + 2^-52),   f(z) = z^2 + c,
// so for every double z in a disk D(w, r) around a point w of the exact orbit
//   |F(z) - f(w)| <= r (2|w| + r) + 2^-52 (3.5 a^2 + 1.5 |c|_1),  a = |w| + r,
// using |F(z)|_1 <= 1.5 (a^2 + |c|_1).  Following the image of a disk
// B = D(P, R) along the exact orbit with this radius recurrence (rho), a
// ball that comes back inside B after p steps traps the double loop: F^p(B)
// lies in B and every intermediate image stays far inside the bailout, so a
// double orbit that is in B never escapes and the double loop's result is N.
// A disk is laid at each power-of-two iteration count from kTrapFirst on,
// centred on the FE32 orbit point (float-float), with R = 16 times the
// distance from there to the double orbit (the FE32 and double-loop bounds)
// but at least 2^-22 (on the double-loop frames of a 240-frame 1280x720 zoom
// into -0.743643887037151+0.131825904205330i, 2^-22 traps the most interior
// samples soonest: 2^-36 and 2^-18 took 1.5x and 1.4x as many steps); the
// return is checked at the end of every chunk, and a radius
// above kTrapRhoMax drops the disk.
constexpr float kTrapRMin = 0x1p-22f;
constexpr float kTrapRMax = 0x1p-20f;
constexpr float kTrapRhoMax = 0x1p-4f;
constexpr int kTrapFirst = 1024;
constexpr float kFeBailout = 1024.0f;       // mandelbrot.cpp:58
constexpr float kFeBailout2 = 1048576.0f;   // mandelbrot.cpp:59

// Arithmetic on error bounds, rounded upward.
__device__ __forceinline__ float up_add(float a, float b) { return __fadd_ru(a, b); }
__device__ __forceinline__ float up_mul(float a, float b) { return __fmul_ru(a, b); }
__device__ __forceinline__ float up_fma(float a, float b, float c) { return __fmaf_ru(a, b, c); }

struct alignas(16) FeState {
  FF dr, di;      // delta * 2^-E
  FF er, ei;      // eps * 2^-E
  float err;      // error bound of delta, in the same units
  int32_t E;      // 0: unscaled
  int32_t j, i;   // orbit index, iteration count (getIterations' i)
  int32_t certified;
  int32_t frame;  // frame of a batch
  float e64;      // double-loop views: bound on the double loop's own error
  int32_t pad_;
};

// Finished sample: escape iteration (N: no escape) and |Y|^2 at the escape.
struct alignas(16) FeResult {
  int32_t it;
  int32_t certified;
  FF r2;
};

struct ZFF {  // reference orbit element, float-float
  float hx, hy, lx, ly;
};

template <bool kStaged = false>
__device__ __forceinline__ ZFF fe_load_z(const DeviceView& v, int j) {
  const Flt4 z = orbit_zf<kStaged>(v, j);
  return ZFF{z.x, z.y, z.z, z.w};
}

// The front of a double-loop view (getIterationsHW, mandelbrot.cpp:231-254):
// the reference's cardioid test, then the perturbation start Y_1 = Z_1 + eps =
// the double coordinate the loop starts from; no series skip.
__device__ __forceinline__ bool double_loop_front(const DeviceView& v, int r, int c,
                                                  SeriesFront& f, EscapeValue& out, double& sm,
                                                  bool& undecided) {
  undecided = false;
  if (v.cardioid_mode == CARDIOID_PER_SAMPLE &&
      in_cardioid_dd(v.coord_re[c], v.coord_im[r], undecided)) {
    out = {v.N, 0.0f};
    sm = 0.0;
    return true;
  }
  f.eps = C64{v.eps_re[c], v.eps_im[r]};
  f.dfound = f.eps;
  f.dsize = 1;
  f.eps_e = 0;
  f.d_e = 0;
  return false;
}

// The front of the FE32 path: the double-loop front or the series front.
__device__ __forceinline__ bool fe_front(const DeviceView& v, int r, int c, SeriesFront& f,
                                         EscapeValue& out, double& sm, bool& undecided) {
  if (v.double_loop) return double_loop_front(v, r, c, f, out, sm, undecided);
  return series_front_any(v, r, c, f, out, sm, undecided);
}

// Start state from the front (bit-identical to the FP64 path's).  A
// double-loop view starts at Z index 1 (Y = the loop's start value) with
// iteration count 0, so that the escape test after step `it` sees the
// double loop's z after its step `it`.
__device__ __forceinline__ void fe_start(const DeviceView& v, const SeriesFront& f, FeState& st) {
  // exponent of the larger of |d[found]| and |eps| (their mantissas carry
  // their own exponents d_e, eps_e in floatexp views)
  const double dm = fmax(fabs(f.dfound.re), fabs(f.dfound.im));
  const double em = fmax(fabs(f.eps.re), fabs(f.eps.im));
  const int kNone = -(1 << 30);
  const int mag = max(dm > 0.0 ? ilogb(dm) + f.d_e : kNone, em > 0.0 ? ilogb(em) + f.eps_e : kNone);
  const int E = (mag > kNone && mag < -60) ? mag : 0;
  st.E = E;
  st.dr = ff_from_double(scalbn(f.dfound.re, f.d_e - E));
  st.di = ff_from_double(scalbn(f.dfound.im, f.d_e - E));
  st.er = ff_from_double(scalbn(f.eps.re, f.eps_e - E));
  st.ei = ff_from_double(scalbn(f.eps.im, f.eps_e - E));
  st.err = up_mul(kFeU, up_add(fabsf(st.dr.h), fabsf(st.di.h)));
  st.j = f.dsize;
  st.i = v.double_loop ? 0 : f.dsize;
  st.certified = 1;
  st.frame = 0;
  st.e64 = 0.0f;
  st.pad_ = 0;
}

// ---- the series front on the FP32 pipe ---------------------------------------
//
// The FP64 front (pixel_fp64.cuh, pixel_fe64.cuh) decides two things that the
// FE32 path must reproduce exactly -- the series stop index and whether the
// sample escapes before it -- and computes d[found], which the FE32 path only
// needs to within its error bound.  Here:
//   stop index: the first i with T_i < u, u = |eps3|^2/|eps2|^2 = |eps|^2 in
//     exact arithmetic; the FP64 front's u is within 2^-40 of |eps|^2 and its
//     own thresholds are exact there, so where no threshold T_i lies within
//     2^-18 of the FP32 |eps|^2 (good to 2^-22) both fronts stop at the same i;
//   escape before the stop: impossible when |X[found]|_1 + |d|_1 < 1023.5;
//   d[found] = A eps + B eps^2 + C eps^3 in float-float with exponents, within
//     2^-40 (|A eps| + |B eps^2| + |C eps^3|) of the FP64 front's value, which
//     goes into the starting error bound.
// Any other sample (a threshold in the band, an orbit element near the
// bailout) returns kFront32Undecided and takes the FP64 front.

constexpr int kFront32Ready = 0, kFront32Finished = 1, kFront32Undecided = 2;

struct CFF {  // ((re) + i (im)) * 2^e, float-float mantissas
  FF re, im;
  int e;
};

__device__ __forceinline__ FF ffe_scaled(float h, float l, int d) {
  if (h == 0.0f || d < -140) return FF{0.0f, 0.0f};
  return ff_scale(FF{h, l}, d);
}
__device__ __forceinline__ float cff_l1(const CFF& a) { return fabsf(a.re.h) + fabsf(a.im.h); }
__device__ __forceinline__ CFF cff_mul(const CFF& a, const CFF& b) {
  CFF r;
  ff_cmul_add(a.re, a.im, b.re, b.im, FF{0.0f, 0.0f}, FF{0.0f, 0.0f}, r.re, r.im);
  r.e = a.e + b.e;
  return r;
}
__device__ __forceinline__ CFF cff_of(const CFFE& x) {
  return CFF{FF{x.rh, x.rl}, FF{x.ih, x.il}, x.e};
}
__device__ __forceinline__ bool tfe_less(TFE a, TFE b) {
  return a.e < b.e || (a.e == b.e && a.m < b.m);
}
__device__ __forceinline__ int first_below32(const TFE* t, int lo, int hi, TFE x) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (tfe_less(t[mid], x))
      hi = mid;
    else
      lo = mid + 1;
  }
  return lo;
}
__device__ __forceinline__ TFE tfe_norm(float m, int e) {
  if (!(m > 0.0f)) return TFE{0.0f, kTfeZero};
  const int k = ilogbf(m);
  return TFE{ldexpf(m, -k), e + k};
}

__device__ __forceinline__ int fe_front32(const DeviceView& v, int r, int c, FeState& st) {
  if (v.cardioid_mode == CARDIOID_PER_SAMPLE || !v.sa_min32) return kFront32Undecided;
  const FFE er = v.eps32_re[c], ei = v.eps32_im[r];
  const int ee = er.h == 0.0f ? ei.e : ei.h == 0.0f ? er.e : max(er.e, ei.e);
  const CFF eps{ffe_scaled(er.h, er.l, er.e - ee), ffe_scaled(ei.h, ei.l, ei.e - ee), ee};
  const int n = v.xlen;
  int fire = n;
  const float s = fmaf(eps.re.h, eps.re.h, eps.im.h * eps.im.h);  // |eps|^2 * 2^-2ee
  if (s > 0.0f) {
    const TFE u = tfe_norm(s, 2 * ee);
    // both ends normalised (m in [1, 2)): the comparison is lexicographic
    const TFE hi = tfe_norm(u.m * (1.0f + 0x1p-18f), u.e), lo = tfe_norm(u.m * (1.0f - 0x1p-18f), u.e);
    const int i1 = first_below32(v.sa_min32, 1, n, hi);
    if (i1 < n) {
      if (first_below32(v.sa_min32, i1, n, lo) != i1) return kFront32Undecided;
      fire = i1;
    }
  }
  const int dsize = fire < n ? (fire - 3 < 1 ? 1 : fire - 3) : n;
  const int found = dsize - 1;
  // d[found] and its distance bound, both at exponent de
  CFF d;
  float dbound;  // in units of 2^d.e
  if (found == 0) {
    d = eps;
    dbound = up_mul(0x1p-46f, cff_l1(eps));
  } else {
    const CFF e2 = cff_mul(eps, eps), e3 = cff_mul(eps, e2);
    const CFF A = cff_of(v.sa_a32[found]), B = cff_of(v.sa_b32[found]), C = cff_of(v.sa_c32[found]);
    const CFF ta = cff_mul(A, eps), tb = cff_mul(B, e2), tc = cff_mul(C, e3);
    const float ma = cff_l1(ta), mb = cff_l1(tb), mc = cff_l1(tc);
    int de = ma > 0.0f ? ta.e : -(1 << 29);
    if (mb > 0.0f) de = max(de, tb.e);
    if (mc > 0.0f) de = max(de, tc.e);
    if (de == -(1 << 29)) de = ta.e;
    d.e = de;
    d.re = FF{0.0f, 0.0f};
    d.im = FF{0.0f, 0.0f};
    // products of the inputs' magnitudes bound each term's rounding
    const float l1e = cff_l1(eps);
    float mag = 0.0f;
    const CFF* terms[3] = {&ta, &tb, &tc};
    const float mags[3] = {up_mul(cff_l1(A), l1e), up_mul(up_mul(cff_l1(B), l1e), l1e),
                           up_mul(up_mul(up_mul(cff_l1(C), l1e), l1e), l1e)};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int sh = terms[k]->e - de;
      const float mk = up_add(mags[k], cff_l1(*terms[k]));
      if (sh < -100) {  // below 2^-95 of the sum: dropped, its size in the bound
        mag = up_add(mag, fmaxf(ldexpf(mk, sh + 40), 0x1p-126f));
        continue;
      }
      d.re = ff_add(d.re, ff_scale(terms[k]->re, sh));
      d.im = ff_add(d.im, ff_scale(terms[k]->im, sh));
      mag = up_add(mag, fmaxf(ldexpf(mk, sh), 0x1p-126f));
    }
    dbound = up_mul(0x1p-40f, mag);
  }
  // escape before the stop is impossible when |X[found]| + |d| < 1023.5
  {
    const ZFF x = fe_load_z(v, found + 1);
    const float dl1 = ldexpf(up_add(cff_l1(d), dbound), d.e);
    const float xl1 = up_mul(up_add(fabsf(x.hx), fabsf(x.hy)), 1.0f + 0x1p-20f);
    if (!(up_add(xl1, up_mul(dl1, 1.0f + 0x1p-20f)) < 1023.5f)) return kFront32Undecided;
  }
  // the state: delta and eps share exponent E below 2^-60, as fe_start does
  const float dm = fmaxf(fabsf(d.re.h), fabsf(d.im.h));
  const float em = fmaxf(fabsf(eps.re.h), fabsf(eps.im.h));
  const int kNone = -(1 << 30);
  const int mag = max(dm > 0.0f ? ilogbf(dm) + d.e : kNone, em > 0.0f ? ilogbf(em) + eps.e : kNone);
  const int E = (mag > kNone && mag < kFeScaledBelow) ? mag : 0;
  st.E = E;
  st.dr = ffe_scaled(d.re.h, d.re.l, d.e - E);
  st.di = ffe_scaled(d.im.h, d.im.l, d.e - E);
  st.er = ffe_scaled(eps.re.h, eps.re.l, eps.e - E);
  st.ei = ffe_scaled(eps.im.h, eps.im.l, eps.e - E);
  st.err = up_add(fmaxf(ldexpf(dbound, d.e - E), 0.0f),
                  up_mul(kFeU, up_add(fabsf(st.dr.h), fabsf(st.di.h))));
  st.j = dsize;
  st.i = dsize;
  st.certified = 1;
  st.frame = 0;
  st.e64 = 0.0f;
  st.pad_ = 0;
  return kFront32Ready;
}

// The FE32 start state of sample (r, c): the FP32 front where it decides,
// else the FP64 front.  True when the sample is finished in the front (out,
// sm set); `fp64` tells which front ran.
__device__ __forceinline__ bool fe_front_start(const DeviceView& v, int r, int c, FeState& st,
                                               EscapeValue& out, double& sm, bool& undecided,
                                               bool& fp64) {
  undecided = false;
  fp64 = false;
  if (!v.double_loop && fe_front32(v, r, c, st) == kFront32Ready) return false;
  fp64 = !v.double_loop;
  SeriesFront f;
  if (fe_front(v, r, c, f, out, sm, undecided)) return true;
  fe_start(v, f, st);
  return false;
}

// sqrt(x) from the hardware reciprocal square root (relative error below
// 2^-21; 0 for x = 0).
// sqrt(x) from the hardware reciprocal square root (relative error below
// 2^-22.9; with the product's rounding within 2^-21).  Below x = 2^-120 the
// result is 2^-60, above sqrt(x): the FE32 step only uses the estimate of |Y|
// as an upper bound (its error amplification, the bailout gap 1024 - |Y|),
// and the flush-to-zero form needs no subnormal handling.
__device__ __forceinline__ float approx_sqrt(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return x > 0x1p-120f ? x * r : 0x1p-60f;
}
__device__ __forceinline__ float approx_norm(float x, float y) {
  return approx_sqrt(fmaf(x, x, y * y));
}

// x^2 + y^2 in float-float.
__device__ __forceinline__ FF ff_norm2(FF x, FF y) {
  const float p1 = x.h * x.h, e1 = fmaf(x.h, x.h, -p1);
  const float p2 = y.h * y.h, e2 = fmaf(y.h, y.h, -p2);
  const FF s = ff_two_sum(p1, p2);
  float lo = s.l + e1 + e2;
  lo = fmaf(2.0f * x.h, x.l, lo);
  lo = fmaf(2.0f * y.h, y.l, lo);
  return ff_fast_two_sum(s.h, lo);
}

// The bailout test on Y = Z + delta (unscaled, float-float).  Returns true
// when |Y|^2 > 2^20; clears `certified` when the error bound `yerr` on |Y|
// reaches across 1024.
__device__ __forceinline__ bool fe_escape_test(FF yr, FF yi, float yerr, bool& certified,
                                               FF& r2) {
  r2 = ff_norm2(yr, yi);
  const float d = (r2.h - kFeBailout2) + r2.l;  // r2.h - 2^20 is exact near 2^20
  // | |Y| - 1024 | <= 2 yerr  <=>  | |Y|^2 - 2^20 | <= (2048 + 2 yerr) 2 yerr
  if (fabsf(d) <= up_fma(up_fma(2.0f, yerr, 2048.0f), up_mul(2.0f, yerr), up_mul(0x1p-40f, r2.h)))
    certified = false;
  return d > 0.0f;
}

// The smoothing term of mandelbrot.cpp:133-136, 1 - log2(log|Y|^2 / (2 log 1024)),
// in FP32 from the float-float |Y|^2 (good to about 2^-22 absolute; the value is
// stored as a float).  0 for a sample that did not escape.
__device__ __forceinline__ float fe_smoothing(const DeviceView& v, const FeResult& res) {
  if (res.it >= v.N) return 0.0f;
  return 1.0f - log2f(0.5f * logf(res.r2.h + res.r2.l) / (float)v.log_bailout);
}

__device__ __forceinline__ void fe_renormalise(FeState& st) {
  const float mag = fmaxf(fabsf(st.dr.h), fabsf(st.di.h));
  if (!(mag > 0.0f)) return;
  const int e = ilogbf(mag);
  st.dr = ff_scale(st.dr, -e);
  st.di = ff_scale(st.di, -e);
  st.er = ff_scale(st.er, -e);
  st.ei = ff_scale(st.ei, -e);
  st.err = ldexpf(st.err, -e);
  st.E += e;
  if (st.E >= kFeScaledBelow) {  // large enough for plain FP32
    st.dr = ff_scale(st.dr, st.E);
    st.di = ff_scale(st.di, st.E);
    st.er = ff_scale(st.er, st.E);
    st.ei = ff_scale(st.ei, st.E);
    st.err = ldexpf(st.err, st.E);
    st.E = 0;
  }
}

// Steps while delta is scaled: Y = Z to working precision, so the events are
// the reference's own escape, the end of the orbit, and Z passing so close to
// 0 that |Y| < |delta| could hold (left to the FP64 kernel: uncertified).
template <bool kStaged = false, bool kRawT = false>
__device__ __forceinline__ bool fe_scaled_steps(const DeviceView& v, FeState& st, int steps,
                                             FeResult& res, unsigned long long& executed,
                                             unsigned long long& rebases) {
  const int zlast = v.zlen - 1;
  const int stop = min(v.N, st.i + steps);
  const int start = st.i;
  ZFF z = fe_load_z<kStaged>(v, st.j);
  bool done = false;
  // delta * 2^E as a float-float (0 below 2^-140, as in fe_renormalise's
  // range): E stays fixed through these steps, and for -140 <= E the factor
  // 2^E is a float (subnormal below 2^-126), so x * 2^E rounds once, exactly
  // as ldexpf(x, E) does
  const float sfac = st.E < -140 ? 0.0f
                     : st.E >= -126 ? __int_as_float((st.E + 127) << 23)
                                    : __int_as_float(1 << (st.E + 149));
  auto unscaled = [&](FF d) { return FF{d.h * sfac, d.l * sfac}; };
  for (; st.i < stop; st.i++) {
    const FF sd_r = unscaled(st.dr);
    const FF sd_i = unscaled(st.di);
    const FF tr = fe_twice_plus<kRawT>(z.hx, z.lx, sd_r);
    const FF ti = fe_twice_plus<kRawT>(z.hy, z.ly, sd_i);
    const float zl1 = up_add(fabsf(z.hx), fabsf(z.hy)), dl1 = up_add(fabsf(st.dr.h), fabsf(st.di.h));
    FF nr, ni;
    ff_cmul_add(tr, ti, st.dr, st.di, st.er, st.ei, nr, ni);
    {
      // scaled units: e' = 2 (|Z| + |delta|) e + e^2 2^E + u (|t||delta| + |eps|)
      //                     + u_z (2|Z| + |delta|) |delta|
      const float dmag = fmaxf(ldexpf(dl1, st.E), 0x1p-126f);
      const float amp = up_add(up_mul(2.0f, up_add(zl1, dmag)),
                               fmaxf(ldexpf(st.err, st.E), 0x1p-126f));
      const float loc = up_fma(kRawT ? kFeUTRaw : kFeUT, up_mul(up_fma(2.0f, zl1, dmag), dl1),
                               up_mul(kFeU, up_add(fabsf(st.er.h), fabsf(st.ei.h))));
      st.err = up_fma(amp, st.err, loc);
    }
    st.dr = nr;
    st.di = ni;
    st.j++;
    z = fe_load_z<kStaged>(v, st.j);
    const float zm2 = fmaf(z.hx, z.hx, z.hy * z.hy);
    // Y = Z + delta, formed where it is used (the escape test, the rebase)
    auto y_of = [&](FF& yr, FF& yi) {
      yr = ff_add(FF{z.hx, z.lx}, unscaled(st.dr));
      yi = ff_add(FF{z.hy, z.ly}, unscaled(st.di));
    };
    if (zm2 > kFeBailout2 * (1.0f - 0x1p-10f)) {
      FF yr, yi;
      y_of(yr, yi);
      const float yerr = up_add(fmaxf(ldexpf(st.err, st.E), 0x1p-126f),
                                up_mul(kFeUZ, up_add(fabsf(z.hx), fabsf(z.hy))));
      bool cert = st.certified != 0;
      FF r2;
      if (fe_escape_test(yr, yi, yerr, cert, r2)) {
        st.certified = cert ? 1 : 0;
        res.it = st.i;
        res.r2 = r2;
        done = true;
        st.i++;
        break;
      }
      st.certified = cert ? 1 : 0;
    }
    const float dmag = ldexpf(dl1, st.E);
    if (fabsf(z.hx) + fabsf(z.hy) <= 4.0f * dmag) st.certified = 0;  // |Y| < |delta| possible
    if (!st.certified) {  // the FP64 kernel renders this sample
      st.i++;
      done = true;
      break;
    }
    if (st.j == zlast) {  // orbit exhausted: rebase to Z[0], now unscaled
      const float e_abs = up_add(up_add(fmaxf(ldexpf(st.err, st.E), 0x1p-126f), kFeUZ * 2048.0f),
                                 up_mul(kFeU, up_add(zl1, dmag)));
      FF yr, yi;
      y_of(yr, yi);
      st.dr = yr;
      st.di = yi;
      st.er = ff_scale(st.er, st.E);
      st.ei = ff_scale(st.ei, st.E);
      st.err = e_abs;
      st.E = 0;
      st.j = 0;
      rebases++;
      st.i++;
      break;
    }
    if (fmaxf(fabsf(st.dr.h), fabsf(st.di.h)) > 0x1p60f) {
      st.i++;
      break;
    }
  }
  executed += (unsigned long long)(st.i - start);
  if (!done && st.E != 0) fe_renormalise(st);
  if (done) return true;
  if (st.i >= v.N) {
    res.it = v.N;
    res.r2 = FF{0.f, 0.f};
    return true;
  }
  return false;
}

// Up to `steps` iterations; true when the sample is finished: either
// certified with res filled, or uncertified (st.certified == 0), in which case
// the iteration stops at once and res is not meaningful -- the sample goes to
// the FP64 kernel.
// The unscaled steps; kDl: a double-loop view (second bound e64, trapping).
template <bool kDl, bool kStaged = false, bool kRawT = false>
__device__ __forceinline__ bool fe_unscaled_steps(const DeviceView& v, FeState& st, int steps,
                                                  FeResult& res, unsigned long long& executed,
                                                  unsigned long long& rebases, FeTrap* trap) {
  const int zlast = v.zlen - 1;
  const int stop = min(v.N, st.i + steps);
  const int start = st.i;
  const float lo_band = kFeBailout2 * (1.0f - 0x1p-10f);
  const float ueps = up_mul(kFeU, up_add(fabsf(st.er.h), fabsf(st.ei.h)));
  const FF er = st.er, ei = st.ei;
  FF dr = st.dr, di = st.di;
  float err = st.err;
  float e64 = st.e64;
  constexpr bool dloop = kDl;
  // the radius of the followed trapping disk's image (a sample starts at i = 0)
  float rho = (kDl && trap && st.i > 0) ? trap->rho : 0.0f;
  int j = st.j, i = st.i;
  bool certified = st.certified != 0;
  ZFF z = fe_load_z<kStaged>(v, j);
  // |Y| of the current state (for the error bound's amplification 2|Y|),
  // from the hardware reciprocal square root: within 2^-21 of |Y_h|, which
  // the 2^-20 (|Z| + |delta|) margins below cover together with the hi parts'
  // own error (2^-22)
  float ym = approx_norm(z.hx + dr.h, z.hy + di.h);
  bool done = false;
  for (; i < stop; i++) {
    const FF tr = fe_twice_plus<kRawT>(z.hx, z.lx, dr);
    const FF ti = fe_twice_plus<kRawT>(z.hy, z.ly, di);
    const float zl1 = up_add(fabsf(z.hx), fabsf(z.hy)), dl1 = up_add(fabsf(dr.h), fabsf(di.h));
    const float ym_up = up_fma(0x1p-20f, up_add(zl1, dl1), ym);
    const float loc = up_fma(kRawT ? kFeUTRaw : kFeUT, up_mul(up_fma(2.0f, zl1, dl1), dl1), ueps);
    const float err_old = err;
    err = up_fma(up_fma(2.0f, ym_up, err), err, loc);  // 2|Y| e + e^2 + local rounding
    FF nr, ni;
    ff_cmul_add(tr, ti, dr, di, er, ei, nr, ni);
    dr = nr;
    di = ni;
    j++;
    z = fe_load_z<kStaged>(v, j);
    const float yr = z.hx + dr.h, yi = z.hy + di.h;
    const float r2 = fmaf(yr, yr, yi * yi);
    ym = approx_sqrt(r2);
    // error of Y = Z + delta held in float-float (the rebase value)
    auto y_err = [&]() {
      const float zn1 = up_add(fabsf(z.hx), fabsf(z.hy)), dn1 = up_add(fabsf(dr.h), fabsf(di.h));
      return up_add(err, up_fma(kFeUZ, zn1, up_mul(kFeU, up_add(zn1, dn1))));
    };
    // The bailout test: evaluated in full near the bailout, on a double-loop
    // view (whose second bound e64 is propagated every step), at the orbit's
    // last point, or once the bound has grown past kFeQuickErr; otherwise it
    // is decided (|Y| below 1024 by more than the band) -- see kFeQuickErr.
    if (dloop || r2 > lo_band || !(err < kFeQuickErr) || j == zlast) {
      const float zn1 = up_add(fabsf(z.hx), fabsf(z.hy)), dn1 = up_add(fabsf(dr.h), fabsf(di.h));
      float yerr = y_err();
      if (dloop) {
        // The double loop's own distance from exact arithmetic, d' <= (|z| + |w|) d
        // + its rounding: with |w| <= |Y| + e (the exact orbit) and |z| <= |w| + d,
        // d' <= (2(|Y| + e) + d) d + 2^-52 (2 |z|^2 + |z'|_1); its bailout test
        // rounds |z|^2 by 2^-52 more.  The tests below take the sum of both bounds.
        const float w_old = up_add(ym_up, err_old);
        const float z_old = up_add(w_old, e64);
        const float z_new = up_add(up_add(zn1, dn1), up_add(err, e64));
        const float l64 = up_mul(0x1p-52f, up_fma(up_mul(2.0f, z_old), z_old, z_new));
        e64 = up_fma(up_fma(2.0f, w_old, e64), e64, l64);
        yerr = up_add(yerr, up_fma(0x1p-52f, z_new, e64));
        if (rho > 0.0f) {  // the image of the trapping disk around the exact orbit
          const float a = up_add(w_old, rho);
          const float l64r = up_mul(0x1p-52f, up_fma(up_mul(3.5f, a), a, up_mul(1.5f, v.c_abs)));
          rho = up_fma(up_fma(2.0f, w_old, rho), rho, l64r);
          // dropped where the disk's image could reach the bailout or grow past
          // the linear regime
          if (!(up_add(rho, err) <= kTrapRhoMax) || !(r2 <= lo_band)) rho = 0.0f;
        }
      }
      if (r2 <= lo_band) {
        // |Y| is below the bailout by more than 2^-11 of it; the estimate ym
        // is good to 2^-20 (|Z| + |delta|), so the test is decided unless the
        // bound covers the whole gap
        if (up_mul(2.0f, up_fma(0x1p-20f, up_add(zn1, dn1), yerr)) >= __fsub_rd(kFeBailout, ym)) {
          certified = false;  // the FP64 kernel renders this sample
          done = true;
          i++;
          break;
        }
      } else {
        FF r2ff;
        if (fe_escape_test(ff_add(FF{z.hx, z.lx}, dr), ff_add(FF{z.hy, z.ly}, di), yerr,
                           certified, r2ff)) {
          res.it = i;
          res.r2 = r2ff;
          done = true;
          i++;
          break;
        }
        if (!certified) {
          done = true;
          i++;
          break;
        }
      }
    }
    const float d2 = fmaf(dr.h, dr.h, di.h * di.h);
    if (r2 < d2 || j == zlast) {  // rebase to Z[0]: delta = Y in float-float
      const float yerr_fe = y_err();
      const FF nyr = ff_add(FF{z.hx, z.lx}, dr);
      const FF nyi = ff_add(FF{z.hy, z.ly}, di);
      dr = nyr;
      di = nyi;
      err = yerr_fe;
      j = 0;
      z = fe_load_z<kStaged>(v, 0);
      ym = approx_norm(dr.h, di.h);
      rebases++;
    }
  }
  if (kDl && trap && !done && certified && i < v.N) {
    // P: the FE32 orbit point Y = Z + delta in float-float, to mgn of Y; the
    // exact orbit within cerr of Y, the double loop's within e64 of it
    const float zn1 = up_add(fabsf(z.hx), fabsf(z.hy)), dn1 = up_add(fabsf(dr.h), fabsf(di.h));
    const FF px = ff_add(FF{z.hx, z.lx}, dr), py = ff_add(FF{z.hy, z.ly}, di);
    const float mgn = up_mul(0x1p-43f, up_add(zn1, dn1));
    const float cerr = up_add(err, up_mul(kFeUZ, zn1));
    if (rho > 0.0f) {
      // back inside: D(exact orbit, rho) within the disk D(P_saved, R)
      const FF ddx = ff_add(px, FF{-trap->pxh, -trap->pxl});
      const FF ddy = ff_add(py, FF{-trap->pyh, -trap->pyl});
      const float dist = up_add(up_add(up_add(fabsf(ddx.h), fabsf(ddx.l)),
                                       up_add(fabsf(ddy.h), fabsf(ddy.l))),
                                up_mul(0x1p-43f, up_add(up_add(zn1, dn1), up_add(
                                    fabsf(trap->pxh), fabsf(trap->pyh)))));
      if (up_add(up_add(dist, up_add(mgn, cerr)), rho) <= trap->R) {
        done = true;
        res.it = v.N;
        res.r2 = FF{0.f, 0.f};
      }
    }
    // a new disk at each power of two from kTrapFirst on, when the double
    // orbit lies well inside it: D(exact orbit, rho) covers D(P, R)
    if (!done && i >= kTrapFirst && __clz(i) < __clz(start > 0 ? start : 1)) {
      const float R = fmaxf(kTrapRMin, up_mul(16.0f, up_add(up_add(cerr, e64), mgn)));
      if (R <= kTrapRMax) {
        trap->pxh = px.h;
        trap->pxl = px.l;
        trap->pyh = py.h;
        trap->pyl = py.l;
        trap->R = R;
        rho = up_add(up_add(R, mgn), cerr);
      }
    }
    trap->rho = rho;
  }
  executed += (unsigned long long)(i - start);
  st.dr = dr;
  st.di = di;
  st.err = err;
  st.e64 = e64;
  st.j = j;
  st.i = i;
  st.certified = certified ? 1 : 0;
  if (done) return true;
  if (i >= v.N) {
    res.it = v.N;
    res.r2 = FF{0.f, 0.f};
    return true;
  }
  return false;
}

template <bool kStaged = false, bool kRawT = false>
__device__ __forceinline__ bool fe_advance(const DeviceView& v, FeState& st, int steps,
                                           FeResult& res, unsigned long long& executed,
                                           unsigned long long& rebases, FeTrap* trap = nullptr) {
  if (st.E != 0) {
    if (v.double_loop) {  // a start below 2^-60: left to the double loop
      st.certified = 0;
      return true;
    }
    return fe_scaled_steps<kStaged, kRawT>(v, st, steps, res, executed, rebases);
  }
  if (v.double_loop)
    return fe_unscaled_steps<true, kStaged, kRawT>(v, st, steps, res, executed, rebases, trap);
  return fe_unscaled_steps<false, kStaged, kRawT>(v, st, steps, res, executed, rebases, nullptr);
}

}  // namespace nmg
