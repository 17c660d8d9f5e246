// Float-float arithmetic: a value held as the unevaluated sum hi + lo of two
// FP32 numbers (about 46 significant bits), on the FP32 pipe.  Error-free
// transformations after Knuth (TwoSum), Dekker (FastTwoSum) and the FMA
// product error; the "sloppy" add drops the lo*lo cross terms' own error.
#pragma once

#include "view_device.cuh"

namespace nmg {

struct FF {
  float h, l;
};

#if defined(__CUDA_ARCH__)
NM_HD float fadd_(float a, float b) { return __fadd_rn(a, b); }
NM_HD float fsub_(float a, float b) { return __fsub_rn(a, b); }
NM_HD float fmul_(float a, float b) { return __fmul_rn(a, b); }
NM_HD float ffma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
inline float fadd_(float a, float b) { return a + b; }
inline float fsub_(float a, float b) { return a - b; }
inline float fmul_(float a, float b) { return a * b; }
inline float ffma_(float a, float b, float c) { return std::fma(a, b, c); }
#endif

// a + b = s + e exactly.
NM_HD FF ff_two_sum(float a, float b) {
  const float s = fadd_(a, b);
  const float bb = fsub_(s, a);
  return {s, fadd_(fsub_(a, fsub_(s, bb)), fsub_(b, bb))};
}
// a + b = s + e exactly when |a| >= |b|.
NM_HD FF ff_fast_two_sum(float a, float b) {
  const float s = fadd_(a, b);
  return {s, fsub_(b, fsub_(s, a))};
}
NM_HD FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.h, b.h);
  return ff_fast_two_sum(s.h, fadd_(s.l, fadd_(a.l, b.l)));
}
// ff_add({2 a.h, 2 a.l}, b) with the doubling folded into fused multiply-adds:
// 2x is exact in floats, so fma(2, x, y) = RN(2x + y) = RN(RN(2x) + y) and
// every value below is the same bits as ff_add's on the doubled operand.
NM_HD FF ff_add_twice(float ah, float al, FF b) {
  const float s = ffma_(2.0f, ah, b.h);           // fadd_(2 ah, b.h)
  const float bb = ffma_(-2.0f, ah, s);           // fsub_(s, 2 ah)
  const float e = fadd_(ffma_(2.0f, ah, -fsub_(s, bb)), fsub_(b.h, bb));
  return ff_fast_two_sum(s, fadd_(e, ffma_(2.0f, al, b.l)));
}
// ff_add_twice without the final renormalisation: h = RN(2 ah + b.h), l = its
// exact error plus 2 al + b.l (rounded twice).  h + l is ff_add_twice's value
// (the renormalisation is exact), but l is not bounded by half an ulp of h:
// |l| <= 2^-23 (2|ah| + |b.h|), and more than |h| where 2 ah + b.h cancels.
// For operands that only enter products (the FE32 step's t = 2Z + delta).
NM_HD FF ff_add_twice_raw(float ah, float al, FF b) {
  const float s = ffma_(2.0f, ah, b.h);
  const float bb = ffma_(-2.0f, ah, s);
  const float e = fadd_(ffma_(2.0f, ah, -fsub_(s, bb)), fsub_(b.h, bb));
  return FF{s, fadd_(e, ffma_(2.0f, al, b.l))};
}
NM_HD FF ff_from_double(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
NM_HD double ff_to_double(FF a) { return (double)a.h + (double)a.l; }
NM_HD FF ff_scale(FF a, int e) {  // a * 2^e (exact unless it underflows)
#if defined(__CUDA_ARCH__)
  return {ldexpf(a.h, e), ldexpf(a.l, e)};
#else
  return {std::ldexp(a.h, e), std::ldexp(a.l, e)};
#endif
}

// a.re*b.re - a.im*b.im + c  and  a.re*b.im + a.im*b.re + d, each in
// float-float with one rounding of the high parts' sum.
NM_HD void ff_cmul_add(FF ar, FF ai, FF br, FF bi, FF c, FF d, FF& outr, FF& outi) {
  // real part
  {
    const float p1 = fmul_(ar.h, br.h), e1 = ffma_(ar.h, br.h, -p1);
    const float p2 = fmul_(ai.h, bi.h), e2 = ffma_(ai.h, bi.h, -p2);
    const FF s = ff_two_sum(p1, -p2);
    const FF s2 = ff_two_sum(s.h, c.h);
    float lo = fadd_(fadd_(s.l, s2.l), fsub_(e1, e2));
    lo = ffma_(ar.h, br.l, lo);
    lo = ffma_(ar.l, br.h, lo);
    lo = ffma_(-ai.h, bi.l, lo);
    lo = ffma_(-ai.l, bi.h, lo);
    lo = fadd_(lo, c.l);
    outr = ff_fast_two_sum(s2.h, lo);
  }
  // imaginary part
  {
    const float p1 = fmul_(ar.h, bi.h), e1 = ffma_(ar.h, bi.h, -p1);
    const float p2 = fmul_(ai.h, br.h), e2 = ffma_(ai.h, br.h, -p2);
    const FF s = ff_two_sum(p1, p2);
    const FF s2 = ff_two_sum(s.h, d.h);
    float lo = fadd_(fadd_(s.l, s2.l), fadd_(e1, e2));
    lo = ffma_(ar.h, bi.l, lo);
    lo = ffma_(ar.l, bi.h, lo);
    lo = ffma_(ai.h, br.l, lo);
    lo = ffma_(ai.l, br.h, lo);
    lo = fadd_(lo, d.l);
    outi = ff_fast_two_sum(s2.h, lo);
  }
}

}  // namespace nmg
