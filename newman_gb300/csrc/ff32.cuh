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

// ---- the same on packed pairs (Blackwell's FP32x2 instructions) -------------
// A complex float-float value as two 64-bit registers, each holding the
// real part's word in its low half and the imaginary part's in its high half:
// one packed instruction does the real and the imaginary part's operation.
// Every lane performs exactly the operations of the scalar functions above,
// in the same order and rounding, so the results are the same bits.
#if defined(__CUDA_ARCH__)
typedef unsigned long long F2;
struct FF2 {
  F2 h, l;  // {re.h, im.h}, {re.l, im.l}
};

__device__ __forceinline__ F2 f2_pack(float x, float y) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
  return r;
}
__device__ __forceinline__ float f2_x(F2 a) {
  float x, y;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a));
  return x;
}
__device__ __forceinline__ float f2_y(F2 a) {
  float x, y;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(a));
  return y;
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ F2 f2_sub(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ F2 f2_fma(F2 a, F2 b, F2 c) {
  F2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}

// ff_add_twice on both parts: t = 2 z + d.
__device__ __forceinline__ FF2 ff2_add_twice(F2 zh, F2 zl, FF2 d) {
  const F2 two = f2_pack(2.0f, 2.0f), mtwo = f2_pack(-2.0f, -2.0f);
  const F2 s = f2_fma(two, zh, d.h);                                  // fadd_(2 zh, d.h)
  const F2 bb = f2_fma(mtwo, zh, s);                                  // fsub_(s, 2 zh)
  const F2 e = f2_add(f2_fma(two, zh, f2_sub(bb, s)), f2_sub(d.h, bb));  // bb - s = -(s - bb)
  const F2 lo = f2_add(e, f2_fma(two, zl, d.l));
  const F2 th = f2_add(s, lo);                                        // ff_fast_two_sum
  return FF2{th, f2_sub(lo, f2_sub(th, s))};
}

// ff_cmul_add(t.re, t.im, d.re, d.im, c.re, c.im) on both parts at once: with
// i d = (-d.im, d.re), t d = t.re d + t.im (i d), so the real part's
// subtraction becomes an addition of an exactly negated product.
__device__ __forceinline__ FF2 ff2_cmul_add(FF2 t, FF2 d, FF2 c) {
  const F2 mone = f2_pack(-1.0f, -1.0f);
  const float trh = f2_x(t.h), tih = f2_y(t.h), trl = f2_x(t.l), til = f2_y(t.l);
  const F2 TR = f2_pack(trh, trh), TI = f2_pack(tih, tih);
  const F2 TRL = f2_pack(trl, trl), TIL = f2_pack(til, til);
  const F2 nd = f2_mul(d.h, mone);                          // exactly -d.h (signed zeros too)
  const F2 id = f2_pack(f2_y(nd), f2_x(d.h));               // i d: (-d.im.h, d.re.h)
  const F2 nid = f2_pack(f2_y(d.h), f2_x(nd));              // -(i d)
  const F2 idl = f2_pack(f2_y(f2_mul(d.l, mone)), f2_x(d.l));
  const F2 p1 = f2_mul(TR, d.h);
  const F2 e1 = f2_fma(TR, d.h, f2_mul(TR, nd));            // fma(a, b, -p1)
  const F2 p2 = f2_mul(TI, id);                             // (-p2 re, p2 im)
  const F2 e2 = f2_fma(TI, id, f2_mul(TI, nid));
  // s = two_sum(p1, p2)
  const F2 s = f2_add(p1, p2);
  F2 bb = f2_sub(s, p1);
  const F2 sl = f2_add(f2_sub(p1, f2_sub(s, bb)), f2_sub(p2, bb));
  // s2 = two_sum(s, c.h)
  const F2 s2 = f2_add(s, c.h);
  bb = f2_sub(s2, s);
  const F2 s2l = f2_add(f2_sub(s, f2_sub(s2, bb)), f2_sub(c.h, bb));
  F2 lo = f2_add(f2_add(sl, s2l), f2_add(e1, e2));
  lo = f2_fma(TR, d.l, lo);
  lo = f2_fma(TRL, d.h, lo);
  lo = f2_fma(TI, idl, lo);
  lo = f2_fma(TIL, id, lo);
  lo = f2_add(lo, c.l);
  const F2 h = f2_add(s2, lo);                              // ff_fast_two_sum
  return FF2{h, f2_sub(lo, f2_sub(h, s2))};
}
#endif

}  // namespace nmg
