// FP64 with an unbounded exponent: a value is m * 2^e with m a double in
// [1, 2) (or 0) and e a 32-bit int.  Every operation rounds the exact result
// to 53 bits, round-to-nearest-even, exactly as an IEEE double operation would
// if the exponent range had no limits -- so on values that never under- or
// overflow it gives the plain double results bit for bit, and below 2^-1022
// it carries on where doubles would go subnormal or flush to zero.
//
// The mantissa arithmetic is one FP64 add or multiply per operation; the
// exponent handling (alignment, normalisation) is integer work on the
// double's bit pattern, which runs beside the FP64 pipe.
//
//   add:  align the smaller operand to the larger one's exponent by setting
//         its exponent field (exact for a shift of at most 60 bits); past 60
//         bits it is below half an ulp of the larger and the sum rounds to
//         the larger operand, as in unbounded arithmetic.
//   mul:  the product of two mantissas in [1, 2) lies in [1, 4): no range
//         limit is touched, so the FP64 multiply rounds exactly.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "view_device.cuh"

namespace nmg {

struct XD {
  double m;   // 0 or |m| in [1, 2)
  int32_t e;  // value = m * 2^e
};

constexpr int32_t kXdZeroExp = -(1 << 29);  // exponent of 0: below every value

NM_HD int64_t xd_bits_(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  int64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}
NM_HD double xd_from_bits_(int64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

// x (a normal double or 0) times 2^e, normalised.
NM_HD XD xd_norm(double x, int32_t e) {
  const int64_t b = xd_bits_(x);
  const int32_t f = (int32_t)((b >> 52) & 0x7ff);
  if (f == 0) return XD{0.0, kXdZeroExp};  // 0 (subnormals do not arise here)
  const double m = xd_from_bits_((b & ~(0x7ffll << 52)) | (1023ll << 52));
  return XD{m, e + f - 1023};
}

// Any finite double (normal, subnormal or 0), exactly.
NM_HD XD xd_of(double x) {
  const int64_t b = xd_bits_(x);
  if (((b >> 52) & 0x7ff) == 0 && (b & ~(1ll << 63)) != 0)  // subnormal: scale up first
    return xd_norm(x * 0x1p200, -200);
  return xd_norm(x, 0);
}

// m * 2^e for a mantissa m of any magnitude (an FE front's output).
NM_HD XD xd_of(double m, int32_t e) {
  XD r = xd_of(m);
  if (r.m != 0.0) r.e += e;
  return r;
}

// The double nearest to x (x must be inside the double range: used for
// values near the bailout radius).
NM_HD double xd_to_double(XD x) {
  if (x.m == 0.0) return 0.0;
#if defined(__CUDA_ARCH__)
  return scalbn(x.m, x.e);
#else
  return std::scalbn(x.m, x.e);
#endif
}

NM_HD XD xd_neg(XD a) { return XD{-a.m, a.e}; }
NM_HD XD xd_twice(XD a) { return a.m == 0.0 ? a : XD{a.m, a.e + 1}; }

NM_HD XD xd_add(XD a, XD b) {
  if (a.e < b.e) {
    const XD t = a;
    a = b;
    b = t;
  }
  if (b.m == 0.0) return a;
  const int32_t d = a.e - b.e;
  if (d > 60) return a;  // |b| < 2^-59 |a|: below half an ulp of a
  // b.m * 2^-d: set the exponent field of b.m (1023 for [1, 2)) to 1023 - d
  const double bs = xd_from_bits_(xd_bits_(b.m) - ((int64_t)d << 52));
#if defined(__CUDA_ARCH__)
  const double s = __dadd_rn(a.m, bs);
#else
  const double s = a.m + bs;
#endif
  return xd_norm(s, a.e);
}
NM_HD XD xd_sub(XD a, XD b) { return xd_add(a, xd_neg(b)); }

NM_HD XD xd_mul(XD a, XD b) {
#if defined(__CUDA_ARCH__)
  const double p = __dmul_rn(a.m, b.m);
#else
  const double p = a.m * b.m;
#endif
  return xd_norm(p, a.e + b.e);
}

// a > b for a, b >= 0.
NM_HD bool xd_gt(XD a, XD b) { return a.e > b.e || (a.e == b.e && a.m > b.m); }

}  // namespace nmg
