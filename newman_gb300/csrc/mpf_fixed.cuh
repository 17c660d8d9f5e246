// Arbitrary-precision floats with the results of GMP's mpf functions, at a
// precision fixed at compile time -- for the GPU (and the host) to continue
// the reference's per-pixel iteration in the arbitrary precision it uses
// (mandelbrot.cpp:209-224, the gmpxx expressions of complex.h and :102-103)
// and get the same bits.
//
// GMP's mpf functions do not round correctly: each truncates its operands at
// limb boundaries that depend on the destination's precision, then truncates
// the result.  What they compute, for a destination of P limbs of precision
// (GMP's _mp_prec; mpf_init2(x, bits) gives P = (bits + 127) / 64, and a value
// holds up to P + 1 limbs), was established here by calling GMP 6.3.0
// (libgmp.so.10) on millions of structured random operands and comparing
// values limb for limb (tests/native/mpf_conformance.cpp keeps that check):
//
//   mul(u, v)  both operands cut to their top P limbs, exact product, cut to
//              its top P + 1 limbs;
//   add(u, v)  same signs: both cut at limb position E - P, E the larger
//              exponent, exact sum (P + 1 limbs when it carries);
//              opposite signs: leading limbs that cancel exactly are skipped
//              first -- limbs equal in both (equal exponents), then a
//              difference of 1 followed by limb pairs (0, 2^64 - 1), which
//              cancel to a 1 one limb lower -- and both operands are cut
//              P + 1 limbs below the position so reached; exact difference;
//   get_d(x)   x truncated toward zero to a double (into the subnormal
//              range too; +0 when nothing is left, of either sign; infinity
//              beyond the double range);
//   set_d(x)   exact.
//
// A value is sign, limb exponent e and the D = P + 1 limbs d[0..P], most
// significant first, value = sign * sum_i d[i] * 2^(64 (e - 1 - i)), with
// d[0] != 0 unless the value is 0.  Limbs below the value's own are zero;
// trailing zero limbs never change a result (every cut is at a limb position
// fixed by exponents and operand values, not by limb counts).
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define MPF_HD __host__ __device__ __forceinline__
#else
#define MPF_HD inline
#endif

namespace nmg {

template <int P>
struct Mpfx {
  static_assert(P >= 2, "GMP's smallest mpf precision is 2 limbs (64 bits)");
  static constexpr int D = P + 1;
  uint64_t d[D];
  int32_t e;
  int32_t s;  // -1, 0, +1
};

namespace mpf_detail {

MPF_HD void mul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
#if defined(__CUDA_ARCH__)
  lo = a * b;
  hi = __umul64hi(a, b);
#else
  const unsigned __int128 p = (unsigned __int128)a * b;
  lo = (uint64_t)p;
  hi = (uint64_t)(p >> 64);
#endif
}

MPF_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// a + b + c (c in {0, 1}); c becomes the carry out.  On the GPU through the
// hardware carry flag: c sets it (c + 2^64 - 1 carries exactly when c = 1).
MPF_HD uint64_t addc(uint64_t a, uint64_t b, uint64_t& c) {
#if defined(__CUDA_ARCH__)
  uint64_t r;
  asm volatile(
      "{\n\t.reg .u64 t;\n\t"
      "add.cc.u64 t, %2, 0xffffffffffffffff;\n\t"
      "addc.cc.u64 %0, %3, %4;\n\t"
      "addc.u64 %1, 0, 0;\n\t}"
      : "=l"(r), "=l"(c)
      : "l"(c), "l"(a), "l"(b));
  return r;
#else
  const uint64_t t = a + b;
  const uint64_t c1 = t < a;
  const uint64_t u = t + c;
  c = c1 | (uint64_t)(u < t);
  return u;
#endif
}

// a - b - br (br in {0, 1}); br becomes the borrow out.  On the GPU through
// the hardware borrow flag: 0 - br borrows exactly when br = 1.
MPF_HD uint64_t subb(uint64_t a, uint64_t b, uint64_t& br) {
#if defined(__CUDA_ARCH__)
  uint64_t r, bo;
  asm volatile(
      "{\n\t.reg .u64 t;\n\t"
      "sub.cc.u64 t, 0, %2;\n\t"
      "subc.cc.u64 %0, %3, %4;\n\t"
      "subc.u64 %1, 0, 0;\n\t}"
      : "=l"(r), "=l"(bo)
      : "l"(br), "l"(a), "l"(b));
  br = bo ? 1 : 0;  // the borrow out comes as 0 or 2^64 - 1
  return r;
#else
  const uint64_t t = a - b;
  const uint64_t b1 = a < b;
  const uint64_t u = t - br;
  br = b1 | (uint64_t)(t < br);
  return u;
#endif
}

// d[k] for a runtime k, 0 outside [0, D): on the GPU by selects over the
// limbs, so that they stay in registers; on the host by indexing.
template <int D>
MPF_HD uint64_t limb_at(const uint64_t (&d)[D], int k) {
#if defined(__CUDA_ARCH__)
  uint64_t r = 0;
#pragma unroll
  for (int j = 0; j < D; j++) r = (k == j) ? d[j] : r;
  return r;
#else
  return (k >= 0 && k < D) ? d[k] : 0;
#endif
}

}  // namespace mpf_detail

template <int P>
MPF_HD Mpfx<P> mpf_zero() {
  Mpfx<P> r;
#pragma unroll
  for (int i = 0; i < Mpfx<P>::D; i++) r.d[i] = 0;
  r.e = 0;
  r.s = 0;
  return r;
}

template <int P>
MPF_HD Mpfx<P> mpf_neg(Mpfx<P> a) {
  a.s = -a.s;
  return a;
}

// -1, 0, 1 as |a| is below, equal to or above |b|.
template <int P>
MPF_HD int mpf_cmp_abs(const Mpfx<P>& a, const Mpfx<P>& b) {
  if (a.s == 0 || b.s == 0) return (a.s != 0) - (b.s != 0);
  if (a.e != b.e) return a.e < b.e ? -1 : 1;
  int r = 0;
#pragma unroll
  for (int i = 0; i < Mpfx<P>::D; i++)
    if (r == 0 && a.d[i] != b.d[i]) r = a.d[i] < b.d[i] ? -1 : 1;
  return r;
}

// mpf_cmp: -1, 0, 1 as a is below, equal to or above b.
template <int P>
MPF_HD int mpf_cmp(const Mpfx<P>& a, const Mpfx<P>& b) {
  if (a.s != b.s) return a.s < b.s ? -1 : 1;
  const int m = mpf_cmp_abs(a, b);
  return a.s < 0 ? -m : m;
}

// mpf_mul into a destination of P limbs of precision.
template <int P>
MPF_HD Mpfx<P> mpf_mul(const Mpfx<P>& a, const Mpfx<P>& b) {
  using namespace mpf_detail;
  constexpr int D = P + 1;
  if (a.s == 0 || b.s == 0) return mpf_zero<P>();
  // the top P limbs of each, little-endian, and their exact product
  uint64_t r[2 * P];
#pragma unroll
  for (int k = 0; k < 2 * P; k++) r[k] = 0;
#if defined(__CUDA_ARCH__)
  // row i: r[i .. i+P] += a_i * b, the low halves of the products in one
  // carry chain, their high halves in a second (the row's sum fits: the
  // final carry is 0)
#pragma unroll
  for (int i = 0; i < P; i++) {
    const uint64_t ai = a.d[P - 1 - i];
    asm volatile("mad.lo.cc.u64 %0, %1, %2, %0;" : "+l"(r[i]) : "l"(ai), "l"(b.d[P - 1]));
#pragma unroll
    for (int j = 1; j < P; j++)
      asm volatile("madc.lo.cc.u64 %0, %1, %2, %0;"
                   : "+l"(r[i + j])
                   : "l"(ai), "l"(b.d[P - 1 - j]));
    asm volatile("addc.u64 %0, 0, 0;" : "=l"(r[i + P]));
    asm volatile("mad.hi.cc.u64 %0, %1, %2, %0;" : "+l"(r[i + 1]) : "l"(ai), "l"(b.d[P - 1]));
#pragma unroll
    for (int j = 1; j < P - 1; j++)
      asm volatile("madc.hi.cc.u64 %0, %1, %2, %0;"
                   : "+l"(r[i + 1 + j])
                   : "l"(ai), "l"(b.d[P - 1 - j]));
    asm volatile("madc.hi.u64 %0, %1, %2, %0;" : "+l"(r[i + P]) : "l"(ai), "l"(b.d[0]));
  }
#else
#pragma unroll
  for (int i = 0; i < P; i++) {
    const uint64_t ai = a.d[P - 1 - i];
    uint64_t carry = 0;
#pragma unroll
    for (int j = 0; j < P; j++) {
      uint64_t lo, hi;
      mul64(ai, b.d[P - 1 - j], lo, hi);
      uint64_t c = 0;
      lo = addc(lo, r[i + j], c);
      hi += c;
      c = 0;
      lo = addc(lo, carry, c);
      hi += c;
      r[i + j] = lo;
      carry = hi;
    }
    r[i + P] = carry;
  }
#endif
  // top limb zero: one limb lower
  const bool adj = r[2 * P - 1] == 0;
  Mpfx<P> o;
#pragma unroll
  for (int k = 0; k < D; k++) {
    const uint64_t hi = r[2 * P - 1 - k];
    const uint64_t lo = (2 * P - 2 - k >= 0) ? r[(2 * P - 2 - k) >= 0 ? 2 * P - 2 - k : 0] : 0;
    o.d[k] = adj ? lo : hi;
  }
  o.e = a.e + b.e - (adj ? 1 : 0);
  o.s = a.s * b.s;
  return o;
}

// mpf_mul(r, two, a) with two = 2.0: 2 times the top P limbs of a, exactly.
template <int P>
MPF_HD Mpfx<P> mpf_mul2(const Mpfx<P>& a) {
  constexpr int D = P + 1;
  if (a.s == 0) return a;
  Mpfx<P> o;
  const uint64_t top = a.d[0] >> 63;
  if (top) {  // the product gains a limb
    o.d[0] = 1;
#pragma unroll
    for (int k = 1; k < D; k++)
      o.d[k] = (a.d[k - 1] << 1) | ((k < P) ? (a.d[k < P ? k : 0] >> 63) : 0);
    o.e = a.e + 1;
  } else {
#pragma unroll
    for (int k = 0; k < D; k++)
      o.d[k] = (k < P) ? ((a.d[k < P ? k : 0] << 1) | ((k + 1 < P) ? (a.d[k + 1 < P ? k + 1 : 0] >> 63) : 0))
                       : 0;
    o.e = a.e;
  }
  o.s = a.s;
  return o;
}

// mpf_add (and mpf_sub = mpf_add with -b) into a destination of P limbs.
template <int P>
MPF_HD Mpfx<P> mpf_add(const Mpfx<P>& a, const Mpfx<P>& b) {
  using namespace mpf_detail;
  constexpr int D = P + 1;
  if (a.s == 0) return b;
  if (b.s == 0) return a;
  Mpfx<P> o;
  if (a.s == b.s) {
    // both cut at limb position E - P: the top P limbs below E
    const bool a_hi = a.e >= b.e;
    const Mpfx<P>& u = a_hi ? a : b;
    const Mpfx<P>& v = a_hi ? b : a;
    const int off = u.e - v.e;  // v's limb k sits at u's index k + off
    uint64_t sum[P];
    uint64_t c = 0;
#pragma unroll
    for (int i = P - 1; i >= 0; i--) sum[i] = addc(u.d[i], limb_at(v.d, i - off), c);
    if (c) {
      o.d[0] = 1;
#pragma unroll
      for (int k = 1; k < D; k++) o.d[k] = sum[k - 1];
      o.e = u.e + 1;
    } else {
#pragma unroll
      for (int k = 0; k < P; k++) o.d[k] = sum[k];
      o.d[P] = 0;
      o.e = u.e;
    }
    o.s = u.s;
    return o;
  }
  // opposite signs: U the larger magnitude
  const int m = mpf_cmp_abs(a, b);
  if (m == 0) return mpf_zero<P>();
  const Mpfx<P>& U = m > 0 ? a : b;
  const Mpfx<P>& W = m > 0 ? b : a;
  const int off = U.e - W.e;  // W's limb k sits at U's index k + off; off >= 0
  {
    // The common case: U's top limb exceeds W's limb at the same place by 2 or
    // more, so no leading limbs cancel, no borrow chain forms and the window's
    // top word stays at least 1 -- the window below is U's D limbs less W's
    // (t = s0 = z = 0), with U's limbs at fixed indexes.
    const uint64_t top = U.d[0] - (off == 0 ? W.d[0] : 0ull);
    if (top >= 2) {
      uint64_t br = 0;
#pragma unroll
      for (int i = D - 1; i >= 1; i--) o.d[i] = subb(U.d[i], limb_at(W.d, i - off), br);
      o.d[0] = top - br;
      o.e = U.e;
      o.s = U.s;
      return o;
    }
  }
  // first index where the limbs differ (equal exponents: equal leading limbs
  // cancel)
  int t = 0;
  if (off == 0) {
    bool eq = true;
#pragma unroll
    for (int i = 0; i < D; i++) {
      eq = eq && U.d[i] == W.d[i];
      t += eq ? 1 : 0;
    }
  }
  // U[t] - W[t] == 1 followed by (0, 2^64 - 1) pairs: they cancel to a 1 at
  // the last pair's index
  const uint64_t ut = limb_at(U.d, t), wt = limb_at(W.d, t - off);
  int s0 = t;
  uint64_t topw = ut - wt;
  if (topw == 1) {
    int j = t + 1;
    // bounded: W's limbs end D + off indexes down
    for (int k = 0; k < D + 1; k++) {
      if (limb_at(U.d, j) == 0 && limb_at(W.d, j - off) == ~0ull)
        j++;
      else
        break;
    }
    s0 = j - 1;
  }
  // window of D limbs from index s0: the top word is topw (1 after a chain),
  // the D - 1 below are U - W with borrows
  uint64_t w[D];
  uint64_t br = 0;
#pragma unroll
  for (int i = D - 1; i >= 1; i--) w[i] = subb(limb_at(U.d, s0 + i), limb_at(W.d, s0 + i - off), br);
  w[0] = topw - br;
  // normalise: leading zero limbs
  int z = 0;
  bool lead = true;
#pragma unroll
  for (int i = 0; i < D; i++) {
    lead = lead && w[i] == 0;
    z += lead ? 1 : 0;
  }
  if (z == D) return mpf_zero<P>();
#pragma unroll
  for (int k = 0; k < D; k++) o.d[k] = limb_at(w, k + z);
  o.e = U.e - s0 - z;
  o.s = U.s;
  return o;
}

template <int P>
MPF_HD Mpfx<P> mpf_sub(const Mpfx<P>& a, const Mpfx<P>& b) {
  return mpf_add(a, mpf_neg(b));
}

// mpf_get_d: truncation toward zero.
template <int P>
MPF_HD double mpf_get_d(const Mpfx<P>& a) {
  using namespace mpf_detail;
  if (a.s == 0) return 0.0;
  const int lz = clz64(a.d[0]);
  uint64_t m = a.d[0] << lz;  // the top 64 bits, leading bit set
  if (lz) m |= a.d[1] >> (64 - lz);
  const long top = 64L * (a.e - 1) + (63 - lz);  // weight 2^top of the leading bit
  union {
    double f;
    uint64_t u;
  } r;
  if (top > 1023) {
    r.u = 0x7ff0000000000000ull;  // infinity
  } else if (top >= -1022) {      // normal: the top 53 bits
    r.u = ((uint64_t)(top + 1023) << 52) | ((m >> 11) & ((1ull << 52) - 1));
  } else {                        // subnormal: multiples of 2^-1074, truncated
    const long sh = -1074 - (top - 63);
    r.u = sh >= 64 ? 0 : m >> sh;
    if (r.u == 0) return 0.0;
  }
  if (a.s < 0) r.u |= 1ull << 63;
  return r.f;
}

// mpf_get_d_2exp: the value as m * 2^exp with 0.5 <= |m| < 1, m truncated
// toward zero to 53 bits (m = 0, exp = 0 for zero).
template <int P>
MPF_HD double mpf_get_d_2exp(long* exp, const Mpfx<P>& a) {
  using namespace mpf_detail;
  if (a.s == 0) {
    *exp = 0;
    return 0.0;
  }
  const int lz = clz64(a.d[0]);
  uint64_t m = a.d[0] << lz;
  if (lz) m |= a.d[1] >> (64 - lz);
  m >>= 11;
  *exp = 64L * a.e - lz;
  const double x = (double)m * 0x1p-53;
  return a.s < 0 ? -x : x;
}

// mpf_set_d: a finite double exactly.
template <int P>
MPF_HD Mpfx<P> mpf_from_double(double x) {
  Mpfx<P> o = mpf_zero<P>();
  if (x == 0.0) return o;
  union {
    double f;
    uint64_t u;
  } b;
  b.f = x;
  o.s = (b.u >> 63) ? -1 : 1;
  int be = (int)((b.u >> 52) & 0x7ff);
  uint64_t m = b.u & ((1ull << 52) - 1);
  if (be) {
    m |= 1ull << 52;
  } else {
    be = 1;  // subnormal
  }
  // value = m * 2^(be - 1075); top bit of m at bit h
  const int h = 63 - mpf_detail::clz64(m);
  const int top = be - 1075 + h;        // weight 2^top of the leading bit
  const int e = (top >> 6) + 1;         // limb exponent (floor division)
  const int bit = top - 64 * (e - 1);   // leading bit's place in limb e - 1
  const int sh = bit - h;               // m's bit 0 lands at this bit of limb e - 1
  if (sh >= 0) {
    o.d[0] = m << sh;
  } else {
    o.d[0] = m >> (-sh);
    o.d[1] = m << (64 + sh);
  }
  o.e = e;
  return o;
}

// ---- the reference's arbitrary-precision step, gmpxx order -----------------
// computeOrbit / getIterations (mandelbrot.cpp:102-103, :213-214):
//   re = X.re * X.re - X.im * X.im + X0.re;   im = 2.0 * (X.re * X.im) + X0.im
template <int P>
MPF_HD void mpf_orbit_step(const Mpfx<P>& xr, const Mpfx<P>& xi, const Mpfx<P>& x0r,
                           const Mpfx<P>& x0i, Mpfx<P>& nr, Mpfx<P>& ni) {
  const Mpfx<P> t1 = mpf_sub(mpf_mul(xr, xr), mpf_mul(xi, xi));
  const Mpfx<P> t3 = mpf_mul2(mpf_mul(xr, xi));
  nr = mpf_add(t1, x0r);
  ni = mpf_add(t3, x0i);
}

// bailedOut (mandelbrot.cpp:58-61): sqMag(descend(z)) > 1024^2 in doubles,
// unfused.
template <int P>
MPF_HD double mpf_sq_mag_d(const Mpfx<P>& re, const Mpfx<P>& im) {
  const double a = mpf_get_d(re), b = mpf_get_d(im);
#if defined(__CUDA_ARCH__)
  return __dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b));
#else
  volatile double aa = a * a, bb = b * b;
  return aa + bb;
#endif
}
// r2_out, when given, is set where the test returns true.  Components below
// 701 in magnitude (zero, a limb exponent of at most 0, or an integer limb of
// at most 700) decide it without the doubles: get_d truncates toward zero, so
// both doubles are at most 701 and r2 <= 2 * 701^2 (1 + 2^-52)^2 < 2^20.
template <int P>
MPF_HD bool mpf_bailed_out(const Mpfx<P>& re, const Mpfx<P>& im, double* r2_out = nullptr) {
  auto small = [](const Mpfx<P>& x) { return x.s == 0 || x.e <= 0 || (x.e == 1 && x.d[0] <= 700); };
  if (small(re) && small(im)) return false;
  const double r2 = mpf_sq_mag_d(re, im);
  if (r2_out) *r2_out = r2;
  return r2 > 1024.0 * 1024.0;
}

// inCardioid (mandelbrot.cpp:63-71) in the view's precision: fourth and one
// are 0.25 and 1.0.
template <int P>
MPF_HD bool mpf_in_cardioid(const Mpfx<P>& zr, const Mpfx<P>& zi) {
  const Mpfx<P> fourth = mpf_from_double<P>(0.25), one = mpf_from_double<P>(1.0);
  const Mpfx<P> xmf = mpf_sub(zr, fourth);
  const Mpfx<P> y2 = mpf_mul(zi, zi);
  const Mpfx<P> q = mpf_add(mpf_mul(xmf, xmf), y2);
  const Mpfx<P> lhs = mpf_mul(q, mpf_add(q, xmf));
  const Mpfx<P> rhs = mpf_mul(fourth, y2);
  if (mpf_cmp(lhs, rhs) < 0) return true;
  const Mpfx<P> q2 = mpf_add(zr, one);
  const Mpfx<P> lhs2 = mpf_add(mpf_mul(q2, q2), y2);
  return mpf_cmp(lhs2, mpf_mul(fourth, fourth)) < 0;
}

}  // namespace nmg
