// Conformance of newman_gb300/csrc/mpf_fixed.cuh (host build) with GMP's mpf
// functions in the runtime library libgmp.so.10: every operation the
// reference's per-pixel arithmetic uses (mpf_mul, mpf_add, mpf_sub with the
// gmpxx temporaries at the destination's precision, 2.0 * x, mpf_get_d,
// mpf_set_d, mpf_cmp), on structured random operands -- limbs of 0, 1,
// 2^63, 2^64 - 1 and random, exponents a few limbs apart, operands that
// cancel in whole limbs -- and whole orbits of the reference's step
// (mandelbrot.cpp:102-103) from random starting points near the set's
// boundary.  Results are compared as values, limb for limb.
//
// Test infrastructure: built and run by tests/test_mpf_fixed.py.
// Usage: mpf_conformance [cases_per_precision] [seed]; exit status 0 when
// every result agrees.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "gmp_abi.h"
#include "mpf_fixed.cuh"

using nmg::Mpfx;

namespace {

std::mt19937_64 rng;
long failures = 0, checked = 0;

uint64_t rand_limb() {
  switch (rng() % 7) {
    case 0: return 0;
    case 1: return ~0ull;
    case 2: return 1;
    case 3: return 1ull << 63;
    case 4: return rng() >> (rng() % 64);
    default: return rng();
  }
}

template <int P>
Mpfx<P> rand_mpf(int max_limbs, int exp_lo, int exp_hi) {
  Mpfx<P> x = nmg::mpf_zero<P>();
  const int n = 1 + (int)(rng() % (unsigned)(max_limbs < Mpfx<P>::D ? max_limbs : Mpfx<P>::D));
  for (int i = 0; i < n; i++) x.d[i] = rand_limb();
  if (x.d[0] == 0) x.d[0] = 1 + (rng() & 0xffff);
  x.e = exp_lo + (int)(rng() % (unsigned)(exp_hi - exp_lo + 1));
  x.s = (rng() & 1) ? 1 : -1;
  return x;
}

// A value close to x: some limbs replaced, or the (1, 0..0) / (0, ff..ff)
// pattern that cancels with borrows.
template <int P>
Mpfx<P> near(const Mpfx<P>& x) {
  Mpfx<P> y = x;
  const int kind = (int)(rng() % 3);
  if (kind == 0) {
    for (int i = 0; i < Mpfx<P>::D; i++)
      if (rng() % 3 == 0) y.d[i] = rand_limb();
  } else {
    const int at = (int)(rng() % Mpfx<P>::D);
    if (y.d[at] == 0) y.d[at] = 1;
    y.d[at] -= 1;
    for (int i = at + 1; i < Mpfx<P>::D; i++) y.d[i] = (rng() % 5) ? ~0ull : rand_limb();
    if (kind == 2 && at == 0 && y.d[0] == 0) {  // across the exponent step
      for (int i = 0; i + 1 < Mpfx<P>::D; i++) y.d[i] = y.d[i + 1];
      y.d[Mpfx<P>::D - 1] = rand_limb();
      y.e -= 1;
    }
  }
  if (y.d[0] == 0) y.d[0] = 3;
  return y;
}

struct G {  // an mpf_t with capacity for any operand here
  mpf_t v;
  explicit G(unsigned long bits) { mpf_init2(v, bits); }
  ~G() { mpf_clear(v); }
};

template <int P>
void to_gmp(const Mpfx<P>& x, mpf_ptr g) {
  int n = Mpfx<P>::D;
  while (n > 0 && x.d[n - 1] == 0) n--;
  if (x.s == 0 || n == 0) {
    g->_mp_size = 0;
    g->_mp_exp = 0;
    return;
  }
  for (int i = 0; i < n; i++) g->_mp_d[n - 1 - i] = x.d[i];
  g->_mp_size = x.s < 0 ? -n : n;
  g->_mp_exp = x.e;
}

template <int P>
bool same(mpf_srcptr g, const Mpfx<P>& x) {
  int n = g->_mp_size < 0 ? -g->_mp_size : g->_mp_size;
  const int s = g->_mp_size < 0 ? -1 : (g->_mp_size > 0);
  // GMP may keep low zero limbs; compare values
  uint64_t gd[64] = {0};
  for (int i = 0; i < n && i < 64; i++) gd[i] = g->_mp_d[n - 1 - i];
  while (n > 0 && gd[n - 1] == 0) n--;
  if (n == 0) return x.s == 0;
  if (x.s != s || x.e != g->_mp_exp || n > Mpfx<P>::D) return false;
  for (int i = 0; i < Mpfx<P>::D; i++)
    if (x.d[i] != (i < n ? gd[i] : 0)) return false;
  return true;
}

template <int P>
void report(const char* op, const Mpfx<P>& a, const Mpfx<P>& b, mpf_srcptr g, const Mpfx<P>& m) {
  if (++failures > 10) return;
  std::printf("MISMATCH P=%d %s\n", P, op);
  auto show = [](const char* t, int s, long e, const uint64_t* d, int n) {
    std::printf("  %s s=%d e=%ld [", t, s, e);
    for (int i = 0; i < n; i++) std::printf(" %016llx", (unsigned long long)d[i]);
    std::printf(" ]\n");
  };
  show("a", a.s, a.e, a.d, Mpfx<P>::D);
  show("b", b.s, b.e, b.d, Mpfx<P>::D);
  uint64_t gd[64] = {0};
  const int n = g->_mp_size < 0 ? -g->_mp_size : g->_mp_size;
  for (int i = 0; i < n && i < 64; i++) gd[i] = g->_mp_d[n - 1 - i];
  show("gmp", g->_mp_size < 0 ? -1 : (g->_mp_size > 0), g->_mp_exp, gd, n);
  show("here", m.s, m.e, m.d, Mpfx<P>::D);
}

template <int P>
void check_ops(long cases) {
  const unsigned long bits = 64ul * (P - 1);  // mpf_init2 precision giving P limbs
  G r(bits), u(64 * 80), v(64 * 80), two(64);
  if (r.v->_mp_prec != P) {
    std::printf("precision mapping: %lu bits gave %d limbs, expected %d\n", bits, r.v->_mp_prec, P);
    failures++;
    return;
  }
  mpf_set_d(two.v, 2.0);
  for (long it = 0; it < cases; it++) {
    Mpfx<P> a = rand_mpf<P>(Mpfx<P>::D, -3, 3);
    Mpfx<P> b = (rng() % 2) ? near(a) : rand_mpf<P>(Mpfx<P>::D, a.e - 3, a.e + 1);
    if (rng() % 4 == 0) b.s = -a.s;
    if (rng() % 16 == 0) b = nmg::mpf_zero<P>();
    to_gmp(a, u.v);
    to_gmp(b, v.v);
    // mul
    mpf_mul(r.v, u.v, v.v);
    Mpfx<P> m = nmg::mpf_mul(a, b);
    checked++;
    if (!same(r.v, m)) report("mul", a, b, r.v, m);
    // add
    mpf_add(r.v, u.v, v.v);
    m = nmg::mpf_add(a, b);
    checked++;
    if (!same(r.v, m)) report("add", a, b, r.v, m);
    // sub
    mpf_sub(r.v, u.v, v.v);
    m = nmg::mpf_sub(a, b);
    checked++;
    if (!same(r.v, m)) report("sub", a, b, r.v, m);
    // 2.0 * a
    mpf_mul(r.v, two.v, u.v);
    m = nmg::mpf_mul2(a);
    checked++;
    if (!same(r.v, m)) report("mul2", a, b, r.v, m);
    // cmp
    const int gc = mpf_cmp(u.v, v.v), hc = nmg::mpf_cmp(a, b);
    checked++;
    if ((gc > 0) - (gc < 0) != hc) {
      if (++failures <= 10) std::printf("MISMATCH P=%d cmp\n", P);
    }
    // get_d_2exp (any exponent)
    {
      long ge = 0, he = 0;
      const double gm = mpf_get_d_2exp(&ge, u.v), hm = nmg::mpf_get_d_2exp(&he, a);
      checked++;
      if ((std::memcmp(&gm, &hm, 8) != 0 || ge != he) && ++failures <= 10)
        std::printf("MISMATCH P=%d get_d_2exp %a %ld / %a %ld\n", P, gm, ge, hm, he);
    }
    // get_d, also below and above the double range
    {
      if (rng() % 4 == 0) {
        a.e = (rng() & 1) ? -14 - (int)(rng() % 6) : 14 + (int)(rng() % 4);
        to_gmp(a, u.v);
      }
      const double gd = mpf_get_d(u.v), hd = nmg::mpf_get_d(a);
      checked++;
      if (std::memcmp(&gd, &hd, 8) != 0 && ++failures <= 10)
        std::printf("MISMATCH P=%d get_d %a %a\n", P, gd, hd);
    }
  }
  // set_d
  for (long it = 0; it < cases / 4; it++) {
    double x;
    const uint64_t bitsx = rng();
    std::memcpy(&x, &bitsx, 8);
    if (!std::isfinite(x)) continue;
    if (rng() % 2) x = std::ldexp((double)(rng() >> 11), (int)(rng() % 200) - 150);
    mpf_set_d(r.v, x);
    const Mpfx<P> m = nmg::mpf_from_double<P>(x);
    checked++;
    if (!same(r.v, m)) {
      if (++failures <= 10) std::printf("MISMATCH P=%d set_d %a\n", P, x);
    }
  }
}

// Whole orbits: X <- X^2 + c in the reference's gmpxx order, GMP and here,
// from c near the boundary, compared at every step.
template <int P>
void check_orbits(int orbits, int steps) {
  const unsigned long bits = 64ul * (P - 1);
  G xr(bits), xi(bits), cr(bits), ci(bits), t1(bits), t2(bits), t3(bits), nr(bits), ni(bits),
      two(64);
  mpf_set_d(two.v, 2.0);
  for (int k = 0; k < orbits; k++) {
    // c = a point near the boundary (a seahorse-valley neighbourhood), with
    // random low limbs below the double
    const double base_r = -0.7436438870371510 + std::ldexp((double)(int64_t)(rng() >> 20), -60);
    const double base_i = 0.1318259042053300 + std::ldexp((double)(int64_t)(rng() >> 20), -60);
    Mpfx<P> hr = nmg::mpf_from_double<P>(base_r), hi = nmg::mpf_from_double<P>(base_i);
    for (int i = 2; i < Mpfx<P>::D; i++) {
      hr.d[i] = rng();
      hi.d[i] = rng();
    }
    to_gmp(hr, cr.v);
    to_gmp(hi, ci.v);
    mpf_set(xr.v, cr.v);
    mpf_set(xi.v, ci.v);
    Mpfx<P> zr = hr, zi = hi;
    for (int i = 0; i < steps; i++) {
      mpf_mul(t1.v, xr.v, xr.v);
      mpf_mul(t2.v, xi.v, xi.v);
      mpf_sub(t1.v, t1.v, t2.v);
      mpf_mul(t3.v, xr.v, xi.v);
      mpf_mul(t3.v, two.v, t3.v);
      mpf_add(nr.v, t1.v, cr.v);
      mpf_add(ni.v, t3.v, ci.v);
      Mpfx<P> mr, mi;
      nmg::mpf_orbit_step(zr, zi, hr, hi, mr, mi);
      checked++;
      if (!same(nr.v, mr) || !same(ni.v, mi)) {
        if (++failures <= 10) std::printf("MISMATCH P=%d orbit %d step %d\n", P, k, i);
        break;
      }
      const bool gb = mpf_get_d(nr.v) * mpf_get_d(nr.v) + mpf_get_d(ni.v) * mpf_get_d(ni.v) >
                      1024.0 * 1024.0;
      if (gb != nmg::mpf_bailed_out(mr, mi)) {
        if (++failures <= 10) std::printf("MISMATCH P=%d bailout %d step %d\n", P, k, i);
        break;
      }
      if (gb) break;
      mpf_set(xr.v, nr.v);
      mpf_set(xi.v, ni.v);
      zr = mr;
      zi = mi;
    }
  }
}

template <int P>
void check(long cases, int orbits, int steps) {
  check_ops<P>(cases);
  check_orbits<P>(orbits, steps);
}

}  // namespace

int main(int argc, char** argv) {
  const long cases = argc > 1 ? std::atol(argv[1]) : 200000;
  rng.seed(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 2026);
  check<2>(cases, 200, 4000);
  check<3>(cases, 100, 4000);
  check<4>(cases, 50, 4000);
  check<5>(cases / 2, 20, 2000);
  check<8>(cases / 2, 20, 2000);
  check<12>(cases / 4, 10, 1000);
  check<18>(cases / 4, 10, 1000);
  check<19>(cases / 4, 10, 1000);
  std::printf("%ld checks, %ld mismatches\n", checked, failures);
  return failures ? 1 : 0;
}
