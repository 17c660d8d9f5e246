// The FP64 step's shortcut decisions (pixel_fp64.cuh) against the tests they
// stand for, on the host build of the same header: bailout_and_rebase against
// forming r2 = yr^2 + yi^2 and d2 = dr^2 + di^2 and comparing them as the
// reference order does; no_event_before_y against the whole step's tests; the
// double loop's skipped bailout sum.  Seeded structured random operands:
// exponent boundaries, zeros, subnormals, near-equal |Y| and |delta|.
// Prints "... <m> mismatches".
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "pixel_fp64.cuh"

using namespace nmg;

static double bailout2 = 1024.0 * 1024.0;

// the tests as delta_steps made them before the shortcuts
static int reference_event(double yr, double yi, double dr, double di, bool last, double& r2) {
  r2 = add_(mul_(yr, yr), mul_(yi, yi));
  if (above_bits(r2, bailout2)) return 2;
  if (last) return 1;
  if (clearly_larger(yr, yi, dr, di)) return 0;
  return above_bits(add_(mul_(dr, dr), mul_(di, di)), r2) ? 1 : 0;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
  std::mt19937_64 g(argc > 2 ? std::atoll(argv[2]) : 1);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  auto scale = [&](int lo, int hi) {
    return std::ldexp(1.0, (int)(lo + (long)(g() % (unsigned long)(hi - lo + 1))));
  };
  auto pick = [&](double s) {
    switch (g() % 8) {
      case 0: return 0.0;
      case 1: return u(g) * 4.9e-324 * (double)(g() % 5);  // subnormal
      default: return u(g) * s;
    }
  };
  long checks = 0, bad = 0, estimated = 0, skipped_y = 0;
  for (long k = 0; k < n; k++) {
    // Y and delta: random scales, or delta near |Y| (the rebase test's edge)
    const double sy = scale(-80, 12), sd = (g() % 3 == 0) ? sy : scale(-80, 12);
    double yr = pick(sy), yi = pick(sy), dr = pick(sd), di = pick(sd);
    if (g() % 4 == 0) {  // |delta| within a few ulp of |Y|
      const double f = 1.0 + u(g) * std::ldexp(1.0, -(int)(g() % 40));
      dr = yr * f;
      di = yi * f;
      if (g() % 2) std::swap(dr, di);
    }
    if (g() % 16 == 0) {  // around the bailout radius and the 2^8 boundary
      yr = std::ldexp(1.0, 8) * (1.0 + u(g) * 1e-3);
      yi = u(g) * 724.1;
    }
    const bool last = g() % 50 == 0;
    double r2a = -1.0, r2b = -1.0;
    const int a = bailout_and_rebase(yr, yi, dr, di, last, bailout2, r2a);
    const int b = reference_event(yr, yi, dr, di, last, r2b);
    checks++;
    if (a != b || (a == 2 && r2a != r2b)) {
      if (bad++ < 10)
        std::printf("bailout_and_rebase: Y (%a, %a) delta (%a, %a) last %d: %d, reference %d\n",
                    yr, yi, dr, di, (int)last, a, b);
    }
    // the FP32 estimate on its own, where it decides
    const int q = rebase_by_estimate(yr, yi, dr, di);
    if (q >= 0) {
      estimated++;
      checks++;
      const double r2 = add_(mul_(yr, yr), mul_(yi, yi));
      const int e = above_bits(add_(mul_(dr, dr), mul_(di, di)), r2) ? 1 : 0;
      if (q != e && bad++ < 10)
        std::printf("rebase_by_estimate: Y (%a, %a) delta (%a, %a): %d, exact %d\n", yr, yi, dr,
                    di, q, e);
    }
    // no_event_before_y: Z and the new delta
    const Dbl2 zn{pick(scale(-20, 8)), pick(scale(-20, 8))};
    const double nr = pick(scale(-40, 8)), ni = pick(scale(-40, 8));
    if (no_event_before_y(zn, nr, ni)) {
      skipped_y++;
      double r2;
      const double y1 = add_(zn.x, nr), y2 = add_(zn.y, ni);
      checks++;
      if (reference_event(y1, y2, nr, ni, false, r2) != 0) {
        if (bad++ < 10)
          std::printf("no_event_before_y: Z (%a, %a) delta (%a, %a)\n", zn.x, zn.y, nr, ni);
      }
    }
    // the double loop: both squares below 2^19 never bail out
    const double zr = u(g) * 800.0, zi = u(g) * 800.0;
    const double sr = mul_(zr, zr), si = mul_(zi, zi);
    if (exp_field(sr) < 1042 && exp_field(si) < 1042) {
      checks++;
      if (above_bits(add_(sr, si), bailout2)) {
        if (bad++ < 10) std::printf("double loop: z (%a, %a)\n", zr, zi);
      }
    }
  }
  std::printf("%ld checks (%ld decided by the estimate, %ld steps without Y), %ld mismatches\n",
              checks, estimated, skipped_y, bad);
  return bad ? 1 : 0;
}
