// Host-side arbitrary-precision work of one render.  Everything here is
// per-view or per-row/column, never per-pixel: the view arithmetic of the
// reference's `Mandelbrot` (mandelbrot.cpp:8-56, 285-316), the reference
// orbit and series coefficients (mandelbrot.cpp:73-131), and their FP64
// export for the GPU.  The arbitrary-precision operations are GMP mpf calls in
// the same order and at the same precision as the reference's gmpxx
// expressions, so the exported doubles are the values the reference reads.
#include "mpview.hpp"

#include "mpf_fixed.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>

namespace nmg {
namespace {

constexpr double kBailout2 = 1024.0 * 1024.0;  // mandelbrot.cpp:58-59

inline bool bailed_out(mpf_srcptr re, mpf_srcptr im) {  // mandelbrot.cpp:61
  double x = mpf_get_d(re), y = mpf_get_d(im);
  return x * x + y * y > kBailout2;
}

// Temporaries of one z^2 + c / series step at the working precision.
struct StepTemps {
  Mpf t1, t2, t3, two, one;
  explicit StepTemps(unsigned long bits) : t1(bits), t2(bits), t3(bits), two(64), one(64) {
    mpf_set_d(two.p(), 2.0);
    mpf_set_d(one.p(), 1.0);
  }
};

// (nre, nim) = (xr^2 - xi^2 + cr, 2.0 * (xr * xi) + ci), the reference's
// grouping (mandelbrot.cpp:102-103).
inline void square_add(mpf_ptr nre, mpf_ptr nim, mpf_srcptr xr, mpf_srcptr xi, mpf_srcptr cr,
                       mpf_srcptr ci, StepTemps& s) {
  mpf_mul(s.t1.p(), xr, xr);
  mpf_mul(s.t2.p(), xi, xi);
  mpf_sub(s.t1.p(), s.t1.p(), s.t2.p());
  mpf_mul(s.t3.p(), xr, xi);
  mpf_mul(s.t3.p(), s.two.p(), s.t3.p());
  mpf_add(nre, s.t1.p(), cr);
  mpf_add(nim, s.t3.p(), ci);
}

// Orbit length of computeOrbit(c) (mandelbrot.cpp:97-110) without storing it.
int orbit_length(mpf_srcptr cr, mpf_srcptr ci, int N, unsigned long bits) {
  StepTemps s(bits);
  Mpf ar(bits), ai(bits), br(bits), bi(bits);
  mpf_set(ar.p(), cr);
  mpf_set(ai.p(), ci);
  for (int i = 1; i < N; i++) {
    square_add(br.p(), bi.p(), ar.p(), ai.p(), cr, ci, s);
    if (bailed_out(br.p(), bi.p())) return i;
    ar.swap(br);
    ai.swap(bi);
  }
  return N;
}

// ---- the same arithmetic on fixed-precision limbs (mpf_fixed.cuh) -----------
// GMP's results bit for bit without a library call per operation: the probe
// search, the winner's orbit and its series run here for precisions of
// kFixedMinP .. kFixedMaxP limbs (64 .. 448 bits); above, GMP's own
// multiplication is the faster (measured on the 1e-300 view's orbit and
// series: 314 bits 0.19 s here against 0.24 s with GMP, 600 bits 0.65 s
// against 0.50 s, 1100 bits 2.5 s against 1.6 s).
constexpr int kFixedMinP = 2, kFixedMaxP = 8;

template <int P>
Mpfx<P> fixed_of(mpf_srcptr x) {
  Mpfx<P> r = mpf_zero<P>();
  const int size = x->_mp_size;
  const int n = size < 0 ? -size : size;
  if (n == 0) return r;
  for (int i = 0; i < Mpfx<P>::D && i < n; i++) r.d[i] = x->_mp_d[n - 1 - i];
  r.e = (int32_t)x->_mp_exp;
  r.s = size < 0 ? -1 : 1;
  return r;
}

template <int P>
void record_of(const Mpfx<P>& x, uint64_t* out) {
  out[0] = ((uint64_t)(uint32_t)(x.s ? x.e : 0) << 32) | (uint32_t)x.s;
  for (int i = 0; i < Mpfx<P>::D; i++) out[1 + i] = x.d[i];
}

template <int P>
int fixed_orbit_length(const Mpfx<P>& cr, const Mpfx<P>& ci, int N) {
  Mpfx<P> xr = cr, xi = ci;
  for (int i = 1; i < N; i++) {
    Mpfx<P> nr, ni;
    mpf_orbit_step(xr, xi, cr, ci, nr, ni);
    if (mpf_bailed_out(nr, ni)) return i;
    xr = nr;
    xi = ni;
  }
  return N;
}

// get_d of a complex value as floatexp with one exponent (cfe_of below).
template <int P>
CFE fixed_cfe(const Mpfx<P>& re, const Mpfx<P>& im) {
  long er = 0, ei = 0;
  const double dr = mpf_get_d_2exp(&er, re), di = mpf_get_d_2exp(&ei, im);
  if (dr == 0.0 && di == 0.0) return {0.0, 0.0, 0};
  const long e = dr == 0.0 ? ei : di == 0.0 ? er : std::max(er, ei);
  return {std::ldexp(dr, (int)(er - e)), std::ldexp(di, (int)(ei - e)), (int32_t)e};
}

// The winner's orbit X and series A, B, C (mandelbrot.cpp:97-131) in one pass,
// exported as MPView::precompute's GMP loop exports them.  Returns true when
// the orbit escaped (its escaped element then ends od.z).
template <int P>
bool fixed_orbit_series(mpf_srcptr cr_g, mpf_srcptr ci_g, int N, OrbitData& od, bool keep_mp) {
  const Mpfx<P> cr = fixed_of<P>(cr_g), ci = fixed_of<P>(ci_g);
  const Mpfx<P> one = mpf_from_double<P>(1.0);
  Mpfx<P> xr = cr, xi = ci;
  Mpfx<P> ar = one, ai = mpf_zero<P>(), br = mpf_zero<P>(), bi = mpf_zero<P>();
  Mpfx<P> c_r = mpf_zero<P>(), c_i = mpf_zero<P>();
  const int w = mp_record_words(Mpfx<P>::D);
  auto split = [](const Mpfx<P>& v, double& hi, double& lo) {
    hi = mpf_get_d(v);
    lo = mpf_get_d(mpf_sub(v, mpf_from_double<P>(hi)));
  };
  Mpfx<P> nxr, nxi;
  for (int i = 0;; i++) {
    D2 hi, lo;
    split(xr, hi.x, lo.x);
    split(xi, hi.y, lo.y);
    od.xhi.push_back(hi);
    od.xlo.push_back(lo);
    od.z.push_back(hi);
    if (keep_mp) {
      const size_t at = od.xmp.size();
      od.xmp.resize(at + 2 * (size_t)w);
      record_of(xr, &od.xmp[at]);
      record_of(xi, &od.xmp[at + w]);
    }
    od.a.push_back({mpf_get_d(ar), mpf_get_d(ai)});
    od.b.push_back({mpf_get_d(br), mpf_get_d(bi)});
    od.c.push_back({mpf_get_d(c_r), mpf_get_d(c_i)});
    od.a_fe.push_back(fixed_cfe(ar, ai));
    od.b_fe.push_back(fixed_cfe(br, bi));
    od.c_fe.push_back(fixed_cfe(c_r, c_i));
    if (i + 1 >= N) return false;  // X.resize(N) is full
    mpf_orbit_step(xr, xi, cr, ci, nxr, nxi);
    if (mpf_bailed_out(nxr, nxi)) {
      od.z.push_back({mpf_get_d(nxr), mpf_get_d(nxi)});  // the element that escaped
      return true;
    }
    // A, B, C at i + 1 from X[i] in the reference's grouping (:122-129)
    const Mpfx<P> nar = mpf_add(mpf_mul2(mpf_sub(mpf_mul(xr, ar), mpf_mul(xi, ai))), one);
    const Mpfx<P> nai = mpf_mul2(mpf_add(mpf_mul(xr, ai), mpf_mul(xi, ar)));
    const Mpfx<P> nbr = mpf_sub(
        mpf_add(mpf_mul2(mpf_sub(mpf_mul(xr, br), mpf_mul(xi, bi))), mpf_mul(nar, nar)),
        mpf_mul(nai, nai));
    const Mpfx<P> nbi = mpf_mul2(
        mpf_add(mpf_add(mpf_mul(xr, bi), mpf_mul(xi, br)), mpf_mul(nar, nai)));
    const Mpfx<P> ncr = mpf_mul2(mpf_sub(
        mpf_add(mpf_sub(mpf_mul(xr, c_r), mpf_mul(xi, c_i)), mpf_mul(nar, nbr)),
        mpf_mul(nai, nbi)));
    const Mpfx<P> nci = mpf_mul2(mpf_add(
        mpf_add(mpf_add(mpf_mul(xr, c_i), mpf_mul(xi, c_r)), mpf_mul(nar, nbi)),
        mpf_mul(nai, nbr)));
    ar = nar; ai = nai;
    br = nbr; bi = nbi;
    c_r = ncr; c_i = nci;
    xr = nxr;
    xi = nxi;
  }
}

// Probe lengths and the winner's orbit and series at P limbs: probe k's
// coordinates are (pr[k], pi[k]).
template <int P>
void fixed_probe_lengths(const std::vector<Mpf>& pr, const std::vector<Mpf>& pi, int N,
                         int threads, std::vector<int>& len) {
  std::atomic<size_t> next{0};
  auto worker = [&]() {
    for (;;) {
      const size_t k = next.fetch_add(1);
      if (k >= pr.size()) break;
      len[k] = fixed_orbit_length(fixed_of<P>(pr[k].p()), fixed_of<P>(pi[k].p()), N);
    }
  };
  const int T = std::max(1, std::min<int>(threads, (int)pr.size()));
  std::vector<std::thread> pool;
  for (int t = 1; t < T; t++) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
}

template <int P>
bool fixed_dispatch(int p, const std::vector<Mpf>& pr, const std::vector<Mpf>& pi, int N,
                    int threads, std::vector<int>& len, mpf_srcptr* winner, OrbitData* od,
                    bool keep_mp, bool* escaped) {
  if constexpr (P > kFixedMaxP) {
    return false;
  } else {
    if (p != P)
      return fixed_dispatch<P + 1>(p, pr, pi, N, threads, len, winner, od, keep_mp, escaped);
    if (!winner)
      fixed_probe_lengths<P>(pr, pi, N, threads, len);
    else
      *escaped = fixed_orbit_series<P>(winner[0], winner[1], N, *od, keep_mp);
    return true;
  }
}

// Interval arithmetic in double with outward slack, for the view-box
// cardioid classification.
struct Iv {
  double lo, hi;
};
inline Iv widen(Iv a) {
  double m = std::max(std::fabs(a.lo), std::fabs(a.hi)) * 4e-16 + 1e-300;
  return {a.lo - m, a.hi + m};
}
inline Iv iadd(Iv a, Iv b) { return widen({a.lo + b.lo, a.hi + b.hi}); }
inline Iv isub(Iv a, Iv b) { return widen({a.lo - b.hi, a.hi - b.lo}); }
inline Iv imul(Iv a, Iv b) {
  double p[4] = {a.lo * b.lo, a.lo * b.hi, a.hi * b.lo, a.hi * b.hi};
  return widen({*std::min_element(p, p + 4), *std::max_element(p, p + 4)});
}
inline Iv isq(Iv a) {
  if (a.lo >= 0) return widen({a.lo * a.lo, a.hi * a.hi});
  if (a.hi <= 0) return widen({a.hi * a.hi, a.lo * a.lo});
  return widen({0.0, std::max(a.lo * a.lo, a.hi * a.hi)});
}

}  // namespace

MPView::MPView(int nr, int nc) : nr_(nr), nc_(nc) {
  // mandelbrot.cpp:8-17
  mpf_set_d(cre_.p(), -0.5);
  mpf_set_d(cim_.p(), 0.0);
  mpf_set_d(sre_.p(), 4.0 / nc);
  mpf_set_d(sim_.p(), 3.0 / nr);
  set_precision();
}

void MPView::set_precision() {
  // bits = max(64, (int)(64 - e + log2(1e-20))), sz.re = m 2^e, 0.5 <= |m| < 1
  const double log_alpha = std::log2(1.0e-20);
  long e = 0;
  mpf_get_d_2exp(&e, sre_.p());
  int b = (int)(64 - e + log_alpha);
  if (b < 64) b = 64;
  if ((unsigned long)b < min_bits_) b = (int)min_bits_;
  bits_ = (unsigned long)b;
  mpf_set_prec(cre_.p(), bits_);
  mpf_set_prec(cim_.p(), bits_);
  mpf_set_prec(sre_.p(), bits_);
  mpf_set_prec(sim_.p(), bits_);
}

int MPView::set_view(const char* cre, const char* cim, const char* sre, const char* sim, int N,
                     double tol, int min_bits) {
  if (!cre || !cim || !sre || !sim || N < 1 || !(tol >= 0.0)) return 1;
  Mpf probe(4096);
  if (mpf_set_str(probe.p(), sre, 10) != 0) return 2;
  Mpf t(64);
  if (mpf_set_str(t.p(), cre, 10) != 0 || mpf_set_str(t.p(), cim, 10) != 0 ||
      mpf_set_str(t.p(), sim, 10) != 0)
    return 2;
  min_bits_ = min_bits > 0 ? (unsigned long)min_bits : 0;
  no_hardware_ = false;
  mpf_set_prec(sre_.p(), 4096);
  mpf_set(sre_.p(), probe.p());
  set_precision();
  mpf_set_str(cre_.p(), cre, 10);
  mpf_set_str(cim_.p(), cim, 10);
  mpf_set_str(sre_.p(), sre, 10);
  mpf_set_str(sim_.p(), sim, 10);
  N_ = N;
  tol_ = tol;
  return 0;
}

void MPView::set_iterations(int N) { N_ = N; }

bool MPView::use_hardware() const {
  const double minpreview = 1.5e-16;
  return !no_hardware_ && sre_.d() >= minpreview && sim_.d() >= minpreview;
}

void MPView::scale_up(int sc) {
  nr_ *= sc;
  nc_ *= sc;
  mpf_div_ui(sre_.p(), sre_.p(), (unsigned long)sc);  // sz.re = sz.re / sc
  mpf_div_ui(sim_.p(), sim_.p(), (unsigned long)sc);
  set_precision();
}

void MPView::scale_down(int sc) {
  nr_ /= sc;
  nc_ /= sc;
  mpf_mul_ui(sre_.p(), sre_.p(), (unsigned long)sc);  // sz.re = sz.re * sc
  mpf_mul_ui(sim_.p(), sim_.p(), (unsigned long)sc);
  set_precision();
}

// out = base + k * step for a signed machine integer k (gmpxx's int * mpf_class
// goes through mpf_mul_ui and a negation).
static void offset(mpf_ptr out, mpf_srcptr base, long k, mpf_srcptr step, mpf_ptr tmp, bool sub) {
  mpf_mul_ui(tmp, step, (unsigned long)(k < 0 ? -k : k));
  if (k < 0) mpf_neg(tmp, tmp);
  if (sub)
    mpf_sub(out, base, tmp);
  else
    mpf_add(out, base, tmp);
}

void MPView::coord_re(int c, Mpf& out, Mpf& tmp) const {
  offset(out.p(), cre_.p(), (long)c - nc_ / 2, sre_.p(), tmp.p(), false);
}
void MPView::coord_im(int r, Mpf& out, Mpf& tmp) const {
  offset(out.p(), cim_.p(), (long)(nr_ / 2) - r - 1, sim_.p(), tmp.p(), false);
}

void MPView::point_at(int r, int c, int sc, Mpf& re, Mpf& im) const {
  Mpf tmp(bits_);
  mpf_set_prec(re.p(), bits_);
  mpf_set_prec(im.p(), bits_);
  offset(re.p(), cre_.p(), (long)sc * c - nc_ / 2, sre_.p(), tmp.p(), false);
  offset(im.p(), cim_.p(), (long)(nr_ / 2) - (long)sc * r - 1, sim_.p(), tmp.p(), false);
}

void MPView::translate(int dr, int dc, int sc) {
  Mpf tmp(bits_);
  // center.re = center.re - dc * sc * sz.re; center.im = center.im + dr * sc * sz.im
  offset(cre_.p(), cre_.p(), (long)dc * sc, sre_.p(), tmp.p(), true);
  offset(cim_.p(), cim_.p(), (long)dr * sc, sim_.p(), tmp.p(), false);
}

void MPView::zoom(float scale) {
  Mpf f(64);
  mpf_set_d(f.p(), 1.0 / scale);  // sz *= (1.0 / scale)
  mpf_mul(sre_.p(), sre_.p(), f.p());
  mpf_mul(sim_.p(), sim_.p(), f.p());
  set_precision();
}

void MPView::zoom_at(float scale, int r, int c, int sc) {
  Mpf pre(bits_), pim(bits_), tmp(bits_), f(64);
  point_at(r, c, sc, pre, pim);
  mpf_set_d(f.p(), 1.0 / scale);
  mpf_mul(sre_.p(), sre_.p(), f.p());
  mpf_mul(sim_.p(), sim_.p(), f.p());
  offset(cre_.p(), pre.p(), (long)sc * c - nc_ / 2, sre_.p(), tmp.p(), true);
  offset(cim_.p(), pim.p(), (long)(nr_ / 2) - (long)sc * r - 1, sim_.p(), tmp.p(), true);
  set_precision();
}

int MPView::load_legacy(const char* path) {
  FILE* fp = std::fopen(path, "r");
  if (!fp) return 1;  // the reference ignores a missing file; the caller reports it
  char buf[4096];
  int n = 0;
  int ok = std::fscanf(fp, "%d\n", &n) == 1;
  Mpf* dst[4] = {&cre_, &cim_, &sre_, &sim_};
  for (int k = 0; ok && k < 4; k++) {
    ok = std::fscanf(fp, "%4095s\n", buf) == 1;
    // parsed at the precision the field already has (gmpxx assignment)
    if (ok) ok = mpf_set_str(dst[k]->p(), buf, 10) == 0;
  }
  std::fclose(fp);
  if (!ok) return 2;
  N_ = n;
  no_hardware_ = false;  // a loaded view is nobody's preview
  Mpf f(64);
  mpf_set_d(f.p(), 800.0 / nc_);
  mpf_mul(sre_.p(), sre_.p(), f.p());
  mpf_set_d(f.p(), 600.0 / nr_);
  mpf_mul(sim_.p(), sim_.p(), f.p());
  set_precision();
  return 0;
}

std::string MPView::to_string(const Mpf& f) {
  mp_exp_t e;
  char* s = mpf_get_str(nullptr, &e, 10, 0, f.p());
  std::string out;
  if (s[0] == 0)
    out = "0";
  else if (s[0] == '-')
    out = std::string("-0.") + (s + 1) + "e" + std::to_string((long)e);
  else
    out = std::string("0.") + s + "e" + std::to_string((long)e);
  std::free(s);
  return out;
}

int MPView::save(const char* path) const {
  FILE* fp = std::fopen(path, "w");
  if (!fp) return 1;
  std::fprintf(fp, "%d\n%s\n%s\n%s\n%s\n", N_, to_string(cre_).c_str(), to_string(cim_).c_str(),
               to_string(sre_).c_str(), to_string(sim_).c_str());
  std::fclose(fp);
  return 0;
}

void MPView::coordinates(std::vector<D2>& re, std::vector<D2>& im) const {
  re.resize(nc_);
  im.resize(nr_);
  Mpf p(bits_), t(bits_), h(64);
  for (int c = 0; c < nc_; c++) {
    coord_re(c, p, t);
    double hi = p.d();
    mpf_set_d(h.p(), hi);
    mpf_sub(t.p(), p.p(), h.p());
    re[c] = {hi, t.d()};
  }
  for (int r = 0; r < nr_; r++) {
    coord_im(r, p, t);
    double hi = p.d();
    mpf_set_d(h.p(), hi);
    mpf_sub(t.p(), p.p(), h.p());
    im[r] = {hi, t.d()};
  }
}

void mp_record(mpf_srcptr x, int limbs, uint64_t* out) {
  const int size = x->_mp_size;
  const int n = size < 0 ? -size : size;
  const int32_t s = size < 0 ? -1 : (size > 0 ? 1 : 0);
  out[0] = ((uint64_t)(uint32_t)(int32_t)(s ? x->_mp_exp : 0) << 32) | (uint32_t)s;
  for (int i = 0; i < limbs; i++) out[1 + i] = i < n ? x->_mp_d[n - 1 - i] : 0;
}

void MPView::coordinates_mp(std::vector<uint64_t>& re, std::vector<uint64_t>& im) const {
  const int limbs = mp_limbs_for_bits(bits_), w = mp_record_words(limbs);
  re.assign((size_t)nc_ * w, 0);
  im.assign((size_t)nr_ * w, 0);
  Mpf p(bits_), t(bits_);
  for (int c = 0; c < nc_; c++) {
    coord_re(c, p, t);
    mp_record(p.p(), limbs, &re[(size_t)c * w]);
  }
  for (int r = 0; r < nr_; r++) {
    coord_im(r, p, t);
    mp_record(p.p(), limbs, &im[(size_t)r * w]);
  }
}

void MPView::eps_tables(const OrbitData&, std::vector<double>& er, std::vector<double>& ei) const {
  // Y.re = Y0.re - X[0].re; eps.re = Y.re.get_d()   (mandelbrot.cpp:155-159)
  er.resize(nc_);
  ei.resize(nr_);
  Mpf p(bits_), t(bits_);
  for (int c = 0; c < nc_; c++) {
    coord_re(c, p, t);
    mpf_sub(t.p(), p.p(), x0re_.p());
    er[c] = t.d();
  }
  for (int r = 0; r < nr_; r++) {
    coord_im(r, p, t);
    mpf_sub(t.p(), p.p(), x0im_.p());
    ei[r] = t.d();
  }
}

void MPView::eps_tables_fe(std::vector<RFE>& er, std::vector<RFE>& ei) const {
  er.resize(nc_);
  ei.resize(nr_);
  Mpf p(bits_), t(bits_);
  long e = 0;
  for (int c = 0; c < nc_; c++) {
    coord_re(c, p, t);
    mpf_sub(t.p(), p.p(), x0re_.p());
    const double m = mpf_get_d_2exp(&e, t.p());
    er[c] = {m, m == 0.0 ? 0 : (int32_t)e};
  }
  for (int r = 0; r < nr_; r++) {
    coord_im(r, p, t);
    mpf_sub(t.p(), p.p(), x0im_.p());
    const double m = mpf_get_d_2exp(&e, t.p());
    ei[r] = {m, m == 0.0 ? 0 : (int32_t)e};
  }
}

// get_d of a complex mpf value as a floatexp pair with one exponent: the same
// truncated mantissas mpf_get_d_2exp returns, rescaled exactly.
static CFE cfe_of(mpf_srcptr re, mpf_srcptr im) {
  long er = 0, ei = 0;
  const double dr = mpf_get_d_2exp(&er, re), di = mpf_get_d_2exp(&ei, im);
  if (dr == 0.0 && di == 0.0) return {0.0, 0.0, 0};
  const long e = dr == 0.0 ? ei : di == 0.0 ? er : std::max(er, ei);
  return {std::ldexp(dr, (int)(er - e)), std::ldexp(di, (int)(ei - e)), (int32_t)e};
}

static bool rfe_less_host(RFE x, RFE y) {
  if (!(x.m > 0.0)) return y.m > 0.0 || (x.m < y.m);
  if (!(y.m > 0.0)) return false;
  if (std::isinf(x.m) || std::isinf(y.m)) return x.m < y.m;
  const int ex = std::ilogb(x.m) + x.e, ey = std::ilogb(y.m) + y.e;
  if (ex != ey) return ex < ey;
  return std::scalbn(x.m, x.e - ex) < std::scalbn(y.m, y.e - ey);
}

int MPView::precompute(int threads, OrbitData& od, int reference_mode, bool keep_mp,
                       ProbeLengths probe_lengths, void* probe_ctx) {
  od = OrbitData();
  const int mp_limbs = mp_limbs_for_bits(bits_), mp_w = mp_record_words(mp_limbs);
  if (keep_mp) od.mp_limbs = mp_limbs;
  // Probe points of findProbe (mandelbrot.cpp:77-83), in the reference's order,
  // or the view center alone: pointAt(nr/2 - 1, nc/2) is exactly the center.
  std::vector<std::pair<int, int>> pts;
  if (reference_mode == REFERENCE_CENTER) {
    pts.push_back({nr_ / 2 - 1, nc_ / 2});
  } else {
    for (int c = 0; c < nc_; c += 2) {
      pts.push_back({nr_ / 4, c});
      pts.push_back({nr_ / 2, c});
      pts.push_back({3 * nr_ / 4, c});
    }
    for (int r = 0; r < nr_; r += 2) pts.push_back({r, nc_ / 2});
  }

  std::vector<int> len(pts.size(), N_);
  const int P = (int)((bits_ + 127) / 64);  // GMP's limbs of precision
  const bool fixed = P >= kFixedMinP && P <= kFixedMaxP;
  bool probed = false;
  if (pts.size() > 1 && probe_lengths) {
    const int limbs = mp_limbs_for_bits(bits_), w = mp_record_words(limbs);
    std::vector<uint64_t> re(pts.size() * w), im(pts.size() * w);
    Mpf p(bits_), tmp(bits_);
    for (size_t k = 0; k < pts.size(); k++) {
      coord_re(pts[k].second, p, tmp);
      mp_record(p.p(), limbs, &re[k * w]);
      coord_im(pts[k].first, p, tmp);
      mp_record(p.p(), limbs, &im[k * w]);
    }
    probed = probe_lengths(probe_ctx, limbs, re, im, N_, len);
  }
  if (probed) {
    // lengths from the GPU
  } else if (pts.size() > 1 && fixed) {
    std::vector<Mpf> pr(pts.size(), Mpf(bits_)), pi(pts.size(), Mpf(bits_));
    Mpf tmp(bits_);
    for (size_t k = 0; k < pts.size(); k++) {
      coord_re(pts[k].second, pr[k], tmp);
      coord_im(pts[k].first, pi[k], tmp);
    }
    fixed_dispatch<kFixedMinP>(P, pr, pi, N_, threads, len, nullptr, nullptr, false, nullptr);
  } else if (pts.size() > 1) {
  std::atomic<size_t> next{0};
  auto worker = [&]() {
    Mpf pr(bits_), pi(bits_), tmp(bits_);
    for (;;) {
      size_t k = next.fetch_add(1);
      if (k >= pts.size()) break;
      coord_re(pts[k].second, pr, tmp);
      coord_im(pts[k].first, pi, tmp);
      len[k] = orbit_length(pr.p(), pi.p(), N_, bits_);
    }
  };
  int T = std::max(1, std::min<int>(threads, (int)pts.size()));
  std::vector<std::thread> pool;
  for (int t = 1; t < T; t++) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  }
  // Longest orbit wins, earliest probe on ties (the strict '>' at :90).  With
  // a single probe its length is found by the orbit loop below.
  int best = 0;
  for (size_t k = 1; k < pts.size(); k++)
    if (len[k] > len[best]) best = (int)k;
  od.probe_index = best;

  // Orbit and series of the winner in one pass: X[i] (mandelbrot.cpp:102-103)
  // then A[i], B[i], C[i] from X[i-1] (mandelbrot.cpp:122-129).
  Mpf cr(bits_), ci(bits_), tmp(bits_);
  coord_re(pts[best].second, cr, tmp);
  coord_im(pts[best].first, ci, tmp);
  x0re_ = cr;
  x0im_ = ci;
  const size_t cap = (size_t)std::min(N_, 1 << 20) + 2;
  od.z.reserve(cap);
  od.z.push_back({0.0, 0.0});
  if (fixed) {
    mpf_srcptr winner[2] = {cr.p(), ci.p()};
    bool escaped = false;
    fixed_dispatch<kFixedMinP>(P, {}, {}, N_, threads, len, winner, &od, keep_mp, &escaped);
    od.xlen = (int)od.xhi.size();
    finish_thresholds(od);
    return 0;
  }
  StepTemps s(bits_);
  Mpf xr(bits_), xi(bits_), nxr(bits_), nxi(bits_);
  Mpf ar(bits_), ai(bits_), br(bits_), bi(bits_), c_r(bits_), c_i(bits_);
  Mpf nar(bits_), nai(bits_), nbr(bits_), nbi(bits_), ncr(bits_), nci(bits_), h(64);
  mpf_set(xr.p(), cr.p());
  mpf_set(xi.p(), ci.p());
  mpf_set_d(ar.p(), 1.0);
  mpf_set_d(ai.p(), 0.0);
  mpf_set_d(br.p(), 0.0);
  mpf_set_d(bi.p(), 0.0);
  mpf_set_d(c_r.p(), 0.0);
  mpf_set_d(c_i.p(), 0.0);
  auto split = [&](mpf_srcptr v, double& hi, double& lo) {
    hi = mpf_get_d(v);
    mpf_set_d(h.p(), hi);
    mpf_sub(s.t3.p(), v, h.p());
    lo = mpf_get_d(s.t3.p());
  };
  mpf_ptr t1 = s.t1.p(), t2 = s.t2.p();
  bool escaped = false;
  for (int i = 0;; i++) {
    D2 hi, lo;
    split(xr.p(), hi.x, lo.x);
    split(xi.p(), hi.y, lo.y);
    od.xhi.push_back(hi);
    od.xlo.push_back(lo);
    od.z.push_back(hi);
    if (keep_mp) {
      const size_t at = od.xmp.size();
      od.xmp.resize(at + 2 * (size_t)mp_w);
      mp_record(xr.p(), mp_limbs, &od.xmp[at]);
      mp_record(xi.p(), mp_limbs, &od.xmp[at + mp_w]);
    }
    od.a.push_back({ar.d(), ai.d()});
    od.b.push_back({br.d(), bi.d()});
    od.c.push_back({c_r.d(), c_i.d()});
    od.a_fe.push_back(cfe_of(ar.p(), ai.p()));
    od.b_fe.push_back(cfe_of(br.p(), bi.p()));
    od.c_fe.push_back(cfe_of(c_r.p(), c_i.p()));
    if (i + 1 >= N_) break;  // X.resize(N) is full
    // X[i+1]; computeOrbit stops at the first element that bails out
    square_add(nxr.p(), nxi.p(), xr.p(), xi.p(), cr.p(), ci.p(), s);
    if (bailed_out(nxr.p(), nxi.p())) {
      escaped = true;
      break;
    }
    {
      // A[i+1].re = 2.0 * (X.re * A.re - X.im * A.im) + 1.0
      mpf_mul(t1, xr.p(), ar.p()); mpf_mul(t2, xi.p(), ai.p()); mpf_sub(t1, t1, t2);
      mpf_mul(t1, s.two.p(), t1); mpf_add(nar.p(), t1, s.one.p());
      // A[i+1].im = 2.0 * (X.re * A.im + X.im * A.re)
      mpf_mul(t1, xr.p(), ai.p()); mpf_mul(t2, xi.p(), ar.p()); mpf_add(t1, t1, t2);
      mpf_mul(nai.p(), s.two.p(), t1);
      // B[i+1].re = 2.0 * (X.re * B.re - X.im * B.im) + A'.re * A'.re - A'.im * A'.im
      mpf_mul(t1, xr.p(), br.p()); mpf_mul(t2, xi.p(), bi.p()); mpf_sub(t1, t1, t2);
      mpf_mul(t1, s.two.p(), t1);
      mpf_mul(t2, nar.p(), nar.p()); mpf_add(t1, t1, t2);
      mpf_mul(t2, nai.p(), nai.p()); mpf_sub(nbr.p(), t1, t2);
      // B[i+1].im = 2.0 * (X.re * B.im + X.im * B.re + A'.re * A'.im)
      mpf_mul(t1, xr.p(), bi.p()); mpf_mul(t2, xi.p(), br.p()); mpf_add(t1, t1, t2);
      mpf_mul(t2, nar.p(), nai.p()); mpf_add(t1, t1, t2);
      mpf_mul(nbi.p(), s.two.p(), t1);
      // C[i+1].re = 2.0 * (X.re * C.re - X.im * C.im + A'.re * B'.re - A'.im * B'.im)
      mpf_mul(t1, xr.p(), c_r.p()); mpf_mul(t2, xi.p(), c_i.p()); mpf_sub(t1, t1, t2);
      mpf_mul(t2, nar.p(), nbr.p()); mpf_add(t1, t1, t2);
      mpf_mul(t2, nai.p(), nbi.p()); mpf_sub(t1, t1, t2);
      mpf_mul(ncr.p(), s.two.p(), t1);
      // C[i+1].im = 2.0 * (X.re * C.im + X.im * C.re + A'.re * B'.im + A'.im * B'.re)
      mpf_mul(t1, xr.p(), c_i.p()); mpf_mul(t2, xi.p(), c_r.p()); mpf_add(t1, t1, t2);
      mpf_mul(t2, nar.p(), nbi.p()); mpf_add(t1, t1, t2);
      mpf_mul(t2, nai.p(), nbr.p()); mpf_add(t1, t1, t2);
      mpf_mul(nci.p(), s.two.p(), t1);
      ar.swap(nar); ai.swap(nai);
      br.swap(nbr); bi.swap(nbi);
      c_r.swap(ncr); c_i.swap(nci);
    }
    xr.swap(nxr);
    xi.swap(nxi);
  }
  od.xlen = (int)od.xhi.size();
  if (escaped) od.z.push_back({nxr.d(), nxi.d()});  // the element that escaped
  finish_thresholds(od);
  return 0;
}

void MPView::finish_thresholds(OrbitData& od) const {
  const int xlen = od.xlen;
  // Series instability thresholds: term i fires when tol |b|^2 < |c|^2, which
  // in exact arithmetic is  tol |B_i|^2 / |C_i|^2 < |eps3|^2 / |eps2|^2.
  od.sa_min.assign(xlen, INFINITY);
  double run = INFINITY;
  double bmax = 0.0, cmax = 0.0;
  for (int i = 1; i < xlen; i++) {
    double nb = std::hypot(od.b[i].x, od.b[i].y);
    double ncm = std::hypot(od.c[i].x, od.c[i].y);
    double t = ncm == 0.0 ? INFINITY : tol_ * (nb / ncm) * (nb / ncm);
    if (std::isnan(t)) t = 0.0;  // non-finite coefficients fire at once
    run = std::min(run, t);
    od.sa_min[i] = run;
    bmax = std::max(bmax, nb);
    cmax = std::max(cmax, ncm);
  }
  // FP64 terms of the farthest and nearest samples stay normal and finite.
  double w = std::max(std::fabs(sre_.d()) * nc_, std::fabs(sim_.d()) * nr_) * 1.5;
  double e_min = std::min(std::fabs(sre_.d()), std::fabs(sim_.d()));
  od.sa_fp64_ok = std::isfinite(bmax) && std::isfinite(cmax) && cmax * w * w * w < 1e140 &&
                  bmax * w * w < 1e140 && e_min > 1e-45;

  // The same thresholds in floatexp, for views outside the FP64 range.
  od.sa_min_fe.assign(xlen, RFE{INFINITY, 0});
  RFE runf{INFINITY, 0};
  for (int i = 1; i < xlen; i++) {
    const CFE& B = od.b_fe[i];
    const CFE& C = od.c_fe[i];
    const double nb = std::hypot(B.re, B.im), ncm = std::hypot(C.re, C.im);
    RFE t{INFINITY, 0};
    if (ncm != 0.0) {
      t.m = tol_ * (nb / ncm) * (nb / ncm);
      t.e = 2 * (B.e - C.e);
    }
    if (rfe_less_host(t, runf)) runf = t;
    od.sa_min_fe[i] = runf;
  }
}

int MPView::precompute_center_orbit(OrbitData& od, unsigned long orbit_bits) {
  od = OrbitData();
  od.double_loop = true;
  od.probe_index = 0;
  const unsigned long bits = orbit_bits > bits_ ? orbit_bits : bits_;
  Mpf cr(bits), ci(bits), tmp(bits_), pre(bits_);
  // pointAt(nr/2 - 1, nc/2) is exactly the center; taken at the view's
  // precision, then iterated at `bits`
  coord_re(nc_ / 2, pre, tmp);
  mpf_set(cr.p(), pre.p());
  coord_im(nr_ / 2 - 1, pre, tmp);
  mpf_set(ci.p(), pre.p());
  x0re_ = cr;
  x0im_ = ci;
  StepTemps s(bits);
  Mpf xr(bits), xi(bits), nxr(bits), nxi(bits), h(64);
  mpf_set(xr.p(), cr.p());
  mpf_set(xi.p(), ci.p());
  od.z.reserve((size_t)std::min(N_, 1 << 20) + 2);
  od.z.push_back({0.0, 0.0});
  auto split = [&](mpf_srcptr v, double& hi, double& lo) {
    hi = mpf_get_d(v);
    mpf_set_d(h.p(), hi);
    mpf_sub(s.t3.p(), v, h.p());
    lo = mpf_get_d(s.t3.p());
  };
  bool escaped = false;
  for (int i = 0;; i++) {
    D2 hi, lo;
    split(xr.p(), hi.x, lo.x);
    split(xi.p(), hi.y, lo.y);
    od.xhi.push_back(hi);
    od.xlo.push_back(lo);
    od.z.push_back(hi);
    if (i + 1 >= N_) break;
    square_add(nxr.p(), nxi.p(), xr.p(), xi.p(), cr.p(), ci.p(), s);
    if (bailed_out(nxr.p(), nxi.p())) {
      escaped = true;
      break;
    }
    xr.swap(nxr);
    xi.swap(nxi);
  }
  od.xlen = (int)od.xhi.size();
  if (escaped) od.z.push_back({nxr.d(), nxi.d()});
  od.sa_fp64_ok = true;
  return 0;
}

void MPView::eps_tables_double_loop(const std::vector<double>& px, const std::vector<double>& py,
                                    std::vector<double>& er, std::vector<double>& ei) const {
  const unsigned long bits = mpf_get_prec(x0re_.p()) + 64;
  Mpf t(bits), x(bits);
  er.resize(px.size());
  ei.resize(py.size());
  for (size_t c = 0; c < px.size(); c++) {
    mpf_set_d(x.p(), px[c]);
    mpf_sub(t.p(), x.p(), x0re_.p());
    er[c] = t.d();
  }
  for (size_t r = 0; r < py.size(); r++) {
    mpf_set_d(x.p(), py[r]);
    mpf_sub(t.p(), x.p(), x0im_.p());
    ei[r] = t.d();
  }
}

bool MPView::view_outside_cardioid() const {
  std::vector<D2> re, im;
  Mpf p(bits_), t(bits_);
  coord_re(0, p, t);
  double x0 = p.d();
  coord_re(nc_ - 1, p, t);
  double x1 = p.d();
  coord_im(0, p, t);
  double y0 = p.d();
  coord_im(nr_ - 1, p, t);
  double y1 = p.d();
  Iv x = widen({std::min(x0, x1), std::max(x0, x1)});
  Iv y = widen({std::min(y0, y1), std::max(y0, y1)});
  Iv xmf = isub(x, {0.25, 0.25});
  Iv y2 = isq(y);
  Iv q = iadd(isq(xmf), y2);
  Iv g1 = isub(imul(q, iadd(q, xmf)), imul({0.25, 0.25}, y2));
  Iv xp1 = iadd(x, {1.0, 1.0});
  Iv g2 = isub(iadd(isq(xp1), y2), {0.0625, 0.0625});
  return g1.lo > 0.0 && g2.lo > 0.0;
}

}  // namespace nmg
