// Host-side arbitrary-precision view state of one render: the center, the
// pixel step, the iteration count and the precision rule of the reference's
// `Mandelbrot` object (mandelbrot.h:7-53), plus the sequential precompute
// (probe search, reference orbit, series coefficients) that feeds the GPU.
#pragma once

#include <algorithm>
#include <cmath>

#include <cstdint>
#include <string>
#include <vector>

#include "gmp_abi.h"
#include "view_device.cuh"

namespace nmg {

// One mpf_t with value semantics (copying keeps the precision).
class Mpf {
 public:
  explicit Mpf(unsigned long bits = 64) { mpf_init2(v_, bits); }
  Mpf(const Mpf& o) {
    mpf_init2(v_, mpf_get_prec(o.v_));
    mpf_set(v_, o.v_);
  }
  Mpf& operator=(const Mpf& o) {
    if (this != &o) {
      mpf_set_prec(v_, mpf_get_prec(o.v_));
      mpf_set(v_, o.v_);
    }
    return *this;
  }
  ~Mpf() { mpf_clear(v_); }
  void swap(Mpf& o) {  // exchanges the limb buffers, no copy
    __mpf_struct t = v_[0];
    v_[0] = o.v_[0];
    o.v_[0] = t;
  }
  mpf_ptr p() { return v_; }
  mpf_srcptr p() const { return v_; }
  double d() const { return mpf_get_d(v_); }

 private:
  mpf_t v_;
};

struct D2 {
  double x, y;
};

// What one precompute hands to the device, all as FP64 values read from the
// arbitrary-precision state with get_d (truncation toward zero, like
// complex.h:33-35 `descend`).
struct OrbitData {
  int xlen = 0;                 // X.size() of the reference after findProbe
  int probe_index = -1;         // which probe won (mandelbrot.cpp:85-94)
  std::vector<D2> z;            // 0, X[0..xlen), and the escaped element if any
  std::vector<D2> xhi, xlo;     // X[k] = xhi + xlo (+ < 2^-106 |X|)
  std::vector<D2> a, b, c;      // series coefficients A, B, C
  std::vector<double> sa_min;   // prefix minimum of tol |B_i|^2 / |C_i|^2 (index 0 unused)
  bool sa_fp64_ok = true;       // FP64 series terms stay in the normal range
  // Floatexp copies (FP64 mantissa, int exponent), used when !sa_fp64_ok:
  std::vector<CFE> a_fe, b_fe, c_fe;
  std::vector<RFE> sa_min_fe;
  // The orbit alone, for the FE32 path on a view the reference renders with
  // its double loop (no series: those samples start at iteration 0).
  bool double_loop = false;
  // The orbit X[0..xlen) in the view's arbitrary precision, for the
  // reference-exact path (filled when precompute is asked for it): per
  // element the records of re and im, each mp_record_words(limbs) words.
  int mp_limbs = 0;
  std::vector<uint64_t> xmp;
};

// One arbitrary-precision value as device words: word 0 holds the limb
// exponent (high 32 bits) and the sign (low 32 bits, -1, 0 or 1), then
// `limbs` limbs, most significant first, zero below the value's own.
inline int mp_record_words(int limbs) { return limbs + 1; }
// Limbs a value of the view's precision holds: GMP's P + 1 for mpf_init2(bits).
inline int mp_limbs_for_bits(unsigned long bits) { return (int)((bits + 127) / 64) + 1; }
void mp_record(mpf_srcptr x, int limbs, uint64_t* out);

// Where the reference orbit starts.
enum ReferenceMode {
  REFERENCE_PROBES = 0,  // the reference's probe search (findProbe, mandelbrot.cpp:73-95)
  REFERENCE_CENTER = 1   // the view center only (one orbit; for deep views)
};

class MPView {
 public:
  MPView(int nr, int nc);

  int rows() const { return nr_; }
  int cols() const { return nc_; }
  int iterations() const { return N_; }
  double tolerance() const { return tol_; }
  unsigned long bits() const { return bits_; }

  // center / step as decimal strings, N, series tolerance, precision floor.
  int set_view(const char* cre, const char* cim, const char* sre, const char* sim, int N,
               double tol, int min_bits);
  void set_iterations(int N);
  void set_tolerance(double tol) { tol_ = tol; }

  bool use_hardware() const;  // mandelbrot.cpp:256-259
  // A preview that stands for a finer view (nm_preview): it keeps the finer
  // view's precision through scale_down, and renders by perturbation wherever
  // the finer view does, whatever its own step.
  void stand_in_for(const MPView& fine) {
    min_bits_ = std::max(min_bits_, fine.bits_);
    no_hardware_ = !fine.use_hardware();
  }
  double step_max() const { return std::max(std::fabs(sre_.d()), std::fabs(sim_.d())); }
  void scale_up(int sc);      // mandelbrot.cpp:334-346 (geometry)
  void scale_down(int sc);    // mandelbrot.cpp:348-360 (geometry)
  void zoom(float scale);     // mandelbrot.cpp:297-302
  void zoom_at(float scale, int r, int c, int sc);  // mandelbrot.cpp:304-316
  void translate(int dr, int dc, int sc);           // mandelbrot.cpp:292-295
  void point_at(int r, int c, int sc, Mpf& re, Mpf& im) const;  // mandelbrot.cpp:285-290
  int load_legacy(const char* path);                // mandelbrot.cpp:19-35
  int save(const char* path) const;                 // viewer.cpp:12-23 format

  std::string center_re_str() const { return to_string(cre_); }
  std::string center_im_str() const { return to_string(cim_); }
  std::string step_re_str() const { return to_string(sre_); }
  std::string step_im_str() const { return to_string(sim_); }
  static std::string to_string(const Mpf& f);

  // Per-column real and per-row imaginary sample coordinates (computeRow's
  // pt.re / pt.im, mandelbrot.cpp:271,275), as hi + lo doubles.
  void coordinates(std::vector<D2>& re, std::vector<D2>& im) const;
  // eps = get_d(pt - X[0]) per column / row (mandelbrot.cpp:155-159).
  void eps_tables(const OrbitData& od, std::vector<double>& er, std::vector<double>& ei) const;
  // The same as floatexp (mantissa and exponent of the truncated value).
  void eps_tables_fe(std::vector<RFE>& er, std::vector<RFE>& ei) const;

  // findProbe + computeSeries (mandelbrot.cpp:73-131), probes on `threads`
  // host threads (or the view center only, REFERENCE_CENTER).  Fills `out`.
  // The probe lengths can be handed to `probe_lengths` (records of the probe
  // points' coordinates, mp_record_words(mp_limbs_for_bits(bits())) words
  // each); when it returns false they are found on the host threads.
  using ProbeLengths = bool (*)(void* ctx, int limbs, const std::vector<uint64_t>& re,
                                const std::vector<uint64_t>& im, int N, std::vector<int>& len);
  int precompute(int threads, OrbitData& out, int reference_mode = REFERENCE_PROBES,
                 bool keep_mp = false, ProbeLengths probe_lengths = nullptr,
                 void* probe_ctx = nullptr);
  // computeRow's pt.re per column and pt.im per row (mandelbrot.cpp:271,275)
  // as arbitrary-precision records (mp_record) of mp_limbs_for_bits(bits())
  // limbs.
  void coordinates_mp(std::vector<uint64_t>& re, std::vector<uint64_t>& im) const;

  // For the FE32 path on a double-loop view: the orbit of the view center at
  // `orbit_bits` of precision (no series), and per column / row the exact
  // offset of the double coordinate the double loop starts from,
  // get_d(get_d(pt) - X[0]) (the inner get_d is computeRow's pt handed to
  // getIterationsHW, mandelbrot.cpp:242).
  int precompute_center_orbit(OrbitData& out, unsigned long orbit_bits);
  void eps_tables_double_loop(const std::vector<double>& px, const std::vector<double>& py,
                              std::vector<double>& er, std::vector<double>& ei) const;

  // Box in which every sample lies is provably outside both the main
  // cardioid and the period-2 disk.
  bool view_outside_cardioid() const;

 private:
  void set_precision();  // mandelbrot.cpp:37-56
  // The series thresholds of od (sa_min, sa_fp64_ok, sa_min_fe) from its
  // coefficients.
  void finish_thresholds(OrbitData& od) const;
  void coord_re(int c, Mpf& out, Mpf& tmp) const;
  void coord_im(int r, Mpf& out, Mpf& tmp) const;

  int nr_, nc_;
  int N_ = 256;
  double tol_ = 1e-10;
  unsigned long bits_ = 64, min_bits_ = 0;
  bool no_hardware_ = false;
  Mpf cre_, cim_, sre_, sim_;
  Mpf x0re_, x0im_;  // X[0] of the last precompute
};

}  // namespace nmg
