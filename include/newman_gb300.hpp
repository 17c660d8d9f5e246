// Header-only C++ face of the C ABI, with the method names of the reference's
// `Mandelbrot` class (mandelbrot.h:7-53 of axnjaxn/newman), so that a
// caller written against that class (viewer.cpp's render loop, beauty
// render, zoom handling) maps onto it call for call.  Errors become
// newman_gb300::Error exceptions; the object is copyable by value like the
// reference's (viewer.cpp:193,251).
#ifndef NEWMAN_GB300_HPP
#define NEWMAN_GB300_HPP

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "newman_gb300.h"

namespace newman_gb300 {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
  if (rc != NM_OK) throw Error(rc, nm_last_error());
}

// RenderGrid::EscapeValue (grid.h:8-14).
using EscapeValue = nm_escape_value;

// A complex number as two decimal strings (the reference keeps mpf_class).
struct DecimalComplex {
  std::string re, im;
};

class Mandelbrot {
 public:
  Mandelbrot() : Mandelbrot(1, 1) {}
  Mandelbrot(int nr, int nc) : h_(nm_create(nr, nc)) {
    if (!h_) throw Error(NM_ERR_ARG, nm_last_error());
  }
  Mandelbrot(const Mandelbrot& o) : h_(nm_copy(o.h_)) {
    if (!h_) throw Error(NM_ERR_CUDA, nm_last_error());
  }
  Mandelbrot& operator=(const Mandelbrot& o) {
    if (this != &o) {
      nm_handle* c = nm_copy(o.h_);
      if (!c) throw Error(NM_ERR_CUDA, nm_last_error());
      nm_destroy(h_);
      h_ = c;
    }
    return *this;
  }
  Mandelbrot(Mandelbrot&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  Mandelbrot& operator=(Mandelbrot&& o) noexcept {
    std::swap(h_, o.h_);
    return *this;
  }
  ~Mandelbrot() { nm_destroy(h_); }

  // public fields of the reference: N, error_tolerance, center, sz
  int N() const { return nm_get_iterations(h_); }
  void setN(int n) { check(nm_set_iterations(h_, n)); }
  void setErrorTolerance(double tol) { check(nm_set_tolerance(h_, tol)); }
  DecimalComplex center() const { return {field(0), field(1)}; }
  DecimalComplex sz() const { return {field(2), field(3)}; }
  // center, step, N, tolerance at once (the fields of a save file)
  void setView(const DecimalComplex& center, const DecimalComplex& sz, int n, double tol = 1e-10,
               int min_bits = 0) {
    check(nm_set_view(h_, center.re.c_str(), center.im.c_str(), sz.re.c_str(), sz.im.c_str(), n,
                      tol, min_bits));
  }

  void loadLegacy(const char* fn) { check(nm_load_legacy(h_, fn)); }
  void save(const char* fn) const { check(nm_save(h_, fn)); }

  int rows() const { return nm_rows(h_); }
  int cols() const { return nm_cols(h_); }

  bool useHardware() const { return nm_use_hardware(h_) == 1; }
  void precompute() { check(nm_precompute(h_)); }
  void computeRow(int r) { check(nm_compute_row(h_, r)); }
  // all rows at once (the row loop of viewer.cpp:166-171 in one launch)
  void render() { check(nm_render(h_)); }
  void cancel() { check(nm_cancel(h_)); }

  DecimalComplex pointAt(int r, int c, int sc = 1) const {
    std::vector<char> a(1 << 16), b(1 << 16);
    check(nm_point_at(h_, r, c, sc, a.data(), b.data(), (int)a.size()));
    return {a.data(), b.data()};
  }
  void translate(int dr, int dc, int sc = 1) { check(nm_translate(h_, dr, dc, sc)); }
  void zoom(float scale) { check(nm_zoom(h_, scale)); }
  void zoomAt(float scale, int r, int c, int sc = 1) { check(nm_zoom_at(h_, scale, r, c, sc)); }

  EscapeValue at(int r, int c) {
    EscapeValue e;
    check(nm_at(h_, r, c, &e));
    return e;
  }
  EscapeValue at(int r, int c, int sc) {
    EscapeValue e;
    check(nm_at_sc(h_, r, c, sc, &e));
    return e;
  }
  void scaleUp(int sc) { check(nm_scale_up(h_, sc)); }
  void scaleDown(int sc) { check(nm_scale_down(h_, sc)); }

  // the whole grid, row-major r*cols()+c (RenderGrid::values)
  std::vector<EscapeValue> grid() {
    std::vector<EscapeValue> v((size_t)rows() * cols());
    check(nm_get_grid(h_, v.data()));
    return v;
  }
  void setPath(int path) { check(nm_set_path(h_, path)); }
  nm_handle* handle() { return h_; }

 private:
  std::string field(int which) const {
    std::vector<char> buf(1 << 16);
    check(nm_get_view(h_, which, buf.data(), (int)buf.size()));
    return buf.data();
  }
  nm_handle* h_;
};

}  // namespace newman_gb300

#endif  // NEWMAN_GB300_HPP
