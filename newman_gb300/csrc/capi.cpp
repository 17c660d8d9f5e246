// The C ABI (include/newman_gb300.h): one nm_handle per reference
// `Mandelbrot` object.  Host arbitrary-precision state in nmg::MPView, GPU
// buffers and launches here.  There is no CPU path for per-sample work: if
// the CUDA runtime or device is missing, every render call fails.
#include "newman_gb300.h"

#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "engine.hpp"
#include "handle.hpp"
#include "mpview.hpp"

using nmg::Dbl2;
using nmg::EscapeValue;

using nmg::DevBuf;
using nmg::fail;
using namespace nmg::scratch;

namespace {

thread_local std::string g_last_error;

// Precision of the view-center orbit for the FE32 path on a double-loop view:
// the certificate takes that orbit as exact to the 2^-52 of its FP64 copy.
constexpr unsigned long kDoubleLoopOrbitBits = 256;

// The FE32 path on a double-loop view certifies against the double loop's own
// rounding, which grows with the zoom: below a sample step of 2^-33 most
// samples cannot be certified (measured on a 1280x720 zoom into
// -0.743643887037151+0.131825904205330i: reworked fraction 7 % at step 6e-10,
// 24 % at 1e-10, over 90 % below 1e-13), so there the FE32
// path renders with the double loop directly -- the same escape counts.
constexpr double kDoubleLoopFe32MinStep = 0x1p-33;

// Orbit entries staged in shared memory by default on views whose series
// leaves the double range (NM_OPT_ORBIT_STAGE -1).
constexpr int kAutoOrbitStage = 1024;

// An upper bound on |c|_1 over the samples of the view (their coordinates as
// the double loop takes them), as a float.
float coord_abs_bound(const nm_handle* h) {
  double mr = 0.0, mi = 0.0;
  for (const Dbl2& x : h->coord_re) mr = std::max(mr, std::fabs(x.x) + std::fabs(x.y));
  for (const Dbl2& y : h->coord_im) mi = std::max(mi, std::fabs(y.x) + std::fabs(y.y));
  return std::nextafter((float)((mr + mi) * (1.0 + 0x1p-40)), INFINITY);
}

bool double_loop_direct(const nm_handle* h) {
  return h->path == NM_PATH_FE32 && h->view.use_hardware() &&
         h->view.step_max() < kDoubleLoopFe32MinStep;
}

}  // namespace

int nmg::fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

namespace {

// The CUDA side of a handle is created on first use, so that the host-only
// calls (view edits, the arbitrary-precision precompute) work without a GPU.
}  // namespace

int nmg::ensure_device(nm_handle* h) {
  if (h->stream) return NM_OK;
  NM_CUDA(cudaGetDevice(&h->device));
  NM_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  NM_CUDA(cudaHostAlloc(&h->cancel_host, sizeof(int), cudaHostAllocMapped));
  *h->cancel_host = 0;
  NM_CUDA(cudaHostGetDevicePointer((void**)&h->cancel_dev, h->cancel_host, 0));
  NM_CUDA(h->d_scratch.reserve(kScratchWords));
  NM_CUDA(cudaMemsetAsync(h->d_scratch.p, 0, kScratchWords * 8, h->stream));
  for (cudaEvent_t& e : h->ev) NM_CUDA(cudaEventCreate(&e));
  return NM_OK;
}

namespace {

using nmg::ensure_device;

int ensure_grid(nm_handle* h) {
  if (int rc = ensure_device(h)) return rc;
  const int nr = h->view.rows(), nc = h->view.cols();
  if (h->grid.p && h->grid_nr == nr && h->grid_nc == nc &&
      (!h->keep_smooth64 || h->smooth64.p))
    return NM_OK;
  const size_t n = (size_t)nr * nc;
  if (!(h->grid.p && h->grid_nr == nr && h->grid_nc == nc)) {
    NM_CUDA(h->grid.reserve(n));
    NM_CUDA(cudaMemsetAsync(h->grid.p, 0, n * sizeof(EscapeValue), h->stream));
  }
  if (h->keep_smooth64) {
    NM_CUDA(h->smooth64.reserve(n));
    NM_CUDA(cudaMemsetAsync(h->smooth64.p, 0, n * sizeof(double), h->stream));
  }
  h->grid_nr = nr;
  h->grid_nc = nc;
  h->generation++;
  return NM_OK;
}

template <typename T>
int upload(DevBuf<T>& d, const std::vector<T>& v, cudaStream_t s) {
  NM_CUDA(d.reserve(v.size()));
  if (!v.empty())
    NM_CUDA(cudaMemcpyAsync(d.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return NM_OK;
}

int ensure_coords(nm_handle* h) {
  if (h->coords_valid) return NM_OK;
  std::vector<nmg::D2> re, im;
  h->view.coordinates(re, im);
  h->coord_re.resize(re.size());
  h->coord_im.resize(im.size());
  for (size_t i = 0; i < re.size(); i++) h->coord_re[i] = {re[i].x, re[i].y};
  for (size_t i = 0; i < im.size(); i++) h->coord_im[i] = {im[i].x, im[i].y};
  h->outside_cardioid = h->view.view_outside_cardioid();
  if (h->path == NM_PATH_MP) {
    h->view.coordinates_mp(h->coord_re_mp, h->coord_im_mp);
  } else {
    h->coord_re_mp.clear();
    h->coord_im_mp.clear();
  }
  h->coords_valid = true;
  h->uploaded = false;
  return NM_OK;
}

int do_upload(nm_handle* h) {
  int rc;
  if ((rc = ensure_device(h))) return rc;
  if ((rc = upload(h->d_coord_re, h->coord_re, h->stream))) return rc;
  if ((rc = upload(h->d_coord_im, h->coord_im, h->stream))) return rc;
  if (!h->coord_re_mp.empty()) {
    if ((rc = upload(h->d_coord_re_mp, h->coord_re_mp, h->stream))) return rc;
    if ((rc = upload(h->d_coord_im_mp, h->coord_im_mp, h->stream))) return rc;
  }
  // a sharing preview reads its source's orbit and series (uploaded there)
  if (h->tables_stale()) return fail(NM_ERR_STATE, kStalePreview);
  if (h->orbit_src && !h->orbit_src->uploaded)
    if ((rc = do_upload(h->orbit_src))) return rc;
  const bool own = h->orbit_src == nullptr;
  if (own && h->precomputed && !h->od.xmp.empty())
    if ((rc = upload(h->d_x_mp, h->od.xmp, h->stream))) return rc;
  if (h->precomputed) {
    if ((rc = upload(h->d_eps_re, h->eps_re, h->stream))) return rc;
    if ((rc = upload(h->d_eps_im, h->eps_im, h->stream))) return rc;
  }
  if (h->precomputed && own) {
    auto cv = [](const std::vector<nmg::D2>& v) {
      std::vector<Dbl2> o(v.size());
      std::memcpy(o.data(), v.data(), v.size() * sizeof(Dbl2));
      return o;
    };
    const size_t zlen = h->od.z.size();
    std::vector<nmg::Flt4> zf(2 * zlen);
    for (size_t k = 0; k < zlen; k++) {
      const float hx = (float)h->od.z[k].x, hy = (float)h->od.z[k].y;
      zf[k] = {hx, hy, (float)(h->od.z[k].x - hx), (float)(h->od.z[k].y - hy)};
    }
    static_assert(sizeof(nmg::Flt4) == sizeof(Dbl2), "orbit entries");
    std::memcpy(zf.data() + zlen, h->od.z.data(), zlen * sizeof(Dbl2));
    if ((rc = upload(h->d_zf, zf, h->stream))) return rc;
    if ((rc = upload(h->d_xhi, cv(h->od.xhi), h->stream))) return rc;
    if ((rc = upload(h->d_xlo, cv(h->od.xlo), h->stream))) return rc;
    if ((rc = upload(h->d_a, cv(h->od.a), h->stream))) return rc;
    if ((rc = upload(h->d_b, cv(h->od.b), h->stream))) return rc;
    if ((rc = upload(h->d_c, cv(h->od.c), h->stream))) return rc;
    if ((rc = upload(h->d_sa_min, h->od.sa_min, h->stream))) return rc;
    if (!h->od.double_loop) {
      if ((rc = upload(h->d_a32, h->a32, h->stream))) return rc;
      if ((rc = upload(h->d_b32, h->b32, h->stream))) return rc;
      if ((rc = upload(h->d_c32, h->c32, h->stream))) return rc;
      if ((rc = upload(h->d_sa_min32, h->sa_min32, h->stream))) return rc;
    }
    if (!h->od.sa_fp64_ok) {
      if ((rc = upload(h->d_a_fe, h->od.a_fe, h->stream))) return rc;
      if ((rc = upload(h->d_b_fe, h->od.b_fe, h->stream))) return rc;
      if ((rc = upload(h->d_c_fe, h->od.c_fe, h->stream))) return rc;
      if ((rc = upload(h->d_sa_min_fe, h->od.sa_min_fe, h->stream))) return rc;
    }
  }
  if (h->precomputed && !h->od.double_loop) {  // per row / column, every handle its own
    if ((rc = upload(h->d_eps32_re, h->eps32_re, h->stream))) return rc;
    if ((rc = upload(h->d_eps32_im, h->eps32_im, h->stream))) return rc;
  }
  if (h->precomputed && !h->od.sa_fp64_ok) {
    if ((rc = upload(h->d_eps_re_fe, h->eps_re_fe, h->stream))) return rc;
    if ((rc = upload(h->d_eps_im_fe, h->eps_im_fe, h->stream))) return rc;
  }
  // The vectors above are pageable; the copies are complete when the stream
  // reaches this point, so wait before the host may touch them again.
  NM_CUDA(cudaStreamSynchronize(h->stream));
  h->uploaded = true;
  h->generation++;
  return NM_OK;
}

// ---- tables of the FP32 series front ------------------------------------
nmg::FFE ffe_of(double m, int e) {
  if (m == 0.0 || !std::isfinite(m)) return {0.0f, 0.0f, 0, 0};
  const int k = std::ilogb(m);
  const double x = std::scalbn(m, -k);  // [1, 2)
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi), e + k, 0};
}
nmg::CFFE cffe_of(double re, double im, int e) {
  const double mx = std::max(std::fabs(re), std::fabs(im));
  if (mx == 0.0 || !std::isfinite(mx)) return {0.0f, 0.0f, 0.0f, 0.0f, 0, {0, 0, 0}};
  const int k = std::ilogb(mx);
  const double xr = std::scalbn(re, -k), xi = std::scalbn(im, -k);
  const float rh = (float)xr, ih = (float)xi;
  return {rh, (float)(xr - (double)rh), ih, (float)(xi - (double)ih), e + k, {0, 0, 0}};
}
nmg::TFE tfe_of(double m, int e) {
  if (std::isinf(m) && m > 0.0) return {1.0f, nmg::kTfeInf};
  if (!(m > 0.0)) return {0.0f, nmg::kTfeZero};  // 0 or NaN: below every threshold
  int k = std::ilogb(m);
  float x = (float)std::scalbn(m, -k);
  if (x >= 2.0f) {
    x *= 0.5f;
    k++;
  }
  return {x, e + k};
}

// The series front's values in float-float with int exponents: eps per
// column / row, A, B, C and the thresholds per index.  Deep views only.
void build_front32_tables(nm_handle* h, bool series = true) {
  const nmg::OrbitData& od = h->od;
  const int n = series ? od.xlen : 0;
  h->a32.resize(n);
  h->b32.resize(n);
  h->c32.resize(n);
  h->sa_min32.resize(n);
  if (od.sa_fp64_ok) {
    for (int i = 0; i < n; i++) {
      h->a32[i] = cffe_of(od.a[i].x, od.a[i].y, 0);
      h->b32[i] = cffe_of(od.b[i].x, od.b[i].y, 0);
      h->c32[i] = cffe_of(od.c[i].x, od.c[i].y, 0);
      h->sa_min32[i] = tfe_of(od.sa_min[i], 0);
    }
    h->eps32_re.resize(h->eps_re.size());
    h->eps32_im.resize(h->eps_im.size());
    for (size_t c = 0; c < h->eps_re.size(); c++) h->eps32_re[c] = ffe_of(h->eps_re[c], 0);
    for (size_t r = 0; r < h->eps_im.size(); r++) h->eps32_im[r] = ffe_of(h->eps_im[r], 0);
  } else {
    for (int i = 0; i < n; i++) {
      h->a32[i] = cffe_of(od.a_fe[i].re, od.a_fe[i].im, od.a_fe[i].e);
      h->b32[i] = cffe_of(od.b_fe[i].re, od.b_fe[i].im, od.b_fe[i].e);
      h->c32[i] = cffe_of(od.c_fe[i].re, od.c_fe[i].im, od.c_fe[i].e);
      h->sa_min32[i] = tfe_of(od.sa_min_fe[i].m, od.sa_min_fe[i].e);
    }
    h->eps32_re.resize(h->eps_re_fe.size());
    h->eps32_im.resize(h->eps_im_fe.size());
    for (size_t c = 0; c < h->eps_re_fe.size(); c++)
      h->eps32_re[c] = ffe_of(h->eps_re_fe[c].m, h->eps_re_fe[c].e);
    for (size_t r = 0; r < h->eps_im_fe.size(); r++)
      h->eps32_im[r] = ffe_of(h->eps_im_fe[r].m, h->eps_im_fe[r].e);
  }
}

int check_handle(const nm_handle* h) {
  if (!h) return fail(NM_ERR_ARG, "null handle");
  return NM_OK;
}

// Views outside the FP64 range run their series front in floatexp.
void set_fe_tables(const nm_handle* h, nmg::DeviceView& v) {
  const nm_handle* t = h->tables();  // the orbit and series (a sharing preview: its source's)
  v.sa_scan = 0;
  if (!h->od.double_loop && !t->a32.empty()) {
    v.eps32_re = h->d_eps32_re.p;
    v.eps32_im = h->d_eps32_im.p;
    v.sa_a32 = t->d_a32.p;
    v.sa_b32 = t->d_b32.p;
    v.sa_c32 = t->d_c32.p;
    v.sa_min32 = t->d_sa_min32.p;
  }
  v.sa_fe = h->od.sa_fp64_ok ? 0 : 1;
  if (!v.sa_fe) return;
  v.eps_re_fe = h->d_eps_re_fe.p;
  v.eps_im_fe = h->d_eps_im_fe.p;
  v.sa_a_fe = t->d_a_fe.p;
  v.sa_b_fe = t->d_b_fe.p;
  v.sa_c_fe = t->d_c_fe.p;
  v.sa_min_fe = t->d_sa_min_fe.p;
}

}  // namespace

int nmg::prepare_view(nm_handle* h, int r0, int r1, nmg::DeviceView& v, nmg::KernelKind& kind) {
  const int nr = h->view.rows(), nc = h->view.cols();
  const bool hw = h->view.use_hardware() &&
                  (h->path == NM_PATH_REFERENCE || h->path == NM_PATH_MP || double_loop_direct(h));
  const int mp_limbs = nmg::mp_limbs_for_bits(h->view.bits());
  if (h->tables_stale()) return fail(NM_ERR_STATE, kStalePreview);
  if (h->path == NM_PATH_MP) {
    if (mp_limbs < nmg::kMpMinLimbs || mp_limbs > nmg::kMpMaxLimbs)
      return fail(NM_ERR_UNSUPPORTED, "the reference-exact path takes 64 to %d bits of precision "
                  "(the view has %lu)", 64 * (nmg::kMpMaxLimbs - 2), h->view.bits());
    if (!hw && h->precomputed && h->od.mp_limbs != mp_limbs)
      return fail(NM_ERR_STATE, "precomputed without the arbitrary-precision orbit; "
                                "nm_precompute again after choosing NM_PATH_MP");
    if (!hw && h->precomputed && !h->od.sa_fp64_ok)
      return fail(NM_ERR_UNSUPPORTED, "the reference-exact path needs series terms in the double "
                                      "range (the reference renders no other view)");
  }
  if (!hw && !h->precomputed)
    return fail(NM_ERR_STATE, "deep view: nm_precompute must run before rendering");
  if (!hw && h->od.double_loop && h->path != NM_PATH_FE32)
    return fail(NM_ERR_STATE, "precomputed for the FE32 path on a double-loop view; "
                              "nm_precompute again after changing the path");
  if (int rc = ensure_grid(h)) return rc;
  if (int rc = ensure_coords(h)) return rc;
  if (!h->uploaded)
    if (int rc = do_upload(h)) return rc;
  std::memset(&v, 0, sizeof v);
  v.nr = nr;
  v.nc = nc;
  v.N = h->effective_N();
  v.cardioid_mode = h->outside_cardioid ? nmg::CARDIOID_NONE : nmg::CARDIOID_PER_SAMPLE;
  v.tol = h->view.tolerance();
  v.bailout2 = 1024.0 * 1024.0;
  v.log_bailout = std::log(1024.0);
  v.tile_w = h->tile_w;
  v.tile_h = h->tile_h;
  v.row0 = r0;
  v.row1 = r1;
  v.tiles_x = (nc + h->tile_w - 1) / h->tile_w;
  v.tiles_y = (r1 - r0 + h->tile_h - 1) / h->tile_h;
  v.total = (long long)v.tiles_x * v.tiles_y * h->tile_w * h->tile_h;
  v.coord_re = h->d_coord_re.p;
  v.coord_im = h->d_coord_im.p;
  v.c_abs = coord_abs_bound(h);
  if (!hw) {
    const nm_handle* t = h->tables();  // a sharing preview: its source's orbit and series
    v.eps_re = h->d_eps_re.p;
    v.eps_im = h->d_eps_im.p;
    v.z = t->orbit_z();
    v.zf = t->d_zf.p;
    v.zlen = (int)t->zlen();
    v.xlen = h->od.xlen;
    v.xhi = t->d_xhi.p;
    v.xlo = t->d_xlo.p;
    v.sa_a = t->d_a.p;
    v.sa_b = t->d_b.p;
    v.sa_c = t->d_c.p;
    v.sa_min = t->d_sa_min.p;
    set_fe_tables(h, v);
    v.double_loop = h->od.double_loop ? 1 : 0;
    if (h->od.double_loop) {  // the FE32 path on a double-loop view: trapping records
      NM_CUDA(h->d_fe_trap.reserve((size_t)v.total));
      v.trap = h->d_fe_trap.p;
    }
  }
  v.grid = h->grid.p;
  v.smooth64 = h->keep_smooth64 ? h->smooth64.p : nullptr;
  const bool whole = r0 == 0 && r1 == nr;
  const long long ntiles = (long long)v.tiles_x * v.tiles_y;
  const bool host_order = !h->tile_order.empty() && (long long)h->tile_order.size() == ntiles;
  const bool device_order = h->tile_order_on_device && h->tile_order_n == ntiles;
  if (whole && (host_order || device_order) && h->tile_order_w == h->tile_w &&
      h->tile_order_h == h->tile_h) {
    if (host_order && !h->tile_order_uploaded) {
      if (int rc = upload(h->d_tile_order, h->tile_order, h->stream)) return rc;
      NM_CUDA(cudaStreamSynchronize(h->stream));
      h->tile_order_uploaded = true;
    }
    v.tile_order = h->d_tile_order.p;
  }
  if (h->path == NM_PATH_MP) {
    v.mp_limbs = mp_limbs;
    v.coord_re_mp = h->d_coord_re_mp.p;
    v.coord_im_mp = h->d_coord_im_mp.p;
    v.x_mp = hw ? nullptr : h->tables()->d_x_mp.p;
    kind = hw ? nmg::KERNEL_HW_MP : nmg::KERNEL_MP;
    return NM_OK;
  }
  kind = hw ? nmg::KERNEL_HW : (h->path == NM_PATH_FE32 ? nmg::KERNEL_FE32 : nmg::KERNEL_DELTA64);
  return NM_OK;
}



extern "C" {

const char* nm_last_error(void) { return g_last_error.c_str(); }

nm_handle* nm_create(int nr, int nc) {
  if (nr < 1 || nc < 1) {
    fail(NM_ERR_ARG, "grid size %d x %d", nr, nc);
    return nullptr;
  }
  return new nm_handle(nr, nc);
}

nm_handle* nm_copy(const nm_handle* src) {
  if (!src) {
    fail(NM_ERR_ARG, "null handle");
    return nullptr;
  }
  std::unique_ptr<nm_handle> h(new nm_handle(1, 1));
  h->view = src->view;
  h->path = src->path;
  h->tile_w = src->tile_w;
  h->tile_h = src->tile_h;
  h->chunk = src->chunk;
  h->blocks = src->blocks;
  h->threads = src->threads;
  h->renorm = src->renorm;
  h->keep_smooth64 = src->keep_smooth64;
  h->coord_re = src->coord_re;
  h->coord_im = src->coord_im;
  h->coord_re_mp = src->coord_re_mp;
  h->coord_im_mp = src->coord_im_mp;
  h->eps_re = src->eps_re;
  h->eps_im = src->eps_im;
  h->eps_re_fe = src->eps_re_fe;
  h->eps_im_fe = src->eps_im_fe;
  h->eps32_re = src->eps32_re;
  h->eps32_im = src->eps32_im;
  h->a32 = src->a32;
  h->b32 = src->b32;
  h->c32 = src->c32;
  h->sa_min32 = src->sa_min32;
  h->reference_mode = src->reference_mode;
  h->fe_single_pass = src->fe_single_pass;
  h->fe_overlap = src->fe_overlap;
  h->z_stage = src->z_stage;
  h->l2_window = src->l2_window;
  h->tile_order = src->tile_order;
  if (src->tile_order_on_device && src->d_tile_order.p) {  // the copy holds it on the host
    h->tile_order.resize((size_t)src->tile_order_n);
    if (cudaStreamSynchronize(src->stream) != cudaSuccess ||
        cudaMemcpy(h->tile_order.data(), src->d_tile_order.p, h->tile_order.size() * 4,
                   cudaMemcpyDeviceToHost) != cudaSuccess) {
      fail(NM_ERR_CUDA, "copy of a device tile order");
      return nullptr;
    }
  }
  h->tile_order_w = src->tile_order_w;
  h->tile_order_h = src->tile_order_h;
  h->log_costs = src->log_costs;
  h->od = src->od;
  h->od_zlen = src->od_zlen;
  h->orbit_src = src->orbit_src;
  h->src_stamp = src->src_stamp;
  h->iter_cap = src->iter_cap;
  h->precomputed = src->precomputed;
  h->coords_valid = src->coords_valid;
  h->outside_cardioid = src->outside_cardioid;
  if (!src->stream) return h.release();  // nothing on the GPU yet
  if (ensure_grid(h.get()) != NM_OK) return nullptr;
  cudaError_t e = cudaStreamSynchronize(src->stream);
  const size_t n = (size_t)src->grid_nr * src->grid_nc;
  if (e == cudaSuccess)
    e = cudaMemcpy(h->grid.p, src->grid.p, n * sizeof(EscapeValue), cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess && src->keep_smooth64 && src->smooth64.p)
    e = cudaMemcpy(h->smooth64.p, src->smooth64.p, n * sizeof(double), cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) {
    fail(NM_ERR_CUDA, "copy: %s", cudaGetErrorString(e));
    return nullptr;
  }
  return h.release();
}

void nm_destroy(nm_handle* h) {
  if (h) {
    if (h->stream) cudaStreamSynchronize(h->stream);
    delete h;
  }
}

int nm_set_view(nm_handle* h, const char* cre, const char* cim, const char* sre, const char* sim,
                int N, double tol, int min_bits) {
  if (int rc = check_handle(h)) return rc;
  if (N < 1) return fail(NM_ERR_ARG, "N must be >= 1 (got %d)", N);
  if (!(tol >= 0.0)) return fail(NM_ERR_ARG, "tolerance must be >= 0");
  int rc = h->view.set_view(cre, cim, sre, sim, N, tol, min_bits);
  if (rc == 1) return fail(NM_ERR_ARG, "null view string");
  if (rc == 2) return fail(NM_ERR_PARSE, "view string does not parse as a decimal number");
  h->invalidate();
  return NM_OK;
}

int nm_get_view(const nm_handle* h, int which, char* buf, int buflen) {
  if (int rc = check_handle(h)) return rc;
  if (!buf || which < 0 || which > 3) return fail(NM_ERR_ARG, "bad view field %d", which);
  std::string s = which == 0 ? h->view.center_re_str()
                : which == 1 ? h->view.center_im_str()
                : which == 2 ? h->view.step_re_str()
                             : h->view.step_im_str();
  if ((int)s.size() + 1 > buflen) return fail(NM_ERR_ARG, "buffer too small (%zu)", s.size() + 1);
  std::memcpy(buf, s.c_str(), s.size() + 1);
  return NM_OK;
}

int nm_set_iterations(nm_handle* h, int N) {
  if (int rc = check_handle(h)) return rc;
  if (N < 1) return fail(NM_ERR_ARG, "N must be >= 1 (got %d)", N);
  h->view.set_iterations(N);
  h->precomputed = false;
  h->uploaded = false;
  h->generation++;
  return NM_OK;
}
int nm_get_iterations(const nm_handle* h) { return h ? h->view.iterations() : -1; }
int nm_set_tolerance(nm_handle* h, double tol) {
  if (int rc = check_handle(h)) return rc;
  if (!(tol >= 0.0)) return fail(NM_ERR_ARG, "tolerance must be >= 0");
  h->view.set_tolerance(tol);
  h->precomputed = false;
  h->uploaded = false;
  h->generation++;
  return NM_OK;
}
int nm_rows(const nm_handle* h) { return h ? h->view.rows() : -1; }
int nm_cols(const nm_handle* h) { return h ? h->view.cols() : -1; }
int nm_use_hardware(const nm_handle* h) { return h ? (h->view.use_hardware() ? 1 : 0) : -1; }

int nm_set_path(nm_handle* h, int path) {
  if (int rc = check_handle(h)) return rc;
  if (path < NM_PATH_REFERENCE || path > NM_PATH_MP) return fail(NM_ERR_ARG, "bad path %d", path);
  if ((path == NM_PATH_MP) != (h->path == NM_PATH_MP)) {
    h->coords_valid = false;  // the arbitrary-precision coordinate tables come and go
    h->uploaded = false;
  }
  h->path = path;
  h->generation++;
  return NM_OK;
}

int nm_set_option(nm_handle* h, int opt, long long value) {
  if (int rc = check_handle(h)) return rc;
  h->generation++;
  switch (opt) {
    case NM_OPT_TILE_W:
    case NM_OPT_TILE_H:
      if (value < 1 || value > 1024) return fail(NM_ERR_ARG, "tile size %lld", value);
      (opt == NM_OPT_TILE_W ? h->tile_w : h->tile_h) = (int)value;
      return NM_OK;
    case NM_OPT_CHUNK:
      if (value < 1 || value > (1 << 20)) return fail(NM_ERR_ARG, "chunk %lld", value);
      h->chunk = (int)value;
      return NM_OK;
    case NM_OPT_KEEP_SMOOTH64:
      h->keep_smooth64 = value != 0;
      return h->stream ? ensure_grid(h) : NM_OK;
    case NM_OPT_THREADS:
      if (value < 0) return fail(NM_ERR_ARG, "threads %lld", value);
      h->threads = (int)value;
      return NM_OK;
    case NM_OPT_BLOCKS:
      if (value < 0 || value > (1 << 20)) return fail(NM_ERR_ARG, "blocks %lld", value);
      h->blocks = (int)value;
      return NM_OK;
    case NM_OPT_RENORM:
      if (value < 0 || value > 256) return fail(NM_ERR_ARG, "renorm interval %lld", value);
      h->renorm = (int)value;
      return NM_OK;
    case NM_OPT_FE32_SINGLE_PASS:
      h->fe_single_pass = value != 0;
      return NM_OK;
    case NM_OPT_FE32_OVERLAP:
      h->fe_overlap = value != 0;
      return NM_OK;
    case NM_OPT_LOG_TILE_COSTS:
      h->log_costs = value != 0;
      return NM_OK;
    case NM_OPT_ORBIT_STAGE:
      if (value < -1 || value > 3072)
        return fail(NM_ERR_ARG, "orbit stage %lld (-1..3072)", value);
      h->z_stage = (int)value;
      return NM_OK;
    case NM_OPT_L2_WINDOW:
      h->l2_window = value != 0;
      return NM_OK;
    case NM_OPT_ITER_CAP:
      if (value < 0 || value > (1ll << 31) - 1) return fail(NM_ERR_ARG, "iteration cap %lld", value);
      h->iter_cap = (int)value;
      return NM_OK;
    case NM_OPT_REFERENCE:
      if (value != nmg::REFERENCE_PROBES && value != nmg::REFERENCE_CENTER)
        return fail(NM_ERR_ARG, "reference mode %lld", value);
      h->reference_mode = (int)value;
      h->precomputed = false;
      h->uploaded = false;
      return NM_OK;
  }
  return fail(NM_ERR_ARG, "unknown option %d", opt);
}

int nm_get_stat(nm_handle* h, int stat, long long* value) {
  if (int rc = check_handle(h)) return rc;
  if (!value) return fail(NM_ERR_ARG, "null output");
  if (stat >= 0 && stat < nmg::STAT_COUNT) {
    unsigned long long v = 0;
    if (!h->stream) {
      *value = 0;
      return NM_OK;
    }
    NM_CUDA(cudaStreamSynchronize(h->stream));
    const int slot = stat == nmg::STAT_REWORK ? kReworkCount : kStatsMain + stat;
    NM_CUDA(cudaMemcpy(&v, h->d_scratch.p + slot, 8, cudaMemcpyDeviceToHost));
    *value = (long long)v;
    return NM_OK;
  }
  switch (stat) {
    case NM_STAT_ORBIT_LENGTH: *value = h->precomputed ? h->od.xlen : 0; return NM_OK;
    case NM_STAT_PROBE_INDEX: *value = h->precomputed ? h->od.probe_index : -1; return NM_OK;
    case NM_STAT_PRECISION_BITS: *value = (long long)h->view.bits(); return NM_OK;
    case NM_STAT_PRECOMPUTE_US: *value = (long long)h->precompute_us; return NM_OK;
    case NM_STAT_KERNEL_LAUNCHES: *value = nmg::launches_so_far(); return NM_OK;
    case NM_STAT_KERNEL_NS:
    case NM_STAT_REWORK_KERNEL_NS:
    case NM_STAT_ITER_KERNEL_NS: {
      *value = 0;
      if (!h->stream || (stat == NM_STAT_REWORK_KERNEL_NS && !h->timed_rework) ||
          (stat == NM_STAT_ITER_KERNEL_NS && !h->timed_iter))
        return NM_OK;
      cudaEvent_t a = stat == NM_STAT_KERNEL_NS ? h->ev[0]
                    : stat == NM_STAT_REWORK_KERNEL_NS ? h->ev[1] : h->ev[3];
      cudaEvent_t b = stat == NM_STAT_KERNEL_NS ? h->ev[1]
                    : stat == NM_STAT_REWORK_KERNEL_NS ? h->ev[2] : h->ev[4];
      if (cudaEventSynchronize(b) != cudaSuccess) return NM_OK;  // never recorded
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) *value = (long long)(ms * 1e6);
      return NM_OK;
    }
  }
  return fail(NM_ERR_ARG, "unknown stat %d", stat);
}

// findProbe's orbit lengths on the handle's GPU (the same arithmetic as the
// host's, bit for bit); false when no GPU is at hand or the precision has no
// kernel, and the host threads find them.
static bool gpu_probe_lengths(void* ctx, int limbs, const std::vector<uint64_t>& re,
                              const std::vector<uint64_t>& im, int N, std::vector<int>& len) {
  nm_handle* h = static_cast<nm_handle*>(ctx);
  if (limbs < nmg::kMpMinLimbs || limbs > nmg::kMpMaxLimbs) return false;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return false;
  }
  if (ensure_device(h) != NM_OK) return false;
  const int n = (int)len.size();
  DevBuf<uint64_t> d_re, d_im;
  DevBuf<int32_t> d_len;
  if (d_re.reserve(re.size()) || d_im.reserve(im.size()) || d_len.reserve((size_t)n)) return false;
  cudaStream_t s = h->stream;
  if (cudaMemcpyAsync(d_re.p, re.data(), re.size() * 8, cudaMemcpyHostToDevice, s) ||
      cudaMemcpyAsync(d_im.p, im.data(), im.size() * 8, cudaMemcpyHostToDevice, s) ||
      nmg::launch_probes(limbs, d_re.p, d_im.p, n, N, d_len.p, s) ||
      cudaMemcpyAsync(len.data(), d_len.p, (size_t)n * 4, cudaMemcpyDeviceToHost, s) ||
      cudaStreamSynchronize(s))
    return false;
  return true;
}

int nm_precompute(nm_handle* h) {
  if (int rc = check_handle(h)) return rc;
  auto t0 = std::chrono::steady_clock::now();
  h->coords_valid = false;
  if (int rc = ensure_coords(h)) return rc;
  h->precomputed = false;
  h->orbit_src = nullptr;  // from here on the handle's own orbit
  h->od_zlen = 0;
  h->tables_stamp++;  // previews sharing the old orbit no longer render
  if (double_loop_direct(h)) {
    // rendered by the double loop: nothing to precompute
  } else if (h->view.use_hardware() && h->path == NM_PATH_FE32) {
    // the FE32 path on a view the reference renders with its double loop:
    // the view-center orbit at 256 bits or more, offsets of the loop's start
    if (h->view.precompute_center_orbit(h->od, kDoubleLoopOrbitBits))
      return fail(NM_ERR_STATE, "precompute failed");
    std::vector<double> px(h->coord_re.size()), py(h->coord_im.size());
    for (size_t c = 0; c < px.size(); c++) px[c] = h->coord_re[c].x;
    for (size_t r = 0; r < py.size(); r++) py[r] = h->coord_im[r].x;
    h->view.eps_tables_double_loop(px, py, h->eps_re, h->eps_im);
    h->precomputed = true;
  } else if (!h->view.use_hardware() ||
             (h->path != NM_PATH_REFERENCE && h->path != NM_PATH_MP)) {
    int threads = h->threads > 0 ? h->threads : (int)std::thread::hardware_concurrency();
    if (h->view.precompute(threads, h->od, h->reference_mode, h->path == NM_PATH_MP,
                           gpu_probe_lengths, h))
      return fail(NM_ERR_STATE, "precompute failed");
    h->view.eps_tables(h->od, h->eps_re, h->eps_im);
    if (!h->od.sa_fp64_ok) h->view.eps_tables_fe(h->eps_re_fe, h->eps_im_fe);
    build_front32_tables(h);
    h->precomputed = true;
  }
  h->precompute_us =
      std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
  h->uploaded = false;  // copied to the GPU by nm_upload or the next render
  h->generation++;
  return NM_OK;
}

int nm_get_orbit(nm_handle* h, double* x, double* xlo, double* a, double* b, double* c, int n) {
  if (int rc = check_handle(h)) return rc;
  if (h->orbit_src && h->precomputed) h = h->orbit_src;
  if (!h->precomputed || h->od.double_loop) return fail(NM_ERR_STATE, "no precomputed orbit and series");
  if (n != h->od.xlen) return fail(NM_ERR_ARG, "%d entries for an orbit of %d", n, h->od.xlen);
  for (int i = 0; i < n; i++) {
    if (x) x[2 * i] = h->od.xhi[i].x, x[2 * i + 1] = h->od.xhi[i].y;
    if (xlo) xlo[2 * i] = h->od.xlo[i].x, xlo[2 * i + 1] = h->od.xlo[i].y;
    if (a) a[2 * i] = h->od.a[i].x, a[2 * i + 1] = h->od.a[i].y;
    if (b) b[2 * i] = h->od.b[i].x, b[2 * i + 1] = h->od.b[i].y;
    if (c) c[2 * i] = h->od.c[i].x, c[2 * i + 1] = h->od.c[i].y;
  }
  return NM_OK;
}

int nm_upload(nm_handle* h) {
  if (int rc = check_handle(h)) return rc;
  if (int rc = ensure_coords(h)) return rc;
  return do_upload(h);
}

// The FP64 rework of the FE32 path: the rework list, its length and claim
// counter, and statistics of its own.
static nmg::RenderCtl rework_ctl(nm_handle* h, const nmg::RenderCtl& main) {
  nmg::RenderCtl re = main;
  re.next = h->d_scratch.p + kNextRework;
  re.stats = h->d_scratch.p + kStatsRework;
  re.list = h->d_rework.p;
  re.count_ptr = h->d_scratch.p + kReworkCount;
  re.first = 0;
  re.count = 0;
  re.rework = nullptr;
  re.rework_n = nullptr;
  return re;
}

int nm_render_rows(nm_handle* h, int r0, int r1, void* stream_arg) {
  if (int rc = check_handle(h)) return rc;
  const int nr = h->view.rows(), nc = h->view.cols();
  if (r0 < 0 || r1 > nr || r0 > r1) return fail(NM_ERR_ARG, "rows [%d, %d) of %d", r0, r1, nr);
  nmg::DeviceView v;
  nmg::KernelKind kind;
  if (int rc = prepare_view(h, r0, r1, v, kind)) return rc;
  cudaStream_t s = stream_arg ? (cudaStream_t)stream_arg : h->stream;
  h->render_stream = s;
  h->last_overlapped = false;
  nmg::RenderCtl ctl;
  std::memset(&ctl, 0, sizeof ctl);
  ctl.next = h->d_scratch.p + kNextMain;
  ctl.stats = h->d_scratch.p + kStatsMain;
  ctl.cancel = h->cancel_dev;
  ctl.first = 0;
  ctl.count = v.total;
  if (kind == nmg::KERNEL_FE32) {
    NM_CUDA(h->d_rework.reserve((size_t)v.total));
    ctl.rework = h->d_rework.p;
    ctl.rework_n = h->d_scratch.p + kReworkCount;
  }
  if (h->log_costs && r0 == 0 && r1 == nr) {
    const long long tiles = (long long)v.tiles_x * v.tiles_y;
    NM_CUDA(h->d_tile_cost.reserve((size_t)tiles));
    NM_CUDA(cudaMemsetAsync(h->d_tile_cost.p, 0, (size_t)tiles * 8, s));
    v.tile_cost = h->d_tile_cost.p;
    h->cost_tiles = tiles;
  }
  *h->cancel_host = 0;
  h->expected_samples = (long long)(r1 - r0) * nc;
  NM_CUDA(cudaMemsetAsync(h->d_scratch.p, 0, kScratchWords * 8, s));
  if (v.total == 0) return NM_OK;
  int blocks = h->blocks > 0 ? h->blocks : nmg::persistent_blocks(kind, h->device);
  long long max_useful = (v.total + 31) / 32;  // one warp per 32 samples at most
  long long warps_per_block = nmg::kernel_threads(kind) / 32;
  long long need_blocks = (max_useful + warps_per_block - 1) / warps_per_block;
  if (blocks > need_blocks) blocks = (int)need_blocks;
  if (blocks < 1) blocks = 1;
  int chunk = h->chunk;
  if (kind == nmg::KERNEL_FE32)  // the FE32 kernel renormalises per chunk
    chunk = h->renorm > 0 ? h->renorm : (v.sa_fe ? 32 : 64);
  NM_CUDA(cudaEventRecord(h->ev[0], s));
  h->timed_iter = false;
  if (kind == nmg::KERNEL_FE32 && !h->fe_single_pass) {
    // FE32 pass pipeline: FP64 front, FP32 iteration and smoothing
    NM_CUDA(h->d_fe_state.reserve((size_t)v.total * nmg::kFeStateBytes));
    NM_CUDA(h->d_work.reserve((size_t)v.total));
    nmg::FePassBuffers b;
    b.state = reinterpret_cast<nmg::FeState*>(h->d_fe_state.p);
    b.work = h->d_work.p;
    b.work_n = h->d_scratch.p + kWorkCount;
    nmg::OverlapCtl o;
    if (h->fe_overlap) {
      // the FP64 side reads list entries until they differ from the sentinel
      NM_CUDA(cudaMemsetAsync(h->d_rework.p, 0xff, (size_t)v.total * sizeof(unsigned int), s));
      o.rework = rework_ctl(h, ctl);
      o.fe_warps_done = h->d_scratch.p + kFeWarpsDone;
      o.timeouts = h->d_scratch.p + kStatsMain + nmg::STAT_WAIT_TIMEOUTS;
      o.chunk = h->chunk;
    }
    // Staging the orbit's first entries: measured on the 3840x2160 view at
    // width 1e-300 (floatexp series) 32.3 -> 31.4 ms with 1024 entries (31.7
    // with 2048); on the 1920x1080x16 view at 1e-12 no change with 1024 and
    // 12 % slower with 2048 (3 blocks an SM instead of 4).
    const int stage = h->z_stage >= 0 ? h->z_stage : (v.sa_fe ? kAutoOrbitStage : 0);
    NM_CUDA(nmg::launch_fe32_passes(v, b, ctl, s, h->device, h->blocks, chunk, h->ev[3],
                                    h->ev[4], h->fe_overlap ? &o : nullptr, stage,
                                    h->l2_window));
    h->timed_iter = true;
    h->last_overlapped = h->fe_overlap;
    h->last_view = v;
  } else {
    NM_CUDA(nmg::launch_render(kind, v, ctl, s, blocks, chunk));
  }
  NM_CUDA(cudaEventRecord(h->ev[1], s));
  h->timed_rework = kind == nmg::KERNEL_FE32;
  if (kind == nmg::KERNEL_FE32) {
    // Samples the FE32 kernel could not certify: the plain FP64 kernel
    // renders them again, reading the list and its length from the GPU (after
    // an overlapped iteration pass: only the entries it left unclaimed).
    const nmg::RenderCtl re = rework_ctl(h, ctl);
    int rblocks = h->blocks > 0 ? h->blocks : nmg::persistent_blocks(nmg::KERNEL_REWORK, h->device);
    NM_CUDA(nmg::launch_render(nmg::KERNEL_REWORK, v, re, s, rblocks, h->chunk));
    NM_CUDA(cudaEventRecord(h->ev[2], s));
  }
  return NM_OK;
}

int nm_synchronize(nm_handle* h) {
  if (int rc = check_handle(h)) return rc;
  if (!h->stream) return NM_OK;
  cudaStream_t s = h->render_stream ? h->render_stream : h->stream;
  NM_CUDA(cudaStreamSynchronize(s));
  if (s != h->stream) NM_CUDA(cudaStreamSynchronize(h->stream));
  if (h->last_overlapped) {
    // An overlapped FP64 consumer skips a rework entry it claimed but could not
    // read within its poll limit (counted in STAT_WAIT_TIMEOUTS).  Every entry
    // is written once the launch has ended, so the whole list is rendered
    // again in FP64 -- the same results for the samples already rendered.
    h->last_overlapped = false;
    unsigned long long lost = 0;
    NM_CUDA(cudaMemcpy(&lost, h->d_scratch.p + kStatsMain + nmg::STAT_WAIT_TIMEOUTS, 8,
                       cudaMemcpyDeviceToHost));
    if (lost && !*h->cancel_host) {
      nmg::RenderCtl main{};
      main.cancel = h->cancel_dev;
      const nmg::RenderCtl re = rework_ctl(h, main);
      NM_CUDA(cudaMemsetAsync(h->d_scratch.p + kNextRework, 0, 8, s));
      NM_CUDA(nmg::launch_render(nmg::KERNEL_REWORK, h->last_view, re, s,
                                 nmg::persistent_blocks(nmg::KERNEL_REWORK, h->device), h->chunk));
      NM_CUDA(cudaStreamSynchronize(s));
    }
  }
  if (*h->cancel_host) {
    unsigned long long done = 0;
    NM_CUDA(cudaMemcpy(&done, h->d_scratch.p + kStatsMain + nmg::STAT_SAMPLES, 8,
                       cudaMemcpyDeviceToHost));
    if ((long long)done < h->expected_samples)
      return fail(NM_ERR_CANCELLED, "render cancelled after %llu of %lld samples", done,
                  h->expected_samples);
  }
  return NM_OK;
}

int nm_render(nm_handle* h) {
  if (int rc = nm_render_rows(h, 0, h ? h->view.rows() : 0, nullptr)) return rc;
  return nm_synchronize(h);
}

int nm_compute_row(nm_handle* h, int r) {
  if (int rc = nm_render_rows(h, r, r + 1, nullptr)) return rc;
  return nm_synchronize(h);
}

int nm_tiles(nm_handle* h, int* tiles_x, int* tiles_y) {
  if (int rc = check_handle(h)) return rc;
  if (!tiles_x || !tiles_y) return fail(NM_ERR_ARG, "null output");
  *tiles_x = (h->view.cols() + h->tile_w - 1) / h->tile_w;
  *tiles_y = (h->view.rows() + h->tile_h - 1) / h->tile_h;
  return NM_OK;
}

int nm_set_tile_order(nm_handle* h, const int* order, int n) {
  if (int rc = check_handle(h)) return rc;
  if (!order || n == 0) {
    h->tile_order_on_device = false;
    h->tile_order.clear();
    h->generation++;
    return NM_OK;
  }
  int tx = 0, ty = 0;
  nm_tiles(h, &tx, &ty);
  if ((long long)n != (long long)tx * ty)
    return fail(NM_ERR_ARG, "tile order of %d entries for %d x %d tiles", n, tx, ty);
  std::vector<char> seen((size_t)n, 0);
  for (int k = 0; k < n; k++) {
    if (order[k] < 0 || order[k] >= n || seen[(size_t)order[k]])
      return fail(NM_ERR_ARG, "tile order is not a permutation (entry %d = %d)", k, order[k]);
    seen[(size_t)order[k]] = 1;
  }
  h->generation++;
  h->tile_order_on_device = false;
  h->tile_order.assign(order, order + n);
  h->tile_order_w = h->tile_w;
  h->tile_order_h = h->tile_h;
  h->tile_order_uploaded = false;
  return NM_OK;
}

int nm_get_tile_order(nm_handle* h, int* out, int n) {
  if (int rc = check_handle(h)) return rc;
  if (!out) return fail(NM_ERR_ARG, "null output");
  if (h->tile_order_on_device) {
    if ((long long)n != h->tile_order_n)
      return fail(NM_ERR_ARG, "%d entries for an order of %lld tiles", n, h->tile_order_n);
    NM_CUDA(cudaStreamSynchronize(h->stream));
    NM_CUDA(cudaMemcpy(out, h->d_tile_order.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
    return NM_OK;
  }
  if (h->tile_order.empty()) return fail(NM_ERR_STATE, "no tile order set (static order)");
  if ((size_t)n != h->tile_order.size())
    return fail(NM_ERR_ARG, "%d entries for an order of %zu tiles", n, h->tile_order.size());
  std::memcpy(out, h->tile_order.data(), (size_t)n * 4);
  return NM_OK;
}

int nm_get_tile_costs(nm_handle* h, unsigned long long* out, int n) {
  if (int rc = check_handle(h)) return rc;
  if (!out) return fail(NM_ERR_ARG, "null output");
  if (h->cost_tiles == 0 || !h->stream)
    return fail(NM_ERR_STATE, "no logged render (set NM_OPT_LOG_TILE_COSTS, render the whole grid)");
  if ((long long)n != h->cost_tiles)
    return fail(NM_ERR_ARG, "%d entries for a log of %lld tiles", n, h->cost_tiles);
  NM_CUDA(cudaStreamSynchronize(h->stream));
  NM_CUDA(cudaMemcpy(out, h->d_tile_cost.p, (size_t)n * 8, cudaMemcpyDeviceToHost));
  return NM_OK;
}

nm_handle* nm_preview(const nm_handle* src, int factor) {
  if (!src || factor < 1) {
    fail(NM_ERR_ARG, "preview of %s at factor %d", src ? "a view" : "a null handle", factor);
    return nullptr;
  }
  if (src->view.rows() % factor || src->view.cols() % factor) {
    fail(NM_ERR_ARG, "grid %d x %d is not a multiple of the preview factor %d", src->view.rows(),
         src->view.cols(), factor);
    return nullptr;
  }
  std::unique_ptr<nm_handle> h(new nm_handle(1, 1));
  h->view = src->view;
  h->view.stand_in_for(src->view);  // the source's precision and arithmetic
  h->view.scale_down(factor);
  h->path = src->path;
  h->chunk = src->chunk;
  h->threads = src->threads;
  h->renorm = src->renorm;
  h->reference_mode = src->reference_mode;
  h->fe_overlap = src->fe_overlap;
  if (src->precomputed && (src->reference_mode == nmg::REFERENCE_CENTER || src->od.double_loop)) {
    // the orbit at the view center and its series do not depend on the grid:
    // only the per-row / per-column tables are the preview's own
    if (src->od.double_loop) {
      h->od = src->od;
    } else {
      // the orbit and series stay with their owner, read in place (host
      // vectors and device tables): only their sizes and flags come along
      const nm_handle* owner = src->tables();
      h->orbit_src = const_cast<nm_handle*>(owner);
      h->src_stamp = owner->tables_stamp;
      h->od_zlen = owner->zlen();
      h->od.xlen = src->od.xlen;
      h->od.probe_index = src->od.probe_index;
      h->od.sa_fp64_ok = src->od.sa_fp64_ok;
      h->od.double_loop = false;
      h->od.mp_limbs = src->od.mp_limbs;
    }
    if (ensure_coords(h.get()) != NM_OK) return nullptr;
    if (h->od.double_loop) {
      std::vector<double> px(h->coord_re.size()), py(h->coord_im.size());
      for (size_t c = 0; c < px.size(); c++) px[c] = h->coord_re[c].x;
      for (size_t r = 0; r < py.size(); r++) py[r] = h->coord_im[r].x;
      h->view.eps_tables_double_loop(px, py, h->eps_re, h->eps_im);
    } else {
      h->view.eps_tables(h->od, h->eps_re, h->eps_im);
      if (!h->od.sa_fp64_ok) h->view.eps_tables_fe(h->eps_re_fe, h->eps_im_fe);
      build_front32_tables(h.get(), /*series=*/false);
    }
    h->precomputed = true;
  }
  return h.release();
}

int nm_cancel(nm_handle* h) {
  if (int rc = check_handle(h)) return rc;
  *(volatile int*)h->cancel_host = 1;
  return NM_OK;
}

int nm_at(nm_handle* h, int r, int c, nm_escape_value* out) {
  if (int rc = check_handle(h)) return rc;
  if (int rc = ensure_grid(h)) return rc;
  if (!out || r < 0 || c < 0 || r >= h->grid_nr || c >= h->grid_nc)
    return fail(NM_ERR_ARG, "at(%d, %d) outside %d x %d", r, c, h->grid_nr, h->grid_nc);
  NM_CUDA(cudaStreamSynchronize(h->stream));
  NM_CUDA(cudaMemcpy(out, h->grid.p + (size_t)r * h->grid_nc + c, sizeof(EscapeValue),
                     cudaMemcpyDeviceToHost));
  return NM_OK;
}

int nm_at_sc(nm_handle* h, int r, int c, int sc, nm_escape_value* out) {
  if (int rc = check_handle(h)) return rc;
  if (int rc = ensure_grid(h)) return rc;
  if (!out || sc < 1 || r < 0 || c < 0 || (long long)sc * (r + 1) > h->grid_nr ||
      (long long)sc * (c + 1) > h->grid_nc)
    return fail(NM_ERR_ARG, "at(%d, %d, %d) outside %d x %d", r, c, sc, h->grid_nr, h->grid_nc);
  NM_CUDA(cudaStreamSynchronize(h->stream));
  std::vector<EscapeValue> block((size_t)sc * sc);
  for (int r1 = 0; r1 < sc; r1++)
    NM_CUDA(cudaMemcpy(block.data() + (size_t)r1 * sc,
                       h->grid.p + (size_t)(sc * r + r1) * h->grid_nc + (size_t)sc * c,
                       sc * sizeof(EscapeValue), cudaMemcpyDeviceToHost));
  // mandelbrot.cpp:322-330
  float sum = 0.0f;
  for (const EscapeValue& e : block) sum += e.iterations + e.smoothing;
  sum /= sc * sc;
  out->iterations = (int)sum;
  out->smoothing = sum - out->iterations;
  return NM_OK;
}

int nm_reduce(nm_handle* h, int sc, nm_escape_value* host_out) {
  if (int rc = check_handle(h)) return rc;
  if (int rc = ensure_grid(h)) return rc;
  if (!host_out || sc < 1) return fail(NM_ERR_ARG, "bad reduce arguments");
  const int nr = h->grid_nr / sc, nc = h->grid_nc / sc;
  DevBuf<EscapeValue> tmp;
  NM_CUDA(tmp.reserve((size_t)nr * nc));
  NM_CUDA(nmg::launch_reduce(h->grid.p, nr, nc, sc, tmp.p, h->stream));
  NM_CUDA(cudaMemcpyAsync(host_out, tmp.p, (size_t)nr * nc * sizeof(EscapeValue),
                          cudaMemcpyDeviceToHost, h->stream));
  NM_CUDA(cudaStreamSynchronize(h->stream));
  return NM_OK;
}

int nm_scale_up(nm_handle* h, int sc) {
  if (int rc = check_handle(h)) return rc;
  if (sc < 1) return fail(NM_ERR_ARG, "scale %d", sc);
  if (!h->stream) {  // no grid on the GPU yet: all zeros, nothing to duplicate
    h->view.scale_up(sc);
    h->invalidate();
    return NM_OK;
  }
  if (int rc = ensure_grid(h)) return rc;
  const int nr = h->grid_nr, nc = h->grid_nc;
  DevBuf<EscapeValue> bigger;
  NM_CUDA(bigger.reserve((size_t)nr * sc * nc * sc));
  NM_CUDA(nmg::launch_duplicate(h->grid.p, nr, nc, sc, bigger.p, h->stream));
  NM_CUDA(cudaStreamSynchronize(h->stream));
  std::swap(h->grid.p, bigger.p);
  std::swap(h->grid.n, bigger.n);
  h->grid_nr = nr * sc;
  h->grid_nc = nc * sc;
  h->smooth64.release();
  h->view.scale_up(sc);
  h->invalidate();
  return ensure_grid(h);
}

int nm_scale_down(nm_handle* h, int sc) {
  if (int rc = check_handle(h)) return rc;
  if (sc < 1) return fail(NM_ERR_ARG, "scale %d", sc);
  if (!h->stream) {  // no grid on the GPU yet: the mean of zeros is zero
    h->view.scale_down(sc);
    h->invalidate();
    return NM_OK;
  }
  if (int rc = ensure_grid(h)) return rc;
  const int nr = h->grid_nr / sc, nc = h->grid_nc / sc;
  DevBuf<EscapeValue> smaller;
  NM_CUDA(smaller.reserve((size_t)nr * nc));
  NM_CUDA(nmg::launch_reduce(h->grid.p, nr, nc, sc, smaller.p, h->stream));
  NM_CUDA(cudaStreamSynchronize(h->stream));
  std::swap(h->grid.p, smaller.p);
  std::swap(h->grid.n, smaller.n);
  h->grid_nr = nr;
  h->grid_nc = nc;
  h->smooth64.release();
  h->view.scale_down(sc);
  h->invalidate();
  return ensure_grid(h);
}

int nm_get_grid(nm_handle* h, nm_escape_value* host_out) {
  if (int rc = check_handle(h)) return rc;
  if (int rc = ensure_grid(h)) return rc;
  if (!host_out) return fail(NM_ERR_ARG, "null output");
  NM_CUDA(cudaMemcpyAsync(host_out, h->grid.p, (size_t)h->grid_nr * h->grid_nc * 8,
                          cudaMemcpyDeviceToHost, h->stream));
  NM_CUDA(cudaStreamSynchronize(h->stream));
  return NM_OK;
}

int nm_get_smoothing64(nm_handle* h, double* host_out) {
  if (int rc = check_handle(h)) return rc;
  if (int rc = ensure_grid(h)) return rc;
  if (!host_out) return fail(NM_ERR_ARG, "null output");
  if (!h->keep_smooth64 || !h->smooth64.p)
    return fail(NM_ERR_STATE, "NM_OPT_KEEP_SMOOTH64 is off");
  NM_CUDA(cudaMemcpyAsync(host_out, h->smooth64.p, (size_t)h->grid_nr * h->grid_nc * 8,
                          cudaMemcpyDeviceToHost, h->stream));
  NM_CUDA(cudaStreamSynchronize(h->stream));
  return NM_OK;
}

int nm_device_grid(nm_handle* h, nm_escape_value** grid, double** smooth64) {
  if (int rc = check_handle(h)) return rc;
  if (int rc = ensure_grid(h)) return rc;
  if (grid) *grid = reinterpret_cast<nm_escape_value*>(h->grid.p);
  if (smooth64) *smooth64 = h->keep_smooth64 ? h->smooth64.p : nullptr;
  return NM_OK;
}

int nm_point_at(const nm_handle* h, int r, int c, int sc, char* re, char* im, int buflen) {
  if (int rc = check_handle(h)) return rc;
  if (!re || !im) return fail(NM_ERR_ARG, "null output");
  nmg::Mpf pr(64), pi(64);
  h->view.point_at(r, c, sc, pr, pi);
  std::string a = nmg::MPView::to_string(pr), b = nmg::MPView::to_string(pi);
  if ((int)std::max(a.size(), b.size()) + 1 > buflen) return fail(NM_ERR_ARG, "buffer too small");
  std::memcpy(re, a.c_str(), a.size() + 1);
  std::memcpy(im, b.c_str(), b.size() + 1);
  return NM_OK;
}

int nm_translate(nm_handle* h, int dr, int dc, int sc) {
  if (int rc = check_handle(h)) return rc;
  h->view.translate(dr, dc, sc);
  h->invalidate();
  return NM_OK;
}

int nm_zoom(nm_handle* h, float scale) {
  if (int rc = check_handle(h)) return rc;
  if (!(scale > 0.0f)) return fail(NM_ERR_ARG, "zoom scale must be > 0");
  h->view.zoom(scale);
  h->invalidate();
  return NM_OK;
}

int nm_zoom_at(nm_handle* h, float scale, int r, int c, int sc) {
  if (int rc = check_handle(h)) return rc;
  if (!(scale > 0.0f)) return fail(NM_ERR_ARG, "zoom scale must be > 0");
  h->view.zoom_at(scale, r, c, sc);
  h->invalidate();
  return NM_OK;
}

int nm_load_legacy(nm_handle* h, const char* path) {
  if (int rc = check_handle(h)) return rc;
  if (!path) return fail(NM_ERR_ARG, "null path");
  int rc = h->view.load_legacy(path);
  if (rc == 1) return fail(NM_ERR_IO, "cannot open %s", path);
  if (rc == 2) return fail(NM_ERR_PARSE, "malformed view file %s", path);
  h->invalidate();
  return NM_OK;
}

int nm_save(const nm_handle* h, const char* path) {
  if (int rc = check_handle(h)) return rc;
  if (!path) return fail(NM_ERR_ARG, "null path");
  if (h->view.save(path)) return fail(NM_ERR_IO, "cannot write %s", path);
  return NM_OK;
}

}  // extern "C"

namespace nmg {

void noalloc_fail(const std::string& why) { g_last_error = why; }

// The device view of a handle whose tables are already on the GPU, for the
// allocation-free entry point (noalloc.cu): only reads the handle.
int noalloc_view(nm_handle* h, DeviceView& v, int& device, std::string& why, KernelKind& kind) {
  kind = double_loop_direct(h) ? KERNEL_HW : KERNEL_FE32;
  if (h->tables_stale()) {
    why = kStalePreview;
    return NM_ERR_STATE;
  }
  if (!h->uploaded || !h->stream ||
      (kind == KERNEL_FE32 && (!h->precomputed || !h->tables()->d_zf.p || !h->tables()->uploaded))) {
    why = "the view's tables are not on the GPU: call nm_precompute and nm_upload first";
    return NM_ERR_STATE;
  }
  const int nr = h->view.rows(), nc = h->view.cols();
  std::memset(&v, 0, sizeof v);
  v.nr = nr;
  v.nc = nc;
  v.N = h->effective_N();
  v.cardioid_mode = h->outside_cardioid ? CARDIOID_NONE : CARDIOID_PER_SAMPLE;
  v.tol = h->view.tolerance();
  v.bailout2 = 1024.0 * 1024.0;
  v.log_bailout = std::log(1024.0);
  v.tile_w = h->tile_w;
  v.tile_h = h->tile_h;
  v.row0 = 0;
  v.row1 = nr;
  v.tiles_x = (nc + h->tile_w - 1) / h->tile_w;
  v.tiles_y = (nr + h->tile_h - 1) / h->tile_h;
  v.total = (long long)v.tiles_x * v.tiles_y * h->tile_w * h->tile_h;
  v.coord_re = h->d_coord_re.p;
  v.coord_im = h->d_coord_im.p;
  v.eps_re = h->d_eps_re.p;
  v.eps_im = h->d_eps_im.p;
  const nm_handle* t = h->tables();
  v.z = t->orbit_z();
  v.zf = t->d_zf.p;
  v.zlen = (int)t->zlen();
  v.xlen = h->od.xlen;
  v.xhi = t->d_xhi.p;
  v.xlo = t->d_xlo.p;
  v.sa_a = t->d_a.p;
  v.sa_b = t->d_b.p;
  v.sa_c = t->d_c.p;
  v.sa_min = t->d_sa_min.p;
  set_fe_tables(h, v);
  v.double_loop = h->od.double_loop ? 1 : 0;
  v.c_abs = coord_abs_bound(h);
  device = h->device;
  return NM_OK;
}

}  // namespace nmg
