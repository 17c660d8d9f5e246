// Internal declarations shared by the C ABI's translation units (capi.cpp,
// batch.cpp): the handle behind nm_handle, device buffers, error reporting.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <string>
#include <vector>

#include "engine.hpp"
#include "mpview.hpp"
#include "newman_gb300.h"

namespace nmg {

// Records the message of the failing call (nm_last_error) and returns code.
int fail(int code, const char* fmt, ...);


#define NM_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail(NM_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                  __LINE__);                                                           \
  } while (0)

// Device buffer that grows on demand.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t reserve(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, (count ? count : 1) * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
};

static_assert(sizeof(nm_escape_value) == sizeof(EscapeValue), "grid layout");

// Device scratch words of a handle: the persistent kernels' work counters and
// statistics, and the length of the FE32 rework list.
namespace scratch {
constexpr int kNextMain = 0;
constexpr int kStatsMain = 1;
constexpr int kNextRework = kStatsMain + nmg::STAT_COUNT;
constexpr int kStatsRework = kNextRework + 1;
constexpr int kReworkCount = kStatsRework + nmg::STAT_COUNT;
constexpr int kWorkCount = kReworkCount + 1;  // FE32 pass pipeline: samples to iterate
constexpr int kFeWarpsDone = kWorkCount + 1;  // overlapped rework: FP32 warps finished
constexpr int kScratchWords = kFeWarpsDone + 1;
}  // namespace scratch

}  // namespace nmg

struct nm_handle {
  template <typename T>
  using DevBuf = nmg::DevBuf<T>;
  using EscapeValue = nmg::EscapeValue;
  using Dbl2 = nmg::Dbl2;
  nmg::MPView view;
  int device = 0;
  int path = NM_PATH_REFERENCE;
  // renorm 0: 64 steps a chunk, 32 on floatexp views (measured: 1920x1080x16 at
  // width 1e-12 190 -> 185 ms with 64; 3840x2160 at width 1e-300 31 -> 33 ms)
  int tile_w = 16, tile_h = 16, chunk = 32, blocks = 0, threads = 0, renorm = 0;
  bool keep_smooth64 = false;
  cudaStream_t stream = nullptr;

  // grid
  DevBuf<EscapeValue> grid;
  DevBuf<double> smooth64;
  int grid_nr = 0, grid_nc = 0;

  // per-view tables
  std::vector<Dbl2> coord_re, coord_im;
  std::vector<double> eps_re, eps_im;
  nmg::OrbitData od;
  bool precomputed = false;   // od + eps valid for the current view
  bool coords_valid = false;  // coord tables valid for the current view
  bool uploaded = false;      // device copies current
  bool outside_cardioid = false;
  double precompute_us = 0.0;
  DevBuf<Dbl2> d_coord_re, d_coord_im, d_xhi, d_xlo, d_a, d_b, d_c;
  // the reference orbit, zlen entries as float-float (zf) followed by zlen as
  // FP64 pairs (z): one allocation, so that one L2 access-policy window covers
  // both copies
  DevBuf<nmg::Flt4> d_zf;
  const Dbl2* orbit_z() const {
    return reinterpret_cast<const Dbl2*>(d_zf.p ? d_zf.p + zlen() : nullptr);
  }
  size_t zlen() const { return od_zlen ? od_zlen : od.z.size(); }
  size_t od_zlen = 0;  // a sharing preview: its source's orbit length
  DevBuf<double> d_eps_re, d_eps_im, d_sa_min;
  // floatexp tables (views outside the FP64 range)
  std::vector<nmg::RFE> eps_re_fe, eps_im_fe;
  DevBuf<nmg::RFE> d_eps_re_fe, d_eps_im_fe, d_sa_min_fe;
  DevBuf<nmg::CFE> d_a_fe, d_b_fe, d_c_fe;
  // tables of the FP32 series front
  std::vector<nmg::FFE> eps32_re, eps32_im;
  std::vector<nmg::CFFE> a32, b32, c32;
  std::vector<nmg::TFE> sa_min32;
  DevBuf<nmg::FFE> d_eps32_re, d_eps32_im;
  DevBuf<nmg::CFFE> d_a32, d_b32, d_c32;
  DevBuf<nmg::TFE> d_sa_min32;
  int reference_mode = nmg::REFERENCE_PROBES;
  // FE32 iteration pass: orbit entries staged in shared memory by the TMA unit
  // (orbit_stage.cuh), and a persisting L2 access-policy window on the orbit
  int z_stage = -1;  // -1: kAutoOrbitStage on floatexp views, else none
  bool l2_window = false;
  // renders stop every sample at min(N, iter_cap) iterations (0: N); for
  // previews that estimate where the work lies
  int iter_cap = 0;
  // A preview made by nm_preview reads its source's orbit and series tables
  // (host and device) instead of holding copies; od then carries only the
  // tables' sizes and flags.  The source must outlive the preview.
  nm_handle* orbit_src = nullptr;
  // Bumped whenever the handle's own orbit and series are replaced or dropped
  // (nm_precompute, invalidate); a sharing preview records its source's stamp
  // and refuses to render once the source has moved on.
  unsigned long long tables_stamp = 0;
  unsigned long long src_stamp = 0;
  bool tables_stale() const {
    return orbit_src && (!orbit_src->precomputed || orbit_src->tables_stamp != src_stamp);
  }
  nm_handle* tables() { return orbit_src ? orbit_src : this; }
  const nm_handle* tables() const { return orbit_src ? orbit_src : this; }
  int effective_N() const {
    return iter_cap > 0 && iter_cap < view.iterations() ? iter_cap : view.iterations();
  }

  // scratch: work counters, statistics, and the FE32 rework list
  DevBuf<unsigned long long> d_scratch;  // kScratchWords, layout below
  DevBuf<unsigned int> d_rework;
  int* cancel_host = nullptr;
  int* cancel_dev = nullptr;
  long long expected_samples = 0;
  // events around the last render's kernels: [0] before, [1] after the main
  // kernel (or FE32 passes), [2] after the FE32 rework kernel, [3]/[4] around
  // the FE32 iteration pass
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  bool timed_rework = false, timed_iter = false;
  bool fe_single_pass = false;  // FE32 in one persistent kernel instead of the passes
  bool fe_overlap = true;       // FE32 passes: FP64 rework inside the iteration pass
  DevBuf<char> d_fe_state;
  DevBuf<nmg::FeTrap> d_fe_trap;  // double-loop views on the FE32 path
  // the reference-exact path: sample coordinates in arbitrary precision
  std::vector<uint64_t> coord_re_mp, coord_im_mp;
  DevBuf<uint64_t> d_coord_re_mp, d_coord_im_mp, d_x_mp;
  DevBuf<unsigned int> d_work;

  // scheduling: the order in which whole-grid renders hand out their tiles (a
  // permutation of the tiles at tile_order_w x tile_order_h; empty: row-major)
  // and the per-tile cost log of the last whole-grid render
  std::vector<int32_t> tile_order;
  int tile_order_w = 0, tile_order_h = 0;
  bool tile_order_uploaded = false;
  DevBuf<int32_t> d_tile_order;
  // an order computed on the GPU (nm_order_tiles): d_tile_order holds
  // tile_order_n entries and the host vector is empty
  bool tile_order_on_device = false;
  long long tile_order_n = 0;
  bool log_costs = false;
  DevBuf<unsigned long long> d_tile_cost;
  long long cost_tiles = 0;

  // Bumped by every change that can alter what a render of this handle
  // launches (view, N, tolerance, path, options, tables, their upload, the
  // grid): a batch records it per frame when it captures its graph and
  // rebuilds the graph when it differs.
  unsigned long long generation = 0;
  // The stream of the last nm_render_rows (the handle's own or the caller's),
  // which nm_synchronize waits for.
  cudaStream_t render_stream = nullptr;
  // The last render's device view, when it was an FE32 render with the FP64
  // rework overlapped: nm_synchronize re-renders its rework list if any of the
  // overlapped pass's bounded waits ran out.
  bool last_overlapped = false;
  nmg::DeviceView last_view{};

  nm_handle(int nr, int nc) : view(nr, nc) {}
  ~nm_handle() {
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
    if (cancel_host) cudaFreeHost(cancel_host);
  }
  void invalidate() {
    precomputed = false;
    coords_valid = false;
    uploaded = false;
    orbit_src = nullptr;
    od_zlen = 0;
    tables_stamp++;
    generation++;
  }
};

// The error of a render of a preview whose source changed its orbit and series
// (or dropped them) after nm_preview.
inline constexpr const char* kStalePreview =
    "the preview's source view changed or was precomputed again since nm_preview: make a new preview";

namespace nmg {

// Everything a render of rows [r0, r1) of h needs on the GPU (grid, tables),
// and the device view and kernel that render them (capi.cpp).
int prepare_view(nm_handle* h, int r0, int r1, DeviceView& v, KernelKind& kind);
// The handle's stream, scratch and events, created on first use.
int ensure_device(nm_handle* h);

}  // namespace nmg
