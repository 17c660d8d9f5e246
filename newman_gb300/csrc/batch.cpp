// Batches of frames (nm_batch_*): every frame of, say, a zoom video -- each
// with its own view, reference orbit, series skip and iteration count --
// rendered by one CUDA graph launch that holds all of the batch's kernels
// (render_batch.cu), and multisample-reduced into one frame-major array.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "engine.hpp"
#include "handle.hpp"

using nmg::DevBuf;
using nmg::fail;

struct nm_batch {
  int sc = 1;
  std::vector<nm_handle*> frames;
  int tile_w = 16, tile_h = 16, chunk = 32, fe_chunk = 64;  // fe_chunk 64: the 240-frame zoom 1399 -> 1340 ms
  bool use_graph = true;
  bool overlap = true;  // FP64 work inside the FE32 iteration pass
  int fp64_warps = 0;   // of 8 a block in that pass; 0: chosen from the batch

  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool built = false;
  cudaGraphExec_t exec = nullptr;
  long long graph_kernels = 0;  // kernel launches captured in exec
  nmg::BatchLaunch L{};
  // what the graph was built against, to notice changed frames: each frame's
  // generation (nm_handle::generation) and buffers
  std::vector<unsigned long long> seen_gen;
  std::vector<const void*> seen_grid, seen_orbit;

  DevBuf<nmg::DeviceView> d_views_fe, d_views_hw, d_views_fp64;
  DevBuf<long long> d_off_fe, d_off_hw, d_off_fp64;
  DevBuf<char> d_fe_state;
  DevBuf<unsigned int> d_work, d_rework;
  DevBuf<unsigned long long> d_scratch;
  DevBuf<nmg::ReduceJob> d_reduce;
  DevBuf<nmg::EscapeValue> d_reduced;
  long long reduced_pixels = 0;

  ~nm_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }
  void invalidate() {
    built = false;
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
  }
};

namespace {

// scratch words of a batch launch
enum {
  kFeNext = 0,
  kFeStats = 1,
  kReworkNext = kFeStats + nmg::STAT_COUNT,
  kReworkStats = kReworkNext + 1,
  kReworkN = kReworkStats + nmg::STAT_COUNT,
  kWorkN = kReworkN + 1,
  kHwNext = kWorkN + 1,
  kHwStats = kHwNext + 1,
  kFp64Next = kHwStats + nmg::STAT_COUNT,
  kFp64Stats = kFp64Next + 1,
  kFeWarpsDone = kFp64Stats + nmg::STAT_COUNT,
  kBatchWords = kFeWarpsDone + 1
};

template <typename T>
int upload_vec(DevBuf<T>& d, const std::vector<T>& v, cudaStream_t s) {
  NM_CUDA(d.reserve(v.size()));
  if (!v.empty())
    NM_CUDA(cudaMemcpyAsync(d.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return NM_OK;
}

nmg::BatchGroup group(const DevBuf<nmg::DeviceView>& views, const DevBuf<long long>& off,
                      const std::vector<long long>& host_off) {
  nmg::BatchGroup g{};
  g.views = views.p;
  g.offsets = off.p;
  g.n = (int)host_off.size() - 1;
  g.total = host_off.empty() ? 0 : host_off.back();
  return g;
}

nmg::RenderCtl ctl_at(unsigned long long* words, int next, int stats, long long count) {
  nmg::RenderCtl c{};
  c.next = words + next;
  c.stats = words + stats;
  c.first = 0;
  c.count = count;
  return c;
}

int build(nm_batch* b) {
  b->invalidate();
  std::vector<nmg::DeviceView> fe, hw, fp64;
  std::vector<long long> off_fe{0}, off_hw{0}, off_fp64{0};
  std::vector<nmg::ReduceJob> red;
  long long red_total = 0;
  b->seen_gen.clear();
  b->seen_grid.clear();
  b->seen_orbit.clear();
  for (nm_handle* h : b->frames) {
    h->tile_w = b->tile_w;
    h->tile_h = b->tile_h;
    nmg::DeviceView v;
    nmg::KernelKind kind;
    if (int rc = nmg::prepare_view(h, 0, h->view.rows(), v, kind)) return rc;
    if (kind == nmg::KERNEL_MP || kind == nmg::KERNEL_HW_MP)
      return fail(NM_ERR_UNSUPPORTED, "a batch renders the FE32, FP64 and double-loop paths; "
                                      "render reference-exact frames alone");
    if (kind == nmg::KERNEL_FE32) {
      fe.push_back(v);
      off_fe.push_back(off_fe.back() + v.total);
    } else if (kind == nmg::KERNEL_HW) {
      hw.push_back(v);
      off_hw.push_back(off_hw.back() + v.total);
    } else {
      fp64.push_back(v);
      off_fp64.push_back(off_fp64.back() + v.total);
    }
    if (b->sc > 1) {
      nmg::ReduceJob j;
      j.in = h->grid.p;
      j.sc = b->sc;
      j.nc = h->view.cols() / b->sc;
      j.offset = red_total;
      j.out = nullptr;  // set once d_reduced exists
      red.push_back(j);
      red_total += (long long)(h->view.rows() / b->sc) * j.nc;
    }
    b->seen_gen.push_back(h->generation);
    b->seen_grid.push_back(h->grid.p);
    b->seen_orbit.push_back(h->tables()->d_zf.p);
  }
  if (off_fe.back() > 0xffffffffll)
    return fail(NM_ERR_ARG, "batch of %lld FE32 samples exceeds 2^32", off_fe.back());
  cudaStream_t s = b->stream;
  if (int rc = upload_vec(b->d_views_fe, fe, s)) return rc;
  if (int rc = upload_vec(b->d_views_hw, hw, s)) return rc;
  if (int rc = upload_vec(b->d_views_fp64, fp64, s)) return rc;
  if (int rc = upload_vec(b->d_off_fe, off_fe, s)) return rc;
  if (int rc = upload_vec(b->d_off_hw, off_hw, s)) return rc;
  if (int rc = upload_vec(b->d_off_fp64, off_fp64, s)) return rc;
  const size_t nfe = (size_t)off_fe.back();
  NM_CUDA(b->d_fe_state.reserve(nfe * nmg::kFeStateBytes));
  NM_CUDA(b->d_work.reserve(nfe));
  NM_CUDA(b->d_rework.reserve(nfe));
  NM_CUDA(b->d_scratch.reserve(kBatchWords));
  NM_CUDA(b->d_reduced.reserve((size_t)red_total));
  for (auto& j : red) j.out = b->d_reduced.p + j.offset;
  if (int rc = upload_vec(b->d_reduce, red, s)) return rc;
  NM_CUDA(cudaStreamSynchronize(s));
  b->reduced_pixels = red_total;

  nmg::BatchLaunch& L = b->L;
  std::memset(&L, 0, sizeof L);
  L.device = b->device;
  L.fe = group(b->d_views_fe, b->d_off_fe, off_fe);
  L.hw = group(b->d_views_hw, b->d_off_hw, off_hw);
  L.fp64 = group(b->d_views_fp64, b->d_off_fp64, off_fp64);
  unsigned long long* w = b->d_scratch.p;
  L.fe_buf.state = reinterpret_cast<nmg::FeState*>(b->d_fe_state.p);
  L.fe_buf.work = b->d_work.p;
  L.fe_buf.work_n = w + kWorkN;
  L.fe_ctl = ctl_at(w, kFeNext, kFeStats, 0);
  L.fe_ctl.list = b->d_work.p;
  L.fe_ctl.count_ptr = w + kWorkN;
  L.fe_ctl.rework = b->d_rework.p;
  L.fe_ctl.rework_n = w + kReworkN;
  L.rework_ctl = ctl_at(w, kReworkNext, kReworkStats, 0);
  L.rework_ctl.list = b->d_rework.p;
  L.rework_ctl.count_ptr = w + kReworkN;
  L.hw_ctl = ctl_at(w, kHwNext, kHwStats, L.hw.total);
  L.fp64_ctl = ctl_at(w, kFp64Next, kFp64Stats, L.fp64.total);
  L.fe_chunk = b->fe_chunk;
  L.chunk = b->chunk;
  L.overlap = b->overlap;
  L.fp64_warps = b->fp64_warps;
  L.overlap_ctl.rework = L.rework_ctl;
  L.overlap_ctl.fe_warps_done = w + kFeWarpsDone;
  L.overlap_ctl.timeouts = w + kFeStats + nmg::STAT_WAIT_TIMEOUTS;
  L.overlap_ctl.chunk = b->chunk;
  L.reduce = b->d_reduce.p;
  L.nreduce = (int)red.size();
  L.reduce_total = red_total;

  if (b->use_graph) {
    cudaGraph_t graph = nullptr;
    const long long launches0 = nmg::launches_so_far();
    NM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(b->d_scratch.p, 0, kBatchWords * 8, s);
    if (e == cudaSuccess) e = nmg::launch_batch(L, s);
    cudaError_t e2 = cudaStreamEndCapture(s, &graph);
    // captured, not run: a replay counts them
    b->graph_kernels = nmg::launches_so_far() - launches0;
    nmg::note_launches(-b->graph_kernels);
    if (e != cudaSuccess || e2 != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return fail(NM_ERR_CUDA, "batch graph capture: %s",
                  cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(NM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  }
  b->built = true;
  return NM_OK;
}

bool stale(const nm_batch* b) {
  if (!b->built || b->seen_grid.size() != b->frames.size()) return true;
  for (size_t k = 0; k < b->frames.size(); k++) {
    const nm_handle* h = b->frames[k];
    if (!h->uploaded || h->tables_stale() || h->generation != b->seen_gen[k] ||
        h->grid.p != b->seen_grid[k] || h->tables()->d_zf.p != b->seen_orbit[k])
      return true;
  }
  return false;
}

}  // namespace

extern "C" {

nm_batch* nm_batch_create(int sc) {
  if (sc < 1) {
    fail(NM_ERR_ARG, "multisample factor %d", sc);
    return nullptr;
  }
  nm_batch* b = new nm_batch();
  b->sc = sc;
  return b;
}

void nm_batch_destroy(nm_batch* b) {
  if (b && b->stream) cudaStreamSynchronize(b->stream);
  delete b;
}

int nm_batch_add(nm_batch* b, nm_handle* frame) {
  if (!b || !frame) return fail(NM_ERR_ARG, "null batch or frame");
  if (frame->path == NM_PATH_MP)
    return fail(NM_ERR_UNSUPPORTED, "a batch renders the FE32, FP64 and double-loop paths; "
                                    "render reference-exact frames alone");
  if (frame->view.rows() % b->sc || frame->view.cols() % b->sc)
    return fail(NM_ERR_ARG, "frame %d x %d is not a multiple of the multisample factor %d",
                frame->view.rows(), frame->view.cols(), b->sc);
  b->frames.push_back(frame);
  b->invalidate();
  return NM_OK;
}

int nm_batch_set_option(nm_batch* b, int opt, long long value) {
  if (!b) return fail(NM_ERR_ARG, "null batch");
  switch (opt) {
    case NM_OPT_TILE_W:
    case NM_OPT_TILE_H:
      if (value < 1 || value > 1024) return fail(NM_ERR_ARG, "tile size %lld", value);
      (opt == NM_OPT_TILE_W ? b->tile_w : b->tile_h) = (int)value;
      break;
    case NM_OPT_CHUNK:
      if (value < 1 || value > (1 << 20)) return fail(NM_ERR_ARG, "chunk %lld", value);
      b->chunk = (int)value;
      break;
    case NM_OPT_RENORM:
      if (value < 1 || value > 256) return fail(NM_ERR_ARG, "renorm interval %lld", value);
      b->fe_chunk = (int)value;
      break;
    case NM_OPT_BATCH_GRAPH:
      b->use_graph = value != 0;
      break;
    case NM_OPT_FE32_OVERLAP:
      b->overlap = value != 0;
      break;
    case NM_OPT_BATCH_FP64_WARPS:
      if (value != 0 && value != 2 && value != 4 && value != 6)
        return fail(NM_ERR_ARG, "FP64 warps a block %lld (0, 2, 4 or 6)", value);
      b->fp64_warps = (int)value;
      break;
    default:
      return fail(NM_ERR_ARG, "option %d does not apply to a batch", opt);
  }
  b->invalidate();
  return NM_OK;
}

int nm_batch_render(nm_batch* b) {
  if (!b) return fail(NM_ERR_ARG, "null batch");
  if (b->frames.empty()) return fail(NM_ERR_STATE, "empty batch");
  if (!b->stream) {
    NM_CUDA(cudaGetDevice(&b->device));
    NM_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    NM_CUDA(cudaEventCreate(&b->ev0));
    NM_CUDA(cudaEventCreate(&b->ev1));
  }
  if (stale(b))
    if (int rc = build(b)) return rc;
  NM_CUDA(cudaEventRecord(b->ev0, b->stream));
  if (b->use_graph) {
    NM_CUDA(cudaGraphLaunch(b->exec, b->stream));
    nmg::note_launches(b->graph_kernels);
  } else {
    NM_CUDA(cudaMemsetAsync(b->d_scratch.p, 0, kBatchWords * 8, b->stream));
    NM_CUDA(nmg::launch_batch(b->L, b->stream));
  }
  NM_CUDA(cudaEventRecord(b->ev1, b->stream));
  NM_CUDA(cudaStreamSynchronize(b->stream));
  if (b->overlap && b->L.fe.n > 0 && b->L.fe.total > 0) {
    // An overlapped FP64 consumer skips a rework entry it claimed but could not
    // read within its poll limit (counted as a wait timeout).  Every entry is
    // written once the launches have ended: render the whole rework list again
    // in FP64 (the same results for the samples already rendered) and reduce
    // the frames again.
    unsigned long long lost = 0;
    NM_CUDA(cudaMemcpy(&lost, b->d_scratch.p + kFeStats + nmg::STAT_WAIT_TIMEOUTS, 8,
                       cudaMemcpyDeviceToHost));
    if (lost) {
      NM_CUDA(cudaMemsetAsync(b->d_scratch.p + kReworkNext, 0, 8, b->stream));
      NM_CUDA(nmg::launch_batch_rework(b->L, b->stream));
      NM_CUDA(cudaStreamSynchronize(b->stream));
    }
  }
  return NM_OK;
}

int nm_batch_get_stat(nm_batch* b, int stat, long long* value) {
  if (!b || !value) return fail(NM_ERR_ARG, "null batch or output");
  *value = 0;
  if (stat == NM_STAT_KERNEL_LAUNCHES) {
    *value = nmg::launches_so_far();
    return NM_OK;
  }
  if (!b->built) return NM_OK;
  if (stat == NM_STAT_KERNEL_NS) {
    float ms = 0.f;
    NM_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    *value = (long long)(ms * 1e6);
    return NM_OK;
  }
  unsigned long long w[kBatchWords];
  NM_CUDA(cudaMemcpy(w, b->d_scratch.p, sizeof w, cudaMemcpyDeviceToHost));
  if (stat == NM_STAT_FP64_REWORK) {
    *value = (long long)w[kReworkN];
    return NM_OK;
  }
  if (stat < 0 || stat >= nmg::STAT_COUNT) return fail(NM_ERR_ARG, "unknown stat %d", stat);
  *value = (long long)(w[kFeStats + stat] + w[kHwStats + stat] + w[kFp64Stats + stat]);
  if (stat == nmg::STAT_EXECUTED_ITERS) *value += (long long)w[kReworkStats + stat];
  return NM_OK;
}

int nm_batch_frames(nm_batch* b, nm_escape_value* host_out) {
  if (!b || !host_out) return fail(NM_ERR_ARG, "null batch or output");
  if (!b->built) return fail(NM_ERR_STATE, "batch not rendered");
  if (b->sc > 1) {
    NM_CUDA(cudaMemcpy(host_out, b->d_reduced.p, (size_t)b->reduced_pixels * 8,
                       cudaMemcpyDeviceToHost));
    return NM_OK;
  }
  size_t at = 0;
  for (nm_handle* h : b->frames) {
    const size_t n = (size_t)h->view.rows() * h->view.cols();
    NM_CUDA(cudaMemcpy(host_out + at, h->grid.p, n * 8, cudaMemcpyDeviceToHost));
    at += n;
  }
  return NM_OK;
}

int nm_batch_autotune(nm_batch* b, int stride, int* tile_w, int* tile_h, int* renorm) {
  if (!b || stride < 1) return fail(NM_ERR_ARG, "bad autotune arguments");
  if (b->frames.empty()) return fail(NM_ERR_STATE, "empty batch");
  const int ow = b->tile_w, oh = b->tile_h, orn = b->fe_chunk, ofw = b->fp64_warps;
  // a sub-batch of every stride-th frame, same options
  nm_batch sub;
  sub.sc = b->sc;
  sub.use_graph = b->use_graph;
  sub.overlap = b->overlap;
  sub.chunk = b->chunk;
  sub.fp64_warps = b->fp64_warps;
  for (size_t k = 0; k < b->frames.size(); k += (size_t)stride) sub.frames.push_back(b->frames[k]);
  static const int tiles[][2] = {{8, 8}, {16, 16}, {32, 8}, {32, 32}, {64, 16}, {64, 64}};
  static const int renorms[] = {8, 16, 32, 64, 128, 256};
  float best = 1e30f;
  int bw = b->tile_w, bh = b->tile_h, br = b->fe_chunk;
  for (const auto& t : tiles)
    for (int rn : renorms) {
      sub.tile_w = t[0];
      sub.tile_h = t[1];
      sub.fe_chunk = rn;
      sub.invalidate();
      if (int rc = nm_batch_render(&sub)) return rc;  // builds and warms up
      float ms = 0.f;
      for (int rep = 0; rep < 2; rep++) {
        if (int rc = nm_batch_render(&sub)) return rc;
        float m = 0.f;
        NM_CUDA(cudaEventElapsedTime(&m, sub.ev0, sub.ev1));
        ms += m;
      }
      if (ms < best) {
        best = ms;
        bw = t[0];
        bh = t[1];
        br = rn;
      }
    }
  // then the FP64 side's share of each block, at the chosen tiles
  int bfw = b->fp64_warps;
  if (b->overlap) {
    sub.tile_w = bw;
    sub.tile_h = bh;
    sub.fe_chunk = br;
    float best_w = 1e30f;
    for (int fw : {2, 4, 6}) {
      sub.fp64_warps = fw;
      sub.invalidate();
      if (int rc = nm_batch_render(&sub)) return rc;
      float ms = 0.f;
      for (int rep = 0; rep < 2; rep++) {
        if (int rc = nm_batch_render(&sub)) return rc;
        float m = 0.f;
        NM_CUDA(cudaEventElapsedTime(&m, sub.ev0, sub.ev1));
        ms += m;
      }
      if (ms < best_w) {
        best_w = ms;
        bfw = fw;
      }
    }
  }
  // Last, the tuned settings against the batch's own on the whole batch (a
  // sub-batch can miss the few frames that dominate it): the faster stays.
  auto set = [&](int tw, int th, int rn, int fw) {
    b->tile_w = tw;
    b->tile_h = th;
    b->fe_chunk = rn;
    b->fp64_warps = fw;
    b->invalidate();
    // frames are prepared with the batch's tile shape when it is built
    for (nm_handle* h : b->frames) {
      h->tile_w = tw;
      h->tile_h = th;
    }
  };
  auto time_whole = [&](float& out) -> int {
    if (int rc = nm_batch_render(b)) return rc;  // builds and warms up
    out = 0.f;
    for (int rep = 0; rep < 2; rep++) {
      if (int rc = nm_batch_render(b)) return rc;
      float m = 0.f;
      NM_CUDA(cudaEventElapsedTime(&m, b->ev0, b->ev1));
      out += m;
    }
    return NM_OK;
  };
  if (bw != ow || bh != oh || br != orn || bfw != ofw) {
    float t_tuned = 0.f, t_own = 0.f;
    set(bw, bh, br, bfw);
    if (int rc = time_whole(t_tuned)) return rc;
    set(ow, oh, orn, ofw);
    if (int rc = time_whole(t_own)) return rc;
    if (t_own <= t_tuned) {
      bw = ow;
      bh = oh;
      br = orn;
      bfw = ofw;
    }
  }
  set(bw, bh, br, bfw);
  if (tile_w) *tile_w = bw;
  if (tile_h) *tile_h = bh;
  if (renorm) *renorm = br;
  return NM_OK;
}

}  // extern "C"
