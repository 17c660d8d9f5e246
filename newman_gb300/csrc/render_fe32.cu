// FP32 floatexp perturbation kernels with certified escape counts
// (the iteration and its certificate: fe_core.cuh).
//
// Two arrangements of the same arithmetic:
//
// * The pass pipeline (the FE32 path of nm_render_rows):
//     fe_front_kernel   one thread per sample: the series front of
//                       getIterations -- its stop index searched in FP32 with
//                       a guard band, the FP64 front (pixel_fp64.cuh,
//                       bit-identical to the plain FP64 path) only where that
//                       search cannot decide; writes the sample's start state
//                       and appends it to a work list, or finishes it
//                       (cardioid, escape before the skip point).
//     fe_overlap_kernel persistent and warp-refilled over the work list: six
//                       warps a block run the FP32 delta iteration and the
//                       smoothing term, appending every sample they cannot
//                       certify to the rework list, which the other two warps
//                       render in FP64 meanwhile (fe_iter_kernel: the FP32
//                       warps alone, the rework after the pass).
//   followed by the plain FP64 kernel over what is left of the rework list.
//   FP64 runs only in converged warps: GB300 issues FP64 at about 1/75 of the
//   FP32 rate, and a warp instruction costs the FP64 pipe the same whatever
//   its active lanes.
//
// * The single-pass kernel fe32_kernel: front, iteration and smoothing in one
//   persistent kernel (the FP64 front inside the refill loop).  Its scratch is only the
//   work counters and the rework list, which lets the allocation-free entry
//   point (noalloc.cu) run it from a fixed static array.
#include <type_traits>

#include "engine.hpp"
#include "fe_core.cuh"
#include "jobs_fp64.cuh"
#include "orbit_stage.cuh"
#include "persistent.cuh"

namespace nmg {

namespace {

template <bool kRawT>
struct FeJob {
  using State = FeState;
  static constexpr bool kCertifies = true;
  static constexpr int kCostWeight = 1;
  static __device__ __forceinline__ bool init(const DeviceView& v, int r, int c, State& st,
                                              EscapeValue& out, double& sm, bool& und) {
    bool fp64;
    return fe_front_start(v, r, c, st, out, sm, und, fp64);
  }
  static __device__ __forceinline__ bool steps(const DeviceView& v, State& st, int n,
                                               EscapeValue& out, double& sm,
                                               unsigned long long& executed,
                                               unsigned long long& rebases) {
    FeResult res;
    if (!fe_advance<false, kRawT>(v, st, n, res, executed, rebases)) return false;
    const float s = fe_smoothing(v, res);
    sm = s;
    out = {res.it, s};
    return true;
  }
  static __device__ __forceinline__ bool certified(const State& st) {
    return st.certified != 0;
  }
};

template <bool kRawT>
__global__ void __launch_bounds__(kPersistentThreads) fe32_kernel(DeviceView v, RenderCtl ctl,
                                                                    int chunk) {
  persistent_loop<FeJob<kRawT>>(v, ctl, chunk);
}

// ---- pass pipeline ------------------------------------------------------------

__global__ void __launch_bounds__(256) fe_front_kernel(DeviceView v, FePassBuffers b,
                                                       long long total,
                                                       unsigned long long* stats) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  unsigned long long finished = 0, undecided = 0, fp64_fronts = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  // whole warps step together so that the list appends can be aggregated
  const long long span = ((total + 31) / 32) * 32;
  for (long long sid = blockIdx.x * (long long)blockDim.x + threadIdx.x; sid - lane < span;
       sid += stride) {
    int r = 0, c = 0;
    bool needs_iteration = false;
    if (sid < total && sample_rc(v, sid, r, c)) {
      EscapeValue out;
      double sm = 0.0;
      bool und = false, fp64 = false;
      FeState st;
      if (fe_front_start(v, r, c, st, out, sm, und, fp64)) {
        store_sample(v, r, c, out, sm);
        finished++;
      } else {
        b.state[sid] = st;
        needs_iteration = true;
      }
      undecided += und ? 1 : 0;
      fp64_fronts += fp64 ? 1 : 0;
    }
    const unsigned want = __ballot_sync(kFull, needs_iteration);
    if (want) {
      const int leader = __ffs(want) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(b.work_n, (unsigned long long)__popc(want));
      base = __shfl_sync(kFull, base, leader);
      if (needs_iteration)
        b.work[base + __popc(want & ((1u << lane) - 1))] = (unsigned int)sid;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    finished += __shfl_xor_sync(kFull, finished, o);
    undecided += __shfl_xor_sync(kFull, undecided, o);
    fp64_fronts += __shfl_xor_sync(kFull, fp64_fronts, o);
  }
  if (lane == 0) {
    if (finished) atomicAdd(&stats[STAT_SAMPLES], finished);
    if (undecided) atomicAdd(&stats[STAT_CARDIOID_UNDECIDED], undecided);
    if (fp64_fronts) atomicAdd(&stats[STAT_FRONT_FP64], fp64_fronts);
  }
}

static_assert(sizeof(FeState) == kFeStateBytes, "FE32 state record");
static_assert(sizeof(FeResult) == kFeResultBytes, "FE32 result record");

// Persistent and warp-refilled like persistent_loop, over the work list: the
// start state comes from the front pass, the result goes to the grid.
template <bool kStaged = false, bool kRawT = false>
__device__ __forceinline__ void fe_iter_warp(const DeviceView& v, const FePassBuffers& b,
                                             const RenderCtl& ctl, int chunk) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  FeState st;
  unsigned int sid = 0;
  bool active = false, exhausted = false;
  unsigned long long executed = 0, rebases = 0, finished = 0, exec0 = 0;
  const unsigned long long end = *ctl.count_ptr;
  for (;;) {
    const unsigned need = __ballot_sync(kFull, !active && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) {
        if (ctl.cancel && *ctl.cancel)
          base = ~0ull;
        else
          base = atomicAdd(ctl.next, (unsigned long long)__popc(need));
      }
      base = __shfl_sync(kFull, base, leader);
      if (!active && !exhausted) {
        const unsigned long long mine =
            base == ~0ull ? ~0ull : base + __popc(need & ((1u << lane) - 1));
        if (mine >= end) {
          exhausted = true;
        } else {
          sid = ctl.list[mine];
          st = b.state[sid];
          active = true;
          exec0 = executed;
        }
      }
    }
    if (!__any_sync(kFull, active)) break;
    if (active) {
      FeResult res;
      if (fe_advance<kStaged, kRawT>(v, st, chunk, res, executed, rebases,
                              v.trap ? v.trap + sid : nullptr)) {
        int r = 0, c = 0;
        sample_rc(v, sid, r, c);
        if (st.certified) {
          const float s = fe_smoothing(v, res);
          store_sample(v, r, c, EscapeValue{res.it, s}, s);
        } else {  // rendered by the FP64 kernel
          const unsigned long long k = atomicAdd(ctl.rework_n, 1ull);
          ctl.rework[k] = sid;
        }
        log_cost(v, r, c, executed - exec0, 1);
        finished++;
        active = false;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    executed += __shfl_xor_sync(kFull, executed, o);
    rebases += __shfl_xor_sync(kFull, rebases, o);
    finished += __shfl_xor_sync(kFull, finished, o);
  }
  if (lane == 0) {
    atomicAdd(&ctl.stats[STAT_EXECUTED_ITERS], executed);
    atomicAdd(&ctl.stats[STAT_SAMPLES], finished);
    if (rebases) atomicAdd(&ctl.stats[STAT_REBASES], rebases);
  }
}

template <bool kRawT>
__global__ void __launch_bounds__(kPersistentThreads) fe_iter_kernel(DeviceView v,
                                                                       FePassBuffers b,
                                                                       RenderCtl ctl, int chunk) {
  fe_iter_warp<false, kRawT>(v, b, ctl, chunk);
}

// The iteration pass with the FP64 rework overlapped: the last two warps of
// every block render uncertified samples in FP64 (the FP64 pipe is idle under
// the FP32 iteration) from the start and drain the list to its end; the other
// warps iterate in FP32 and leave when the FP32 work list is exhausted (the
// FP64 code under this kernel's 64-register cap spills; a warp joining it
// made a 3840x2160 (2x2) view of width 1e-413 5 % slower and helped nowhere).
// Capped at 64 registers so that 4 blocks fit on an SM.  On the 1920x1080
// (4x4 samples) view of width 1e-12, N 50,000 (2.7 % of the samples
// reworked): 191 ms with two FP64 warps a block, 245 ms with one, 221 ms with
// three, 243 ms with the rework after the pass.  Views whose FP64 side is the
// longer one take three (fp64_warps_for): the 1e-300 view 31.3 -> 29.3 ms,
// a 3840x2160 (2x2) view of width 1e-412 with N 2,000,000 1,317 -> 1,175 ms,
// against 170 -> 182 ms on the 1e-12 view above; four are slower on both deep
// views (31.3 and 1,350 ms).
int fp64_warps_for(const DeviceView& v) { return (v.sa_fe || v.N > 200000) ? 3 : 2; }

// The FP64 side, out of line: its register pressure (the FP64 series front)
// then stays out of the FP32 iteration's allocation.
template <bool kStaged>
__device__ __noinline__ void overlap_fp64_side(const DeviceView& v, const OverlapCtl& o,
                                               unsigned long long producers,
                                               SamplePool<typename Fp64AnyJobT<kStaged>::State>* pool) {
  drain_loop<Fp64AnyJobT<kStaged>>(OneView{v}, o.rework, o.fe_warps_done, producers, o.timeouts,
                                   o.chunk, pool);
}

// kStaged: the launch stages the orbit's first v.z_stage entries in its
// dynamic shared memory (orbit_stage.cuh) and both sides read them there.
// kRawT: the FP32 step's t = 2Z + delta unnormalised (fe_core.cuh, kFeUTRaw).
// kFp64Warps: the warps of a block on the FP64 side.
template <bool kStaged, bool kRawT, int kFp64Warps>
__global__ void __launch_bounds__(kPersistentThreads, 4) fe_overlap_kernel(
    DeviceView v, FePassBuffers b, RenderCtl ctl, OverlapCtl o, int chunk) {
  __shared__ SamplePool<typename Fp64AnyJobT<kStaged>::State> pool;
  if (kStaged) stage_orbit_prefix(v, ctl.stats + STAT_STAGE_FALLBACKS);
  pool_init(&pool);
  const int warp = threadIdx.x >> 5;
  const int fe_warps = kPersistentThreads / 32 - kFp64Warps;
  if (warp < fe_warps) {
    fe_iter_warp<kStaged, kRawT>(v, b, ctl, chunk);
    producer_warp_done(o.fe_warps_done);
    return;
  }
  overlap_fp64_side<kStaged>(v, o, (unsigned long long)gridDim.x * fe_warps, &pool);
}

int blocks_for(const void* kernel, int threads, int device, size_t dyn_smem = 0) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, dyn_smem);
  return sms * (per_sm < 1 ? 1 : per_sm);
}

// The persisting L2 set-aside of this process's context on `device`, once:
// as much of the orbit as the device allows.  A context setting; it ends
// with the process.
void ensure_l2_set_aside(int device, size_t bytes) {
  static size_t done[64] = {};
  if (device < 0 || device >= 64 || done[device] >= bytes) return;
  int max_persist = 0;
  cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, device);
  const size_t want = bytes < (size_t)max_persist ? bytes : (size_t)max_persist;
  if (want > 0 && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) == cudaSuccess)
    done[device] = bytes;
  cudaGetLastError();
}

}  // namespace

int fe32_blocks_per_sm() {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fe32_kernel<true>, kPersistentThreads, 0);
  int per_sm_norm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_norm, fe32_kernel<false>,
                                                kPersistentThreads, 0);
  if (per_sm_norm < per_sm) per_sm = per_sm_norm;
  return per_sm;
}

cudaError_t launch_fe32(const DeviceView& v, const RenderCtl& ctl, cudaStream_t stream,
                        int blocks, int chunk) {
  note_launches(1);
  if (!fe_raw_t(v))  // the arithmetic of the pass pipeline (launch_fe32_passes)
    fe32_kernel<false><<<blocks, kPersistentThreads, 0, stream>>>(v, ctl, chunk);
  else
    fe32_kernel<true><<<blocks, kPersistentThreads, 0, stream>>>(v, ctl, chunk);
  return cudaGetLastError();
}

cudaError_t launch_fe32_passes(const DeviceView& v, const FePassBuffers& b, const RenderCtl& ctl,
                               cudaStream_t stream, int device, int blocks, int chunk,
                               cudaEvent_t iter_begin, cudaEvent_t iter_end,
                               const OverlapCtl* overlap, int z_stage, bool l2_window) {
  const long long total = v.total;
  if (total <= 0) return cudaSuccess;
  note_launches(2);
  fe_front_kernel<<<blocks_for((const void*)fe_front_kernel, 256, device), 256, 0, stream>>>(
      v, b, total, ctl.stats);
  if (iter_begin) cudaEventRecord(iter_begin, stream);
  RenderCtl it = ctl;
  it.list = b.work;
  it.count_ptr = b.work_n;
  if (overlap) {
    DeviceView vs = v;
    vs.z_stage = z_stage < 0 ? 0 : (z_stage > v.zlen ? v.zlen : z_stage);
    const size_t dyn = 32 * (size_t)vs.z_stage;
    // Views in the FP64 range take the unnormalised t (C2: 182 -> 170 ms); on
    // floatexp views its larger bound reworks more samples, and their frame
    // time is set by the reworked tail (1e-300 view: 31.3 -> 32.9 ms).
    const bool raw_t = fe_raw_t(v);
    const bool three = fp64_warps_for(v) == 3;
    auto pick = [&](auto staged, auto raw) {
      return three ? fe_overlap_kernel<decltype(staged)::value, decltype(raw)::value, 3>
                   : fe_overlap_kernel<decltype(staged)::value, decltype(raw)::value, 2>;
    };
    using T_ = std::true_type;
    using F_ = std::false_type;
    auto kfn = vs.z_stage > 0 ? (raw_t ? pick(T_{}, T_{}) : pick(T_{}, F_{}))
                              : (raw_t ? pick(F_{}, T_{}) : pick(F_{}, F_{}));
    const void* kernel = (const void*)kfn;
    if (dyn > 48 * 1024)
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    const int oblocks =
        blocks > 0 ? blocks : blocks_for(kernel, kPersistentThreads, device, dyn);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(oblocks);
    cfg.blockDim = dim3(kPersistentThreads);
    cfg.dynamicSmemBytes = dyn;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    if (l2_window && v.zlen > 0) {
      int max_window = 0;
      cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, device);
      size_t bytes = 32 * (size_t)v.zlen;  // zf, then z, in one allocation
      if (max_window > 0 && bytes > (size_t)max_window) bytes = (size_t)max_window;
      ensure_l2_set_aside(device, bytes);
      attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
      attr[0].val.accessPolicyWindow.base_ptr = (void*)v.zf;
      attr[0].val.accessPolicyWindow.num_bytes = bytes;
      attr[0].val.accessPolicyWindow.hitRatio = 1.0f;
      attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
      attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
    }
    cudaError_t e = cudaLaunchKernelEx(&cfg, kfn, vs, b, it, *overlap, chunk);
    if (e != cudaSuccess) return e;
  } else {
    auto kfn = fe_raw_t(v) ? fe_iter_kernel<true> : fe_iter_kernel<false>;  // as the overlap kernel
    const int iblocks =
        blocks > 0 ? blocks : blocks_for((const void*)kfn, kPersistentThreads, device);
    kfn<<<iblocks, kPersistentThreads, 0, stream>>>(v, b, it, chunk);
  }
  if (iter_end) cudaEventRecord(iter_end, stream);
  return cudaGetLastError();
}

}  // namespace nmg
