// Batched rendering: many frames (each its own view, orbit, series skip and
// iteration count) in one sequence of launches that the host captures into a
// single CUDA graph.  Frames are grouped by the kernel that renders them:
//
//   FE32 frames:  batch_front_kernel (series front: FP32 stop-index search,
//                                     the FP64 front where it cannot decide),
//                 batch_overlap_kernel (FP32 iteration and smoothing,
//                                     persistent over all FE32 frames'
//                                     samples at once, with the double-path
//                                     frames and the FP64 rework of the
//                                     uncertified samples on the FP64 pipe
//                                     alongside) -- or batch_iter_kernel
//                                     without the FP64 side,
//                 batch_list_kernel<Fp64AnyJob> over the uncertified samples
//                                     (those not yet rendered);
//   double-path frames (the reference's useHardware views):
//                 batch_list_kernel<HwJob> over all their samples (those
//                                     not yet rendered);
//   FP64 frames:  batch_list_kernel<Delta64Job> over all their samples;
//   then batch_reduce_kernel: every frame's multisample mean.
//
// A global sample index g runs over the frames of a group in order; the frame
// of g is found by binary search in the group's prefix sums of samples.
#include "engine.hpp"
#include "fe_core.cuh"
#include "jobs_fp64.cuh"
#include "persistent.cuh"

namespace nmg {

namespace {

__device__ __forceinline__ int frame_of(const BatchGroup& g, long long s) {
  int lo = 0, hi = g.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (g.offsets[mid] <= s)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// The samples of a group of frames for sample_loop / drain_loop.
struct Frames {
  const BatchGroup& g;
  __device__ __forceinline__ const DeviceView& view(int f) const { return g.views[f]; }
  __device__ __forceinline__ bool locate(long long s, int& f, int& r, int& c) const {
    f = frame_of(g, s);
    return sample_rc(g.views[f], s - g.offsets[f], r, c);
  }
};

__global__ void __launch_bounds__(256) batch_front_kernel(BatchGroup grp, FePassBuffers b,
                                                          unsigned long long* stats) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  unsigned long long finished = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long span = ((grp.total + 31) / 32) * 32;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g - lane < span;
       g += stride) {
    bool needs_iteration = false;
    if (g < grp.total) {
      const int f = frame_of(grp, g);
      const DeviceView& v = grp.views[f];
      int r = 0, c = 0;
      if (sample_rc(v, g - grp.offsets[f], r, c)) {
        EscapeValue out;
        double sm = 0.0;
        bool und = false, fp64 = false;
        FeState st;
        if (fe_front_start(v, r, c, st, out, sm, und, fp64)) {
          store_sample(v, r, c, out, sm);
          finished++;
        } else {
          st.frame = f;
          b.state[g] = st;
          needs_iteration = true;
        }
      }
    }
    const unsigned want = __ballot_sync(kFull, needs_iteration);
    if (want) {
      const int leader = __ffs(want) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(b.work_n, (unsigned long long)__popc(want));
      base = __shfl_sync(kFull, base, leader);
      if (needs_iteration) b.work[base + __popc(want & ((1u << lane) - 1))] = (unsigned int)g;
    }
  }
  for (int o = 16; o > 0; o >>= 1) finished += __shfl_xor_sync(kFull, finished, o);
  if (lane == 0 && finished) atomicAdd(&stats[STAT_SAMPLES], finished);
}

__device__ __forceinline__ void batch_iter_warp(const BatchGroup& grp, const FePassBuffers& b,
                                                const RenderCtl& ctl, int chunk) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  FeState st;
  unsigned int g = 0;
  int f = 0;
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
          g = ctl.list[mine];
          st = b.state[g];
          f = st.frame;
          active = true;
          exec0 = executed;
        }
      }
    }
    if (!__any_sync(kFull, active)) break;
    if (active) {
      FeResult res;
      const DeviceView& v = grp.views[f];
      // the arithmetic of the frame rendered alone (render_fe32.cu): t = 2Z +
      // delta unnormalised on frames inside the FP64 range
      FeTrap* trap = v.trap ? v.trap + (g - grp.offsets[f]) : nullptr;
      if (fe_raw_t(v) ? fe_advance<false, true>(v, st, chunk, res, executed, rebases, trap)
                      : fe_advance<false, false>(v, st, chunk, res, executed, rebases, trap)) {
        int r = 0, c = 0;
        sample_rc(v, g - grp.offsets[f], r, c);
        log_cost(v, r, c, executed - exec0, 1);
        if (st.certified) {
          const float s = fe_smoothing(v, res);
          store_sample(v, r, c, EscapeValue{res.it, s}, s);
        } else {  // rendered by the FP64 kernel
          const unsigned long long k = atomicAdd(ctl.rework_n, 1ull);
          ctl.rework[k] = g;
        }
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

__global__ void __launch_bounds__(kPersistentThreads) batch_iter_kernel(BatchGroup grp,
                                                                          FePassBuffers b,
                                                                          RenderCtl ctl,
                                                                          int chunk) {
  batch_iter_warp(grp, b, ctl, chunk);
}

// sample_loop over the samples of many frames: a range [0, grp.total) or a
// list of global sample indices (count from device memory).
template <class Job>
__global__ void __launch_bounds__(kPersistentThreads) batch_list_kernel(BatchGroup grp,
                                                                          RenderCtl ctl,
                                                                          int chunk) {
  __shared__ SamplePool<typename Job::State> pool;
  pool_init(&pool);
  sample_loop<Job>(Frames{grp}, ctl, chunk, &pool);
}

// The FE32 iteration of every FE32 frame with the FP64 work overlapped (the
// FP64 pipe is idle under the FP32 iteration): the last kFp64Warps warps of
// every block render the double-path frames' samples and then the
// uncertified FE32 samples as they are appended; the other warps iterate in
// FP32 and, when the FP32 work list is exhausted, join the FP64 side.  Capped
// at 64 registers so that 4 blocks fit on an SM.  The split follows the
// batch's FP64 work: on a 240-frame 1280x720 (2x2 samples) zoom from width 4
// to 1e-200 with 7 double-loop frames, 4 FP64 warps of 8 gave 1,819 ms, 6 gave
// 1,862 ms, 2 gave 2,030 ms (two runs each).

// The FP64 side, out of line: its register pressure (the FP64 series front)
// then stays out of the FP32 iteration's allocation.
__device__ __noinline__ void batch_fp64_side(const BatchGroup& fe, const BatchGroup& hw,
                                             const RenderCtl& hw_ctl, const OverlapCtl& o,
                                             unsigned long long producers,
                                             SamplePool<Fp64AnyJob::State>* pool) {
  if (hw.n > 0) sample_loop<HwJob>(Frames{hw}, hw_ctl, o.chunk);
  drain_loop<Fp64AnyJob>(Frames{fe}, o.rework, o.fe_warps_done, producers, o.timeouts, o.chunk,
                         pool);
}

template <int kFp64Warps>
__global__ void __launch_bounds__(kPersistentThreads, 4)
    batch_overlap_kernel(BatchGroup fe, FePassBuffers b, RenderCtl fe_ctl, BatchGroup hw,
                         RenderCtl hw_ctl, OverlapCtl o, int chunk) {
  __shared__ SamplePool<Fp64AnyJob::State> pool;
  pool_init(&pool);
  const int warp = threadIdx.x >> 5;
  const int fe_warps = kPersistentThreads / 32 - kFp64Warps;
  if (warp < fe_warps) {
    batch_iter_warp(fe, b, fe_ctl, chunk);
    producer_warp_done(o.fe_warps_done);
  }
  batch_fp64_side(fe, hw, hw_ctl, o, (unsigned long long)gridDim.x * fe_warps, &pool);
}

// Multisample mean of every frame (mandelbrot.cpp:320-332), float arithmetic
// in the reference's order, into one frame-major output array.
__global__ void batch_reduce_kernel(const ReduceJob* jobs, int njobs, long long total) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total;
       k += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].offset <= k)
        lo = mid;
      else
        hi = mid - 1;
    }
    const ReduceJob j = jobs[lo];
    const long long p = k - j.offset;
    const int r = (int)(p / j.nc), c = (int)(p - (long long)r * j.nc);
    const long long NC = (long long)j.nc * j.sc;
    float sum = 0.0f;
    for (int r1 = 0; r1 < j.sc; r1++) {
      const EscapeValue* row = j.in + (long long)(j.sc * r + r1) * NC + (long long)j.sc * c;
      for (int c1 = 0; c1 < j.sc; c1++) {
        const EscapeValue e = row[c1];
        sum = __fadd_rn(sum, __fadd_rn((float)e.iterations, e.smoothing));
      }
    }
    sum = __fdiv_rn(sum, (float)(j.sc * j.sc));
    const int it = (int)sum;
    j.out[p] = EscapeValue{it, __fsub_rn(sum, (float)it)};
  }
}

int blocks_of(const void* kernel, int threads, int device) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0);
  return sms * (per_sm < 1 ? 1 : per_sm);
}

template <int kFp64Warps>
void launch_overlap_with(const BatchLaunch& L, cudaStream_t s) {
  note_launches(1);
  batch_overlap_kernel<kFp64Warps>
      <<<blocks_of((const void*)batch_overlap_kernel<kFp64Warps>, kPersistentThreads, L.device),
         kPersistentThreads, 0, s>>>(L.fe, L.fe_buf, L.fe_ctl, L.hw, L.hw_ctl, L.overlap_ctl,
                                     L.fe_chunk);
}

// FP64 warps a block: as set, else 4 when the batch has double-loop frames
// (their FP64 work dominates), else 2 (the FP64 rework alone).
void launch_overlap(const BatchLaunch& L, cudaStream_t s) {
  const int w = L.fp64_warps > 0 ? L.fp64_warps : (L.hw.n > 0 && L.hw.total > 0 ? 4 : 2);
  if (w <= 2)
    launch_overlap_with<2>(L, s);
  else if (w <= 4)
    launch_overlap_with<4>(L, s);
  else
    launch_overlap_with<6>(L, s);
}

void launch_reduce_all(const BatchLaunch& L, cudaStream_t s) {
  if (L.nreduce > 0 && L.reduce_total > 0) {
    long long blocks = (L.reduce_total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    note_launches(1);
    batch_reduce_kernel<<<(int)blocks, 256, 0, s>>>(L.reduce, L.nreduce, L.reduce_total);
  }
}

}  // namespace

cudaError_t launch_batch(const BatchLaunch& L, cudaStream_t s) {
  const int dev = L.device;
  if (L.fe.n > 0 && L.fe.total > 0) {
    if (L.overlap) {
      // the FP64 side reads rework entries until they differ from the sentinel
      cudaError_t e = cudaMemsetAsync(L.fe_ctl.rework, 0xff,
                                      (size_t)L.fe.total * sizeof(unsigned int), s);
      if (e != cudaSuccess) return e;
    }
    note_launches(2);  // the front and the iteration pass
    batch_front_kernel<<<blocks_of((const void*)batch_front_kernel, 256, dev), 256, 0, s>>>(
        L.fe, L.fe_buf, L.fe_ctl.stats);
    if (L.overlap)
      launch_overlap(L, s);
    else
      batch_iter_kernel<<<blocks_of((const void*)batch_iter_kernel, kPersistentThreads, dev),
                          kPersistentThreads, 0, s>>>(L.fe, L.fe_buf, L.fe_ctl, L.fe_chunk);
    note_launches(1);
    batch_list_kernel<Fp64AnyJob>
        <<<blocks_of((const void*)batch_list_kernel<Fp64AnyJob>, kPersistentThreads, dev),
           kPersistentThreads, 0, s>>>(L.fe, L.rework_ctl, L.chunk);
  }
  // after an overlapped FE32 pass the double-path range is already used up
  // (its counter is shared), and this launch only checks that
  if (L.hw.n > 0 && L.hw.total > 0) note_launches(1);
  if (L.hw.n > 0 && L.hw.total > 0)
    batch_list_kernel<HwJob>
        <<<blocks_of((const void*)batch_list_kernel<HwJob>, kPersistentThreads, dev),
           kPersistentThreads, 0, s>>>(L.hw, L.hw_ctl, L.chunk);
  if (L.fp64.n > 0 && L.fp64.total > 0) note_launches(1);
  if (L.fp64.n > 0 && L.fp64.total > 0)
    batch_list_kernel<Delta64Job>
        <<<blocks_of((const void*)batch_list_kernel<Delta64Job>, kPersistentThreads, dev),
           kPersistentThreads, 0, s>>>(L.fp64, L.fp64_ctl, L.chunk);
  launch_reduce_all(L, s);
  return cudaGetLastError();
}

cudaError_t launch_batch_rework(const BatchLaunch& L, cudaStream_t s) {
  if (L.fe.n > 0 && L.fe.total > 0) note_launches(1);
  if (L.fe.n > 0 && L.fe.total > 0)
    batch_list_kernel<Fp64AnyJob>
        <<<blocks_of((const void*)batch_list_kernel<Fp64AnyJob>, kPersistentThreads, L.device),
           kPersistentThreads, 0, s>>>(L.fe, L.rework_ctl, L.chunk);
  launch_reduce_all(L, s);
  return cudaGetLastError();
}

}  // namespace nmg
