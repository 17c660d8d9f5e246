// Batched rendering: many frames (each its own view, orbit, series skip and
// iteration count) in one sequence of launches that the host captures into a
// single CUDA graph.  Frames are grouped by the kernel that renders them:
//
//   FE32 frames:  batch_front_kernel (FP64 series front, converged),
//                 batch_iter_kernel  (FP32 iteration, persistent over all
//                                     FE32 frames' samples at once),
//                 batch_finish_kernel (FP64 smoothing),
//                 batch_list_kernel<Delta64Job> over the uncertified samples;
//   double-path frames (the reference's useHardware views):
//                 batch_list_kernel<HwJob> over all their samples;
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
        SeriesFront fr;
        EscapeValue out;
        double sm = 0.0;
        bool und = false;
        if (series_front_any(v, r, c, fr, out, sm, und)) {
          store_sample(v, r, c, out, sm);
          finished++;
        } else {
          FeState st;
          fe_start(fr, st);
          st.pad_[0] = f;
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

__global__ void __launch_bounds__(kPersistentThreads) batch_iter_kernel(BatchGroup grp,
                                                                          FePassBuffers b,
                                                                          RenderCtl ctl,
                                                                          int chunk) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  FeState st;
  unsigned int g = 0;
  int f = 0;
  bool active = false, exhausted = false;
  unsigned long long executed = 0, rebases = 0, finished = 0;
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
          f = st.pad_[0];
          active = true;
        }
      }
    }
    if (!__any_sync(kFull, active)) break;
    if (active) {
      FeResult res;
      if (fe_advance(grp.views[f], st, chunk, res, executed, rebases)) {
        res.certified = st.certified;
        b.result[g] = res;
        if (!st.certified) {
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

__global__ void __launch_bounds__(256) batch_finish_kernel(BatchGroup grp, FePassBuffers b) {
  const unsigned long long n = *b.work_n;
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned int g = b.work[k];
    const int f = frame_of(grp, g);
    const DeviceView& v = grp.views[f];
    int r = 0, c = 0;
    sample_rc(v, g - grp.offsets[f], r, c);
    const FeResult res = b.result[g];
    const double sm = res.it < v.N ? smoothing_of(ff_to_double(res.r2), v.log_bailout) : 0.0;
    store_sample(v, r, c, EscapeValue{res.it, (float)sm}, sm);
  }
}

// persistent_loop over the samples of many frames: a range [0, grp.total) or
// a list of global sample indices (count from device memory).
template <class Job>
__global__ void __launch_bounds__(kPersistentThreads) batch_list_kernel(BatchGroup grp,
                                                                          RenderCtl ctl,
                                                                          int chunk) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  typename Job::State st;
  bool active = false, exhausted = false;
  int r = 0, c = 0, f = 0;
  unsigned long long executed = 0, rebases = 0, finished = 0;
  const unsigned long long end =
      ctl.count_ptr ? *ctl.count_ptr : (unsigned long long)ctl.count;
  for (;;) {
    for (;;) {
      const unsigned need = __ballot_sync(kFull, !active && !exhausted);
      if (!need) break;
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
          const long long g = ctl.list ? (long long)ctl.list[mine] : (long long)mine;
          f = frame_of(grp, g);
          const DeviceView& v = grp.views[f];
          if (sample_rc(v, g - grp.offsets[f], r, c)) {
            EscapeValue out;
            double sm = 0.0;
            bool und = false;
            if (Job::init(v, r, c, st, out, sm, und)) {
              store_sample(v, r, c, out, sm);
              finished++;
            } else {
              active = true;
            }
          }
        }
      }
    }
    if (!__any_sync(kFull, active)) break;
    if (active) {
      EscapeValue out;
      double sm = 0.0;
      const DeviceView& v = grp.views[f];
      if (Job::steps(v, st, chunk, out, sm, executed, rebases)) {
        store_sample(v, r, c, out, sm);
        finished++;
        active = false;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    executed += __shfl_xor_sync(kFull, executed, o);
    finished += __shfl_xor_sync(kFull, finished, o);
  }
  if (lane == 0) {
    atomicAdd(&ctl.stats[STAT_EXECUTED_ITERS], executed);
    atomicAdd(&ctl.stats[STAT_SAMPLES], finished);
  }
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

}  // namespace

cudaError_t launch_batch(const BatchLaunch& L, cudaStream_t s) {
  const int dev = L.device;
  if (L.fe.n > 0 && L.fe.total > 0) {
    batch_front_kernel<<<blocks_of((const void*)batch_front_kernel, 256, dev), 256, 0, s>>>(
        L.fe, L.fe_buf, L.fe_ctl.stats);
    batch_iter_kernel<<<blocks_of((const void*)batch_iter_kernel, kPersistentThreads, dev),
                        kPersistentThreads, 0, s>>>(L.fe, L.fe_buf, L.fe_ctl, L.fe_chunk);
    batch_finish_kernel<<<blocks_of((const void*)batch_finish_kernel, 256, dev), 256, 0, s>>>(
        L.fe, L.fe_buf);
    batch_list_kernel<Delta64Job>
        <<<blocks_of((const void*)batch_list_kernel<Delta64Job>, kPersistentThreads, dev),
           kPersistentThreads, 0, s>>>(L.fe, L.rework_ctl, L.chunk);
  }
  if (L.hw.n > 0 && L.hw.total > 0)
    batch_list_kernel<HwJob>
        <<<blocks_of((const void*)batch_list_kernel<HwJob>, kPersistentThreads, dev),
           kPersistentThreads, 0, s>>>(L.hw, L.hw_ctl, L.chunk);
  if (L.fp64.n > 0 && L.fp64.total > 0)
    batch_list_kernel<Delta64Job>
        <<<blocks_of((const void*)batch_list_kernel<Delta64Job>, kPersistentThreads, dev),
           kPersistentThreads, 0, s>>>(L.fp64, L.fp64_ctl, L.chunk);
  if (L.nreduce > 0 && L.reduce_total > 0) {
    long long blocks = (L.reduce_total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    batch_reduce_kernel<<<(int)blocks, 256, 0, s>>>(L.reduce, L.nreduce, L.reduce_total);
  }
  return cudaGetLastError();
}

}  // namespace nmg
