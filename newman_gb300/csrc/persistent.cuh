// Persistent, warp-refilled sample loop shared by the per-sample kernels.
//
// Each warp owns 32 samples at a time.  Lanes run `chunk` iterations of their
// sample, then the warp __ballot_sync's the lanes that finished and refills
// exactly those from a global work counter with one atomicAdd per warp, so
// early-escaping samples never leave a lane idle for longer than one chunk.
// Every loop is bounded: a sample runs at most N iterations and the counter
// only grows, so the kernel always ends.  A host-set cancel flag stops the
// hand-out of new samples; samples already started are finished.
//
// Work comes either as a range of sample indices in tile order or as a list
// of sample indices whose length an earlier kernel wrote to device memory.
// A job that certifies its results (Job::kCertifies) appends each sample it
// could not certify to ctl.rework; its provisional result is still stored.
#pragma once

#include "engine.hpp"

namespace nmg {

constexpr int kPersistentThreads = 256;

__device__ __forceinline__ void store_sample(const DeviceView& v, int r, int c,
                                             const EscapeValue& out, double sm) {
  const long long k = (long long)r * v.nc + c;
  v.grid[k] = out;
  if (v.smooth64) v.smooth64[k] = sm;
}

template <class Job>
__device__ __forceinline__ void persistent_loop(const DeviceView& v, const RenderCtl& ctl,
                                                int chunk) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  typename Job::State st;
  bool active = false, exhausted = false;
  int r = 0, c = 0;
  long long sid = 0;
  unsigned long long executed = 0, rebases = 0, finished = 0, undecided = 0;
  const unsigned long long end =
      ctl.count_ptr ? *ctl.count_ptr : (unsigned long long)ctl.count;

  for (;;) {
    // Refill every idle lane (a new sample may finish at once, e.g. inside
    // the cardioid, so repeat until every lane is busy or the work is gone).
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
          sid = ctl.list ? (long long)ctl.list[mine] : ctl.first + (long long)mine;
          if (sample_rc(v, sid, r, c)) {
            EscapeValue out;
            double sm = 0.0;
            bool und = false;
            if (Job::init(v, r, c, st, out, sm, und)) {
              store_sample(v, r, c, out, sm);
              finished++;
            } else {
              active = true;
            }
            undecided += und ? 1 : 0;
          }
        }
      }
    }
    if (!__any_sync(kFull, active)) break;
    if (active) {
      EscapeValue out;
      double sm = 0.0;
      if (Job::steps(v, st, chunk, out, sm, executed, rebases)) {
        store_sample(v, r, c, out, sm);
        if (Job::kCertifies && !Job::certified(st)) {
          const unsigned long long k = atomicAdd(ctl.rework_n, 1ull);
          ctl.rework[k] = (unsigned int)sid;
        }
        finished++;
        active = false;
      }
    }
  }
  // One atomic per warp for the counters.
  for (int o = 16; o > 0; o >>= 1) {
    executed += __shfl_xor_sync(kFull, executed, o);
    rebases += __shfl_xor_sync(kFull, rebases, o);
    finished += __shfl_xor_sync(kFull, finished, o);
    undecided += __shfl_xor_sync(kFull, undecided, o);
  }
  if (lane == 0) {
    atomicAdd(&ctl.stats[STAT_EXECUTED_ITERS], executed);
    atomicAdd(&ctl.stats[STAT_SAMPLES], finished);
    if (rebases) atomicAdd(&ctl.stats[STAT_REBASES], rebases);
    if (undecided) atomicAdd(&ctl.stats[STAT_CARDIOID_UNDECIDED], undecided);
  }
}

}  // namespace nmg
