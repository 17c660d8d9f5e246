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
// could not certify to ctl.rework instead of storing a result: a later FP64
// pass over that list always renders it.
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

// Where the samples of a launch come from: one view (sample index = tile-order
// index of that view), or the frames of a batch (render_batch.cu).  `f` names
// the view of a sample for view(f).
struct OneView {
  const DeviceView& v;
  __device__ __forceinline__ const DeviceView& view(int) const { return v; }
  __device__ __forceinline__ bool locate(long long s, int& f, int& r, int& c) const {
    f = 0;
    return sample_rc(v, s, r, c);
  }
};

// Adds a finished sample's work to its tile's entry of the cost log.
__device__ __forceinline__ void log_cost(const DeviceView& v, int r, int c,
                                         unsigned long long steps, int weight) {
  if (v.tile_cost && steps) atomicAdd(&v.tile_cost[tile_at(v, r, c)], steps * weight);
}

template <class Job, class Src>
__device__ __forceinline__ void sample_loop(const Src& src, const RenderCtl& ctl, int chunk) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  typename Job::State st;
  bool active = false, exhausted = false;
  int r = 0, c = 0, f = 0;
  long long sid = 0;
  unsigned long long executed = 0, rebases = 0, finished = 0, undecided = 0, exec0 = 0;
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
          if (src.locate(sid, f, r, c)) {
            EscapeValue out;
            double sm = 0.0;
            bool und = false;
            if (Job::init(src.view(f), r, c, st, out, sm, und)) {
              store_sample(src.view(f), r, c, out, sm);
              finished++;
            } else {
              active = true;
              exec0 = executed;
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
      if (Job::steps(src.view(f), st, chunk, out, sm, executed, rebases)) {
        if (Job::kCertifies && !Job::certified(st)) {
          const unsigned long long k = atomicAdd(ctl.rework_n, 1ull);
          ctl.rework[k] = (unsigned int)sid;
        } else {
          store_sample(src.view(f), r, c, out, sm);
        }
        log_cost(src.view(f), r, c, executed - exec0, Job::kCostWeight);
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

template <class Job>
__device__ __forceinline__ void persistent_loop(const DeviceView& v, const RenderCtl& ctl,
                                                int chunk) {
  sample_loop<Job>(OneView{v}, ctl, chunk);
}

// ---- a list that other warps of the same launch are still filling ----------
//
// Producers append with k = atomicAdd(count, 1); list[k] = sample, and when a
// producer warp has appended its last entry it fences and bumps `producers_done`.
// Consumers claim entries [next, count) with a compare-and-swap on `next` (so
// a claim never runs past the entries counted so far), read each entry until
// it differs from kListSentinel (the list is filled with the sentinel before
// the launch; the producer's store follows its atomicAdd at once), and stop
// when every producer is done and every counted entry is claimed.  All waits
// are bounded: a consumer that stays idle for kDrainIdlePolls polls leaves
// the rest of the list to the next launch over the same `next` counter, and an
// entry still unwritten after kEntryPolls polls is counted in `timeouts` and
// skipped and left unrendered (the host sees the count).

constexpr unsigned kDrainIdlePolls = 1u << 19;  // about a second of 2 us sleeps
constexpr unsigned kEntryPolls = 1u << 16;

enum ClaimStatus { CLAIM_OK = 0, CLAIM_EMPTY = 1, CLAIM_BUSY = 2 };

__device__ __forceinline__ int claim_entries(unsigned long long* next,
                                             const unsigned long long* count, unsigned want,
                                             unsigned long long& base, unsigned& got) {
  const unsigned long long end = *(const volatile unsigned long long*)count;
  for (int t = 0; t < 32; t++) {
    const unsigned long long c = *(volatile unsigned long long*)next;
    if (c >= end) {
      got = 0;
      return CLAIM_EMPTY;
    }
    const unsigned long long k = end - c < want ? end - c : want;
    if (atomicCAS(next, c, c + k) == c) {
      base = c;
      got = (unsigned)k;
      return CLAIM_OK;
    }
  }
  got = 0;
  return CLAIM_BUSY;
}

__device__ __forceinline__ unsigned int read_entry(const unsigned int* list, unsigned long long k) {
  const volatile unsigned int* p = list + k;
  unsigned int e = *p;
  for (unsigned t = 0; e == kListSentinel && t < kEntryPolls; t++) {
    __nanosleep(256);
    e = *p;
  }
  return e;
}

// Marks the calling warp's appends as complete (every lane of the warp calls it).
__device__ __forceinline__ void producer_warp_done(unsigned long long* producers_done) {
  __threadfence();
  __syncwarp();
  if ((threadIdx.x & 31) == 0) atomicAdd(producers_done, 1ull);
}

template <class Job, class Src>
__device__ __forceinline__ void drain_loop(const Src& src, const RenderCtl& ctl,
                                           const unsigned long long* producers_done,
                                           unsigned long long producers,
                                           unsigned long long* timeouts, int chunk) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  typename Job::State st;
  bool active = false, closed = false;
  int r = 0, c = 0, f = 0;
  unsigned idle = 0;
  unsigned long long executed = 0, rebases = 0, finished = 0, undecided = 0, lost = 0, exec0 = 0;
  for (;;) {
    const unsigned need = __ballot_sync(kFull, !active);
    if (need && !closed) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      unsigned got = 0;
      int status = CLAIM_BUSY;
      bool done = false;
      if (lane == leader) {
        if (ctl.cancel && *ctl.cancel) {
          done = true;
          status = CLAIM_EMPTY;
        } else {
          done = *(const volatile unsigned long long*)producers_done >= producers;
          __threadfence();  // the count read below includes every finished producer's entries
          status = claim_entries(ctl.next, ctl.count_ptr, __popc(need), base, got);
        }
      }
      base = __shfl_sync(kFull, base, leader);
      got = __shfl_sync(kFull, got, leader);
      status = __shfl_sync(kFull, status, leader);
      done = __shfl_sync(kFull, done, leader);
      if (done && status == CLAIM_EMPTY) closed = true;
      if (!active) {
        const unsigned rank = __popc(need & ((1u << lane) - 1));
        if (rank < got) {
          const unsigned int sid = read_entry(ctl.list, base + rank);
          if (sid == kListSentinel) {
            lost++;
          } else if (src.locate(sid, f, r, c)) {
            EscapeValue out;
            double sm = 0.0;
            bool und = false;
            if (Job::init(src.view(f), r, c, st, out, sm, und)) {
              store_sample(src.view(f), r, c, out, sm);
              finished++;
            } else {
              active = true;
              exec0 = executed;
            }
            undecided += und ? 1 : 0;
          }
        }
      }
    }
    if (!__any_sync(kFull, active)) {
      if (closed || ++idle > kDrainIdlePolls) break;
      __nanosleep(2000);
      continue;
    }
    idle = 0;
    if (active) {
      EscapeValue out;
      double sm = 0.0;
      if (Job::steps(src.view(f), st, chunk, out, sm, executed, rebases)) {
        store_sample(src.view(f), r, c, out, sm);
        log_cost(src.view(f), r, c, executed - exec0, Job::kCostWeight);
        finished++;
        active = false;
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    executed += __shfl_xor_sync(kFull, executed, o);
    rebases += __shfl_xor_sync(kFull, rebases, o);
    finished += __shfl_xor_sync(kFull, finished, o);
    undecided += __shfl_xor_sync(kFull, undecided, o);
    lost += __shfl_xor_sync(kFull, lost, o);
  }
  if (lane == 0) {
    atomicAdd(&ctl.stats[STAT_EXECUTED_ITERS], executed);
    atomicAdd(&ctl.stats[STAT_SAMPLES], finished);
    if (rebases) atomicAdd(&ctl.stats[STAT_REBASES], rebases);
    if (undecided) atomicAdd(&ctl.stats[STAT_CARDIOID_UNDECIDED], undecided);
    if (lost) atomicAdd(timeouts, lost);
  }
}

}  // namespace nmg
