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

// ---- block-local compaction of FP64 samples ---------------------------------
//
// The FP64 pipe spends the same time on a warp instruction whatever the number
// of its active lanes (on GB300 one FP64 warp instruction per 80 cycles of an
// SM sub-partition, with 1 or 32 lanes active), so FP64 samples are best
// carried in full warps.  Once the work a warp draws from has run dry, lanes
// whose samples finish stay empty; then the warps of a block pool their
// samples in shared memory (state, position and steps so far) so that fewer,
// fuller warps carry them on:
//   * a warp left with fewer than kCompactBelow samples hands them to the
//     pool -- and, once no more work can arrive, leaves, when the block's
//     other warps can hold every sample;
//   * a warp with empty lanes takes samples from the pool: freely while it
//     keeps running anyway (kCompactBelow samples or more), otherwise only
//     when kCompactBelow samples wait there or no more work can arrive (so
//     that a warp's few samples do not just come back to it);
//   * a warp leaves only through the pool's lock, and never while samples
//     wait in the pool with no other warp of the block left to take them.
// One lock per block guards the pool (short critical sections, bounded spins;
// a warp that cannot take it keeps its samples and tries again later).  The
// order in which samples run does not change their results.

constexpr int kPoolCap = 128;
constexpr int kCompactBelow = 16;
constexpr unsigned kPoolLockSpins = 1u << 12;

template <class State>
struct PoolEntry {
  State st;
  unsigned long long spent;  // steps run so far (the cost log's share)
  int32_t f, r, c, pad_;
};

template <class State>
struct SamplePool {
  PoolEntry<State> e[kPoolCap];
  int32_t count;  // waiting samples: e[0, count)
  int32_t lock;
  int32_t alive;  // warps of the block inside the loop
  int32_t held;   // samples in those warps' lanes (as last reported)
};

// Every thread of the block calls it at the start of the kernel.
template <class State>
__device__ __forceinline__ void pool_init(SamplePool<State>* p) {
  if (threadIdx.x == 0) {
    p->count = 0;
    p->lock = 0;
    p->alive = 0;
    p->held = 0;
  }
  __syncthreads();
}

template <class State>
__device__ __forceinline__ void pool_enter(SamplePool<State>* p) {
  if (p && (threadIdx.x & 31) == 0) atomicAdd(&p->alive, 1);
}

// One exchange with the pool by a full warp (every lane calls it).  `closed`:
// no more work can arrive for this loop.  Returns true when the warp leaves.
template <class Job>
__device__ __forceinline__ bool pool_exchange(SamplePool<typename Job::State>* p, bool closed,
                                              bool& active, typename Job::State& st,
                                              unsigned long long executed,
                                              unsigned long long& exec0, int& f, int& r, int& c,
                                              int& held) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int ok = 0;
  if (lane == 0) {
    for (unsigned t = 0; t < kPoolLockSpins; t++) {
      if (atomicCAS(&p->lock, 0, 1) == 0) {
        ok = 1;
        break;
      }
      __nanosleep(64);
    }
  }
  if (!__shfl_sync(kFull, ok, 0)) return false;
  __syncwarp();
  int count = 0, alive = 0, held_all = 0;
  if (lane == 0) {
    count = *(volatile int32_t*)&p->count;
    alive = *(volatile int32_t*)&p->alive;
    held_all = *(volatile int32_t*)&p->held;
  }
  count = __shfl_sync(kFull, count, 0);
  alive = __shfl_sync(kFull, alive, 0);
  held_all = __shfl_sync(kFull, held_all, 0);
  unsigned am = __ballot_sync(kFull, active);
  int k = __popc(am);
  bool leave = false;
  // hand a few samples over
  if (k > 0 && k < kCompactBelow && count + k <= kPoolCap &&
      (!closed || (alive - 1) * 32 >= held_all - held + k + count)) {
    if (active) {
      PoolEntry<typename Job::State>& e = p->e[count + __popc(am & ((1u << lane) - 1))];
      e.st = st;
      e.spent = executed - exec0;
      e.f = f;
      e.r = r;
      e.c = c;
      active = false;
    }
    count += k;
    k = 0;
    am = 0;
    leave = closed;
    __syncwarp();
  }
  // fill empty lanes
  if (!leave) {
    const int idle = 32 - k;
    int take = 0;
    if (idle > 0 && count > 0 && (k >= kCompactBelow || closed || count >= kCompactBelow))
      take = idle < count ? idle : count;
    if (take > 0) {
      const unsigned free_lanes = ~am;
      const int rank = __popc(free_lanes & ((1u << lane) - 1));
      if (!active && rank < take) {
        const PoolEntry<typename Job::State>& e = p->e[count - take + rank];
        st = e.st;
        exec0 = executed - e.spent;
        f = e.f;
        r = e.r;
        c = e.c;
        active = true;
      }
      count -= take;
      k += take;
    }
    if (k == 0 && closed && count == 0) leave = true;
  }
  __threadfence_block();
  __syncwarp();
  if (lane == 0) {
    p->count = count;
    p->held += (leave ? 0 : k) - held;
    if (leave) p->alive -= 1;
    __threadfence_block();
    atomicExch(&p->lock, 0);
  }
  held = leave ? 0 : k;
  __syncwarp();
  return leave;
}

template <class Job, class Src>
__device__ __forceinline__ void sample_loop(const Src& src, const RenderCtl& ctl, int chunk,
                                            SamplePool<typename Job::State>* pool = nullptr) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  typename Job::State st;
  bool active = false, exhausted = false;
  int r = 0, c = 0, f = 0;
  long long sid = 0;
  unsigned long long executed = 0, rebases = 0, finished = 0, undecided = 0, exec0 = 0;
  const unsigned long long end =
      ctl.count_ptr ? *ctl.count_ptr : (unsigned long long)ctl.count;
  int held = 0;
  unsigned naps = 0;
  if (Job::kCertifies) pool = nullptr;  // a certifying job's samples carry their list index
  pool_enter(pool);

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
    if (pool && __any_sync(kFull, exhausted) &&
        pool_exchange<Job>(pool, true, active, st, executed, exec0, f, r, c, held))
      break;
    if (!__any_sync(kFull, active)) {
      // without a pool, or after leaving it, nothing is left; with one, its
      // lock was busy: try again (bounded)
      if (!pool || ++naps > kPoolLockSpins) break;
      __nanosleep(1000);
      continue;
    }
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
                                                int chunk,
                                                SamplePool<typename Job::State>* pool = nullptr) {
  sample_loop<Job>(OneView{v}, ctl, chunk, pool);
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

// An idle consumer sleeps 20 us between polls, 2^16 polls: about a second.
// (With 2 us sleeps the 1920x1080x16 view at width 1e-12 took 186 ms instead
// of 183 -- the FE32 warps beside the pollers lose issue slots; 100 us was
// slower again.)
constexpr unsigned kDrainNapNs = 20000;
constexpr unsigned kDrainIdlePolls = 1u << 16;
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
                                           unsigned long long* timeouts, int chunk,
                                           SamplePool<typename Job::State>* pool = nullptr) {
  const unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  typename Job::State st;
  bool active = false, closed = false;
  int r = 0, c = 0, f = 0;
  unsigned idle = 0;
  unsigned long long executed = 0, rebases = 0, finished = 0, undecided = 0, lost = 0, exec0 = 0;
  int held = 0;
  pool_enter(pool);
  for (;;) {
    const unsigned need = __ballot_sync(kFull, !active);
    bool dry = need != 0;  // empty lanes the list could not fill
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
      dry = got < (unsigned)__popc(need);
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
    // after kDrainIdlePolls idle polls the rest of the list is left to the
    // next launch; samples waiting in the pool are still carried on here
    const bool fin = closed || idle > kDrainIdlePolls;
    if (pool && (dry || fin) &&
        pool_exchange<Job>(pool, fin, active, st, executed, exec0, f, r, c, held))
      break;
    if (!__any_sync(kFull, active)) {
      if (!pool ? fin : idle > 2 * kDrainIdlePolls) break;
      ++idle;
      __nanosleep(kDrainNapNs);
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
