// Launch interface of the per-sample kernels (host side, C++).
#pragma once

#include <cuda_runtime.h>

#include "view_device.cuh"

namespace nmg {

enum StatIndex {
  STAT_CARDIOID_UNDECIDED = 0,  // double-double cardioid test within 2^-96 of zero
  STAT_EXECUTED_ITERS = 1,      // z -> z^2 + c steps run on the GPU
  STAT_SAMPLES = 2,             // samples finished
  STAT_REBASES = 3,             // rebases of the perturbation delta
  STAT_REWORK = 4,              // samples the FE32 kernel handed to the FP64 kernel
  STAT_WAIT_TIMEOUTS = 5,       // bounded waits of the overlapped rework that ran out
  STAT_FRONT_FP64 = 6,          // FE32 samples whose series front needed FP64
  STAT_STAGE_FALLBACKS = 7,     // blocks whose staged orbit copy they made themselves
  STAT_COUNT = 8
};

// Work distribution and bookkeeping of one persistent launch.  `next` and
// `stats` live in device scratch memory that the caller zeroes.
struct RenderCtl {
  unsigned long long* next;      // work counter, samples handed out so far
  unsigned long long* stats;     // [STAT_COUNT]
  const volatile int* cancel;    // host-mapped flag, may be null
  long long first;               // first sample index (tile order)
  long long count;               // samples in this launch
  // Work from a list instead of a range: item k is sample list[k], and the
  // item count is read from device memory (written by an earlier kernel).
  const unsigned int* list;
  const unsigned long long* count_ptr;
  // Samples whose escape count a kernel could not certify are appended here.
  unsigned int* rework;
  unsigned long long* rework_n;
};

// KERNEL_REWORK: the FE32 path's FP64 rework (the double loop on double-loop
// views, else the FP64 delta path).
// KERNEL_MP: the reference-exact path (the series front, then the reference's
// arbitrary-precision continuation in its own arithmetic, mpf_fixed.cuh);
// KERNEL_HW_MP: the double loop with the cardioid test in that arithmetic.
enum KernelKind {
  KERNEL_HW = 0,
  KERNEL_DELTA64 = 1,
  KERNEL_FE32 = 2,
  KERNEL_REWORK = 3,
  KERNEL_MP = 4,
  KERNEL_HW_MP = 5
};
// Precisions the reference-exact kernels are built for: values of
// kMpMinLimbs .. kMpMaxLimbs limbs (GMP precisions of 64 .. 64 (kMpMaxLimbs - 2)
// bits).
constexpr int kMpMinLimbs = 3, kMpMaxLimbs = 9;
cudaError_t launch_mp(KernelKind kind, const DeviceView& v, const RenderCtl& ctl,
                      cudaStream_t stream, int blocks, int chunk);
// findProbe's orbit lengths on the GPU: n probe points as arbitrary-precision
// records of `limbs` limbs (re[k], im[k]), lengths to len[k] (device memory).
cudaError_t launch_probes(int limbs, const uint64_t* re, const uint64_t* im, int n, int N,
                          int32_t* len, cudaStream_t stream);

// Buffers of the FE32 pass pipeline (render_fe32.cu), one record per sample
// index in tile order.
struct FeState;
constexpr int kFeStateBytes = 64;
constexpr int kFeResultBytes = 16;
struct FePassBuffers {
  FeState* state;              // start state written by the front pass
  unsigned int* work;          // samples that need the iteration pass
  unsigned long long* work_n;  // their count (device scratch)
};

// The FP64 side of the overlapped iteration pass: warps that render the
// uncertified samples in FP64 while other warps of the same launch still
// iterate in FP32 and append to the rework list.  `rework.next` counts the
// list entries claimed; entries not claimed by the end of the launch are left
// to a following FP64 launch over the same list and counter.  The list must
// be filled with kListSentinel before the launch.
struct OverlapCtl {
  RenderCtl rework;                  // list, count_ptr, next, stats of the FP64 work
  unsigned long long* fe_warps_done; // FP32 warps that finished their FP32 work
  unsigned long long* timeouts;      // waits that ran out (stats word)
  int chunk;                         // FP64 steps between refills
};
constexpr unsigned int kListSentinel = 0xffffffffu;

// front pass -> iteration pass (persistent, events around it if given).  ctl
// carries the counters, the stats and the rework list; with `overlap` the
// iteration pass also renders the rework list in FP64 as it grows.
// z_stage > 0: the iteration pass stages orbit entries [0, z_stage) in
// shared memory (orbit_stage.cuh); l2_window: it runs with a persisting L2
// access-policy window over the orbit (both copies, 32 zlen bytes).
cudaError_t launch_fe32_passes(const DeviceView& v, const FePassBuffers& b, const RenderCtl& ctl,
                               cudaStream_t stream, int device, int blocks, int chunk,
                               cudaEvent_t iter_begin, cudaEvent_t iter_end,
                               const OverlapCtl* overlap, int z_stage = 0,
                               bool l2_window = false);

// ---- batches of frames (render_batch.cu) ------------------------------------
// Frames rendered by one kernel: global sample index g of frame f runs over
// [offsets[f], offsets[f+1]).
struct BatchGroup {
  const DeviceView* views;   // [n], device memory
  const long long* offsets;  // [n+1], device memory
  int n;
  long long total;
};
// One frame's multisample mean: (nr*sc x nc*sc) samples -> nr x nc pixels at
// out; its pixels are [offset, offset + nr*nc) of the batch's output.
struct ReduceJob {
  const EscapeValue* in;
  EscapeValue* out;
  int nc, sc;
  long long offset;
};
struct BatchLaunch {
  int device;
  BatchGroup fe, hw, fp64;
  FePassBuffers fe_buf;
  RenderCtl fe_ctl, rework_ctl, hw_ctl, fp64_ctl;
  bool overlap;             // FP64 work inside the FE32 iteration pass
  int fp64_warps;           // FP64 warps of 8 a block in that pass (0: by the batch)
  OverlapCtl overlap_ctl;   // its rework side (= rework_ctl) and counters
  int fe_chunk, chunk;
  const ReduceJob* reduce;  // [nreduce], device memory
  int nreduce;
  long long reduce_total;
};
// Every launch of one batch render, in stream order (capturable).
cudaError_t launch_batch(const BatchLaunch& launch, cudaStream_t stream);
// The FP64 render of the batch's rework list from its claim counter on (the
// caller resets it), then the multisample reduce of every frame.
cudaError_t launch_batch_rework(const BatchLaunch& launch, cudaStream_t stream);

// Kernels launched by this library in this process (all handles; a graph
// replay counts its kernel nodes).  note_launches adds n.
void note_launches(long long n);
long long launches_so_far();

// Persistent, warp-refilled launches: every warp keeps its 32 lanes busy by
// pulling new samples from `ctl.next` as lanes finish.
cudaError_t launch_render(KernelKind kind, const DeviceView& v, const RenderCtl& ctl,
                          cudaStream_t stream, int blocks, int chunk);
int persistent_blocks(KernelKind kind, int device);
int kernel_threads(KernelKind kind);

// Multisample mean (mandelbrot.cpp:320-332): (nr*sc x nc*sc) -> (nr x nc).
cudaError_t launch_reduce(const EscapeValue* in, int nr, int nc, int sc, EscapeValue* out,
                          cudaStream_t stream);
// Value duplication of scaleUp (mandelbrot.cpp:334-341): (nr x nc) -> (nr*sc x nc*sc).
cudaError_t launch_duplicate(const EscapeValue* in, int nr, int nc, int sc, EscapeValue* out,
                             cudaStream_t stream);

}  // namespace nmg
