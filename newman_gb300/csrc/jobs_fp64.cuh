// The per-sample jobs of the FP64 kernels, for the persistent loops: the
// reference's double path (getIterationsHW, mandelbrot.cpp:231-254) and the
// plain FP64 perturbation path (getIterations' series front, then the FP64
// delta continuation).  All reference-order arithmetic inside is written with
// round-to-nearest intrinsics, so it is never contracted whatever the
// compiler's FMA setting.
#pragma once

#include "pixel_fe64.cuh"
#include "pixel_xd.cuh"

namespace nmg {

struct HwJob {
  using State = HwState;
  static constexpr bool kCertifies = false;
  static constexpr int kCostWeight = kCostFp64Step;
  static __device__ __forceinline__ bool certified(const State&) { return true; }
  static __device__ __forceinline__ bool init(const DeviceView& v, int r, int c, State& st,
                                              EscapeValue& out, double& sm, bool& und) {
    return hw_init(v, r, c, st, out, sm, und);
  }
  static __device__ __forceinline__ bool steps(const DeviceView& v, State& st, int n,
                                               EscapeValue& out, double& sm,
                                               unsigned long long& executed,
                                               unsigned long long&) {
    int before = st.it;
    bool done = hw_steps(v, st, n, out, sm);
    // an escape returns before st.it is written; after a detected cycle st.it
    // holds the steps actually run
    executed += (unsigned long long)((done && out.iterations < v.N ? out.iterations + 1
                                                                   : st.it) - before);
    return done;
  }
};

// Views with a floatexp series front iterate in plain doubles while every
// value stays clear of the underflow range and in FP64 with an unbounded
// exponent (pixel_xd.cuh) otherwise, moving between the two at step (plain to
// unbounded) and chunk (back) boundaries -- the results are the unbounded
// form's throughout.  The other views iterate in plain doubles.  kStaged: the
// kernel staged the orbit's leading entries in shared memory.
template <bool kStaged = false>
struct Delta64JobT {
  struct State {
    union {
      DeltaState d;
      DeltaXDState x;
    };
    int32_t xd;  // 1: in the unbounded-exponent form
  };
  static constexpr bool kCertifies = false;
  static constexpr int kCostWeight = kCostFp64Step;
  static __device__ __forceinline__ bool certified(const State&) { return true; }
  static __device__ __forceinline__ bool init(const DeviceView& v, int r, int c, State& st,
                                              EscapeValue& out, double& sm, bool& und) {
    SeriesFront f;
    if (series_front_any(v, r, c, f, out, sm, und)) return true;
    st.xd = 0;
    if (!v.sa_fe) {
      delta_start(f, st.d);
    } else if (!delta_plain_start(f, st.d)) {
      delta_xd_start(f, st.x);
      st.xd = 1;
    }
    return false;
  }
  static __device__ __forceinline__ bool steps(const DeviceView& v, State& st, int n,
                                               EscapeValue& out, double& sm,
                                               unsigned long long& executed,
                                               unsigned long long&) {
    const int before = st.xd ? st.x.i : st.d.i;
    bool done;
    if (!v.sa_fe) {
      done = delta_steps<kStaged>(v, st.d, n, out, sm);
    } else if (st.xd) {
      done = delta_xd_steps<kStaged>(v, st.x, n, out, sm);
      if (!done && delta_xd_to_plain(st.x, st.d)) st.xd = 0;
    } else {
      bool handover;
      done = delta_guarded_steps<kStaged>(v, st.d, n, out, sm, handover);
      if (handover) {  // the rest of the chunk in the unbounded-exponent form
        const int left = n - (st.d.i - before);
        delta_to_xd(st.d, st.x);
        st.xd = 1;
        done = left > 0 ? delta_xd_steps<kStaged>(v, st.x, left, out, sm) : false;
      }
    }
    const int after = st.xd ? st.x.i : st.d.i;
    executed += (unsigned long long)((done ? out.iterations + (out.iterations < v.N ? 1 : 0)
                                           : after) - before);
    return done;
  }
};
using Delta64Job = Delta64JobT<false>;

// The FP64 rework of the FE32 path: the double loop on double-loop views (the
// FE32 path's comparator there), else the FP64 perturbation path.
template <bool kStaged = false>
struct Fp64AnyJobT {
  union State {
    HwJob::State hw;
    typename Delta64JobT<kStaged>::State d;
  };
  static constexpr bool kCertifies = false;
  static constexpr int kCostWeight = kCostFp64Step;
  static __device__ __forceinline__ bool certified(const State&) { return true; }
  static __device__ __forceinline__ bool init(const DeviceView& v, int r, int c, State& st,
                                              EscapeValue& out, double& sm, bool& und) {
    if (v.double_loop) return HwJob::init(v, r, c, st.hw, out, sm, und);
    return Delta64JobT<kStaged>::init(v, r, c, st.d, out, sm, und);
  }
  static __device__ __forceinline__ bool steps(const DeviceView& v, State& st, int n,
                                               EscapeValue& out, double& sm,
                                               unsigned long long& executed,
                                               unsigned long long& rebases) {
    if (v.double_loop) return HwJob::steps(v, st.hw, n, out, sm, executed, rebases);
    return Delta64JobT<kStaged>::steps(v, st.d, n, out, sm, executed, rebases);
  }
};
using Fp64AnyJob = Fp64AnyJobT<false>;

}  // namespace nmg
