// The per-sample jobs of the FP64 kernels, for the persistent loops: the
// reference's double path (getIterationsHW, mandelbrot.cpp:231-254) and the
// plain FP64 perturbation path (getIterations' series front, then the FP64
// delta continuation).  All reference-order arithmetic inside is written with
// round-to-nearest intrinsics, so it is never contracted whatever the
// compiler's FMA setting.
#pragma once

#include "pixel_fe64.cuh"

namespace nmg {

struct HwJob {
  using State = HwState;
  static constexpr bool kCertifies = false;
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

struct Delta64Job {
  struct State {
    DeltaState d;
  };
  static constexpr bool kCertifies = false;
  static __device__ __forceinline__ bool certified(const State&) { return true; }
  static __device__ __forceinline__ bool init(const DeviceView& v, int r, int c, State& st,
                                              EscapeValue& out, double& sm, bool& und) {
    SeriesFront f;
    if (series_front_any(v, r, c, f, out, sm, und)) return true;
    delta_start(f, st.d);
    return false;
  }
  static __device__ __forceinline__ bool steps(const DeviceView& v, State& st, int n,
                                               EscapeValue& out, double& sm,
                                               unsigned long long& executed,
                                               unsigned long long&) {
    int before = st.d.i;
    bool done = delta_steps(v, st.d, n, out, sm);
    executed += (unsigned long long)((done ? out.iterations + (out.iterations < v.N ? 1 : 0)
                                           : st.d.i) - before);
    return done;
  }
};

}  // namespace nmg
