// The reference-exact path (NM_PATH_MP): every sample computed the way the
// reference computes it, bits included.
//
// * Deep views (getIterations, mandelbrot.cpp:144-229): the cardioid test in
//   the view's arbitrary precision, the series front in FP64 (the reference's
//   own doubles, pixel_fp64.cuh), the sums X[k] + d[k] of its bailout test and
//   binary search in arbitrary precision, then the continuation
//   Y <- Y^2 + Y0 in arbitrary precision (:209-224) -- all with GMP mpf's
//   truncations reproduced limb for limb (mpf_fixed.cuh).
// * Double-loop views (getIterationsHW, :231-254): the cardioid test in
//   arbitrary precision, then the plain double loop (pixel_fp64.cuh).
//
// One kernel per precision (kMpMinLimbs .. kMpMaxLimbs limbs a value): the
// limbs of a value then live in registers.  Persistent and warp-refilled
// like the other per-sample kernels (persistent.cuh); the work is 64-bit
// integer multiply-adds on the integer pipes, so no lane pool is kept.
#include "engine.hpp"
#include "mpf_fixed.cuh"
#include "persistent.cuh"
#include "pixel_fp64.cuh"

namespace nmg {

namespace {

template <int P>
__device__ __forceinline__ Mpfx<P> load_mp(const uint64_t* rec) {
  Mpfx<P> x;
  const uint64_t h = rec[0];
  x.e = (int32_t)(h >> 32);
  x.s = (int32_t)(uint32_t)h;
#pragma unroll
  for (int i = 0; i < P + 1; i++) x.d[i] = rec[1 + i];
  return x;
}

template <int P>
__device__ __forceinline__ const uint64_t* mp_rec(const uint64_t* base, long long k) {
  return base + k * (long long)(P + 2);
}

// Y = X[k] + d (mandelbrot.cpp:184-185, 189-190, 202-203): d set exactly
// (mpf_set_d) and added in the view's precision.
template <int P>
__device__ __forceinline__ void x_plus_d(const DeviceView& v, int k, C64 d, Mpfx<P>& yr,
                                         Mpfx<P>& yi) {
  yr = mpf_add(load_mp<P>(mp_rec<P>(v.x_mp, 2ll * k)), mpf_from_double<P>(d.re));
  yi = mpf_add(load_mp<P>(mp_rec<P>(v.x_mp, 2ll * k + 1)), mpf_from_double<P>(d.im));
}

template <int P>
struct MpJob {
  struct State {
    Mpfx<P> yr, yi, y0r, y0i;
    int32_t i;
  };
  static constexpr bool kCertifies = false;
  static constexpr int kCostWeight = 1;
  static __device__ __forceinline__ bool certified(const State&) { return true; }

  static __device__ __forceinline__ bool init(const DeviceView& v, int r, int c, State& st,
                                              EscapeValue& out, double& sm, bool& und) {
    und = false;
    st.y0r = load_mp<P>(mp_rec<P>(v.coord_re_mp, c));
    st.y0i = load_mp<P>(mp_rec<P>(v.coord_im_mp, r));
    if (v.cardioid_mode == CARDIOID_PER_SAMPLE && mpf_in_cardioid(st.y0r, st.y0i)) {
      out = {v.N, 0.0f};
      sm = 0.0;
      return true;
    }
    // the series front (mandelbrot.cpp:155-181) in the reference's doubles
    const C64 eps{v.eps_re[c], v.eps_im[r]};
    const C64 eps2 = c_sq(eps);
    const C64 eps3 = c_mul(eps, eps2);
    const int fire = sa_first_unstable(v, eps, eps2, eps3);
    int dsize = v.xlen;
    if (fire < v.xlen) dsize = fire - 3 < 1 ? 1 : fire - 3;
    int found = dsize - 1;
    x_plus_d<P>(v, found, sa_value(v, found, eps, eps2, eps3), st.yr, st.yi);
    if (mpf_bailed_out(st.yr, st.yi)) {  // :186-207
      int low = 0, high = dsize - 1, mid = dsize / 2;
      while (low <= high) {
        Mpfx<P> mr, mi;
        x_plus_d<P>(v, mid, sa_value(v, mid, eps, eps2, eps3), mr, mi);
        if (!mpf_bailed_out(mr, mi))
          low = mid + 1;
        else {
          high = mid - 1;
          found = mid;
        }
        mid = (low + high) / 2;
      }
      x_plus_d<P>(v, found, sa_value(v, found, eps, eps2, eps3), st.yr, st.yi);
      const double r2 = mpf_sq_mag_d(st.yr, st.yi);
      sm = smoothing_of(r2, v.log_bailout);
      out = {found, (float)sm};
      return true;
    }
    st.i = dsize;
    return false;
  }

  // The continuation (mandelbrot.cpp:209-228), up to n steps.
  static __device__ __forceinline__ bool steps(const DeviceView& v, State& st, int n,
                                               EscapeValue& out, double& sm,
                                               unsigned long long& executed,
                                               unsigned long long&) {
    for (int k = 0; k < n; k++) {
      if (st.i >= v.N) {
        out = {v.N, 0.0f};
        sm = 0.0;
        executed += k;
        return true;
      }
      Mpfx<P> nr, ni;
      mpf_orbit_step(st.yr, st.yi, st.y0r, st.y0i, nr, ni);
      double r2 = 0.0;
      if (mpf_bailed_out(nr, ni, &r2)) {
        sm = smoothing_of(r2, v.log_bailout);
        out = {st.i, (float)sm};
        executed += k + 1;
        return true;
      }
      st.yr = nr;
      st.yi = ni;
      st.i++;
    }
    executed += n;
    return false;
  }
};

// getIterationsHW with the reference's cardioid test in its own precision.
template <int P>
struct HwMpJob {
  using State = HwState;
  static constexpr bool kCertifies = false;
  static constexpr int kCostWeight = kCostFp64Step;
  static __device__ __forceinline__ bool certified(const State&) { return true; }
  static __device__ __forceinline__ bool init(const DeviceView& v, int r, int c, State& st,
                                              EscapeValue& out, double& sm, bool& und) {
    und = false;
    if (v.cardioid_mode == CARDIOID_PER_SAMPLE &&
        mpf_in_cardioid(load_mp<P>(mp_rec<P>(v.coord_re_mp, c)),
                        load_mp<P>(mp_rec<P>(v.coord_im_mp, r)))) {
      out = {v.N, 0.0f};
      sm = 0.0;
      return true;
    }
    hw_start(v.coord_re[c], v.coord_im[r], st);
    return false;
  }
  static __device__ __forceinline__ bool steps(const DeviceView& v, State& st, int n,
                                               EscapeValue& out, double& sm,
                                               unsigned long long& executed,
                                               unsigned long long&) {
    const int before = st.it;
    const bool done = hw_steps(v, st, n, out, sm);
    executed += (unsigned long long)((done && out.iterations < v.N ? out.iterations + 1
                                                                   : st.it) - before);
    return done;
  }
};

// findProbe's orbit lengths (mandelbrot.cpp:85-94, computeOrbit :97-110): one
// thread per probe point, in the view's arbitrary precision.
template <int P>
__global__ void __launch_bounds__(128) probe_kernel(const uint64_t* re, const uint64_t* im,
                                                      int n, int N, int32_t* len) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const Mpfx<P> cr = load_mp<P>(mp_rec<P>(re, k)), ci = load_mp<P>(mp_rec<P>(im, k));
  Mpfx<P> xr = cr, xi = ci;
  int i = 1;
  for (; i < N; i++) {
    Mpfx<P> nr, ni;
    mpf_orbit_step(xr, xi, cr, ci, nr, ni);
    if (mpf_bailed_out(nr, ni)) break;
    xr = nr;
    xi = ni;
  }
  len[k] = i;
}

template <int P>
__global__ void __launch_bounds__(kPersistentThreads) mp_kernel(DeviceView v, RenderCtl ctl,
                                                                  int chunk) {
  persistent_loop<MpJob<P>>(v, ctl, chunk);
}

template <int P>
__global__ void __launch_bounds__(kPersistentThreads) hw_mp_kernel(DeviceView v, RenderCtl ctl,
                                                                     int chunk) {
  persistent_loop<HwMpJob<P>>(v, ctl, chunk);
}

// At most as many blocks as fit on the GPU at once (a persistent kernel).
int resident_blocks(const void* kernel, int blocks) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPersistentThreads, 0);
  const int most = sms * (per_sm < 1 ? 1 : per_sm);
  return blocks < 1 || blocks > most ? most : blocks;
}

template <int P>
void launch_p(KernelKind kind, const DeviceView& v, const RenderCtl& ctl, cudaStream_t s,
              int blocks, int chunk) {
  if (kind == KERNEL_MP)
    mp_kernel<P><<<resident_blocks((const void*)mp_kernel<P>, blocks), kPersistentThreads, 0, s>>>(
        v, ctl, chunk);
  else
    hw_mp_kernel<P><<<resident_blocks((const void*)hw_mp_kernel<P>, blocks), kPersistentThreads, 0,
                      s>>>(v, ctl, chunk);
}

template <int P>
cudaError_t dispatch(KernelKind kind, const DeviceView& v, const RenderCtl& ctl, cudaStream_t s,
                     int blocks, int chunk) {
  if constexpr (P + 1 > kMpMaxLimbs) {
    return cudaErrorInvalidValue;
  } else {
    if (v.mp_limbs == P + 1) {
      launch_p<P>(kind, v, ctl, s, blocks, chunk);
      return cudaGetLastError();
    }
    return dispatch<P + 1>(kind, v, ctl, s, blocks, chunk);
  }
}

template <int P>
cudaError_t probes_p(int limbs, const uint64_t* re, const uint64_t* im, int n, int N,
                     int32_t* len, cudaStream_t s) {
  if constexpr (P + 1 > kMpMaxLimbs) {
    return cudaErrorInvalidValue;
  } else {
    if (limbs != P + 1) return probes_p<P + 1>(limbs, re, im, n, N, len, s);
    probe_kernel<P><<<(n + 127) / 128, 128, 0, s>>>(re, im, n, N, len);
    return cudaGetLastError();
  }
}

}  // namespace

cudaError_t launch_probes(int limbs, const uint64_t* re, const uint64_t* im, int n, int N,
                          int32_t* len, cudaStream_t stream) {
  if (limbs < kMpMinLimbs || limbs > kMpMaxLimbs || n < 1) return cudaErrorInvalidValue;
  note_launches(1);
  return probes_p<kMpMinLimbs - 1>(limbs, re, im, n, N, len, stream);
}

cudaError_t launch_mp(KernelKind kind, const DeviceView& v, const RenderCtl& ctl,
                      cudaStream_t stream, int blocks, int chunk) {
  if (v.mp_limbs < kMpMinLimbs || v.mp_limbs > kMpMaxLimbs) return cudaErrorInvalidValue;
  note_launches(1);
  return dispatch<kMpMinLimbs - 1>(kind, v, ctl, stream, blocks, chunk);
}

}  // namespace nmg
