// FP32 floatexp perturbation kernel with certified escape counts.
//
// Per sample: the FP64 series front of getIterations (cardioid, eps, series
// skip, binary search -- pixel_fp64.cuh, bit-identical to the plain FP64
// path), then the delta iteration on the FP32 pipe:
//     t = 2 Z[j] + delta;  delta = t * delta + eps;  j += 1;  Y = Z[j] + delta
// with delta, eps and the reference orbit Z held as float-float pairs (two
// FP32 words) and, while |delta| < 2^-60, one int exponent E per sample
// (delta = mantissa * 2^E), renormalised at the end of every chunk of `chunk`
// steps and whenever the mantissa passes 2^60.
//
// Certification.  Alongside delta the kernel propagates a bound on the
// absolute error of delta against exact arithmetic from the same start:
//     e' = 2|Y| e + e^2 + u (|t||delta| + |eps|) + u_z 2|Z||delta|
// (u: float-float rounding, u_z: float-float representation of the FP64 orbit).
// The FP64 path's own rounding is 2^-9 of that, so whenever every escape test
// of the sample is decided by more than twice the bound, both paths take the
// same branch at every test and return the same escape count.  A sample with
// an escape test inside the band is "uncertified": its index is appended to
// a rework list and the plain FP64 kernel renders it again, so the grid
// equals the FP64 path's on every sample whose bound held.
#include "engine.hpp"
#include "ff32.cuh"
#include "persistent.cuh"
#include "pixel_fp64.cuh"

namespace nmg {

namespace {

constexpr int kScaledBelow = -60;     // delta kept as mantissa * 2^E below 2^-60
constexpr float kU = 0x1p-44f;        // float-float rounding per step (generous)
constexpr float kUZ = 0x1p-47f;       // float-float representation of Z
constexpr float kBailout = 1024.0f;   // mandelbrot.cpp:58

struct alignas(16) ZFF {  // reference orbit element, float-float
  float hx, hy, lx, ly;
};

struct FeState {
  FF dr, di;      // delta * 2^-E
  FF er, ei;      // eps * 2^-E
  float err;      // error bound of delta, in the same units
  int32_t E;      // 0: unscaled
  int32_t j, i;
  int32_t certified;
};

__device__ __forceinline__ ZFF load_z(const DeviceView& v, int j) {
  const Flt4 z = v.zf[j];
  return ZFF{z.x, z.y, z.z, z.w};
}

__device__ __forceinline__ bool fe_init(const DeviceView& v, int r, int c, FeState& st,
                                        EscapeValue& out, double& sm, bool& und) {
  SeriesFront f;
  if (series_front(v, r, c, f, out, sm, und)) return true;
  const double m = fmax(fmax(fabs(f.dfound.re), fabs(f.dfound.im)),
                        fmax(fabs(f.eps.re), fabs(f.eps.im)));
  int E = 0;
  if (m > 0.0 && m < 0x1p-60) E = ilogb(m);
  st.E = E;
  st.dr = ff_from_double(scalbn(f.dfound.re, -E));
  st.di = ff_from_double(scalbn(f.dfound.im, -E));
  st.er = ff_from_double(scalbn(f.eps.re, -E));
  st.ei = ff_from_double(scalbn(f.eps.im, -E));
  st.err = kU * (fabsf(st.dr.h) + fabsf(st.di.h));
  st.j = f.dsize;
  st.i = f.dsize;
  st.certified = 1;
  return false;
}

// Y = Z[j] + delta (unscaled) in float-float.
__device__ __forceinline__ void y_ff(const ZFF& z, const FeState& st, FF& yr, FF& yi) {
  yr = ff_add(FF{z.hx, z.lx}, st.dr);
  yi = ff_add(FF{z.hy, z.ly}, st.di);
}

__device__ __forceinline__ void renormalise(FeState& st) {
  const float mag = fmaxf(fabsf(st.dr.h), fabsf(st.di.h));
  if (!(mag > 0.0f)) return;
  const int e = ilogbf(mag);
  st.dr = ff_scale(st.dr, -e);
  st.di = ff_scale(st.di, -e);
  st.er = ff_scale(st.er, -e);
  st.ei = ff_scale(st.ei, -e);
  st.err = ldexpf(st.err, -e);
  st.E += e;
  if (st.E >= kScaledBelow) {  // large enough for plain FP32
    st.dr = ff_scale(st.dr, st.E);
    st.di = ff_scale(st.di, st.E);
    st.er = ff_scale(st.er, st.E);
    st.ei = ff_scale(st.ei, st.E);
    st.err = ldexpf(st.err, st.E);
    st.E = 0;
  }
}

// Steps while delta is scaled: Y = Z to working precision, so the only
// events are the reference's own escape and the end of the orbit.
__device__ __noinline__ bool fe_scaled_steps(const DeviceView& v, FeState& st, int steps,
                                             EscapeValue& out, double& sm,
                                             unsigned long long& executed,
                                             unsigned long long& rebases) {
  const int zlast = v.zlen - 1;
  const int stop = min(v.N, st.i + steps);
  const int start = st.i;
  ZFF z = load_z(v, st.j);
  bool done = false;
  for (; st.i < stop; st.i++) {
    const FF sd_r = st.E < -140 ? FF{0.f, 0.f} : ff_scale(st.dr, st.E);
    const FF sd_i = st.E < -140 ? FF{0.f, 0.f} : ff_scale(st.di, st.E);
    const FF tr = ff_add(FF{2.0f * z.hx, 2.0f * z.lx}, sd_r);
    const FF ti = ff_add(FF{2.0f * z.hy, 2.0f * z.ly}, sd_i);
    const float zl1 = fabsf(z.hx) + fabsf(z.hy), dl1 = fabsf(st.dr.h) + fabsf(st.di.h);
    FF nr, ni;
    ff_cmul_add(tr, ti, st.dr, st.di, st.er, st.ei, nr, ni);
    st.err = fmaf(2.0f * zl1, st.err,
                  kU * fmaf(fabsf(tr.h) + fabsf(ti.h), dl1, fabsf(st.er.h) + fabsf(st.ei.h)) +
                      kUZ * 2.0f * zl1 * dl1);
    st.dr = nr;
    st.di = ni;
    st.j++;
    z = load_z(v, st.j);
    const float zm2 = fmaf(z.hx, z.hx, z.hy * z.hy);
    if (zm2 > (float)(v.bailout2 * (1.0 - 0x1p-10))) {
      double yr, yi;
      const Dbl2 zd = v.z[st.j];
      yr = zd.x + scalbn(ff_to_double(st.dr), st.E);
      yi = zd.y + scalbn(ff_to_double(st.di), st.E);
      const double r2 = yr * yr + yi * yi;
      const double ym = sqrt(r2), band = 2.0 * scalbn((double)st.err, st.E) + 1e-12 * ym;
      if (fabs(ym - 1024.0) <= band) st.certified = 0;
      if (r2 > v.bailout2) {
        sm = smoothing_of(r2, v.log_bailout);
        out = {st.i, (float)sm};
        done = true;
        st.i++;
        break;
      }
    }
    if (zm2 < 0x1p-80f || st.j == zlast) {
      // The orbit is exhausted, or it passes so close to 0 that |Y| < |delta|
      // may hold: rebase to Z[0] in FP64 with the unscaled delta.
      const Dbl2 zd = v.z[st.j];
      const double yr = zd.x + scalbn(ff_to_double(st.dr), st.E);
      const double yi = zd.y + scalbn(ff_to_double(st.di), st.E);
      const double dd = scalbn(fabs(ff_to_double(st.dr)) + fabs(ff_to_double(st.di)), st.E);
      if (st.j == zlast || fabs(yr) + fabs(yi) < dd) {
        const float e_abs = (float)scalbn((double)st.err, st.E) + kUZ * 2048.0f;
        st.dr = ff_from_double(yr);
        st.di = ff_from_double(yi);
        st.er = ff_scale(st.er, st.E);
        st.ei = ff_scale(st.ei, st.E);
        st.err = e_abs;
        st.E = 0;
        st.j = 0;
        rebases++;
        st.i++;
        break;
      }
    }
    if (fmaxf(fabsf(st.dr.h), fabsf(st.di.h)) > 0x1p60f) {
      st.i++;
      break;
    }
  }
  executed += (unsigned long long)(st.i - start);
  if (!done && st.E != 0) renormalise(st);
  if (done) return true;
  if (st.i >= v.N) {
    out = {v.N, 0.0f};
    sm = 0.0;
    return true;
  }
  return false;
}

__device__ __forceinline__ bool fe_steps(const DeviceView& v, FeState& st, int steps,
                                         EscapeValue& out, double& sm,
                                         unsigned long long& executed,
                                         unsigned long long& rebases) {
  if (st.E != 0) return fe_scaled_steps(v, st, steps, out, sm, executed, rebases);
  const int zlast = v.zlen - 1;
  const int stop = min(v.N, st.i + steps);
  const int start = st.i;
  const float lo_band = (float)(v.bailout2 * (1.0 - 0x1p-10));
  const float eps_l1 = fabsf(st.er.h) + fabsf(st.ei.h);
  FF dr = st.dr, di = st.di;
  float err = st.err;
  int j = st.j, i = st.i;
  bool certified = st.certified != 0;
  ZFF z = load_z(v, j);
  // |Y| of the current state (for the error bound's amplification 2|Y|)
  float ym = sqrtf(fmaf(z.hx + dr.h, z.hx + dr.h, (z.hy + di.h) * (z.hy + di.h)));
  for (; i < stop; i++) {
    const FF tr = ff_add(FF{2.0f * z.hx, 2.0f * z.lx}, dr);
    const FF ti = ff_add(FF{2.0f * z.hy, 2.0f * z.ly}, di);
    const float zl1 = fabsf(z.hx) + fabsf(z.hy), dl1 = fabsf(dr.h) + fabsf(di.h);
    const float ym_up = ym + 0x1p-22f * (zl1 + dl1);
    err = fmaf(2.0f * ym_up + err, err,
               kU * fmaf(fabsf(tr.h) + fabsf(ti.h), dl1, eps_l1) + kUZ * 2.0f * zl1 * dl1);
    FF nr, ni;
    ff_cmul_add(tr, ti, dr, di, st.er, st.ei, nr, ni);
    dr = nr;
    di = ni;
    j++;
    z = load_z(v, j);
    const float yr = z.hx + dr.h, yi = z.hy + di.h;
    const float r2 = fmaf(yr, yr, yi * yi);
    ym = sqrtf(r2);
    const float zn1 = fabsf(z.hx) + fabsf(z.hy);
    // error of Y = Z + delta held in float-float (the rebase value)
    const float yerr = err + kUZ * zn1 + kU * (zn1 + fabsf(dr.h) + fabsf(di.h));
    if (r2 <= lo_band) {
      // |Y| is below the bailout by more than 2^-11 of it; the hi-part
      // estimate ym is good to 2^-22 (|Z| + |delta|), so the test is decided
      // unless the bound covers the whole gap
      if (2.0f * (yerr + 0x1p-22f * (zn1 + fabsf(dr.h) + fabsf(di.h))) >= kBailout - ym)
        certified = false;
    } else {
      // escape decided on the accurate Y (FP64 from the float-float parts)
      const Dbl2 zd = v.z[j];
      const double ydr = zd.x + ff_to_double(dr), ydi = zd.y + ff_to_double(di);
      const double r2d = ydr * ydr + ydi * ydi;
      const double ymd = sqrt(r2d);
      if (fabs(ymd - 1024.0) <= 2.0 * (double)yerr + 1e-12 * ymd) certified = false;
      if (r2d > v.bailout2) {
        executed += (unsigned long long)(i + 1 - start);
        sm = smoothing_of(r2d, v.log_bailout);
        out = {i, (float)sm};
        st.certified = certified ? 1 : 0;
        return true;
      }
    }
    const float d2 = fmaf(dr.h, dr.h, di.h * di.h);
    if (r2 < d2 || j == zlast) {  // rebase to Z[0]: delta = Y in float-float
      FF nyr, nyi;
      nyr = ff_add(FF{z.hx, z.lx}, dr);
      nyi = ff_add(FF{z.hy, z.ly}, di);
      dr = nyr;
      di = nyi;
      err = yerr;
      j = 0;
      z = load_z(v, 0);
      ym = sqrtf(fmaf(dr.h, dr.h, di.h * di.h));
      rebases++;
    }
  }
  executed += (unsigned long long)(i - start);
  st.dr = dr;
  st.di = di;
  st.err = err;
  st.j = j;
  st.i = i;
  st.certified = certified ? 1 : 0;
  if (i >= v.N) {
    out = {v.N, 0.0f};
    sm = 0.0;
    return true;
  }
  return false;
}

struct FeJob {
  using State = FeState;
  static constexpr bool kCertifies = true;
  static __device__ __forceinline__ bool init(const DeviceView& v, int r, int c, State& st,
                                              EscapeValue& out, double& sm, bool& und) {
    return fe_init(v, r, c, st, out, sm, und);
  }
  static __device__ __forceinline__ bool steps(const DeviceView& v, State& st, int n,
                                               EscapeValue& out, double& sm,
                                               unsigned long long& executed,
                                               unsigned long long& rebases) {
    return fe_steps(v, st, n, out, sm, executed, rebases);
  }
  static __device__ __forceinline__ bool certified(const State& st) {
    return st.certified != 0;
  }
};

__global__ void __launch_bounds__(kPersistentThreads) fe32_kernel(DeviceView v, RenderCtl ctl,
                                                                    int chunk) {
  persistent_loop<FeJob>(v, ctl, chunk);
}

}  // namespace

int fe32_blocks_per_sm() {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fe32_kernel, kPersistentThreads, 0);
  return per_sm;
}

cudaError_t launch_fe32(const DeviceView& v, const RenderCtl& ctl, cudaStream_t stream,
                        int blocks, int chunk) {
  fe32_kernel<<<blocks, kPersistentThreads, 0, stream>>>(v, ctl, chunk);
  return cudaGetLastError();
}

}  // namespace nmg
