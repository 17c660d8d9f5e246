// The per-pixel colour (viewer.cpp:89-124): getColor on every sample and,
// with multisampling, the float mean of the sample colours of each pixel --
// one thread per output pixel, colours from the cached palette in global
// memory (L1/L2-resident: a few MB at most).  Float arithmetic in the host
// restatement's order (colour.cpp), never contracted, so the image is the
// host's byte for byte.
#include <cuda_runtime.h>

#include "engine.hpp"

#include <cstdint>

#include "colour.hpp"
#include "view_device.cuh"

namespace nmg {
namespace {

__device__ __forceinline__ uint8_t clip_byte_d(float x) {
  if (!(x > 0.0f)) return 0;
  if (x >= 255.0f) return 255;
  return (uint8_t)__fadd_rn(x, 0.5f);
}

__device__ __forceinline__ float interp_channel(uint8_t a, uint8_t b, float t) {
  const float s = __fsub_rn(1.0f, t);
  return __fadd_rn(__fmul_rn(s, (float)a), __fmul_rn(t, (float)b));
}

// viewer.cpp:89-94: black inside, the palette entry, or the blend of the
// entries either side of the smoothed count.  (The reference reads pal[-1]
// for a sample escaping at iteration 0 when smoothing; entry 0 is used.)
__device__ __forceinline__ void sample_colour(const EscapeValue e, int N, const Rgb* pal,
                                              int smooth, float& r, float& g, float& b) {
  if (e.iterations >= N) {
    r = g = b = 0.0f;
    return;
  }
  const Rgb c1 = pal[e.iterations];
  if (!smooth) {
    r = c1.r;
    g = c1.g;
    b = c1.b;
    return;
  }
  const Rgb c0 = pal[e.iterations > 0 ? e.iterations - 1 : 0];
  r = clip_byte_d(interp_channel(c0.r, c1.r, e.smoothing));
  g = clip_byte_d(interp_channel(c0.g, c1.g, e.smoothing));
  b = clip_byte_d(interp_channel(c0.b, c1.b, e.smoothing));
}

__global__ void colour_kernel(const EscapeValue* __restrict__ grid, int nr, int nc, int sc, int N,
                              const Rgb* __restrict__ pal, int smooth, uint8_t* __restrict__ out) {
  const int onc = nc / sc;
  const long long n = (long long)(nr / sc) * onc;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(k / onc), c = (int)(k - (long long)r * onc);
    float sr = 0.0f, sg = 0.0f, sb = 0.0f;
    for (int r1 = r * sc; r1 < (r + 1) * sc; r1++)
      for (int c1 = c * sc; c1 < (c + 1) * sc; c1++) {
        float cr, cg, cb;
        sample_colour(grid[(long long)r1 * nc + c1], N, pal, smooth, cr, cg, cb);
        sr = __fadd_rn(sr, cr);
        sg = __fadd_rn(sg, cg);
        sb = __fadd_rn(sb, cb);
      }
    uint8_t* o = out + 3 * k;
    if (sc == 1) {
      o[0] = (uint8_t)sr;
      o[1] = (uint8_t)sg;
      o[2] = (uint8_t)sb;
    } else {
      const float q = (float)(sc * sc);
      o[0] = clip_byte_d(__fdiv_rn(sr, q));
      o[1] = clip_byte_d(__fdiv_rn(sg, q));
      o[2] = clip_byte_d(__fdiv_rn(sb, q));
    }
  }
}

}  // namespace

cudaError_t launch_colour(const EscapeValue* grid, int nr, int nc, int sc, int N, const Rgb* pal,
                          int smooth, uint8_t* out, cudaStream_t s) {
  const long long n = (long long)(nr / sc) * (nc / sc);
  if (n <= 0) return cudaSuccess;
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  nmg::note_launches(1);
  colour_kernel<<<(int)blocks, 256, 0, s>>>(grid, nr, nc, sc, N, pal, smooth, out);
  return cudaGetLastError();
}

}  // namespace nmg
