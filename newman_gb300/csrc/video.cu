// Keyframe interpolation of the zoom video (VideoZoom::nextFrame,
// video.cpp:14-34): between two keyframes rendered at 1.5 times the output
// size, `rate` frames in which the previous keyframe grows from scale 1 and
// the new one from scale 2/3 by the factor v = 1.5^(1/rate) a frame, the new
// one blended over the old with weight i / rate, both centered.  One thread
// per output pixel of every frame (all frames of a keyframe pair in one
// launch); each layer's pixel is the bilinear sample of its keyframe, rounded
// to a byte as the reference materialises the scaled images, then blended.
//
// libbyteimage's ByteImage::scaled / blit / blend are not in the reference
// tree: scaled is restated as bilinear resampling with pixel centres aligned,
// blend as per-channel (1 - t) a + t b, both rounded half up into a byte.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "handle.hpp"

namespace nmg {
namespace {

__device__ __forceinline__ uint8_t clip_u8(float x) {
  if (!(x > 0.0f)) return 0;
  if (x >= 255.0f) return 255;
  return (uint8_t)__fadd_rn(x, 0.5f);
}

// Channel k of the (dh x dw) bilinear rescale of src (sh x sw) at (y, x).
__device__ __forceinline__ uint8_t scaled_at(const uint8_t* __restrict__ src, int sh, int sw,
                                             int dh, int dw, int y, int x, int k) {
  float fy = __fsub_rn(__fmul_rn(__fadd_rn((float)y, 0.5f), __fdiv_rn((float)sh, (float)dh)), 0.5f);
  float fx = __fsub_rn(__fmul_rn(__fadd_rn((float)x, 0.5f), __fdiv_rn((float)sw, (float)dw)), 0.5f);
  fy = fminf(fmaxf(fy, 0.0f), (float)(sh - 1));
  fx = fminf(fmaxf(fx, 0.0f), (float)(sw - 1));
  const int y0 = (int)fy, x0 = (int)fx;
  const int y1 = min(y0 + 1, sh - 1), x1 = min(x0 + 1, sw - 1);
  const float wy = __fsub_rn(fy, (float)y0), wx = __fsub_rn(fx, (float)x0);
  const float p00 = src[((long long)y0 * sw + x0) * 3 + k], p01 = src[((long long)y0 * sw + x1) * 3 + k];
  const float p10 = src[((long long)y1 * sw + x0) * 3 + k], p11 = src[((long long)y1 * sw + x1) * 3 + k];
  const float ux = __fsub_rn(1.0f, wx), uy = __fsub_rn(1.0f, wy);
  const float top = __fadd_rn(__fmul_rn(ux, p00), __fmul_rn(wx, p01));
  const float bot = __fadd_rn(__fmul_rn(ux, p10), __fmul_rn(wx, p11));
  return clip_u8(__fadd_rn(__fmul_rn(uy, top), __fmul_rn(wy, bot)));
}

struct FrameGeom {  // one output frame: the two layers' sizes and offsets, and the weight
  int lh, lw, sh, sw;  // large (previous keyframe) and small (new keyframe) sizes
  int lr, lc, sr, sc;  // their offsets in the canvas
  float t;
};

__global__ void interp_kernel(const uint8_t* __restrict__ prev, const uint8_t* __restrict__ cur,
                              int kh, int kw, int nr, int nc, const FrameGeom* __restrict__ geom,
                              int frames, uint8_t* __restrict__ out) {
  const long long per = (long long)nr * nc;
  const long long n = per * frames;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int f = (int)(q / per);
    const long long p = q - (long long)f * per;
    const int r = (int)(p / nc), c = (int)(p - (long long)r * nc);
    const FrameGeom g = geom[f];
    uint8_t* o = out + q * 3;
    // the large layer covers the canvas (scale >= 1 of a 1.5x keyframe)
    const int ly = r - g.lr, lx = c - g.lc;
    const bool in_small = r - g.sr >= 0 && r - g.sr < g.sh && c - g.sc >= 0 && c - g.sc < g.sw;
    const float ut = __fsub_rn(1.0f, g.t);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      uint8_t v = 0;
      if (ly >= 0 && ly < g.lh && lx >= 0 && lx < g.lw) v = scaled_at(prev, kh, kw, g.lh, g.lw, ly, lx, k);
      if (in_small) {
        const uint8_t s = scaled_at(cur, kh, kw, g.sh, g.sw, r - g.sr, c - g.sc, k);
        v = clip_u8(__fadd_rn(__fmul_rn(ut, (float)v), __fmul_rn(g.t, (float)s)));
      }
      o[k] = v;
    }
  }
}

}  // namespace

// The frames' geometry on the host, in the reference's float arithmetic:
// t = i / rate, and the two scales advanced by v = pow(1.5, 1/rate) a frame.
std::vector<FrameGeom> video_geometry(int kh, int kw, int nr, int nc, int rate) {
  std::vector<FrameGeom> g((size_t)rate);
  const float v = (float)std::pow(1.5, 1.0 / rate);
  float sm = (float)(2.0 / 3.0), lg = 1.0f;
  for (int i = 0; i < rate; i++) {
    FrameGeom& f = g[(size_t)i];
    f.t = (float)i / rate;
    f.sh = (int)(kh * sm);
    f.sw = (int)(kw * sm);
    f.lh = (int)(kh * lg);
    f.lw = (int)(kw * lg);
    f.lr = (nr - f.lh) / 2;
    f.lc = (nc - f.lw) / 2;
    f.sr = (nr - f.sh) / 2;
    f.sc = (nc - f.sw) / 2;
    sm *= v;
    lg *= v;
  }
  return g;
}

}  // namespace nmg

extern "C" int nm_video_interpolate(const unsigned char* prev_rgb, const unsigned char* cur_rgb,
                                    int key_rows, int key_cols, int rows, int cols, int rate,
                                    unsigned char* frames_out) {
  using nmg::fail;
  if (!prev_rgb || !cur_rgb || !frames_out || key_rows < 1 || key_cols < 1 || rows < 1 ||
      cols < 1 || rate < 1)
    return fail(NM_ERR_ARG, "video interpolation arguments");
  // the previous keyframe at scale >= 1 must cover the frame (as the
  // viewer's 1.5x keyframes do), so that no pixel keeps an older frame's value
  if (key_rows < rows || key_cols < cols)
    return fail(NM_ERR_ARG, "keyframes %d x %d smaller than the frames %d x %d", key_rows,
                key_cols, rows, cols);
  const std::vector<nmg::FrameGeom> geom = nmg::video_geometry(key_rows, key_cols, rows, cols, rate);
  for (const nmg::FrameGeom& g : geom)
    if (g.sh < 1 || g.sw < 1 || g.lh < 1 || g.lw < 1)
      return fail(NM_ERR_ARG, "keyframe %d x %d too small to scale", key_rows, key_cols);
  const size_t kbytes = (size_t)key_rows * key_cols * 3;
  const size_t obytes = (size_t)rate * rows * cols * 3;
  nmg::DevBuf<uint8_t> d_prev, d_cur, d_out;
  nmg::DevBuf<nmg::FrameGeom> d_geom;
  NM_CUDA(d_prev.reserve(kbytes));
  NM_CUDA(d_cur.reserve(kbytes));
  NM_CUDA(d_out.reserve(obytes));
  NM_CUDA(d_geom.reserve(geom.size()));
  NM_CUDA(cudaMemcpy(d_prev.p, prev_rgb, kbytes, cudaMemcpyHostToDevice));
  NM_CUDA(cudaMemcpy(d_cur.p, cur_rgb, kbytes, cudaMemcpyHostToDevice));
  NM_CUDA(cudaMemcpy(d_geom.p, geom.data(), geom.size() * sizeof(nmg::FrameGeom),
                     cudaMemcpyHostToDevice));
  const long long n = (long long)rate * rows * cols;
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  nmg::note_launches(1);
  nmg::interp_kernel<<<(int)blocks, 256>>>(d_prev.p, d_cur.p, key_rows, key_cols, rows, cols,
                                           d_geom.p, rate, d_out.p);
  NM_CUDA(cudaGetLastError());
  NM_CUDA(cudaMemcpy(frames_out, d_out.p, obytes, cudaMemcpyDeviceToHost));
  return NM_OK;
}
