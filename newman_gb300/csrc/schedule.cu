// Learned tile scheduling: per-tile features from a coarse preview of a view,
// and a small MLP cost model (FP16 weights, FP32 accumulation) trained and
// evaluated by hand-written kernels.  The model predicts the relative work of
// every tile, and the render hands tiles out longest-first (nm_set_tile_order);
// every sample's computation is independent of the order, so the image is the
// static order's bit for bit.
//
// Features of a tile (kCostFeatures = 18), from the preview samples inside it:
//   x(it) = 1 for samples that reach N, else (log2(1 + it) - lo) / (hi - lo)
//   clamped to [0, 1], lo / hi the min / max of log2(1 + it) over the preview's
//   escaping samples (x = 0 when hi == lo);
//   [0, 16)  fraction of the tile's samples in bin min(15, floor(16 x));
//   16, 17   mean and max of x.
//
// Model: 18 -> 64 -> 64 -> 64 -> 1, ReLU between layers, y = W4 h3 + b4.
// Parameters, FP32 masters in this order (weights row-major [out][in]):
//   W1[64][18] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64] b4[1].
// The forward and backward passes read FP16 copies of the weights (biases
// FP32) and accumulate in FP32; Adam updates the FP32 masters and rewrites the
// FP16 copies.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <memory>
#include <vector>

#include "handle.hpp"

namespace nmg {
namespace {

constexpr int kIn = 18, kH = 64;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kH * kIn, kOffW2 = kOffB1 + kH,
              kOffB2 = kOffW2 + kH * kH, kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kH * kH,
              kOffW4 = kOffB3 + kH, kOffB4 = kOffW4 + kH, kParams = kOffB4 + 1;
static_assert(kParams == NM_COST_PARAMS, "parameter count");
// FP16 weight copies: W1, W2, W3, W4 back to back, same layouts
constexpr int kHW1 = 0, kHW2 = kHW1 + kH * kIn, kHW3 = kHW2 + kH * kH, kHW4 = kHW3 + kH * kH,
              kHalfs = kHW4 + kH;

// ---- features -----------------------------------------------------------------

__device__ __forceinline__ float log_count(int it) { return log2f(1.0f + (float)it); }

// min / max of log2(1 + it) over escaping samples, as the bit patterns of
// non-negative floats (which order like the floats).
__global__ void preview_range_kernel(const EscapeValue* grid, long long n, int N,
                                     unsigned int* lohi) {
  unsigned int lo = 0x7f7fffffu, hi = 0u;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const int it = grid[k].iterations;
    if (it >= N) continue;
    const unsigned int b = __float_as_uint(log_count(it));
    lo = min(lo, b);
    hi = max(hi, b);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&lohi[0], lo);
    atomicMax(&lohi[1], hi);
  }
}

__global__ void tile_features_kernel(const EscapeValue* grid, int nr, int nc, int N, int tw,
                                     int th, int tiles_x, int ntiles, const unsigned int* lohi,
                                     float* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const float lo = __uint_as_float(lohi[0]), hi = __uint_as_float(lohi[1]);
  const float scale = hi > lo ? 1.0f / (hi - lo) : 0.0f;
  const int ty = t / tiles_x, tx = t - ty * tiles_x;
  float hist[16];
#pragma unroll
  for (int b = 0; b < 16; b++) hist[b] = 0.0f;
  float sum = 0.0f, mx = 0.0f;
  int count = 0;
  for (int r = ty * th; r < min(nr, (ty + 1) * th); r++)
    for (int c = tx * tw; c < min(nc, (tx + 1) * tw); c++) {
      const int it = grid[(long long)r * nc + c].iterations;
      float x = it >= N ? 1.0f : (log_count(it) - lo) * scale;
      x = fminf(fmaxf(x, 0.0f), 1.0f);
      const int bin = min(15, (int)(16.0f * x));
#pragma unroll
      for (int b = 0; b < 16; b++) hist[b] += b == bin ? 1.0f : 0.0f;
      sum += x;
      mx = fmaxf(mx, x);
      count++;
    }
  const float inv = count ? 1.0f / (float)count : 0.0f;
  float* o = out + (long long)t * kIn;
#pragma unroll
  for (int b = 0; b < 16; b++) o[b] = hist[b] * inv;
  o[16] = sum * inv;
  o[17] = mx;
}

// ---- the MLP ------------------------------------------------------------------
//
// One block of kH = 64 threads (thread j = neuron j) runs samples one after
// another.  Shared memory holds the FP16 weights twice -- transposed for the
// forward pass (thread j reads column j: consecutive addresses) and as stored
// for the backward pass -- the activations of the current sample, and, when
// training, FP32 gradient accumulators (transposed likewise), which are added
// to the global gradient once per block.

struct MlpShared {
  __half wf1[kIn * kH];   // [in][out]
  __half wf2[kH * kH];
  __half wf3[kH * kH];
  __half w4[kH];
  __half wb2[kH * kH];    // [out][in]
  __half wb3[kH * kH];
  float b1[kH], b2[kH], b3[kH], b4;
  float x[kIn], h1[kH], h2[kH], h3[kH], g3[kH], g2[kH];
  float a1[kH], a2[kH], a3[kH];
  float red[2];
  // gradient accumulators, [in][out]
  float gw1[kIn * kH], gw2[kH * kH], gw3[kH * kH], gw4[kH], gb1[kH], gb2[kH], gb3[kH], gb4;
  float loss;
};

__device__ __forceinline__ float block_sum64(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  const float s = red[0] + red[1];
  __syncthreads();
  return s;
}

// train == false: out[s] = prediction.  train == true: also the gradient of
// loss = mean_s (y_s - t_s)^2, added into grad (FP32, canonical layout), and
// the loss into *loss.
template <bool kTrain>
__global__ void __launch_bounds__(kH) mlp_kernel(const __half* __restrict__ wh,
                                                 const float* __restrict__ params,
                                                 const float* __restrict__ X,
                                                 const float* __restrict__ T, int n,
                                                 float* __restrict__ out, float* grad,
                                                 float* loss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpShared& S = *reinterpret_cast<MlpShared*>(smem_raw);
  const int j = threadIdx.x;
  // weights: forward copies transposed, backward copies as stored
  for (int k = j; k < kH * kIn; k += kH) {
    const int o = k / kIn, i = k - o * kIn;
    S.wf1[i * kH + o] = wh[kHW1 + k];
  }
  for (int k = j; k < kH * kH; k += kH) {
    const int o = k / kH, i = k - o * kH;
    S.wf2[i * kH + o] = wh[kHW2 + k];
    S.wf3[i * kH + o] = wh[kHW3 + k];
    S.wb2[k] = wh[kHW2 + k];
    S.wb3[k] = wh[kHW3 + k];
  }
  S.w4[j] = wh[kHW4 + j];
  S.b1[j] = params[kOffB1 + j];
  S.b2[j] = params[kOffB2 + j];
  S.b3[j] = params[kOffB3 + j];
  if (j == 0) S.b4 = params[kOffB4];
  if (kTrain) {
    for (int k = j; k < kIn * kH; k += kH) S.gw1[k] = 0.0f;
    for (int k = j; k < kH * kH; k += kH) {
      S.gw2[k] = 0.0f;
      S.gw3[k] = 0.0f;
    }
    S.gw4[j] = S.gb1[j] = S.gb2[j] = S.gb3[j] = 0.0f;
    if (j == 0) {
      S.gb4 = 0.0f;
      S.loss = 0.0f;
    }
  }
  __syncthreads();
  const float inv_n = 1.0f / (float)n;
  for (int s = blockIdx.x; s < n; s += gridDim.x) {
    if (j < kIn) S.x[j] = X[(long long)s * kIn + j];
    __syncthreads();
    float a = S.b1[j];
    for (int i = 0; i < kIn; i++) a = fmaf(__half2float(S.wf1[i * kH + j]), S.x[i], a);
    S.a1[j] = a;
    S.h1[j] = fmaxf(a, 0.0f);
    __syncthreads();
    a = S.b2[j];
    for (int i = 0; i < kH; i++) a = fmaf(__half2float(S.wf2[i * kH + j]), S.h1[i], a);
    S.a2[j] = a;
    S.h2[j] = fmaxf(a, 0.0f);
    __syncthreads();
    a = S.b3[j];
    for (int i = 0; i < kH; i++) a = fmaf(__half2float(S.wf3[i * kH + j]), S.h2[i], a);
    S.a3[j] = a;
    S.h3[j] = fmaxf(a, 0.0f);
    __syncthreads();
    const float y = block_sum64(__half2float(S.w4[j]) * S.h3[j], S.red) + S.b4;
    if (!kTrain) {
      if (j == 0) out[s] = y;
      continue;
    }
    const float diff = y - T[s];
    const float dy = 2.0f * diff * inv_n;
    if (j == 0) {
      S.loss += diff * diff * inv_n;
      S.gb4 += dy;
    }
    // layer 4
    S.gw4[j] += dy * S.h3[j];
    const float g3 = S.a3[j] > 0.0f ? dy * __half2float(S.w4[j]) : 0.0f;
    S.g3[j] = g3;
    S.gb3[j] += g3;
    for (int i = 0; i < kH; i++) S.gw3[i * kH + j] += g3 * S.h2[i];
    __syncthreads();
    // layer 3 -> 2: g2_j = sum_k W3[k][j] g3_k
    float g2 = 0.0f;
    for (int k = 0; k < kH; k++) g2 = fmaf(__half2float(S.wb3[k * kH + j]), S.g3[k], g2);
    g2 = S.a2[j] > 0.0f ? g2 : 0.0f;
    S.g2[j] = g2;
    S.gb2[j] += g2;
    for (int i = 0; i < kH; i++) S.gw2[i * kH + j] += g2 * S.h1[i];
    __syncthreads();
    float g1 = 0.0f;
    for (int k = 0; k < kH; k++) g1 = fmaf(__half2float(S.wb2[k * kH + j]), S.g2[k], g1);
    g1 = S.a1[j] > 0.0f ? g1 : 0.0f;
    S.gb1[j] += g1;
    for (int i = 0; i < kIn; i++) S.gw1[i * kH + j] += g1 * S.x[i];
    __syncthreads();
  }
  if (!kTrain) return;
  __syncthreads();
  for (int k = j; k < kIn * kH; k += kH) {  // gw1 [in][out] -> W1 [out][in]
    const int i = k / kH, o = k - i * kH;
    atomicAdd(&grad[kOffW1 + o * kIn + i], S.gw1[k]);
  }
  for (int k = j; k < kH * kH; k += kH) {
    const int i = k / kH, o = k - i * kH;
    atomicAdd(&grad[kOffW2 + o * kH + i], S.gw2[k]);
    atomicAdd(&grad[kOffW3 + o * kH + i], S.gw3[k]);
  }
  atomicAdd(&grad[kOffW4 + j], S.gw4[j]);
  atomicAdd(&grad[kOffB1 + j], S.gb1[j]);
  atomicAdd(&grad[kOffB2 + j], S.gb2[j]);
  atomicAdd(&grad[kOffB3 + j], S.gb3[j]);
  if (j == 0) {
    atomicAdd(&grad[kOffB4], S.gb4);
    atomicAdd(loss, S.loss);
  }
}

// FP32 masters -> FP16 weight copies.
__device__ __forceinline__ int half_index(int p) {
  if (p < kOffB1) return kHW1 + (p - kOffW1);
  if (p >= kOffW2 && p < kOffB2) return kHW2 + (p - kOffW2);
  if (p >= kOffW3 && p < kOffB3) return kHW3 + (p - kOffW3);
  if (p >= kOffW4 && p < kOffB4) return kHW4 + (p - kOffW4);
  return -1;  // a bias: FP32 only
}

__global__ void to_half_kernel(const float* params, __half* wh) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const int h = half_index(p);
  if (h >= 0) wh[h] = __float2half_rn(params[p]);
}

// Adam (Kingma & Ba) on the FP32 masters, step t (1-based); the gradient is
// cleared for the next accumulation.
__global__ void adam_kernel(float* params, float* grad, float* m, float* v, __half* wh, float lr,
                            float b1t, float b2t) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= kParams) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float g = grad[p];
  const float mp = b1 * m[p] + (1.0f - b1) * g;
  const float vp = b2 * v[p] + (1.0f - b2) * g * g;
  m[p] = mp;
  v[p] = vp;
  const float mh = mp / (1.0f - b1t), vh = vp / (1.0f - b2t);
  const float w = params[p] - lr * mh / (sqrtf(vh) + eps);
  params[p] = w;
  grad[p] = 0.0f;
  const int h = half_index(p);
  if (h >= 0) wh[h] = __float2half_rn(w);
}

// ---- longest-first order on the GPU ------------------------------------------
//
// One block sorts the tiles by key = (order-preserving bits of -prediction)
// << 32 | tile id, ascending, in shared memory (bitonic network over the
// next power of two, padding keys all ones): tiles by decreasing prediction,
// ties by id -- the permutation a stable sort of -prediction gives.
constexpr int kMaxOrderTiles = 16384;
constexpr int kSortThreads = 1024;

__device__ __forceinline__ uint32_t order_bits(float x) {
  const uint32_t b = __float_as_uint(x == 0.0f ? 0.0f : x);  // -0 ties with +0
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__global__ void __launch_bounds__(kSortThreads) order_sort_kernel(const float* __restrict__ pred,
                                                                  int n, int p2,
                                                                  int32_t* __restrict__ order) {
  extern __shared__ unsigned long long keys[];
  for (int k = threadIdx.x; k < p2; k += blockDim.x)
    keys[k] = k < n ? ((unsigned long long)order_bits(-pred[k]) << 32) | (unsigned)k : ~0ull;
  __syncthreads();
  for (int size = 2; size <= p2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = threadIdx.x; t < (p2 >> 1); t += blockDim.x) {
        const int lo = 2 * t - (t & (stride - 1));  // t with a 0 inserted at bit log2(stride)
        const int hi = lo + stride;
        const unsigned long long a = keys[lo], b = keys[hi];
        if ((a > b) == ((lo & size) == 0)) {
          keys[lo] = b;
          keys[hi] = a;
        }
      }
      __syncthreads();
    }
  }
  for (int k = threadIdx.x; k < n; k += blockDim.x) order[k] = (int32_t)(keys[k] & 0xffffffffull);
}

int mlp_blocks(int n, int device) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int b = 2 * (sms > 0 ? sms : 1);
  return n < b ? (n > 0 ? n : 1) : b;
}

}  // namespace
}  // namespace nmg

struct nm_costmodel {
  int device = 0;
  cudaStream_t stream = nullptr;
  nmg::DevBuf<float> params, grad, m, v, scratch;
  nmg::DevBuf<__half> wh;
  nmg::DevBuf<float> x, t, y;
  nmg::DevBuf<unsigned int> lohi;  // the preview's log-count range (nm_order_tiles)
  long long step = 0;
  ~nm_costmodel() {
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

using nmg::fail;

int upload_to_half(nm_costmodel* m) {
  nmg::note_launches(1);
  nmg::to_half_kernel<<<(nmg::kParams + 255) / 256, 256, 0, m->stream>>>(m->params.p, m->wh.p);
  NM_CUDA(cudaGetLastError());
  return NM_OK;
}

int stage(nm_costmodel* m, const float* x, const float* t, int n) {
  NM_CUDA(m->x.reserve((size_t)n * nmg::kIn));
  NM_CUDA(cudaMemcpyAsync(m->x.p, x, (size_t)n * nmg::kIn * 4, cudaMemcpyHostToDevice, m->stream));
  if (t) {
    NM_CUDA(m->t.reserve((size_t)n));
    NM_CUDA(cudaMemcpyAsync(m->t.p, t, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream));
  }
  return NM_OK;
}

template <bool kTrain>
int launch_mlp(nm_costmodel* m, int n, float* out, cudaStream_t stream = nullptr) {
  const size_t smem = sizeof(nmg::MlpShared);
  NM_CUDA(cudaFuncSetAttribute(nmg::mlp_kernel<kTrain>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  nmg::note_launches(1);
  nmg::mlp_kernel<kTrain><<<nmg::mlp_blocks(n, m->device), nmg::kH, smem,
                            stream ? stream : m->stream>>>(
      m->wh.p, m->params.p, m->x.p, kTrain ? m->t.p : nullptr, n, out, m->grad.p,
      m->scratch.p);
  NM_CUDA(cudaGetLastError());
  return NM_OK;
}

// splitmix64: the seeded stream of the weight initialisation
uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

}  // namespace

extern "C" {

nm_costmodel* nm_cost_model_create(unsigned long long seed) {
  std::unique_ptr<nm_costmodel> m(new nm_costmodel());
  if (cudaGetDevice(&m->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
      m->params.reserve(nmg::kParams) != cudaSuccess ||
      m->grad.reserve(nmg::kParams) != cudaSuccess || m->m.reserve(nmg::kParams) != cudaSuccess ||
      m->v.reserve(nmg::kParams) != cudaSuccess || m->scratch.reserve(4) != cudaSuccess ||
      m->wh.reserve(nmg::kHalfs) != cudaSuccess) {
    fail(NM_ERR_CUDA, "cost model: device allocation failed");
    return nullptr;
  }
  // He-uniform weights (limit sqrt(6 / fan_in)), zero biases
  std::vector<float> p(nmg::kParams, 0.0f);
  uint64_t s = seed;
  auto uniform = [&](float lim) {
    const double u = (double)(splitmix(s) >> 11) * 0x1p-53;
    return (float)((2.0 * u - 1.0) * lim);
  };
  for (int k = 0; k < nmg::kH * nmg::kIn; k++) p[nmg::kOffW1 + k] = uniform(std::sqrt(6.0f / nmg::kIn));
  for (int k = 0; k < nmg::kH * nmg::kH; k++) p[nmg::kOffW2 + k] = uniform(std::sqrt(6.0f / nmg::kH));
  for (int k = 0; k < nmg::kH * nmg::kH; k++) p[nmg::kOffW3 + k] = uniform(std::sqrt(6.0f / nmg::kH));
  for (int k = 0; k < nmg::kH; k++) p[nmg::kOffW4 + k] = uniform(std::sqrt(6.0f / nmg::kH));
  if (nm_cost_model_set_params(m.get(), p.data(), nmg::kParams) != NM_OK) return nullptr;
  return m.release();
}

void nm_cost_model_destroy(nm_costmodel* m) {
  if (m && m->stream) cudaStreamSynchronize(m->stream);
  delete m;
}

int nm_cost_model_set_params(nm_costmodel* m, const float* in, int n) {
  if (!m || !in || n != nmg::kParams) return fail(NM_ERR_ARG, "cost model parameters: %d", n);
  NM_CUDA(cudaMemcpyAsync(m->params.p, in, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream));
  NM_CUDA(cudaMemsetAsync(m->grad.p, 0, (size_t)n * 4, m->stream));
  NM_CUDA(cudaMemsetAsync(m->m.p, 0, (size_t)n * 4, m->stream));
  NM_CUDA(cudaMemsetAsync(m->v.p, 0, (size_t)n * 4, m->stream));
  m->step = 0;
  if (int rc = upload_to_half(m)) return rc;
  NM_CUDA(cudaStreamSynchronize(m->stream));
  return NM_OK;
}

int nm_cost_model_params(nm_costmodel* m, float* out, int n) {
  if (!m || !out || n != nmg::kParams) return fail(NM_ERR_ARG, "cost model parameters: %d", n);
  NM_CUDA(cudaStreamSynchronize(m->stream));
  NM_CUDA(cudaMemcpy(out, m->params.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
  return NM_OK;
}

int nm_cost_model_predict(nm_costmodel* m, const float* x, int n, float* y) {
  if (!m || !x || !y || n < 0) return fail(NM_ERR_ARG, "cost model predict");
  if (n == 0) return NM_OK;
  if (int rc = stage(m, x, nullptr, n)) return rc;
  NM_CUDA(m->y.reserve((size_t)n));
  if (int rc = launch_mlp<false>(m, n, m->y.p)) return rc;
  NM_CUDA(cudaMemcpyAsync(y, m->y.p, (size_t)n * 4, cudaMemcpyDeviceToHost, m->stream));
  NM_CUDA(cudaStreamSynchronize(m->stream));
  return NM_OK;
}

int nm_cost_model_gradient(nm_costmodel* m, const float* x, const float* t, int n, float* grad,
                           float* loss) {
  if (!m || !x || !t || !grad || n < 1) return fail(NM_ERR_ARG, "cost model gradient");
  if (int rc = stage(m, x, t, n)) return rc;
  NM_CUDA(cudaMemsetAsync(m->grad.p, 0, (size_t)nmg::kParams * 4, m->stream));
  NM_CUDA(cudaMemsetAsync(m->scratch.p, 0, 4, m->stream));
  if (int rc = launch_mlp<true>(m, n, nullptr)) return rc;
  NM_CUDA(cudaMemcpyAsync(grad, m->grad.p, (size_t)nmg::kParams * 4, cudaMemcpyDeviceToHost,
                          m->stream));
  float l = 0.0f;
  NM_CUDA(cudaMemcpyAsync(&l, m->scratch.p, 4, cudaMemcpyDeviceToHost, m->stream));
  NM_CUDA(cudaMemsetAsync(m->grad.p, 0, (size_t)nmg::kParams * 4, m->stream));
  NM_CUDA(cudaStreamSynchronize(m->stream));
  if (loss) *loss = l;
  return NM_OK;
}

int nm_cost_model_train(nm_costmodel* m, const float* x, const float* t, int n, int epochs,
                        float lr, float* loss) {
  if (!m || !x || !t || n < 1 || epochs < 0 || !(lr > 0.0f)) return fail(NM_ERR_ARG, "cost model train");
  if (int rc = stage(m, x, t, n)) return rc;
  float l = 0.0f;
  for (int e = 0; e < epochs; e++) {
    NM_CUDA(cudaMemsetAsync(m->scratch.p, 0, 4, m->stream));
    if (int rc = launch_mlp<true>(m, n, nullptr)) return rc;
    m->step++;
    const float b1t = (float)std::pow(0.9, (double)m->step);
    const float b2t = (float)std::pow(0.999, (double)m->step);
    nmg::note_launches(1);
    nmg::adam_kernel<<<(nmg::kParams + 255) / 256, 256, 0, m->stream>>>(
        m->params.p, m->grad.p, m->m.p, m->v.p, m->wh.p, lr, b1t, b2t);
    NM_CUDA(cudaGetLastError());
  }
  if (epochs > 0)
    NM_CUDA(cudaMemcpyAsync(&l, m->scratch.p, 4, cudaMemcpyDeviceToHost, m->stream));
  NM_CUDA(cudaStreamSynchronize(m->stream));
  if (loss) *loss = l;
  return NM_OK;
}

int nm_tile_features(nm_handle* preview, int tile_w, int tile_h, float* out, int ntiles) {
  if (!preview || !out || tile_w < 1 || tile_h < 1) return fail(NM_ERR_ARG, "tile features");
  if (!preview->stream || !preview->grid.p) return fail(NM_ERR_STATE, "preview not rendered");
  const int nr = preview->grid_nr, nc = preview->grid_nc;
  const int tx = (nc + tile_w - 1) / tile_w, ty = (nr + tile_h - 1) / tile_h;
  if ((long long)ntiles != (long long)tx * ty)
    return fail(NM_ERR_ARG, "%d feature rows for %d x %d tiles", ntiles, tx, ty);
  cudaStream_t s = preview->stream;
  nmg::DevBuf<unsigned int> lohi;
  nmg::DevBuf<float> d_out;
  NM_CUDA(lohi.reserve(2));
  NM_CUDA(d_out.reserve((size_t)ntiles * nmg::kIn));
  const unsigned int init[2] = {0x7f7fffffu, 0u};
  NM_CUDA(cudaMemcpyAsync(lohi.p, init, 8, cudaMemcpyHostToDevice, s));
  const long long n = (long long)nr * nc;
  const int N = preview->effective_N();  // x = 1 at the preview's own cap
  nmg::note_launches(2);
  nmg::preview_range_kernel<<<256, 256, 0, s>>>(preview->grid.p, n, N, lohi.p);
  nmg::tile_features_kernel<<<(ntiles + 127) / 128, 128, 0, s>>>(
      preview->grid.p, nr, nc, N, tile_w, tile_h, tx, ntiles, lohi.p, d_out.p);
  NM_CUDA(cudaGetLastError());
  NM_CUDA(cudaMemcpyAsync(out, d_out.p, (size_t)ntiles * nmg::kIn * 4, cudaMemcpyDeviceToHost, s));
  NM_CUDA(cudaStreamSynchronize(s));
  return NM_OK;
}

int nm_order_tiles(nm_handle* h, nm_handle* preview, nm_costmodel* m) {
  if (!h || !preview || !m) return fail(NM_ERR_ARG, "order tiles: null argument");
  if (!preview->stream || !preview->grid.p) return fail(NM_ERR_STATE, "preview not rendered");
  const int nr = h->view.rows(), nc = h->view.cols();
  const int pr = preview->grid_nr, pc = preview->grid_nc;
  if (pr < 1 || pc < 1 || nr % pr || nc % pc || nr / pr != nc / pc)
    return fail(NM_ERR_ARG, "a %d x %d preview of a %d x %d view", pr, pc, nr, nc);
  const int f = nr / pr;
  if (h->tile_w % f || h->tile_h % f)
    return fail(NM_ERR_ARG, "tile %d x %d is not a multiple of the preview factor %d", h->tile_w,
                h->tile_h, f);
  const int tw = h->tile_w / f, th = h->tile_h / f;
  const int tx = (nc + h->tile_w - 1) / h->tile_w, ty = (nr + h->tile_h - 1) / h->tile_h;
  const long long ntiles = (long long)tx * ty;  // == the preview's tiles of tw x th
  if (ntiles > nmg::kMaxOrderTiles)
    return fail(NM_ERR_UNSUPPORTED, "%lld tiles (at most %d)", ntiles, nmg::kMaxOrderTiles);
  if (int rc = nmg::ensure_device(h)) return rc;
  cudaStream_t s = h->stream;
  // after the preview's render, and after the model's own pending work
  struct Event {  // destroyed on every return
    cudaEvent_t e = nullptr;
    ~Event() {
      if (e) cudaEventDestroy(e);
    }
  } event;
  NM_CUDA(cudaEventCreateWithFlags(&event.e, cudaEventDisableTiming));
  cudaEvent_t ev = event.e;
  NM_CUDA(cudaEventRecord(ev, preview->render_stream ? preview->render_stream : preview->stream));
  NM_CUDA(cudaStreamWaitEvent(s, ev, 0));
  NM_CUDA(cudaEventRecord(ev, m->stream));
  NM_CUDA(cudaStreamWaitEvent(s, ev, 0));
  NM_CUDA(m->lohi.reserve(2));
  NM_CUDA(m->x.reserve((size_t)ntiles * nmg::kIn));
  NM_CUDA(m->y.reserve((size_t)ntiles));
  NM_CUDA(h->d_tile_order.reserve((size_t)ntiles));
  const unsigned int init[2] = {0x7f7fffffu, 0u};
  NM_CUDA(cudaMemcpyAsync(m->lohi.p, init, 8, cudaMemcpyHostToDevice, s));
  const long long n = (long long)pr * pc;
  const int N = preview->effective_N();
  nmg::note_launches(2);
  nmg::preview_range_kernel<<<256, 256, 0, s>>>(preview->grid.p, n, N, m->lohi.p);
  nmg::tile_features_kernel<<<(int)((ntiles + 127) / 128), 128, 0, s>>>(
      preview->grid.p, pr, pc, N, tw, th, tx, (int)ntiles, m->lohi.p, m->x.p);
  NM_CUDA(cudaGetLastError());
  if (int rc = launch_mlp<false>(m, (int)ntiles, m->y.p, s)) return rc;
  int p2 = 2;
  while (p2 < ntiles) p2 <<= 1;
  const size_t smem = (size_t)p2 * sizeof(unsigned long long);
  NM_CUDA(cudaFuncSetAttribute(nmg::order_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  nmg::note_launches(1);
  nmg::order_sort_kernel<<<1, nmg::kSortThreads, smem, s>>>(m->y.p, (int)ntiles, p2,
                                                              h->d_tile_order.p);
  NM_CUDA(cudaGetLastError());
  // the model's next calls (which reuse x and y) wait for the sort
  NM_CUDA(cudaEventRecord(ev, s));
  NM_CUDA(cudaStreamWaitEvent(m->stream, ev, 0));
  h->tile_order.clear();
  h->tile_order_on_device = true;
  h->tile_order_n = ntiles;
  h->tile_order_w = h->tile_w;
  h->tile_order_h = h->tile_h;
  h->tile_order_uploaded = true;
  h->generation++;
  return NM_OK;
}

}  // extern "C"
