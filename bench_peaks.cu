// Pipe-throughput probes for bench.py: the FP32 and FP64 issue ceilings that
// the per-sample kernels are measured against (the roofline denominators).
// Not part of the library; bench.py builds it into _bench_build/ and loads it
// with ctypes.
//
// Each thread runs 8 independent dependency chains of one instruction kind,
// on every SM, long enough (~100 ms) that launch overhead is negligible.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;

__global__ void fma32_kernel(float* out, int iters, float a, float b) {
  float x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) x[k] = threadIdx.x * 1e-7f + k;
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = __fmaf_rn(x[k], a, b);
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += x[k];
  if (s == 12345.678f) out[0] = s;  // keeps the chains alive
}

__global__ void fma64_kernel(double* out, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) x[k] = threadIdx.x * 1e-7 + k;
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = __fma_rn(x[k], a, b);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += x[k];
  if (s == 12345.678) out[0] = s;
}

// Alternating unfused multiplies and adds: the instruction mix of the
// reference-order FP64 kernels, one flop per instruction.
__global__ void muladd64_kernel(double* out, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) x[k] = threadIdx.x * 1e-7 + k;
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = __dadd_rn(__dmul_rn(x[k], a), b);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += x[k];
  if (s == 12345.678) out[0] = s;
}

}  // namespace

// kind 0: FP32 FMA, 1: FP64 FMA, 2: FP64 unfused multiply + add; flop/s into
// *flops_per_s.  0 on success, 1 for bad arguments, 2 for a CUDA error.
extern "C" int bench_peak_flops(int kind, double* flops_per_s) {
  if (!flops_per_s || kind < 0 || kind > 2) return 1;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 2;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  void* buf = nullptr;
  if (cudaMalloc(&buf, 64) != cudaSuccess) return 2;
  const int threads = 256, blocks = sms * 8;
  const int iters = kind == 0 ? 1 << 19 : 1 << 13;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_ms = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(e0);
    if (kind == 0)
      fma32_kernel<<<blocks, threads>>>((float*)buf, iters, 0.999999f, 1e-6f);
    else if (kind == 1)
      fma64_kernel<<<blocks, threads>>>((double*)buf, iters, 0.999999, 1e-6);
    else
      muladd64_kernel<<<blocks, threads>>>((double*)buf, iters, 0.999999, 1e-6);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best_ms) best_ms = ms;  // first launch is a warm-up
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  if (err != cudaSuccess) return 2;
  const double insts = (double)blocks * threads * iters * kChains;
  const double flops = insts * 2.0;  // one FMA, or one multiply plus one add
  *flops_per_s = flops / (best_ms * 1e-3);
  return 0;
}
