// FP64 per-sample kernels: the reference's double path (getIterationsHW), the
// plain FP64 perturbation path (getIterations' series front plus an FP64
// delta continuation), and the multisample reduce / duplicate of the grid.
//
// Built with --fmad=false; the reference-order arithmetic also uses
// round-to-nearest intrinsics, so no multiply-add is ever contracted.
#include "engine.hpp"
#include "jobs_fp64.cuh"
#include "persistent.cuh"

#include <atomic>

namespace nmg {

__global__ void __launch_bounds__(kPersistentThreads) hw_kernel(DeviceView v, RenderCtl ctl,
                                                                  int chunk) {
  __shared__ SamplePool<HwJob::State> pool;
  pool_init(&pool);
  persistent_loop<HwJob>(v, ctl, chunk, &pool);
}

__global__ void __launch_bounds__(kPersistentThreads) delta64_kernel(DeviceView v, RenderCtl ctl,
                                                                       int chunk) {
  __shared__ SamplePool<Delta64Job::State> pool;
  pool_init(&pool);
  persistent_loop<Delta64Job>(v, ctl, chunk, &pool);
}

__global__ void __launch_bounds__(kPersistentThreads) rework_kernel(DeviceView v, RenderCtl ctl,
                                                                      int chunk) {
  __shared__ SamplePool<Fp64AnyJob::State> pool;
  pool_init(&pool);
  persistent_loop<Fp64AnyJob>(v, ctl, chunk, &pool);
}

cudaError_t launch_fe32(const DeviceView& v, const RenderCtl& ctl, cudaStream_t stream,
                        int blocks, int chunk);
int fe32_blocks_per_sm();

int kernel_threads(KernelKind) { return kPersistentThreads; }

namespace {
std::atomic<long long> g_launches{0};
}
void note_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

int persistent_blocks(KernelKind kind, int device) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  int per_sm = 0;
  if (kind == KERNEL_HW)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hw_kernel, kPersistentThreads, 0);
  else if (kind == KERNEL_DELTA64)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, delta64_kernel, kPersistentThreads, 0);
  else if (kind == KERNEL_REWORK)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rework_kernel, kPersistentThreads, 0);
  else
    per_sm = fe32_blocks_per_sm();
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

cudaError_t launch_render(KernelKind kind, const DeviceView& v, const RenderCtl& ctl,
                          cudaStream_t stream, int blocks, int chunk) {
  if (kind == KERNEL_FE32) return launch_fe32(v, ctl, stream, blocks, chunk);
  if (kind == KERNEL_MP || kind == KERNEL_HW_MP) return launch_mp(kind, v, ctl, stream, blocks, chunk);
  note_launches(1);
  if (kind == KERNEL_HW)
    hw_kernel<<<blocks, kPersistentThreads, 0, stream>>>(v, ctl, chunk);
  else if (kind == KERNEL_DELTA64)
    delta64_kernel<<<blocks, kPersistentThreads, 0, stream>>>(v, ctl, chunk);
  else
    rework_kernel<<<blocks, kPersistentThreads, 0, stream>>>(v, ctl, chunk);
  return cudaGetLastError();
}

// mandelbrot.cpp:320-332, one thread per output pixel, float arithmetic in
// the reference's order: sum += iterations + smoothing; sum /= sc*sc.
__global__ void reduce_kernel(const EscapeValue* __restrict__ in, int nr, int nc, int sc,
                              EscapeValue* __restrict__ out) {
  const long long n = (long long)nr * nc;
  const long long NC = (long long)nc * sc;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(k / nc), c = (int)(k - (long long)r * nc);
    float sum = 0.0f;
    for (int r1 = 0; r1 < sc; r1++) {
      const EscapeValue* row = in + (long long)(sc * r + r1) * NC + (long long)sc * c;
      for (int c1 = 0; c1 < sc; c1++) {
        const EscapeValue e = row[c1];
        sum = __fadd_rn(sum, __fadd_rn((float)e.iterations, e.smoothing));
      }
    }
    sum = __fdiv_rn(sum, (float)(sc * sc));
    const int it = (int)sum;
    out[k] = EscapeValue{it, __fsub_rn(sum, (float)it)};
  }
}

__global__ void duplicate_kernel(const EscapeValue* __restrict__ in, int nr, int nc, int sc,
                                 EscapeValue* __restrict__ out) {
  const long long NC = (long long)nc * sc;
  const long long n = (long long)nr * sc * NC;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const long long r = k / NC, c = k - r * NC;
    out[k] = in[(r / sc) * nc + c / sc];
  }
}

static int grid_for(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

cudaError_t launch_reduce(const EscapeValue* in, int nr, int nc, int sc, EscapeValue* out,
                          cudaStream_t stream) {
  note_launches(1);
  reduce_kernel<<<grid_for((long long)nr * nc), 256, 0, stream>>>(in, nr, nc, sc, out);
  return cudaGetLastError();
}

cudaError_t launch_duplicate(const EscapeValue* in, int nr, int nc, int sc, EscapeValue* out,
                             cudaStream_t stream) {
  note_launches(1);
  duplicate_kernel<<<grid_for((long long)nr * nc * sc * sc), 256, 0, stream>>>(in, nr, nc, sc,
                                                                                 out);
  return cudaGetLastError();
}

}  // namespace nmg
