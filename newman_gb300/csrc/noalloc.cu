// A render entry point that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they render: code
// that records its GPU work into a CUDA graph by stream capture, or a process
// whose device memory belongs to another framework's allocator or to a fixed
// budget.  nm_render_fe32_noalloc renders a handle's view on the FP32
// floatexp path into memory the caller owns, and takes the scratch memory the
// kernels need -- the two work counters, the statistics and the list of
// samples the FP64 kernel re-renders -- from one file-scope device array
// instead of cudaMalloc.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "engine.hpp"
#include "newman_gb300.h"

namespace nmg {
// Reads the device tables of a handle that nm_precompute and nm_upload have
// prepared, without allocating (capi.cpp).  `kind`: KERNEL_FE32, or KERNEL_HW
// for a double-loop view that the FE32 path renders with the double loop.
int noalloc_view(nm_handle* h, DeviceView& v, int& device, std::string& why, KernelKind& kind);
void noalloc_fail(const std::string& why);
}  // namespace nmg

namespace {

constexpr int kWords = 32;  // work counters and statistics (19 used)
constexpr int kNext = 0, kStats = 1, kNextRework = 1 + nmg::STAT_COUNT,
              kStatsRework = kNextRework + 1, kReworkCount = kStatsRework + nmg::STAT_COUNT;
static_assert(kReworkCount < kWords, "scratch words");

struct NoAllocScratch {
  unsigned long long words[kWords];
  unsigned int rework[NM_NOALLOC_MAX_SAMPLES];
};

// One copy per GPU that loads the library, held until the process exits.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_mu;
NoAllocScratch* g_addr[kMaxDevices] = {};

// Device address of the array on `device` (current).  In host code the
// array's name is only a host-side stand-in, so the address is looked up
// once per device and cached.
cudaError_t scratch_on(int device, NoAllocScratch** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = static_cast<NoAllocScratch*>(p);
  }
  *out = g_addr[device];
  return cudaSuccess;
}

}  // namespace

extern "C" int nm_render_fe32_noalloc(nm_handle* h, nm_escape_value* out, void* stream_arg) {
  if (!h || !out) {
    nmg::noalloc_fail("nm_render_fe32_noalloc: null handle or output");
    return NM_ERR_ARG;
  }
  const long long samples = (long long)nm_rows(h) * nm_cols(h);
  if (samples > NM_NOALLOC_MAX_SAMPLES) {
    nmg::noalloc_fail("nm_render_fe32_noalloc: " + std::to_string(samples) +
                      " samples exceed the no-allocation maximum of " +
                      std::to_string(NM_NOALLOC_MAX_SAMPLES));
    return NM_ERR_ARG;
  }
  nmg::DeviceView v;
  int device = 0;
  std::string why;
  nmg::KernelKind kind = nmg::KERNEL_FE32;
  if (int rc = nmg::noalloc_view(h, v, device, why, kind)) {
    nmg::noalloc_fail("nm_render_fe32_noalloc: " + why);
    return rc;
  }
  // The handle's tables, the scratch address looked up below and the kernels
  // all belong to the handle's device, which must be the current one.
  int current = -1;
  if (cudaGetDevice(&current) != cudaSuccess || current != device) {
    nmg::noalloc_fail("nm_render_fe32_noalloc: the handle belongs to device " +
                      std::to_string(device) + " but device " + std::to_string(current) +
                      " is current");
    return NM_ERR_STATE;
  }
  v.grid = reinterpret_cast<nmg::EscapeValue*>(out);
  v.smooth64 = nullptr;
  NoAllocScratch* s = nullptr;
  cudaError_t e = scratch_on(device, &s);
  cudaStream_t st = static_cast<cudaStream_t>(stream_arg);
  // Every call starts from zeroed counters; the rework list needs no clearing.
  if (e == cudaSuccess) e = cudaMemsetAsync(s->words, 0, sizeof s->words, st);
  nmg::RenderCtl ctl{};
  ctl.next = s ? s->words + kNext : nullptr;
  ctl.stats = s ? s->words + kStats : nullptr;
  ctl.first = 0;
  ctl.count = v.total;
  ctl.rework = s ? s->rework : nullptr;
  ctl.rework_n = s ? s->words + kReworkCount : nullptr;
  if (e == cudaSuccess && kind == nmg::KERNEL_HW) {
    e = nmg::launch_render(nmg::KERNEL_HW, v, ctl, st,
                           nmg::persistent_blocks(nmg::KERNEL_HW, device), 32);
  } else if (e == cudaSuccess) {
    e = nmg::launch_render(nmg::KERNEL_FE32, v, ctl, st,
                           nmg::persistent_blocks(nmg::KERNEL_FE32, device), 16);
  }
  if (e == cudaSuccess && kind == nmg::KERNEL_FE32) {
    nmg::RenderCtl re{};
    re.next = s->words + kNextRework;
    re.stats = s->words + kStatsRework;
    re.list = s->rework;
    re.count_ptr = s->words + kReworkCount;
    e = nmg::launch_render(nmg::KERNEL_REWORK, v, re, st,
                           nmg::persistent_blocks(nmg::KERNEL_REWORK, device), 32);
  }
  if (e != cudaSuccess) {
    nmg::noalloc_fail(std::string("nm_render_fe32_noalloc: ") + cudaGetErrorString(e));
    return NM_ERR_CUDA;
  }
  return NM_OK;
}
