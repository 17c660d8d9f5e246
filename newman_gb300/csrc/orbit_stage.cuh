// The leading entries of the reference orbit in shared memory, copied there
// by the TMA unit.
//
// Every sample that rebases (Zhuoran: |Y| < |delta| or the orbit used up)
// restarts at orbit index 0 and walks up from there, so the orbit's first
// entries are read by every block over and over, beside the FP64 side's own
// loads and spills in the same L1.  A launch with v.z_stage = n > 0 copies
// zf[0, n) and z[0, n) (16 bytes an entry each) into the start of its dynamic
// shared memory once per block, with two bulk asynchronous copies
// (cp.async.bulk, non-tensor, no multicast) completing on one mbarrier, and
// the orbit loads (orbit_zf / orbit_z, view_device.cuh) read entries below n
// from there.  The block's dynamic shared memory must be at least 32 n bytes.
//
// Alignment: the copies start at the orbit arrays' bases (cudaMalloc, 256-byte
// aligned) and at the 16-byte aligned dynamic shared memory, and move 16 n
// bytes each.  The wait on the mbarrier is bounded; a block whose copies have
// not arrived by then copies the entries itself with plain loads (the same
// bytes as the bulk copies, which may still land on top) and counts a
// timeout.
#pragma once

#include <cstdint>

#include "view_device.cuh"

namespace nmg {

constexpr unsigned kStageWaitTries = 1u << 16;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Every thread of the block calls it, before any orbit load.
__device__ __forceinline__ void stage_orbit_prefix(const DeviceView& v,
                                                   unsigned long long* timeouts) {
  const int n = v.z_stage;
  if (n <= 0) return;
  __shared__ __align__(8) uint64_t bar;
  Flt4* zf_s = reinterpret_cast<Flt4*>(nm_orbit_smem);
  Dbl2* z_s = reinterpret_cast<Dbl2*>(nm_orbit_smem + 16 * n);
  const uint32_t bar_a = smem_u32(&bar);
  const uint32_t bytes = 16u * (uint32_t)n;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a),
                 "r"(2u * bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(zf_s)),
        "l"(v.zf), "r"(bytes), "r"(bar_a)
        : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(z_s)),
        "l"(v.z), "r"(bytes), "r"(bar_a)
        : "memory");
  }
  uint32_t done = 0;
  for (unsigned t = 0; t < kStageWaitTries && !done; t++) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar_a)
        : "memory");
  }
  if (!done) {
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      zf_s[k] = v.zf[k];
      z_s[k] = v.z[k];
    }
    if (timeouts) atomicAdd(timeouts, 1ull);
  }
  __syncthreads();
}

}  // namespace nmg
