// Tensor-memory-accelerator (TMA) staging of a sweep tile: one elected thread
// issues a 3D bulk tensor copy of the tile's conservative state (all variable
// planes, halos included) into shared memory, completing on an mbarrier.
//
// Every wait is bounded in wall time (the %globaltimer nanosecond clock, with
// an iteration cap besides): a copy that does not land within 2 ms sets bit 1
// of the grid clock's status, and the CTA stops after waiting up to 50 ms more
// for the copy it issued.  A copy that has still not landed then may write into
// shared memory that a later CTA is given, so a status with bit 1 set is fatal
// for the grid: the host stops stepping it.
#pragma once
#include <cuda.h>

#include "fv_common.cuh"

namespace astrea {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// p moved up to the next 128-byte boundary of the shared window, by pointer arithmetic on p
// (which keeps the pointer known to the compiler as shared, so its accesses stay shared loads)
template <typename T> __device__ __forceinline__ T* align128_shared(T* p) {
  const unsigned mis = smem_u32(p) & 127u;
  return p + (mis ? (128u - mis) / sizeof(T) : 0u);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make the initialised barrier visible to the asynchronous (TMA) proxy
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// the same test, letting the thread sleep up to ``hint_ns`` nanoseconds for the phase to complete
__device__ __forceinline__ bool mbar_try_wait_sleep(unsigned long long* bar, unsigned parity, unsigned hint_ns) {
  unsigned done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return done != 0;
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// wait for phase ``parity`` of the barrier for at most ``limit_ns`` nanoseconds of wall
// time (and at most 2^22 polls, each sleeping at most 20 us); false if the limit ran out.
// The polling thread sleeps in the barrier test instead of spinning, which leaves the
// issue slots to the other warps on the SM.
constexpr unsigned long long kCopyWaitNs = 2000000ull;      // a tile's bulk copy: 2 ms (it takes microseconds)
constexpr unsigned long long kDrainWaitNs = 50000000ull;    // after a timeout, for the copy in flight: 50 ms
constexpr unsigned kPollSleepNs = 20000u;
__device__ __forceinline__ bool mbar_wait_timed(unsigned long long* bar, unsigned parity,
                                                unsigned long long limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = globaltimer_ns();
  for (int i = 0; i < (1 << 22); ++i) {
    if (mbar_try_wait_sleep(bar, parity, kPollSleepNs)) return true;
    if (globaltimer_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// 3D tiled bulk copy global -> shared (box origin x innermost); x * element size must be a multiple of 16
// ask the L2 for the 128-byte line holding p (a hint: no data returns to the thread)
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// floor / ceil of x to a multiple of a (a > 0), valid for negative x
constexpr int floor_to(int x, int a) { return x >= 0 ? (x / a) * a : -((-x + a - 1) / a) * a; }
constexpr int ceil_to(int x, int a) { return ((x + a - 1) / a) * a; }

}  // namespace astrea
