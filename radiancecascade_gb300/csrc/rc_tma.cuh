// rc_tma.cuh -- TMA bulk-tensor copies and mbarrier waits (sm_103a inline PTX).
#pragma once

#include <cuda.h>  // CUtensorMap (type only; the driver is reached through the runtime)
#include <stdint.h>

namespace rcx {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes the barrier initialisation visible to the asynchronous (TMA) proxy.
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization may start while the kernel before it in the stream still
// runs; grid_dep_wait() returns once that kernel has completed and its
// writes are visible (at once when the launch was ordinary).
// grid_dep_release() lets the next such kernel start; a kernel calls it only
// after its own wait, so a kernel that starts early still finds every kernel
// before its predecessor complete.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
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

// try_wait that lets the hardware suspend the thread until the phase
// completes or `ns` nanoseconds pass, instead of spinning.
__device__ __forceinline__ bool mbar_try_wait_suspend(uint64_t* bar, uint32_t parity, uint32_t ns) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
      : "memory");
  return done != 0;
}

// Waits for the barrier phase with a time limit (about one second of SM
// clocks); returns false when the limit ran out.  The thread is suspended
// between checks (up to 20 us each), so waiting warps take no issue slots.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long start = clock64();
  while (clock64() - start < 2000000000ll)
    if (mbar_try_wait_suspend(bar, parity, 20000u)) return true;
  return false;
}

// 3-D tiled TMA load of the tensor map's box at (x, y, z) into shared memory,
// completing on `bar` (x must start on a 16-byte boundary: always 0 here).
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// 4-D tiled TMA load of the box at (x, y, z, w) (x on a 16-byte boundary).
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int x, int y, int z, int w,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
      : "memory");
}

// A box of child-averaged radiance ([dir][probe][4] texels) at row y and
// plane z (= direction * planes + plane) of the map: for FP32 a 4-D map
// (channel, x, y, z), for FP16 a 3-D map of 8-byte texels (x, y, z).  The
// box always starts at channel 0 and x = 0.
template <typename T>
__device__ __forceinline__ void tma_load_rgb4(void* dst, const CUtensorMap* map, int y, int z, uint64_t* bar) {
  if (sizeof(T) == 4) tma_load_4d(dst, map, 0, 0, y, z, bar);
  else tma_load_3d(dst, map, 0, y, z, bar);
}

}  // namespace rcx
