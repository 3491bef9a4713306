// rc_check.cuh -- the checked build (compiled with -DRC_CHECKED, library
// librc_checked.so): the kernels' global and shared accesses are tested
// before they are made.
//
// A global access must lie inside one of the device ranges the host has
// registered (every allocation of dev_alloc, the static scratch of the
// allocation-free solve and the caller buffers an entry point borrows); a
// shared access inside the block's shared memory.  A failed test skips the
// access (a load gives 0), counts the failure and keeps the first one's site
// and address in a device status word; nothing traps.  rc_check_status()
// reads and clears the words.  In the ordinary build RC_CHK(p, site) is the
// constant true and compiles away.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "rc_internal.h"

namespace rcx {

// Sites named in rc_check_status's message (rc_host.cpp: check_site_name).
enum CheckSite : int {
  kChkRadiance = 1,  // merged / child-averaged radiance (Store<T>, load_up)
  kChkVolume = 2,    // composed or base voxel volume
  kChkOccupancy = 3, // opacity / emissive bit planes
  kChkMask = 4,      // decimated opacity of a level
  kChkRecord = 5,    // walk records
  kChkTable = 6,     // walk step tables and direction tables
  kChkFluence = 7,   // cascade-0 fluence
  kChkShared = 8,    // shared memory (staged tiles, hit rows)
  kChkHash = 9,      // radiance-cache hash table and hash parts
  kChkCache = 10,    // radiance-cache (R, T), targets, predictions, tile sums
  kChkSpheres = 11,  // emitter regions and sphere lists
};

#ifdef RC_CHECKED
constexpr int kCheckRanges = 1024;
static __device__ CheckRange g_check_range[kCheckRanges];
static __device__ int g_check_n;
static __device__ unsigned long long g_check_first;  // site << 56 | low 56 address bits
static __device__ unsigned int g_check_count;

static __device__ __noinline__ bool check_failed(int site, const void* p) {
  const unsigned long long w = ((unsigned long long)site << 56) | ((unsigned long long)p & ((1ull << 56) - 1));
  atomicCAS(&g_check_first, 0ull, w);
  atomicAdd(&g_check_count, 1u);
  return false;
}

static __device__ __forceinline__ bool check_ptr(const void* p, int bytes, int site) {
  if (__isShared(p)) {
    const uint32_t off = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t total;
    asm("mov.u32 %0, %%total_smem_size;" : "=r"(total));
    // the shared window may start with the system's reserved kilobyte
    if ((uint64_t)off + (uint64_t)bytes <= (uint64_t)total + 1024u) return true;
    return check_failed(site, p);
  }
  if (__isGlobal(p)) {
    const uint64_t a = (uint64_t)p;
    const int n = *(volatile int*)&g_check_n;
    for (int i = 0; i < n; ++i)
      if (a >= g_check_range[i].lo && a + (uint64_t)bytes <= g_check_range[i].hi) return true;
    return check_failed(site, p);
  }
  return true;  // parameter, constant and local space: not a buffer of the library
}

#define RC_CHK(p, site) ::rcx::check_ptr((const void*)(p), (int)sizeof(*(p)), (site))

// Host side of this translation unit's words: upload the registered ranges
// when they changed since the last upload, read (and clear) the status.
static uint64_t g_check_synced[64] = {};  // per device: the version uploaded + 1
static inline cudaError_t check_prepare() {
  int dev = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 != cudaSuccess) return e0;
  uint64_t version = 0;
  const std::vector<CheckRange> r = check_ranges(&version);
  uint64_t& synced = g_check_synced[dev & 63];
  if (synced == version + 1) return cudaSuccess;
  const int n = (int)std::min<size_t>(r.size(), (size_t)kCheckRanges);
  cudaError_t e = cudaSuccess;
  if (n) e = cudaMemcpyToSymbol(g_check_range, r.data() + (r.size() - (size_t)n), n * sizeof(CheckRange));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_check_n, &n, sizeof n);
  if (e == cudaSuccess) synced = version + 1;
  return e;
}
static inline cudaError_t check_read(unsigned long long* first, unsigned* count) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(first, g_check_first, sizeof *first);
  if (e == cudaSuccess) e = cudaMemcpyFromSymbol(count, g_check_count, sizeof *count);
  const unsigned long long z = 0;
  const unsigned zc = 0;
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_check_first, &z, sizeof z);
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_check_count, &zc, sizeof zc);
  return e;
}
#else
#define RC_CHK(p, site) true
static inline cudaError_t check_prepare() { return cudaSuccess; }
#endif

}  // namespace rcx
