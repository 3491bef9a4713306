// rc_batch.cuh -- many scenes of uneven size in one persistent launch (sm_103a).
//
// Every (scene, cascade level, tile) is an item of one work queue.  Items are
// queued top level first across all scenes (depth 0 = every scene's top level,
// depth 1 = the level below, ...), and a block takes the next item with one
// atomic.  An item of level i needs the whole of level i + 1 of its scene: it
// waits on that level's completion counter.  Those items sit earlier in the
// queue, so they were taken by blocks that are already running and can
// always finish -- the launch makes progress whatever the residency.  The
// wait is bounded: on timeout the block sets *err and every block stops.
//
// An item runs the same block routines as the single-scene kernels:
//   kBatchBits    `upi` blocks of the bit-parallel wide-level kernel;
//   kBatchDirect0 `upi` blocks (8 warps each) of the walk-free cascade 0;
//   kBatchWalk    `wpi` walk-queue tasks of one scene's narrow levels (lanes
//                 refill from a block-local counter).  Walks depend only on
//                 the scene, so these items come first and never wait;
//   kBatchMerge   a tile of `ppi` probes x `qpi` parent-texel pairs of a
//                 narrow level, merged from the walk records (waits for the
//                 level above and for its scene's walks);
//   kBatchScalar  a tile of `ppi` probes x `qpi` parent texels with the
//                 scalar walk (levels without a decimated mask).
// The tile shape (ppi, qpi, upi, wpi) is autotuned.  Radiance of the level
// above and the walk records are written during the launch, so every block
// routine reads them with weak loads after the acquire (never through the
// read-only path).
#pragma once

#include "rc_kernels.cuh"
#include "rc_level0.cuh"
#include "rc_walk_bits.cuh"
#include "rc_walk_queue.cuh"

namespace rcx {

enum { kBatchScalar = 0, kBatchBits = 1, kBatchDirect0 = 2, kBatchWalk = 3, kBatchMerge = 4 };

struct BatchLevel {
  LevelArgs a;
  const QueueArgs* q;    // walk: the scene's narrow-level walk queue
  const uint32_t* rec;   // merge: this level's walk records
  int32_t slots;         // merge: record slots per direction
  int32_t up;            // index of the level above in the table, -1 at the top
  int32_t dep2;          // merge: index of the scene's walk entry, else -1
  int32_t ntiles;        // items of this entry
  int32_t ptiles;        // scalar / merge: probe tiles (items = ptiles * texel tiles)
  int32_t units;         // bits / direct0: blocks of the single-scene kernel
  int32_t mode;          // kBatch*
  int32_t is_l0;
  int32_t is_top;
  int32_t pad;
};

struct BatchItem {
  int32_t level;  // index into the level table
  int32_t tile;
};

struct BatchTiles {
  int32_t ppi, qpi, upi, wpi;
};

constexpr int kBatchWalkSteps = 2;  // walk steps per lane between refills (register budget)
constexpr int kBatchThreads = kBitsThreads;  // 8 warps, as the block routines expect
static_assert(kBatchThreads == kL0Threads, "cascade-0 blocks are 8 warps");

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Flattened (probe, parent texel group) units of a scalar / merge tile.
struct TileUnits {
  int64_t p0;
  int np, g0, ng;
};

__device__ __forceinline__ TileUnits tile_units(const BatchLevel& lv, int tile, int ppi, int qpi, int ngroups) {
  TileUnits u;
  const int pt = tile % lv.ptiles, qt = tile / lv.ptiles;
  u.p0 = (int64_t)pt * ppi;
  u.np = (int)min((int64_t)ppi, lv.a.P - u.p0);
  u.g0 = qt * qpi;
  u.ng = min(qpi, ngroups - u.g0);
  return u;
}

// One function per item kind (not inlined), so that each gets its own
// register allocation.
template <typename T, bool L0, bool TOP>
__device__ __noinline__ void bits_item(const LevelArgs& a, int b0, int b1, uint32_t* s_hit) {
  for (int bid = b0; bid < b1; ++bid) level_bits_block<T, L0, TOP, true>(a, bid, s_hit);
}

template <typename T, bool TOP>
__device__ __noinline__ void direct0_item(const LevelArgs& a, int b0, int b1) {
  const int warp = threadIdx.x >> 5;
  for (int blk = b0; blk < b1; ++blk) level0_direct_warp<T, TOP, true>(a, (int64_t)blk * 8 + warp);
}

template <typename T, bool L0, bool TOP>
__device__ __noinline__ void merge_item(const LevelArgs& a, const uint32_t* rec, int slots, TileUnits u) {
  for (int j = threadIdx.x; j < u.np * u.ng; j += blockDim.x)
    merge_probe<T, L0, TOP, true>(a, rec, slots, u.p0 + j % u.np, u.g0 + j / u.np);
}

template <typename T, bool L0, bool TOP>
__device__ __noinline__ void scalar_item(const LevelArgs& a, TileUnits u) {
  for (int j = threadIdx.x; j < u.np * u.ng; j += blockDim.x)
    scalar_probe<T, L0, TOP, true>(a, u.p0 + j % u.np, u.g0 + j / u.np, 1);
}

template <typename T, bool L0, bool TOP>
__device__ __forceinline__ void batch_item(const BatchLevel& lv, int tile, const BatchTiles& ts, uint32_t* s_hit) {
  const LevelArgs& a = lv.a;
  const int hn = a.n >> 1;
  if (lv.mode == kBatchBits) {
    bits_item<T, L0, TOP>(a, tile * ts.upi, min((tile + 1) * ts.upi, lv.units), s_hit);
  } else if (L0 && lv.mode == kBatchDirect0) {
    direct0_item<T, TOP>(a, tile * ts.upi, min((tile + 1) * ts.upi, lv.units));
  } else if (lv.mode == kBatchMerge) {
    merge_item<T, L0, TOP>(a, lv.rec, lv.slots, tile_units(lv, tile, ts.ppi, ts.qpi, L0 ? 1 : hn * hn / 2));
  } else {
    scalar_item<T, L0, TOP>(a, tile_units(lv, tile, ts.ppi, ts.qpi, L0 ? 1 : hn * hn));
  }
}

// A scene's walks replay its step tables when it has them (every level of a
// scene has them or none does), else run their own DDA.  Separate functions,
// so that each walker gets its own register allocation.
__device__ __noinline__ void batch_walk_tables(const QueueArgs& q, unsigned long long* counter, int64_t end) {
  walk_groups<kBatchWalkSteps, TableWalker>(q, counter, end);
}
__device__ __noinline__ void batch_walk_dda(const QueueArgs& q, unsigned long long* counter, int64_t end) {
  walk_groups<kBatchWalkSteps, Walker>(q, counter, end);
}
__device__ __forceinline__ void batch_walk(const QueueArgs& q, unsigned long long* counter, int64_t end) {
  if (q.lv[0].steps)
    batch_walk_tables(q, counter, end);
  else
    batch_walk_dda(q, counter, end);
}

// Bounded wait (about one second of SM clocks) until entry `e` has finished
// all its items; false on timeout or when another block gave up.
__device__ __forceinline__ bool wait_entry(const BatchLevel* levels, const unsigned* done, int e, int* err) {
  const unsigned need = (unsigned)levels[e].ntiles;
  const long long start = clock64();
  while (ld_acquire(&done[e]) < need) {
    if (*(volatile int*)err || clock64() - start > 2000000000ll) {
      atomicExch(err, 1);
      return false;
    }
    __nanosleep(256);
  }
  return true;
}

template <typename T>
__global__ void __launch_bounds__(kBatchThreads, 3)
    k_batch_persistent(const BatchLevel* __restrict__ levels, const BatchItem* __restrict__ items, int nitems,
                       const BatchTiles ts, unsigned* next, unsigned* done, int* err) {
  extern __shared__ uint32_t s_hit[];
  __shared__ int s_item, s_stop;
  __shared__ unsigned long long s_walk;
  for (;;) {
    if (threadIdx.x == 0) {
      s_item = (*(volatile int*)err) ? nitems : (int)atomicAdd(next, 1u);
      s_stop = 0;
    }
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const BatchItem bi = items[it];
    const BatchLevel& lv = levels[bi.level];
    if (threadIdx.x == 0) {
      if ((lv.up >= 0 && !wait_entry(levels, done, lv.up, err)) ||
          (lv.dep2 >= 0 && !wait_entry(levels, done, lv.dep2, err)))
        s_stop = 1;
      if (lv.mode == kBatchWalk) s_walk = (unsigned long long)bi.tile * ts.wpi;
    }
    __syncthreads();
    if (s_stop) break;
    if (lv.mode == kBatchWalk) {
      batch_walk(*lv.q, &s_walk, min((int64_t)(bi.tile + 1) * ts.wpi, lv.q->total));
    } else if (lv.is_l0) {
      if (lv.is_top) batch_item<T, true, true>(lv, bi.tile, ts, s_hit);
      else batch_item<T, true, false>(lv, bi.tile, ts, s_hit);
    } else {
      if (lv.is_top) batch_item<T, false, true>(lv, bi.tile, ts, s_hit);
      else batch_item<T, false, false>(lv, bi.tile, ts, s_hit);
    }
    // Cascade 0 feeds no other item: its stores drain while the block goes
    // on.  Otherwise this block's outputs are visible before the item counts.
    const bool feeds = !lv.is_l0;
    if (feeds) __threadfence();
    __syncthreads();
    if (feeds && threadIdx.x == 0) atomicAdd(&done[bi.level], 1u);
  }
}

}  // namespace rcx
