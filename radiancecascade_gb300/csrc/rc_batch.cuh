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
// An item is a tile of `ppi` probes x `qpi` parent texels (their 4 child
// directions each; level 0: every direction and the fluence), solved with the
// exact scalar walk.  ppi and qpi are the autotuned tile shape.
#pragma once

#include "rc_kernels.cuh"

namespace rcx {

struct BatchLevel {
  LevelArgs a;
  int32_t up;       // index of the level above in the table, -1 at the top
  int32_t ntiles;   // items of this level
  int32_t ptiles;   // probe tiles (items = ptiles * qtiles)
  int32_t is_l0;
  int32_t is_top;
  int32_t pad[3];
};

struct BatchItem {
  int32_t level;  // index into the level table
  int32_t tile;
};

constexpr int kBatchThreads = 128;

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// The next level's child-averaged radiance is written during this launch:
// read it around L1 (coherent at L2).
template <typename T>
__device__ __forceinline__ float load_cg(const T* p);
template <>
__device__ __forceinline__ float load_cg<float>(const float* p) {
  return __ldcg(p);
}
template <>
__device__ __forceinline__ float load_cg<__half>(const __half* p) {
  return __half2float(__ushort_as_half(__ldcg(reinterpret_cast<const unsigned short*>(p))));
}

// One probe of one item: the scalar walk and merge of k_level_scalar.
template <typename T>
__device__ __forceinline__ void batch_probe(const LevelArgs& a, bool L0, bool TOP, int64_t p, int dp0, int ndp) {
  const int mx = (int)(p % a.M[0]);
  const int my = (int)((p / a.M[0]) % a.M[1]);
  const int mz = (int)(p / ((int64_t)a.M[0] * a.M[1]));
  const int h = a.spacing >> 1;
  const int ox = mx * a.spacing + h, oy = my * a.spacing + h, oz = mz * a.spacing + h;
  int64_t tap_off[8];
  float tap_w[8];
  if (!TOP) {
    int q[3][2];
    float w[3][2];
    const int m[3] = {mx, my, mz};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      const int lo = (m[ax] - 1) >> 1;
      w[ax][0] = (m[ax] & 1) ? 0.75f : 0.25f;
      w[ax][1] = 1.0f - w[ax][0];
      q[ax][0] = min(max(lo, 0), a.UM[ax] - 1);
      q[ax][1] = min(max(lo + 1, 0), a.UM[ax] - 1);
    }
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int tx = t & 1, ty = (t >> 1) & 1, tz = t >> 2;
      tap_off[t] = ((int64_t)q[2][tz] * a.UM[1] + q[1][ty]) * a.UM[0] + q[0][tx];
      tap_w[t] = w[2][tz] * w[1][ty] * w[0][tx];
    }
  }
  T* L = static_cast<T*>(a.L);
  const T* Au = static_cast<const T*>(a.A_up);
  const int hn = a.n >> 1;
  const int64_t npar = (int64_t)hn * hn;
  float flu[3] = {0.f, 0.f, 0.f};
  const int nd = L0 ? a.ndirs : 4 * ndp;
  for (int c = 0; c < nd; ++c) {
    int d;
    if (L0) {
      d = c;
    } else {
      const int dp = dp0 + (c >> 2), cc = c & 3;
      d = (2 * (dp / hn) + (cc >> 1)) * a.n + 2 * (dp % hn) + (cc & 1);
    }
    const DirInfo di = a.dirs[d];
    const int64_t hit = walk_interval(a.occ, a.G, a.W, ox + di.start_off[0], oy + di.start_off[1],
                                      oz + di.start_off[2], di, L0);
    float r[3];
    if (hit >= 0) {
      voxel_emission(a.vol, hit, r);
    } else if (TOP) {
      r[0] = r[1] = r[2] = 0.f;
    } else {
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        const T* base = Au + ((int64_t)ch * a.ndirs + d) * a.P_up;
        float s = 0.f;
#pragma unroll
        for (int t = 0; t < 8; ++t) s = fmaf(tap_w[t], load_cg<T>(base + tap_off[t]), s);
        r[ch] = s;
      }
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      Store<T>::store(L + ((int64_t)ch * a.ndirs + d) * a.P + p, r[ch]);
      flu[ch] = L0 ? fmaf(di.omega, r[ch], flu[ch]) : flu[ch] + r[ch];
    }
    if (!L0 && (c & 3) == 3) {
      T* A = static_cast<T*>(a.A_out);
      const int dp = dp0 + (c >> 2);
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) {
        Store<T>::store(A + ((int64_t)ch * npar + dp) * a.P + p, 0.25f * flu[ch]);
        flu[ch] = 0.f;
      }
    }
  }
  if (L0) {
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) a.fluence[p * 3 + ch] = flu[ch];
  }
}

template <typename T>
__global__ void __launch_bounds__(kBatchThreads) k_batch_persistent(const BatchLevel* __restrict__ levels,
                                                                    const BatchItem* __restrict__ items, int nitems,
                                                                    int ppi, int qpi, unsigned* next, unsigned* done,
                                                                    int* err) {
  __shared__ int s_item, s_stop;
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
    if (lv.up >= 0 && threadIdx.x == 0) {
      // bounded wait for the whole level above (about one second of SM clocks)
      const unsigned need = (unsigned)levels[lv.up].ntiles;
      const long long start = clock64();
      while (ld_acquire(&done[lv.up]) < need) {
        if (*(volatile int*)err || clock64() - start > 2000000000ll) {
          atomicExch(err, 1);
          s_stop = 1;
          break;
        }
        __nanosleep(256);
      }
    }
    __syncthreads();
    if (s_stop) break;
    const int pt = bi.tile % lv.ptiles, qt = bi.tile / lv.ptiles;
    const int hn = lv.a.n >> 1;
    const int npar = hn * hn;
    const int dp0 = qt * qpi, ndp = min(qpi, npar - dp0);
    for (int j = threadIdx.x; j < ppi; j += blockDim.x) {
      const int64_t p = (int64_t)pt * ppi + j;
      if (p >= lv.a.P) break;
      if (lv.is_l0) {
        if (lv.is_top) batch_probe<T>(lv.a, true, true, p, 0, 0);
        else batch_probe<T>(lv.a, true, false, p, 0, 0);
      } else {
        if (lv.is_top) batch_probe<T>(lv.a, false, true, p, dp0, ndp);
        else batch_probe<T>(lv.a, false, false, p, dp0, ndp);
      }
    }
    __threadfence();  // this block's outputs are visible before the item counts as done
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&done[bi.level], 1u);
  }
}

}  // namespace rcx
