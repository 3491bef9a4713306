// rc_kernels.cuh -- device code of the radiance-cascade engine (sm_103a).
//
// Data layout in HBM (one scene):
//   vol   rc_voxel[Gz][Gy][Gx]               8 B/voxel composed scene
//   occ   uint32  [Gz][Gy][ceil(Gx/32)]      1 bit/voxel opacity, x fastest
//   L_i   T       [3][dirs_i][Mz][My][Mx]     merged radiance of level i (T = f32 | f16)
//   A_i   T       [dirs_{i-1}][Mz][My][Mx][4] L_i averaged over each 2x2 child-texel
//                                             block, RGB + a zero per (direction, probe);
//                                             read by level i-1's merge.  A_1 read by
//                                             the walk-free cascade 0 is planar instead:
//                                             [3][dirs_0][Mz][My][Mx] (a_out_planar)
//   flu   float   [Mz0][My0][Mx0][3]          cascade-0 fluence
#pragma once

#include <cuda_fp16.h>
#include <stdint.h>

#include "rc_check.cuh"
#include "rc_internal.h"

namespace rcx {

template <typename T>
struct Store;
template <>
struct Store<float> {
  static __device__ __forceinline__ float load(const float* p) { return RC_CHK(p, kChkRadiance) ? __ldg(p) : 0.f; }
  static __device__ __forceinline__ void store(float* p, float v) {
    if (RC_CHK(p, kChkRadiance)) *p = v;
  }
  // write-once outputs: evict-first, so they do not push reused data out of L2
  static __device__ __forceinline__ void stream(float* p, float v) {
    if (RC_CHK(p, kChkRadiance)) __stcs(p, v);
  }
};
template <>
struct Store<__half> {
  static __device__ __forceinline__ float load(const __half* p) {
    return RC_CHK(p, kChkRadiance) ? __half2float(__ldg(p)) : 0.f;
  }
  static __device__ __forceinline__ void store(__half* p, float v) {
    if (RC_CHK(p, kChkRadiance)) *p = __float2half_rn(v);
  }
  static __device__ __forceinline__ void stream(__half* p, float v) {
    if (RC_CHK(p, kChkRadiance)) __stcs(reinterpret_cast<unsigned short*>(p), __half_as_ushort(__float2half_rn(v)));
  }
};

// Reads of the next level's child-averaged radiance.  It is normally written
// by an earlier launch and read through the read-only (non-coherent) path.
// In the batched persistent solve (CG) it is written during the same launch:
// it is read with ordinary weak loads, after an acquire of the producer's
// completion counter, never through the read-only path.  (No line of it can
// sit in L1 before that point: nothing on the SM reads it earlier in the
// launch, and L1 starts empty of it at every launch.)
template <typename T, bool CG>
__device__ __forceinline__ float load_up(const T* p);
template <>
__device__ __forceinline__ float load_up<float, false>(const float* p) {
  return RC_CHK(p, kChkRadiance) ? __ldg(p) : 0.f;
}
template <>
__device__ __forceinline__ float load_up<float, true>(const float* p) {
  return RC_CHK(p, kChkRadiance) ? __ldca(p) : 0.f;
}
template <>
__device__ __forceinline__ float load_up<__half, false>(const __half* p) {
  return RC_CHK(p, kChkRadiance) ? __half2float(__ldg(p)) : 0.f;
}
template <>
__device__ __forceinline__ float load_up<__half, true>(const __half* p) {
  if (!RC_CHK(p, kChkRadiance)) return 0.f;
  return __half2float(__ushort_as_half(__ldca(reinterpret_cast<const unsigned short*>(p))));
}

__device__ __forceinline__ float to_float(float v) { return v; }
__device__ __forceinline__ float to_float(__half v) { return __half2float(v); }

// Child-averaged radiance A_i is stored [parent direction][probe][4]: the
// three channels of one (direction, probe) side by side and a zero, so that
// a blend tap is one 16-byte (FP32) or 8-byte (FP16) load and one TMA copy
// stages every channel.  rgb4_at(A, d, P, probe) is the tap's first value.
template <typename T>
__device__ __forceinline__ const T* rgb4_at(const T* A, int d, int64_t P, int64_t probe) {
  return A + ((int64_t)d * P + probe) * 4;
}
template <typename T>
__device__ __forceinline__ T* rgb4_at(T* A, int d, int64_t P, int64_t probe) {
  return A + ((int64_t)d * P + probe) * 4;
}

__device__ __forceinline__ float3 half4_rgb(uint2 u) {
  const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
  const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
  return make_float3(a.x, a.y, b.x);
}

// One tap from global memory (CG as for load_up).
template <typename T, bool CG>
__device__ __forceinline__ float3 load_rgb(const T* p);
template <>
__device__ __forceinline__ float3 load_rgb<float, false>(const float* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 v = RC_CHK(q, kChkRadiance) ? __ldg(q) : make_float4(0.f, 0.f, 0.f, 0.f);
  return make_float3(v.x, v.y, v.z);
}
template <>
__device__ __forceinline__ float3 load_rgb<float, true>(const float* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 v = RC_CHK(q, kChkRadiance) ? __ldca(q) : make_float4(0.f, 0.f, 0.f, 0.f);
  return make_float3(v.x, v.y, v.z);
}
template <>
__device__ __forceinline__ float3 load_rgb<__half, false>(const __half* p) {
  const uint2* q = reinterpret_cast<const uint2*>(p);
  return half4_rgb(RC_CHK(q, kChkRadiance) ? __ldg(q) : make_uint2(0u, 0u));
}
template <>
__device__ __forceinline__ float3 load_rgb<__half, true>(const __half* p) {
  const uint2* q = reinterpret_cast<const uint2*>(p);
  return half4_rgb(RC_CHK(q, kChkRadiance) ? __ldca(q) : make_uint2(0u, 0u));
}

// One tap from a staged shared-memory tile.
__device__ __forceinline__ float3 lds_rgb(const float* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  const float4 v = RC_CHK(q, kChkShared) ? *q : make_float4(0.f, 0.f, 0.f, 0.f);
  return make_float3(v.x, v.y, v.z);
}
__device__ __forceinline__ float3 lds_rgb(const __half* p) {
  const uint2* q = reinterpret_cast<const uint2*>(p);
  return half4_rgb(RC_CHK(q, kChkShared) ? *q : make_uint2(0u, 0u));
}

// Writes one (direction, probe) of a child average (each channel rounded as
// a single store of it would be).
__device__ __forceinline__ void store_rgb(float* p, float r, float g, float b) {
  float4* q = reinterpret_cast<float4*>(p);
  if (RC_CHK(q, kChkRadiance)) *q = make_float4(r, g, b, 0.f);
}
__device__ __forceinline__ void store_rgb(__half* p, float r, float g, float b) {
  uint2* q = reinterpret_cast<uint2*>(p);
  const __half2 lo = __floats2half2_rn(r, g), hi = __floats2half2_rn(b, 0.f);
  uint2 u;
  u.x = *reinterpret_cast<const uint32_t*>(&lo);
  u.y = *reinterpret_cast<const uint32_t*>(&hi);
  if (RC_CHK(q, kChkRadiance)) *q = u;
}

struct LevelArgs;
template <typename T>
__device__ __forceinline__ void store_avg(const LevelArgs& a, int dp, int64_t p, float r, float g, float b);

struct LevelArgs {
  const uint2* mask;     // this level's decimated (opacity, emissive) bits (bit-parallel walk)
  const uint32_t* emis;  // full-resolution emissive bits, same layout as occ
  int32_t l2s;           // log2(spacing)
  int32_t l2px;          // log2 of the decimated plane row pitch
  int32_t wpp;           // words per decimated plane
  uint32_t rep;          // narrow levels: 1 bit at the start of every row of a word
  int32_t tiles;         // block tiles per direction group
  int32_t up_rows;       // rows of the next level's probes one block stages (k_level_bits_up)
  const uint32_t* occ;
  const uint2* vol;
  int32_t G[3];
  int32_t W;           // occupancy words per x row
  const DirInfo* dirs; // this level's table
  int32_t M[3];        // probes per axis at this level
  int32_t spacing;
  int32_t n;           // direction resolution
  int32_t ndirs;
  int64_t P;           // probes at this level
  void* L;             // out: merged radiance
  void* A_out;         // out: child-averaged radiance (levels >= 1), [parent dir][probe][4]
  int32_t a_out_planar;  // A_out planar [3][parent dir][probe] instead (read by the walk-free cascade 0)
  const void* A_up;    // in: next level's child-averaged radiance (not top), [dir][probe][4]
  int32_t UM[3];       // probes per axis at the next level
  int64_t P_up;
  float* fluence;      // out: level 0 only
};

// One (parent direction dp, probe p) of the level's child average, in its
// output layout.
template <typename T>
__device__ __forceinline__ void store_avg(const LevelArgs& a, int dp, int64_t p, float r, float g, float b) {
  T* A = static_cast<T*>(a.A_out);
  if (a.a_out_planar) {
    const int64_t npar = (int64_t)(a.n >> 1) * (a.n >> 1);
    Store<T>::store(A + (int64_t)dp * a.P + p, r);
    Store<T>::store(A + (npar + dp) * a.P + p, g);
    Store<T>::store(A + (2 * npar + dp) * a.P + p, b);
  } else {
    store_rgb(rgb4_at(A, dp, a.P, p), r, g, b);
  }
}

__device__ __forceinline__ bool opaque_at(const uint32_t* __restrict__ occ, int W, int Gy, int x, int y, int z) {
  const uint32_t* w = &occ[((int64_t)z * Gy + y) * W + (x >> 5)];
  return RC_CHK(w, kChkOccupancy) && ((__ldg(w) >> (x & 31)) & 1u);
}

// Exact integer voxel walk of one interval.  Returns the linear index of the
// first opaque voxel entered inside the interval, or -1 when the ray leaves
// the interval or the grid first.  (x, y, z) is the start voxel: the voxel at
// the probe centre for level 0 (tested first), otherwise the last voxel
// entered before the interval (not tested).
__device__ __forceinline__ int64_t walk_interval(const uint32_t* __restrict__ occ, const int32_t G[3], int W,
                                                 int x, int y, int z, const DirInfo& di, bool test_start) {
  if (test_start && opaque_at(occ, W, G[1], x, y, z)) return ((int64_t)z * G[1] + y) * G[0] + x;
  int tx = di.first_T[0], ty = di.first_T[1], tz = di.first_T[2];
  const int sx = di.sgn[0], sy = di.sgn[1], sz = di.sgn[2];
  const int dx = di.step_T[0], dy = di.step_T[1], dz = di.step_T[2];
  for (int s = di.steps; s > 0; --s) {
    if (tx <= ty && tx <= tz) {
      x += sx;
      tx += dx;
    } else if (ty <= tz) {
      y += sy;
      ty += dy;
    } else {
      z += sz;
      tz += dz;
    }
    if ((unsigned)x >= (unsigned)G[0] || (unsigned)y >= (unsigned)G[1] || (unsigned)z >= (unsigned)G[2]) return -1;
    if (opaque_at(occ, W, G[1], x, y, z)) return ((int64_t)z * G[1] + y) * G[0] + x;
  }
  return -1;
}

__device__ __forceinline__ void voxel_emission(const uint2* __restrict__ vol, int64_t idx, float r[3]) {
  const uint2 v = RC_CHK(&vol[idx], kChkVolume) ? __ldg(&vol[idx]) : make_uint2(0u, 0u);
  r[0] = __half2float(__ushort_as_half((unsigned short)(v.x & 0xFFFFu)));
  r[1] = __half2float(__ushort_as_half((unsigned short)(v.x >> 16)));
  r[2] = __half2float(__ushort_as_half((unsigned short)(v.y & 0xFFFFu)));
}

__device__ __forceinline__ float emission_channel(const uint2* __restrict__ vol, uint32_t idx, int ch) {
  const uint2 v = RC_CHK(&vol[idx], kChkVolume) ? __ldg(&vol[idx]) : make_uint2(0u, 0u);
  const uint32_t w = ch == 2 ? v.y : v.x;
  return __half2float(__ushort_as_half((unsigned short)(ch == 1 ? (w >> 16) : (w & 0xFFFFu))));
}

// One probe p, scalar walk.  Level 0 (L0) walks every direction and reduces
// the fluence; other levels walk the four child directions of each parent
// texel dp0 .. dp0 + ndp - 1 and write their average for the level below.
// Unless TOP, rays that reach the end of their interval take the trilinear
// blend of the 8 nearest next-level probes (child index m sits at parent
// coordinate m/2 - 1/4, clamped at the border) of the child-averaged radiance.
template <typename T, bool L0, bool TOP, bool CG>
__device__ __forceinline__ void scalar_probe(const LevelArgs& a, int64_t p, int dp0, int ndp) {
  // probe coordinates in 32-bit arithmetic (a level has fewer than 2^31 probes)
  const uint32_t pu = (uint32_t)p, rowi = pu / (uint32_t)a.M[0];
  const int mx = (int)(pu - rowi * (uint32_t)a.M[0]);
  const int mz = (int)(rowi / (uint32_t)a.M[1]);
  const int my = (int)(rowi - (uint32_t)mz * (uint32_t)a.M[1]);
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
  const int hn = a.n >> 1;
  float acc[3] = {0.f, 0.f, 0.f};
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
      const T* Au = static_cast<const T*>(a.A_up);
      r[0] = r[1] = r[2] = 0.f;
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const float3 v = load_rgb<T, CG>(rgb4_at(Au, d, a.P_up, tap_off[t]));
        r[0] = fmaf(tap_w[t], v.x, r[0]);
        r[1] = fmaf(tap_w[t], v.y, r[1]);
        r[2] = fmaf(tap_w[t], v.z, r[2]);
      }
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      Store<T>::store(L + ((int64_t)ch * a.ndirs + d) * a.P + p, r[ch]);
      acc[ch] = L0 ? fmaf(di.omega, r[ch], acc[ch]) : acc[ch] + r[ch];
    }
    if (!L0 && (c & 3) == 3) {
      const int dp = dp0 + (c >> 2);
      store_avg<T>(a, dp, p, 0.25f * acc[0], 0.25f * acc[1], 0.25f * acc[2]);
      acc[0] = acc[1] = acc[2] = 0.f;
    }
  }
  if (L0) {
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
      if (RC_CHK(&a.fluence[p * 3 + ch], kChkFluence)) a.fluence[p * 3 + ch] = acc[ch];
  }
}

// One thread per probe; block row blockIdx.y = parent texel (not level 0).
template <typename T, bool L0, bool TOP>
__global__ void __launch_bounds__(128) k_level_scalar(const __grid_constant__ LevelArgs a) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.P) return;
  scalar_probe<T, L0, TOP, false>(a, p, blockIdx.y, 1);
}

// Base volume from boxes: the last box containing a voxel wins.
static __global__ void k_boxes_to_base(uint2* __restrict__ base, int Gx, int Gy, int Gz, const rc_box* __restrict__ boxes,
                                int nb) {
  extern __shared__ rc_box sbox[];
  for (int i = threadIdx.x; i < nb; i += blockDim.x) sbox[i] = boxes[i];
  __syncthreads();
  const int64_t total = (int64_t)Gx * Gy * Gz;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(idx % Gx), y = (int)((idx / Gx) % Gy), z = (int)(idx / ((int64_t)Gx * Gy));
    uint2 v = make_uint2(0u, 0u);
    for (int b = nb - 1; b >= 0; --b) {
      const rc_box& B = sbox[b];
      if (x >= B.lo[0] && x < B.hi[0] && y >= B.lo[1] && y < B.hi[1] && z >= B.lo[2] && z < B.hi[2]) {
        v.x = (uint32_t)B.value.emission[0] | ((uint32_t)B.value.emission[1] << 16);
        v.y = (uint32_t)B.value.emission[2] | ((uint32_t)B.value.albedo_occ << 16);
        break;
      }
    }
    if (RC_CHK(&base[idx], kChkVolume)) base[idx] = v;
  }
}

}  // namespace rcx
