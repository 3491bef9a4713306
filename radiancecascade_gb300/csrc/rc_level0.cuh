// rc_level0.cuh -- cascade 0 without a walk (sm_103a).
//
// With the default cascade shape every cascade-0 interval [0, b_1) holds only
// the voxel the ray starts in (the walk tables give 0 crossings for every
// direction).  That voxel is one of the 8 around the probe's lattice-point
// centre, picked by the signs of the direction (start_off in {-1, 0}^3).  So
// cascade 0 reads the opacity and emissive bits of those 8 voxels once per
// probe and spends the rest on the merge with cascade 1 and the output
// stores, which bound it.
//
// Mapping: one warp = 128 consecutive x-probes of one y row and two z planes;
// lane l owns probes x0 = 4l .. 4l+3 (float4 stores).  The trilinear merge
// reads, per parent row, the float2 of parent columns (2l', 2l'+1) and gets
// columns 2l'-1 and 2l'+2 from the neighbouring lanes.
#pragma once

#include "rc_kernels.cuh"
#include "rc_tma.cuh"

namespace rcx {

constexpr int kL0Threads = 256;

template <typename T>
struct Vec4;
template <>
struct Vec4<float> {
  static __device__ __forceinline__ void stream(float* p, float a, float b, float c, float d) {
    if (RC_CHK(reinterpret_cast<float4*>(p), kChkRadiance)) __stcs(reinterpret_cast<float4*>(p), make_float4(a, b, c, d));
  }
};
template <>
struct Vec4<__half> {
  static __device__ __forceinline__ void stream(__half* p, float a, float b, float c, float d) {
    const __half2 lo = __floats2half2_rn(a, b), hi = __floats2half2_rn(c, d);
    uint2 u;
    u.x = *reinterpret_cast<const uint32_t*>(&lo);
    u.y = *reinterpret_cast<const uint32_t*>(&hi);
    if (RC_CHK(reinterpret_cast<uint2*>(p), kChkRadiance)) __stcs(reinterpret_cast<uint2*>(p), u);
  }
};

// Two adjacent values of the next level's child-averaged radiance (CG: data
// written during the same launch, see load_up).
template <typename T, bool CG>
__device__ __forceinline__ float2 load2(const T* p);
template <>
__device__ __forceinline__ float2 load2<float, false>(const float* p) {
  const float2* q = reinterpret_cast<const float2*>(p);
  return RC_CHK(q, kChkRadiance) ? __ldg(q) : make_float2(0.f, 0.f);
}
template <>
__device__ __forceinline__ float2 load2<float, true>(const float* p) {
  const float2* q = reinterpret_cast<const float2*>(p);
  return RC_CHK(q, kChkRadiance) ? __ldca(q) : make_float2(0.f, 0.f);
}
template <>
__device__ __forceinline__ float2 load2<__half, false>(const __half* p) {
  const __half2* q = reinterpret_cast<const __half2*>(p);
  return RC_CHK(q, kChkRadiance) ? __half22float2(__ldg(q)) : make_float2(0.f, 0.f);
}
template <>
__device__ __forceinline__ float2 load2<__half, true>(const __half* p) {
  const unsigned* q = reinterpret_cast<const unsigned*>(p);
  const unsigned u = RC_CHK(q, kChkRadiance) ? __ldca(q) : 0u;
  return __half22float2(*reinterpret_cast<const __half2*>(&u));
}

// Two adjacent shared-memory values at an even index (one 8- or 4-byte load).
__device__ __forceinline__ float2 lds_pair(const float* p) {
  return RC_CHK(p + 1, kChkShared) ? *reinterpret_cast<const float2*>(p) : make_float2(0.f, 0.f);
}
__device__ __forceinline__ float2 lds_pair(const __half* p) {
  return RC_CHK(p + 1, kChkShared) ? __half22float2(*reinterpret_cast<const __half2*>(p)) : make_float2(0.f, 0.f);
}

// Requires (checked on the host): probe spacing 2 (centres 2m+1, so the 8
// candidate voxels are 2m, 2m+1 per axis), every cascade-0 direction takes 0
// steps, and M[0] % 4 == 0.
// One warp's share: global warp index `wid` (chunk of 128 probes of a row,
// two planes).
template <typename T, bool TOP, bool CG>
__device__ __forceinline__ void level0_direct_warp(const LevelArgs& a, int64_t wid) {
  const int lane = threadIdx.x & 31;
  const int Mx = a.M[0], My = a.M[1], Mz = a.M[2];
  const int chunks = (Mx + 127) >> 7;
  const int cw = (int)(wid % chunks);
  wid /= chunks;
  const int y = (int)(wid % My);
  const int z0 = 2 * (int)(wid / My);
  if (z0 >= Mz) return;  // whole warp
  const int lq = 32 * cw + lane;  // quad index along x
  const int x0 = 4 * lq;
  const bool active = x0 < Mx;
  const bool zok1 = z0 + 1 < Mz;

  // Opacity and emissive bits of the 8 voxels around each of the lane's 4
  // probes in both planes: voxel rows (2y + oy, 2z + oz), x bits 8*lq .. 8*lq+7.
  uint32_t ow[2] = {0u, 0u}, ew[2] = {0u, 0u};  // [zc]: byte (oz * 2 + oy)
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int zc = r >> 2, oz = (r >> 1) & 1, oy = r & 1;
    const int vz = 2 * (z0 + zc) + oz, vy = 2 * y + oy;
    if (active && (zc == 0 || zok1)) {
      const int64_t w = ((int64_t)vz * a.G[1] + vy) * a.W + ((8 * lq) >> 5);
      const int sh = (8 * lq) & 31;
      const uint32_t wo = RC_CHK(&a.occ[w], kChkOccupancy) ? __ldg(&a.occ[w]) : 0u;
      const uint32_t we = RC_CHK(&a.emis[w], kChkOccupancy) ? __ldg(&a.emis[w]) : 0u;
      ow[zc] |= ((wo >> sh) & 0xFFu) << (8 * (r & 3));
      ew[zc] |= ((we >> sh) & 0xFFu) << (8 * (r & 3));
    }
  }

  // For each of the 8 octants o = ox + 2 oy + 4 oz (the start voxel's offset
  // from the probe's lower corner), the 8-bit masks of the lane's children
  // (bit zc * 4 + e) whose start voxel is opaque / emissive.
  uint32_t oct_opq[2] = {0u, 0u}, oct_ems[2] = {0u, 0u};
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    const int ox = o & 1, oy = (o >> 1) & 1, oz = o >> 2;
    uint32_t mo = 0, me = 0;
#pragma unroll
    for (int zc = 0; zc < 2; ++zc) {
      const uint32_t ob = (ow[zc] >> (8 * (oz * 2 + oy))) & 0xFFu, eb = (ew[zc] >> (8 * (oz * 2 + oy))) & 0xFFu;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        mo |= ((ob >> (2 * e + ox)) & 1u) << (zc * 4 + e);
        me |= ((eb >> (2 * e + ox)) & 1u) << (zc * 4 + e);
      }
    }
    oct_opq[o >> 2] |= mo << (8 * (o & 3));
    oct_ems[o >> 2] |= me << (8 * (o & 3));
  }

  // merge geometry: parent rows (qy_lo, qy_hi) with the child row's weights,
  // parent planes (z0/2 - 1, z0/2, z0/2 + 1), own parent columns 2lq, 2lq+1
  const int UMx = a.UM[0], UMy = a.UM[1], UMz = a.UM[2];
  const int ylo = (y - 1) >> 1;
  const float wy_lo = (y & 1) ? 0.75f : 0.25f, wy_hi = 1.0f - wy_lo;
  const int qy[2] = {min(max(ylo, 0), UMy - 1), min(max(ylo + 1, 0), UMy - 1)};
  int qz[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) qz[k] = min(max(z0 / 2 - 1 + k, 0), UMz - 1);
  const int col0 = min(2 * lq, UMx - 2);  // own float2 (always inside the row when active)
  const int lcol = max(2 * lq - 1, 0), rcol = min(2 * lq + 2, UMx - 1);
  // Halo columns 2lq-1 (lane 0) and 2lq+2 (the row's last lane of the warp).
  // At a row's ends they clamp to the lane's own columns; only a row split
  // over several warps (Mx > 128) needs loads for them.
  const bool last_lane = (lane == 31) || (4 * (lq + 1) >= Mx);
  const bool lhalo_load = (lane == 0) && cw > 0;
  const bool rhalo_load = last_lane && 4 * (lq + 1) < Mx;
  int rowoff[2][3];  // element offset of parent row (qy[r], qz[k]) within one direction's plane
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int k = 0; k < 3; ++k) rowoff[r][k] = (qz[k] * UMy + qy[r]) * UMx;

  T* L = static_cast<T*>(a.L);
  const T* Au = static_cast<const T*>(a.A_up);
  const int64_t plane = (int64_t)My * Mx;
  const int64_t p0 = ((int64_t)z0 * My + y) * Mx + x0;  // probe (x0, y, z0)
  // Channel-outer loop: one channel's 8 fluence sums stay in registers.
#pragma unroll 1
  for (int ch = 0; ch < 3; ++ch) {
    float flu[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll 1
    for (int d = 0; d < a.ndirs; ++d) {
      const DirInfo& di = a.dirs[d];
      const int ox = di.start_off[0] + 1, oy = di.start_off[1] + 1, oz = di.start_off[2] + 1;
      const int oct = ox + 2 * oy + 4 * oz;
      const bool hi_oct = oct >= 4;
      const unsigned opq = ((hi_oct ? oct_opq[1] : oct_opq[0]) >> (8 * (oct & 3))) & 0xFFu;
      const unsigned ems = ((hi_oct ? oct_ems[1] : oct_ems[0]) >> (8 * (oct & 3))) & 0xFFu;
      const unsigned valid = active ? (zok1 ? 0xFFu : 0x0Fu) : 0u;
      const bool merge = !TOP && __any_sync(0xFFFFFFFFu, (valid & ~opq) != 0u);
      float mv[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
      if (merge) {
        const T* src = Au + (int64_t)(ch * a.ndirs + d) * a.P_up;
        // z-interpolated parent columns 2lq-1 .. 2lq+2 for both child planes, per parent row
        float zr[2][2][4];  // [zc][row][col]
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          float2 own[3];
          float lh[3], rh[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const T* row = src + rowoff[r][k];
            own[k] = active ? load2<T, CG>(row + col0) : make_float2(0.f, 0.f);
            lh[k] = __shfl_up_sync(0xFFFFFFFFu, own[k].y, 1);
            rh[k] = __shfl_down_sync(0xFFFFFFFFu, own[k].x, 1);
            if (lane == 0) lh[k] = own[k].x;
            if (last_lane) rh[k] = own[k].y;
            if (chunks > 1) {
              if (lhalo_load) lh[k] = load_up<T, CG>(row + lcol);
              if (rhalo_load) rh[k] = load_up<T, CG>(row + rcol);
            }
          }
          const float cols[3][4] = {{lh[0], own[0].x, own[0].y, rh[0]},
                                    {lh[1], own[1].x, own[1].y, rh[1]},
                                    {lh[2], own[2].x, own[2].y, rh[2]}};
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            zr[0][r][c] = fmaf(0.25f, cols[0][c], 0.75f * cols[1][c]);
            zr[1][r][c] = fmaf(0.75f, cols[1][c], 0.25f * cols[2][c]);
          }
        }
#pragma unroll
        for (int zc = 0; zc < 2; ++zc) {
          float v[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) v[c] = fmaf(wy_lo, zr[zc][0][c], wy_hi * zr[zc][1][c]);
          // children e = 0..3 sit at parent coordinates 2lq - 1/4, +1/4, +3/4, +5/4
          mv[zc][0] = fmaf(0.25f, v[0], 0.75f * v[1]);
          mv[zc][1] = fmaf(0.75f, v[1], 0.25f * v[2]);
          mv[zc][2] = fmaf(0.25f, v[1], 0.75f * v[2]);
          mv[zc][3] = fmaf(0.75f, v[2], 0.25f * v[3]);
        }
      }
      const float om = di.omega;
      T* lrow = L + (int64_t)(ch * a.ndirs + d) * a.P + p0;
#pragma unroll
      for (int zc = 0; zc < 2; ++zc) {
        float o[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int bit = zc * 4 + e;
          o[e] = ((opq >> bit) & 1u) ? 0.f : mv[zc][e];
          if ((ems >> bit) & 1u) {  // emissive start voxel (rare)
            const int64_t vx = 2 * (x0 + e) + ox;  // start voxel = probe centre 2m+1 plus start_off
            const int64_t vidx = ((int64_t)(2 * (z0 + zc) + oz) * a.G[1] + (2 * y + oy)) * a.G[0] + vx;
            o[e] = emission_channel(a.vol, (uint32_t)vidx, ch);
          }
          flu[zc][e] = fmaf(om, o[e], flu[zc][e]);
        }
        if ((valid >> (zc * 4)) & 1u) Vec4<T>::stream(lrow + zc * plane, o[0], o[1], o[2], o[3]);
      }
    }
    // fluence channel ch of the lane's 8 probes (RGB interleaved)
#pragma unroll
    for (int zc = 0; zc < 2; ++zc) {
      if (!(active && (zc == 0 || zok1))) continue;
      float* f = a.fluence + (p0 + zc * plane) * 3 + ch;
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (RC_CHK(&f[3 * e], kChkFluence)) f[3 * e] = flu[zc][e];
    }
  }
}

template <typename T, bool TOP>
__global__ void __launch_bounds__(kL0Threads, 3) k_level0_direct(const __grid_constant__ LevelArgs a) {
  level0_direct_warp<T, TOP, false>(a, ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
}

// TMA-staged form of k_level0_direct.  Block = 8 child rows (one per warp) x
// ZC planes of one 128-probe chunk.  For every direction the parent tiles of
// cascade 1's child-averaged radiance -- per channel the full parent row width
// x PY rows x (ZC + 1) planes -- are brought into shared memory by three
// cp.async.bulk.tensor copies while earlier directions' tiles are consumed
// (l0_stages stages); one iteration serves all three channels.  Lanes read
// their 4 parent columns from shared memory.  Each stage has a "full"
// mbarrier the copies complete and an "empty" one every warp arrives at when
// it is done with the stage; thread 0 refills a stage once all warps have
// arrived, so warps never meet at a block barrier and may run a stage apart.
// Every barrier wait is bounded: a wait that runs out marks the block aborted
// (s_abort), every warp leaves its loop at its next wait, the block records
// *err = 1, and thread 0 waits (bounded) for the copies it may still have in
// flight before the block's shared memory goes.
constexpr int kL0TmaRows = 8;
// Parent tiles in flight (S): the copy for iteration it + S - 1 starts at
// iteration it.  Four stages (113.4 against 116.3 us for three at 256^3), five
// for the compiled 32- and 64-wide rows (111.6 us; 69 KB of shared memory per
// block at 64-wide rows, still two blocks per SM -- wider rows keep four).
__host__ __device__ constexpr int l0_stages(int umxc) { return umxc == 32 || umxc == 64 ? 5 : 4; }
// Child planes per block (ZC).  ZC = 1 halves the per-lane accumulators (80
// registers, 3 blocks/SM) but reads 4 parent values per output instead of 3;
// at 256^3 it measured 160 us against 153 us for ZC = 2 (128 registers, 2 blocks/SM).
constexpr int kL0Planes = 2;

// UMXC: cascade 1's row width (UM[0]) fixed at compile time, with tiles of
// kL0TileRows rows (0: both taken from the arguments).  Fixed, every tile and
// stage offset is a constant and the shared-memory addresses need no
// per-direction arithmetic (116.7 against 120.5 us at 256^3).
constexpr int kL0TileRows = 6;
template <typename T, int ZC, int UMXC = 0>
__global__ void __launch_bounds__(kL0Threads, ZC == 1 ? 3 : 2)
    k_level0_tma(const LevelArgs a, const __grid_constant__ CUtensorMap tmap, int py, int* err) {
  static_assert(ZC == 1 || ZC == 2, "one or two child planes per block");
  constexpr int kL0Stages = l0_stages(UMXC);
  const int PY = UMXC ? kL0TileRows : py;
  constexpr int PZ = ZC + 1;  // parent planes in a tile
  extern __shared__ __align__(128) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int Mx = a.M[0], My = a.M[1], Mz = a.M[2];
  const int UMx = UMXC ? UMXC : a.UM[0], UMy = a.UM[1], UMz = a.UM[2];
  // TMA writes to shared memory must start on a 128-byte boundary: both stages
  // start at multiples of 128 from a 128-byte aligned base.
  const int tile_elems = PZ * PY * UMx;
  const uint32_t tile_bytes = (uint32_t)tile_elems * (uint32_t)sizeof(T);
  const uint32_t tile_stride = (tile_bytes + 127u) & ~127u;  // one channel's tile, 128-byte aligned
  const uint32_t stage_bytes = 3u * tile_stride;              // the three channels of one direction
  unsigned char* base = smem + ((128u - (smem_u32(smem) & 127u)) & 127u);
  T* tiles = reinterpret_cast<T*>(base);
  const int stage_elems = (int)(stage_bytes / sizeof(T));
  const int tile_stride_elems = (int)(tile_stride / sizeof(T));
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + kL0Stages * stage_bytes);

  const int chunks = (Mx + 127) >> 7, yblocks = (My + kL0TmaRows - 1) / kL0TmaRows;
  int bid = blockIdx.x;
  const int cw = bid % chunks;
  bid /= chunks;
  const int yb = (bid % yblocks) * kL0TmaRows;
  const int z0 = ZC * (bid / yblocks);
  const int y = yb + warp;
  const int lq = 32 * cw + lane, x0 = 4 * lq;
  const bool active = y < My && x0 < Mx && z0 < Mz;
  const bool zok1 = ZC == 2 && z0 + 1 < Mz;

  // opacity / emissive masks per octant, as in k_level0_direct
  uint32_t ow[2] = {0u, 0u}, ew[2] = {0u, 0u};
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int zc = r >> 2, oz = (r >> 1) & 1, oy = r & 1;
    if (active && (zc == 0 || zok1)) {
      const int64_t w = ((int64_t)(2 * (z0 + zc) + oz) * a.G[1] + (2 * y + oy)) * a.W + ((8 * lq) >> 5);
      const int sh = (8 * lq) & 31;
      const uint32_t wo = RC_CHK(&a.occ[w], kChkOccupancy) ? __ldg(&a.occ[w]) : 0u;
      const uint32_t we = RC_CHK(&a.emis[w], kChkOccupancy) ? __ldg(&a.emis[w]) : 0u;
      ow[zc] |= ((wo >> sh) & 0xFFu) << (8 * (r & 3));
      ew[zc] |= ((we >> sh) & 0xFFu) << (8 * (r & 3));
    }
  }
  uint32_t oct_opq[2] = {0u, 0u}, oct_ems[2] = {0u, 0u};
#pragma unroll
  for (int o = 0; o < 8; ++o) {
    const int ox = o & 1, oy = (o >> 1) & 1, oz = o >> 2;
    uint32_t mo = 0, me = 0;
#pragma unroll
    for (int zc = 0; zc < ZC; ++zc) {
      const uint32_t ob = (ow[zc] >> (8 * (oz * 2 + oy))) & 0xFFu, eb = (ew[zc] >> (8 * (oz * 2 + oy))) & 0xFFu;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        mo |= ((ob >> (2 * e + ox)) & 1u) << (zc * 4 + e);
        me |= ((eb >> (2 * e + ox)) & 1u) << (zc * 4 + e);
      }
    }
    oct_opq[o >> 2] |= mo << (8 * (o & 3));
    oct_ems[o >> 2] |= me << (8 * (o & 3));
  }
  const unsigned valid = active ? (zok1 ? 0xFFu : 0x0Fu) : 0u;

  // tile origin and this warp's parent rows inside it
  const int ys = max(0, min(yb / 2 - 1, UMy - PY));
  const int zs = max(0, min((z0 - 1) >> 1, UMz - PZ));
  // inactive warps and lanes still read the tile: keep their rows and columns inside it
  const int ylo = (min(y, My - 1) - 1) >> 1;
  // Row 0 of rowoff is the parent row of weight 3/4 (ylo + 1 for even y,
  // ylo for odd y), row 1 the one of weight 1/4; with one child plane
  // (ZC = 1) the planes are ordered the same way.  Every 1D blend below is
  // a + 3 b = 4 (a/4 + 3b/4); the three blends' factor 64 is divided out
  // once per value (exact: a power of two).
  const int yfar = (y & 1) ^ 1, zfar = ZC == 1 ? (z0 & 1) ^ 1 : 0;
  int rowoff[2][PZ];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int k = 0; k < PZ; ++k) {
      const int qy = min(max(ylo + (r ^ yfar), 0), UMy - 1);
      const int qz = min(max(((z0 - 1) >> 1) + (ZC == 1 ? (k ^ zfar) : k), 0), UMz - 1);
      rowoff[r][k] = ((qz - zs) * PY + (qy - ys)) * UMx;
    }
  const int c0 = min(2 * lq, UMx - 2), lcol = min(max(2 * lq - 1, 0), UMx - 1), rcol = min(2 * lq + 2, UMx - 1);

  T* L = static_cast<T*>(a.L);
  const int64_t plane = (int64_t)My * Mx;
  const int64_t p0 = ((int64_t)z0 * My + y) * Mx + x0;
  const int64_t chstride = (int64_t)a.ndirs * a.P;  // one channel of L_0
  const int total = a.ndirs;

  // the three channel tiles of direction dd into stage st
  auto issue = [&](int dd, int st) {
    mbar_arrive_expect_tx(&bar[st], 3u * tile_bytes);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
      tma_load_3d(tiles + st * stage_elems + ch * tile_stride_elems, &tmap, 0, ys, (ch * a.ndirs + dd) * UMz + zs,
                  &bar[st]);
  };
  // bar[0 .. S-1]: a stage's copy has landed; bar[S .. 2S-1]: every warp is done with it
  __shared__ int s_abort;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < kL0Stages; ++k) {
      mbar_init(&bar[k], 1);
      mbar_init(&bar[kL0Stages + k], kL0Threads / 32);
    }
    mbar_fence_init();
    s_abort = 0;
  }
  __syncthreads();
  // a destination off its 128-byte boundary is reported and never copied to
  const bool aligned = ((smem_u32(tiles) | tile_stride) & 127u) == 0u;
  if (threadIdx.x == 0) {
    grid_dep_wait();  // cascade 1's child averages: the masks above came from earlier launches
    grid_dep_release();  // the next frame's emitter update may start (it waits before it writes)
    if (aligned) {
      for (int k = 0; k < kL0Stages - 1 && k < total; ++k) issue(k, k);
    } else {
      atomicExch(err, 2);
    }
  }
  // every direction's start octant and solid angle, lane l holding
  // directions l and l + 32 (handed out by shuffles; more than 64 directions
  // read the table in the loop)
  int oct_lane[2] = {0, 0};
  float om_lane[2] = {0.f, 0.f};
#pragma unroll
  for (int h = 0; h < 2; ++h)
    if (lane + 32 * h < total) {
      const DirInfo& dl = a.dirs[lane + 32 * h];
      oct_lane[h] = (dl.start_off[0] + 1) + 2 * (dl.start_off[1] + 1) + 4 * (dl.start_off[2] + 1);
      om_lane[h] = dl.omega;
    }
  float flu[3][ZC][4];
#pragma unroll
  for (int ch = 0; ch < 3; ++ch)
#pragma unroll
    for (int zc = 0; zc < ZC; ++zc) flu[ch][zc][0] = flu[ch][zc][1] = flu[ch][zc][2] = flu[ch][zc][3] = 0.f;
  int it = 0;
  bool failed = false;
#pragma unroll 1
  for (; it < total; ++it) {
    const int d = it;
    const int st = it % kL0Stages;
    const int nx_ = it + kL0Stages - 1;
    // stage nx_ % S last held direction nx_ - S: refill it once every warp is done with that
    if (threadIdx.x == 0 && nx_ < total && aligned) {
      const int prev = nx_ - kL0Stages;
      if (prev >= 0 && !mbar_wait_bounded(&bar[kL0Stages + nx_ % kL0Stages], (uint32_t)(prev / kL0Stages) & 1u))
        atomicExch(&s_abort, 1);
      fence_proxy_async();
      issue(nx_, nx_ % kL0Stages);
    }
    const bool ok = !*(volatile int*)&s_abort && mbar_wait_bounded(&bar[st], (uint32_t)(it / kL0Stages) & 1u);
    if (__any_sync(0xFFFFFFFFu, !ok)) {
      if (lane == 0) atomicExch(&s_abort, 1);
      failed = true;
      break;
    }
    int oct;
    float om;
    if (total <= 64) {
      const bool h = d >= 32;
      oct = __shfl_sync(0xFFFFFFFFu, h ? oct_lane[1] : oct_lane[0], d & 31);
      om = __shfl_sync(0xFFFFFFFFu, h ? om_lane[1] : om_lane[0], d & 31);
    } else {
      const DirInfo& di = a.dirs[d];
      oct = (di.start_off[0] + 1) + 2 * (di.start_off[1] + 1) + 4 * (di.start_off[2] + 1);
      om = di.omega;
    }
    const int ox = oct & 1, oy = (oct >> 1) & 1, oz = oct >> 2;
    const bool hi_oct = oct >= 4;
    const unsigned opq = ((hi_oct ? oct_opq[1] : oct_opq[0]) >> (8 * (oct & 3))) & 0xFFu;
    const unsigned ems = ((hi_oct ? oct_ems[1] : oct_ems[0]) >> (8 * (oct & 3))) & 0xFFu;
    const bool merge = __any_sync(0xFFFFFFFFu, (valid & ~opq) != 0u);
    const unsigned emv = ems & valid;
    // Each output's final scale, taken once per direction for all channels:
    // 1/64 where the start voxel is clear, 0 where it is opaque (the blend of
    // non-negative radiance times 0 is +0, as the plain select gave).
    float sc[ZC][4];
#pragma unroll
    for (int zc = 0; zc < ZC; ++zc)
#pragma unroll
      for (int e = 0; e < 4; ++e) sc[zc][e] = ((opq >> (zc * 4 + e)) & 1u) ? 0.f : (1.f / 64.f);
    T* lrow = L + (int64_t)d * a.P + p0;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      const T* tile = tiles + st * stage_elems + ch * tile_stride_elems;
      float mv[ZC][4];
#pragma unroll
      for (int zc = 0; zc < ZC; ++zc) mv[zc][0] = mv[zc][1] = mv[zc][2] = mv[zc][3] = 0.f;
      if (merge) {
        float zr[ZC][2][4];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          float cv[PZ][4];
#pragma unroll
          for (int k = 0; k < PZ; ++k) {
            const T* row = tile + rowoff[r][k];
            cv[k][0] = RC_CHK(&row[lcol], kChkShared) ? to_float(row[lcol]) : 0.f;
            const float2 own = lds_pair(row + c0);  // c0 and the row offsets are even (UMx is)
            cv[k][1] = own.x;
            cv[k][2] = own.y;
            cv[k][3] = RC_CHK(&row[rcol], kChkShared) ? to_float(row[rcol]) : 0.f;
          }
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            if (ZC == 1) {
              zr[0][r][c] = fmaf(3.f, cv[0][c], cv[PZ - 1][c]);  // plane 0 has weight 3/4
            } else {
              zr[0][r][c] = fmaf(3.f, cv[1][c], cv[0][c]);
              zr[ZC - 1][r][c] = fmaf(3.f, cv[1][c], cv[PZ - 1][c]);
            }
          }
        }
#pragma unroll
        for (int zc = 0; zc < ZC; ++zc) {
          float v[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) v[c] = fmaf(3.f, zr[zc][0][c], zr[zc][1][c]);
          mv[zc][0] = fmaf(3.f, v[1], v[0]) * sc[zc][0];
          mv[zc][1] = fmaf(3.f, v[1], v[2]) * sc[zc][1];
          mv[zc][2] = fmaf(3.f, v[2], v[1]) * sc[zc][2];
          mv[zc][3] = fmaf(3.f, v[2], v[3]) * sc[zc][3];
        }
      }
#pragma unroll
      for (int zc = 0; zc < ZC; ++zc) {
        float o[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) o[e] = mv[zc][e];
        if ((emv >> (zc * 4)) & 0xFu) {  // an emissive start voxel in this plane (rare)
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if ((emv >> (zc * 4 + e)) & 1u) {
              const int64_t vidx =
                  ((int64_t)(2 * (z0 + zc) + oz) * a.G[1] + (2 * y + oy)) * a.G[0] + 2 * (x0 + e) + ox;
              o[e] = emission_channel(a.vol, (uint32_t)vidx, ch);
            }
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) flu[ch][zc][e] = fmaf(om, o[e], flu[ch][zc][e]);
        if ((valid >> (zc * 4)) & 1u) Vec4<T>::stream(lrow + ch * chstride + zc * plane, o[0], o[1], o[2], o[3]);
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&bar[kL0Stages + st]);  // this warp is done with the stage
  }
  if (!failed) {
#pragma unroll
    for (int zc = 0; zc < ZC; ++zc) {
      if (!((valid >> (zc * 4)) & 1u)) continue;
      float* f = a.fluence + (p0 + zc * plane) * 3;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        if (!RC_CHK(&f[3 * e + 2], kChkFluence) || !RC_CHK(&f[3 * e], kChkFluence)) continue;
        f[3 * e] = flu[0][zc][e];
        f[3 * e + 1] = flu[1][zc][e];
        f[3 * e + 2] = flu[2][zc][e];
      }
    }
  }
  if (failed && lane == 0) atomicExch(err, 1);
  if (failed && threadIdx.x == 0) {
    // thread 0 issued the copies up to direction it + S - 1 and waited for those
    // before it: let the others land before the block's shared memory goes
    for (int j = it; j < it + kL0Stages && j < total; ++j)
      (void)mbar_wait_bounded(&bar[j % kL0Stages], (uint32_t)(j / kL0Stages) & 1u);
  }
}

}  // namespace rcx
