// rc_mesh.cuh -- triangle-mesh voxelisation into the static scene (sm_103a).
//
// Vertex positions arrive in grid units rounded to 1/256 voxel (int32), so the
// triangle / voxel-box overlap is decided in exact integer arithmetic: the
// separating-axis test of Akenine-Moeller (2001, "Fast 3D triangle-box overlap
// testing") -- the 3 box axes, the triangle normal and the 9 edge x box-axis
// cross products -- with "touching" counted as overlap (closed boxes, so a
// wall lying exactly on a voxel face marks the voxels on both sides and the
// voxelisation is watertight).  With |coordinate| <= 2048 voxels (2^19 in
// 1/256 units) every product fits int64.
//
// Where triangles overlap, the later triangle wins: pass 1 takes the maximum
// (triangle index + 1) per voxel with atomicMax, pass 2 writes that
// triangle's material -- the same result whatever the thread order.
#pragma once

#include <stdint.h>

#include "rc_internal.h"

namespace rcx {

constexpr int64_t kMeshHalf = 128;  // half a voxel in 1/256 units

// Exact overlap of a triangle (vertices relative to the voxel centre, 1/256
// voxel units) with the closed voxel box [-128, 128]^3.
__host__ __device__ inline bool tri_voxel_overlap(const int64_t* a, const int64_t* b, const int64_t* c) {
  const int64_t h = kMeshHalf;
  // box face axes
  for (int k = 0; k < 3; ++k) {
    const int64_t lo = a[k] < b[k] ? (a[k] < c[k] ? a[k] : c[k]) : (b[k] < c[k] ? b[k] : c[k]);
    const int64_t hi = a[k] > b[k] ? (a[k] > c[k] ? a[k] : c[k]) : (b[k] > c[k] ? b[k] : c[k]);
    if (lo > h || hi < -h) return false;
  }
  const int64_t* v[3] = {a, b, c};
  int64_t e[3][3];
  for (int k = 0; k < 3; ++k) {
    e[0][k] = b[k] - a[k];
    e[1][k] = c[k] - b[k];
    e[2][k] = a[k] - c[k];
  }
  // triangle normal
  {
    const int64_t n0 = e[0][1] * e[1][2] - e[0][2] * e[1][1];
    const int64_t n1 = e[0][2] * e[1][0] - e[0][0] * e[1][2];
    const int64_t n2 = e[0][0] * e[1][1] - e[0][1] * e[1][0];
    const int64_t d = n0 * a[0] + n1 * a[1] + n2 * a[2];
    const int64_t r = h * ((n0 < 0 ? -n0 : n0) + (n1 < 0 ? -n1 : n1) + (n2 < 0 ? -n2 : n2));
    if (d > r || d < -r) return false;
  }
  // edge x box axis: axis u_j, edge e_i -> a = e_i x u_j
  for (int i = 0; i < 3; ++i) {
    const int64_t ex = e[i][0], ey = e[i][1], ez = e[i][2];
    for (int j = 0; j < 3; ++j) {
      int64_t ax, ay, az;
      if (j == 0) { ax = 0; ay = ez; az = -ey; }
      else if (j == 1) { ax = -ez; ay = 0; az = ex; }
      else { ax = ey; ay = -ex; az = 0; }
      int64_t lo = 0, hi = 0;
      for (int k = 0; k < 3; ++k) {
        const int64_t p = ax * v[k][0] + ay * v[k][1] + az * v[k][2];
        if (k == 0 || p < lo) lo = p;
        if (k == 0 || p > hi) hi = p;
      }
      const int64_t r = h * ((ax < 0 ? -ax : ax) + (ay < 0 ? -ay : ay) + (az < 0 ? -az : az));
      if (lo > r || hi < -r) return false;
    }
  }
  return true;
}

__host__ __device__ inline int64_t mesh_floor_div(int64_t a, int64_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// Voxel range [lo, hi] (inclusive) whose closed boxes can touch [mn, mx].
__host__ __device__ inline void mesh_voxel_range(int64_t mn, int64_t mx, int G, int& lo, int& hi) {
  // voxel x spans [256 x, 256 x + 256]
  int64_t l = mesh_floor_div(mn, 256);
  if (mn == l * 256) l -= 1;
  int64_t u = mesh_floor_div(mx, 256);
  lo = (int)(l < 0 ? 0 : l);
  hi = (int)(u > G - 1 ? G - 1 : u);
}

struct MeshArgs {
  const int32_t* verts;     // [nverts][3], 1/256 voxel units
  const uint32_t* indices;  // [ntris][3]
  int64_t ntris;
  uint32_t* owner;          // [Gz][Gy][Gx]: 1 + last overlapping triangle, 0 = none
  int32_t G[3];
  int32_t pad;
};

// One warp per triangle; lanes stride over the voxels of its bounding box.
static __global__ void k_mesh_owner(const __grid_constant__ MeshArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < a.ntris; t += warps) {
    int64_t v[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const uint32_t vi = __ldg(&a.indices[t * 3 + k]);
#pragma unroll
      for (int c = 0; c < 3; ++c) v[k][c] = __ldg(&a.verts[(int64_t)vi * 3 + c]);
    }
    int lo[3], hi[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t mn = min(v[0][c], min(v[1][c], v[2][c])), mx = max(v[0][c], max(v[1][c], v[2][c]));
      mesh_voxel_range(mn, mx, a.G[c], lo[c], hi[c]);
    }
    if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) continue;
    const int nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    const int64_t count = (int64_t)nx * ny * nz;
    for (int64_t q = lane; q < count; q += 32) {
      const int x = lo[0] + (int)(q % nx), y = lo[1] + (int)((q / nx) % ny), z = lo[2] + (int)(q / ((int64_t)nx * ny));
      const int64_t cx = 256 * (int64_t)x + kMeshHalf, cy = 256 * (int64_t)y + kMeshHalf, cz = 256 * (int64_t)z + kMeshHalf;
      int64_t p[3][3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        p[k][0] = v[k][0] - cx;
        p[k][1] = v[k][1] - cy;
        p[k][2] = v[k][2] - cz;
      }
      if (tri_voxel_overlap(p[0], p[1], p[2]))
        atomicMax(&a.owner[((int64_t)z * a.G[1] + y) * a.G[0] + x], (uint32_t)(t + 1));
    }
  }
}

// Materials of the owning triangles into the base volume; clears the owners.
static __global__ void k_mesh_materials(uint32_t* __restrict__ owner, const uint16_t* __restrict__ tri_material,
                                        const rc_voxel* __restrict__ materials, int nmaterials,
                                        uint2* __restrict__ base, int64_t nvox) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nvox; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t o = owner[i];
    uint2 v = make_uint2(0u, 0u);
    if (o) {
      int m = tri_material ? (int)tri_material[o - 1] : 0;
      m = m < nmaterials ? m : nmaterials - 1;
      v = *reinterpret_cast<const uint2*>(&materials[m]);
      owner[i] = 0u;
    }
    base[i] = v;
  }
}

}  // namespace rcx
