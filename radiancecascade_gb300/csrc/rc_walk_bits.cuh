// rc_walk_bits.cuh -- bit-parallel cascade kernel (sm_103a).
//
// Why it works: probe centres are lattice points and the voxel walk is exact
// integer arithmetic, so for one direction every probe of a level visits the
// same sequence of voxel offsets from its own centre.  Probe m (per axis)
// tests voxel m*s + a, where a = s/2 + offset is shared by all probes; with
// phase phi = a mod s and coarse shift c = floor(a / s) that voxel is bit
// (m + c) of the level's phase-phi decimated opacity row.  One lane therefore
// walks 32 probes of an x row at once: per step it loads two 32-bit words,
// funnel-shifts them by c and masks the probes already finished.
//
// Decimated opacity of level i (spacing s = 2^l2s, M probes per axis,
// XW = ceil(Mx/32) words per coarse row):
//   mask[phz][phy][phx][zc][xw][yc]   bit b of word xw <-> coarse x = 32 xw + b
//   = opacity of voxel (xc*s + phx, yc*s + phy, zc*s + phz)
// y is fastest so that the 32 lanes of a warp (consecutive probe rows) read
// 32 consecutive words.
#pragma once

#include "rc_kernels.cuh"

namespace rcx {

constexpr int kTileRows = 32;      // probe rows (y, z) per block
constexpr int kTileDirs = 16;      // directions per block pass
constexpr int kBitsThreads = kTileRows * kTileDirs;
constexpr int kHitStride = 33;     // padded hit-record row (bank spread)
constexpr uint32_t kMiss = 0xFFFFFFFFu;
constexpr size_t kBitsSmem = sizeof(uint32_t) * kTileDirs * kTileRows * kHitStride;

struct MaskLevel {
  uint32_t* base;
  int32_t l2s;
  int32_t M[3];
  int32_t XW;
  int32_t pad;
};

struct MaskSet {
  int32_t n;
  int32_t pad;
  MaskLevel lv[kMaxCascades];
};

__device__ __forceinline__ int64_t mask_word(const MaskLevel& m, int phx, int phy, int phz, int xw, int yc, int zc) {
  const int64_t phase = ((((int64_t)phz << m.l2s) + phy) << m.l2s) + phx;
  return (phase * m.M[2] + zc) * ((int64_t)m.XW * m.M[1]) + (int64_t)xw * m.M[1] + yc;
}

// Updates every level's decimated opacity for the 32 voxels x = 32*wx + lane
// of row (y, z); `bits` is the warp's opacity ballot.  Each (level, phase) bit
// field belongs to exactly one warp, so clear-then-set is race free (a region
// processed twice writes the same values).
__device__ __forceinline__ void update_masks(const MaskSet& ms, int lane, int wx, int x, int y, int z, int Gx,
                                             uint32_t bits) {
  for (int i = 0; i < ms.n; ++i) {
    const MaskLevel& m = ms.lv[i];
    const int s = 1 << m.l2s;
    const int phy = y & (s - 1), yc = y >> m.l2s, phz = z & (s - 1), zc = z >> m.l2s;
    if (s < 32) {
      if (lane < s) {
        const int per = 32 >> m.l2s;  // coarse bits of this phase in the warp's 32 voxels
        uint32_t field = 0;
        for (int j = 0; j < per; ++j) field |= ((bits >> (lane + j * s)) & 1u) << j;
        const int xc0 = (32 * wx) >> m.l2s;
        uint32_t* w = m.base + mask_word(m, lane, phy, phz, xc0 >> 5, yc, zc);
        const int sh = xc0 & 31;
        const uint32_t fmask = (per == 32 ? 0xFFFFFFFFu : ((1u << per) - 1u)) << sh;
        atomicAnd(w, ~fmask);
        if (field) atomicOr(w, field << sh);
      }
    } else if (x < Gx) {
      const int xc = x >> m.l2s;
      uint32_t* w = m.base + mask_word(m, x & (s - 1), phy, phz, xc >> 5, yc, zc);
      const uint32_t b = 1u << (xc & 31);
      if ((bits >> lane) & 1u) atomicOr(w, b);
      else atomicAnd(w, ~b);
    }
  }
}

// Composed volume, full-resolution opacity and every level's decimated
// opacity over a list of regions (see k_compose for the composition rule).
__global__ void k_compose_masks(const uint2* __restrict__ base, uint2* __restrict__ vol, uint32_t* __restrict__ occ,
                                int Gx, int Gy, int Gz, int W, const QSphere* __restrict__ sph, int ns,
                                const Region* __restrict__ regs, const MaskSet ms) {
  const Region r = regs[blockIdx.y];
  const int64_t nw = r.w1 - r.w0, ny = r.y1 - r.y0, nz = r.z1 - r.z0;
  const int64_t words = nw * ny * nz;
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t wstride = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = warp0; w < words; w += wstride) {
    const int wx = r.w0 + (int)(w % nw);
    const int y = r.y0 + (int)((w / nw) % ny);
    const int z = r.z0 + (int)(w / (nw * ny));
    const int x = wx * 32 + lane;
    bool opaque = false;
    if (x < Gx) {
      const int64_t idx = ((int64_t)z * Gy + y) * Gx + x;
      uint2 v = base[idx];
      const int64_t px = (int64_t)(2 * x + 1) * 128, py = (int64_t)(2 * y + 1) * 128, pz = (int64_t)(2 * z + 1) * 128;
      for (int s = 0; s < ns; ++s) {
        const QSphere& S = sph[s];
        const int64_t dx = px - S.c[0], dy = py - S.c[1], dz = pz - S.c[2];
        if (dx > S.r || -dx > S.r || dy > S.r || -dy > S.r || dz > S.r || -dz > S.r) continue;
        if (dx * dx + dy * dy + dz * dz <= S.r * S.r) {
          v.x = (uint32_t)S.value.emission[0] | ((uint32_t)S.value.emission[1] << 16);
          v.y = (uint32_t)S.value.emission[2] | ((uint32_t)S.value.albedo_occ << 16);
        }
      }
      vol[idx] = v;
      opaque = (v.y >> 31) & 1u;
    }
    const unsigned bits = __ballot_sync(0xFFFFFFFFu, opaque);
    if (lane == 0) occ[((int64_t)z * Gy + y) * W + wx] = bits;
    update_masks(ms, lane, wx, x, y, z, Gx, bits);
  }
}

// Phase 1 of k_level_bits: walk the interval of direction `di` for the (up
// to) 32 probes of word `w` in probe row (my, mz); record the first opaque
// voxel of each probe in `hit[b]`.
__device__ __forceinline__ void walk_row_bits(const LevelArgs& a, const DirInfo& di, int w, int my, int mz,
                                              int TX, bool test_start, uint32_t* __restrict__ hit) {
  const int s = a.spacing, l2s = a.l2s, h = s >> 1;
  int ax = h + di.start_off[0], ay = h + di.start_off[1], az = h + di.start_off[2];
  int tx = di.first_T[0], ty = di.first_T[1], tz = di.first_T[2];
  const int sx = di.sgn[0], sy = di.sgn[1], sz = di.sgn[2];
  const int dx = di.step_T[0], dy = di.step_T[1], dz = di.step_T[2];
  const uint32_t valid = TX >= 32 ? 0xFFFFFFFFu : ((1u << TX) - 1u);
  uint32_t done = ~valid;
  const int Mx = a.M[0], My = a.M[1], Mz = a.M[2];
  int k = di.steps;
  bool pending_start = test_start;
  for (;;) {
    if (!pending_start) {
      if (k == 0) break;
      --k;
      if (tx <= ty && tx <= tz) {
        ax += sx;
        tx += dx;
      } else if (ty <= tz) {
        ay += sy;
        ty += dy;
      } else {
        az += sz;
        tz += dz;
      }
    }
    pending_start = false;
    const int zc = mz + (az >> l2s), yc = my + (ay >> l2s);
    if ((unsigned)zc >= (unsigned)Mz || (unsigned)yc >= (unsigned)My) break;  // the row left the grid
    const int X0 = 32 * w + (ax >> l2s);  // coarse x of bit 0
    // bits b with 0 <= X0 + b < Mx are still inside the grid
    const int blo = X0 < 0 ? -X0 : 0;
    const int bhi = Mx - X0;
    uint32_t inr = 0;
    if (blo < 32 && bhi > blo) {
      const uint32_t upto = bhi >= 32 ? 0xFFFFFFFFu : ((1u << bhi) - 1u);
      inr = upto & ~((1u << blo) - 1u);
    }
    done |= ~inr;
    if (done == 0xFFFFFFFFu) break;
    const int64_t phase = ((((int64_t)(az & (s - 1)) << l2s) + (ay & (s - 1))) << l2s) + (ax & (s - 1));
    const uint32_t* row = a.mask + (phase * Mz + zc) * ((int64_t)a.XW * My) + yc;
    const int q = X0 >> 5, sh = X0 & 31;
    const uint32_t lo = (q >= 0 && q < a.XW) ? __ldg(row + (int64_t)q * My) : 0u;
    const uint32_t hi = (q + 1 >= 0 && q + 1 < a.XW) ? __ldg(row + (int64_t)(q + 1) * My) : 0u;
    uint32_t nw = __funnelshift_r(lo, hi, sh) & ~done;
    if (nw) {
      done |= nw;
      const int64_t vyz = ((int64_t)(mz * s + az) * a.G[1] + (my * s + ay)) * a.G[0];
      do {
        const int b = __ffs(nw) - 1;
        nw &= nw - 1;
        hit[b] = (uint32_t)(vyz + (int64_t)(32 * w + b) * s + ax);
      } while (nw);
      if (done == 0xFFFFFFFFu) break;
    }
  }
}

// Bit-parallel cascade level.  Block = 32 probe rows x 16 directions.
// Phase 1: lane (row, direction) walks a 32-probe word and records hits in
// shared memory.  Phase 2: thread (probe) reads the records of all 16
// directions, takes the hit voxel's emission or (below the top level) the
// trilinear blend of the next level's child-averaged radiance, writes L_i
// coalesced along x, and reduces the 2x2-child average (levels >= 1) or the
// fluence (level 0) in registers.
template <typename T, bool L0, bool TOP>
__global__ void __launch_bounds__(kBitsThreads, 2) k_level_bits(const LevelArgs a) {
  extern __shared__ uint32_t s_hit[];
  const int tid = threadIdx.x;
  const int lrow = tid & 31;
  const int ldir = tid >> 5;
  int bid = blockIdx.x;
  const int w = bid % a.XW;
  bid /= a.XW;
  const int rowblk = bid % a.rowblocks;
  const int dgroup = bid / a.rowblocks;  // levels >= 1: group of 4 parent texels
  const int Mx = a.M[0], My = a.M[1];
  const int rows_total = a.M[1] * a.M[2];
  const int TX = min(Mx - 32 * w, 32);
  const int hn = a.n >> 1;
  const int ndir_pass = L0 ? min(a.ndirs, kTileDirs) : kTileDirs;
  const int npass = L0 ? (a.ndirs + kTileDirs - 1) / kTileDirs : 1;

  float flu[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
  for (int pass = 0; pass < npass; ++pass) {
    // ---- phase 1
    {
      uint32_t* hit = s_hit + (ldir * kTileRows + lrow) * kHitStride;
#pragma unroll 8
      for (int b = 0; b < 32; ++b) hit[b] = kMiss;
      const int r = rowblk * kTileRows + lrow;
      int d = -1;
      if (L0) {
        const int dd = pass * kTileDirs + ldir;
        if (ldir < ndir_pass && dd < a.ndirs) d = dd;
      } else {
        const int dp = dgroup * 4 + (ldir >> 2), c = ldir & 3;
        d = (2 * (dp / hn) + (c >> 1)) * a.n + 2 * (dp % hn) + (c & 1);
      }
      if (d >= 0 && r < rows_total) {
        const DirInfo di = a.dirs[d];
        walk_row_bits(a, di, w, r % My, r / My, TX, L0, hit);
      }
    }
    __syncthreads();
    // ---- phase 2
#pragma unroll 1
    for (int j = 0; j < 2; ++j) {
      const int t = tid + kBitsThreads * j;
      if (t >= TX * kTileRows) break;
      const int lr = t / TX, b = t - lr * TX;
      const int r = rowblk * kTileRows + lr;
      if (r >= rows_total) continue;
      const int mx = 32 * w + b, my = r % My, mz = r / My;
      const int64_t p = ((int64_t)mz * My + my) * Mx + mx;
      int tap_off[8];
      float tap_w[8];
      if (!TOP) {
        int q[3][2];
        float wt[3][2];
        const int m[3] = {mx, my, mz};
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          const int lo = (m[ax] - 1) >> 1;
          wt[ax][0] = (m[ax] & 1) ? 0.75f : 0.25f;
          wt[ax][1] = 1.0f - wt[ax][0];
          q[ax][0] = min(max(lo, 0), a.UM[ax] - 1);
          q[ax][1] = min(max(lo + 1, 0), a.UM[ax] - 1);
        }
#pragma unroll
        for (int tp = 0; tp < 8; ++tp) {
          const int ix = tp & 1, iy = (tp >> 1) & 1, iz = tp >> 2;
          tap_off[tp] = (q[2][iz] * a.UM[1] + q[1][iy]) * a.UM[0] + q[0][ix];
          tap_w[tp] = wt[2][iz] * wt[1][iy] * wt[0][ix];
        }
      }
      T* L = static_cast<T*>(a.L);
      float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
      for (int dl = 0; dl < ndir_pass; ++dl) {
        int d;
        if (L0) {
          d = pass * kTileDirs + dl;
          if (d >= a.ndirs) break;
        } else {
          const int dp = dgroup * 4 + (dl >> 2), c = dl & 3;
          d = (2 * (dp / hn) + (c >> 1)) * a.n + 2 * (dp % hn) + (c & 1);
        }
        const uint32_t rec = s_hit[(dl * kTileRows + lr) * kHitStride + b];
        float rv[3];
        if (rec != kMiss) {
          voxel_emission(a.vol, rec, rv);
        } else if (TOP) {
          rv[0] = rv[1] = rv[2] = 0.f;
        } else {
          const T* Au = static_cast<const T*>(a.A_up);
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            const T* src = Au + ((int64_t)ch * a.ndirs + d) * a.P_up;
            float sum = 0.f;
#pragma unroll
            for (int tp = 0; tp < 8; ++tp) sum = fmaf(tap_w[tp], Store<T>::load(src + tap_off[tp]), sum);
            rv[ch] = sum;
          }
        }
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) Store<T>::store(L + ((int64_t)ch * a.ndirs + d) * a.P + p, rv[ch]);
        if (L0) {
          const float om = a.dirs[d].omega;
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) flu[j][ch] = fmaf(om, rv[ch], flu[j][ch]);
        } else {
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) acc[ch] += rv[ch];
          if ((dl & 3) == 3) {
            T* A = static_cast<T*>(a.A_out);
            const int dp = dgroup * 4 + (dl >> 2);
            const int64_t npar = (int64_t)hn * hn;
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
              Store<T>::store(A + ((int64_t)ch * npar + dp) * a.P + p, 0.25f * acc[ch]);
              acc[ch] = 0.f;
            }
          }
        }
      }
    }
    __syncthreads();
  }
  if (L0) {
#pragma unroll 1
    for (int j = 0; j < 2; ++j) {
      const int t = tid + kBitsThreads * j;
      if (t >= TX * kTileRows) break;
      const int lr = t / TX, b = t - lr * TX;
      const int r = rowblk * kTileRows + lr;
      if (r >= rows_total) continue;
      const int64_t p = ((int64_t)(r / My) * My + r % My) * Mx + 32 * w + b;
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) a.fluence[p * 3 + ch] = flu[j][ch];
    }
  }
}

}  // namespace rcx
