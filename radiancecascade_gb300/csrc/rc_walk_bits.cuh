// rc_walk_bits.cuh -- bit-parallel cascade kernel (sm_103a).
//
// Why it works: probe centres are lattice points and the voxel walk is exact
// integer arithmetic, so for one direction every probe of a level visits the
// same sequence of voxel offsets from its own centre.  Probe m (per axis)
// tests voxel m*s + a, where a = s/2 + offset is shared by all probes; with
// phase phi = a mod s and coarse shift c = floor(a / s) that voxel is coarse
// cell (m + c) of the level's phase-phi decimated opacity.  One lane walks the
// 32 probes of one 32-bit word at once: per step it loads two words,
// funnel-shifts them by the shared coarse shift and masks the probes that
// have finished or left the grid.
//
// Decimated opacity of level i (spacing s = 2^l2s, M probes per axis):
//   each (phase, zc) plane of the coarse grid is a row-major bit array with a
//   power-of-two row pitch Px >= Mx bits, packed into wpp = ceil(My*Px/32)
//   words:  mask[phz][phy][phx][zc][word];  bit g = yc*Px + xc of the plane
//   is the opacity of voxel (xc*s + phx, yc*s + phy, zc*s + phz).  Words are
//   uint2 pairs: .x the opacity bits, .y the emissive bits of the same voxels
//   (an emissive voxel is opaque), so a walk that hits a voxel knows from the
//   same load whether to record its index or kBlack.
// Every coarse shift (cx, cy) is a shift of the plane by cy*Px + cx bits, so
// any Mx uses all 32 bits of a lane.
#pragma once

#include <climits>

#include "rc_kernels.cuh"
#include "rc_tma.cuh"

namespace rcx {

constexpr int kTileSlots = 32;     // words (of 32 probes) per block tile
constexpr int kTileDirs = 8;       // directions per block pass
constexpr int kBitsThreads = kTileSlots * kTileDirs;
constexpr int kHitStride = 33;     // padded hit-record row (bank spread)
constexpr uint32_t kMiss = 0xFFFFFFFFu;   // no opaque voxel in the interval
constexpr uint32_t kBlack = 0xFFFFFFFEu;  // opaque voxel without emission
constexpr size_t kBitsSmem = sizeof(uint32_t) * kTileDirs * kTileSlots * kHitStride;

struct MaskLevel {
  uint2* base;  // (opacity, emissive) word pairs
  int32_t l2s;
  int32_t M[3];
  int32_t l2px;  // log2 of the plane row pitch Px
  int32_t wpp;   // words per (phase, zc) plane
};

struct MaskSet {
  int32_t n;
  int32_t pad;
  MaskLevel lv[kMaxCascades];
};

__device__ __forceinline__ int64_t plane_base(const MaskLevel& m, int phx, int phy, int phz, int zc) {
  const int64_t phase = ((((int64_t)phz << m.l2s) + phy) << m.l2s) + phx;
  return (phase * m.M[2] + zc) * (int64_t)m.wpp;
}

__device__ __forceinline__ int64_t plane_base_args(const LevelArgs& a, int phx, int phy, int phz, int zc) {
  const int64_t phase = ((((int64_t)phz << a.l2s) + phy) << a.l2s) + phx;
  return (phase * a.M[2] + zc) * (int64_t)a.wpp;
}

__device__ __forceinline__ uint32_t range_bits(int lo, int hi) {
  // bits [lo, hi) of a word, with lo, hi clamped to [0, 32]
  lo = max(lo, 0);
  hi = min(hi, 32);
  if (hi <= lo) return 0u;
  const uint32_t upto = hi >= 32 ? 0xFFFFFFFFu : ((1u << hi) - 1u);
  return upto & ~((1u << lo) - 1u);
}

// Updates every level's decimated opacity and emissive bits for the 32
// voxels x = 32*wx + lane of row (y, z); `bits` and `ebits` are the warp's
// opacity and emissive ballots.  The coarse cells a
// warp touches in one (level, phase) plane form one bit field that no other
// warp writes, so clear-then-set is race free (a region processed twice
// writes the same values).
__device__ __forceinline__ void update_masks(const MaskSet& ms, int lane, int wx, int x, int y, int z, int Gx,
                                             uint32_t bits, uint32_t ebits) {
  for (int i = 0; i < ms.n; ++i) {
    const MaskLevel& m = ms.lv[i];
    const int s = 1 << m.l2s;
    const int phy = y & (s - 1), yc = y >> m.l2s, phz = z & (s - 1), zc = z >> m.l2s;
    if (s < 32) {
      if (lane < s) {
        const int per = 32 >> m.l2s;  // coarse cells of this phase among the warp's 32 voxels
        const int xc0 = (32 * wx) >> m.l2s;
        const int width = min(per, m.M[0] - xc0);
        if (width > 0) {
          uint32_t field = 0, efield = 0;
          for (int j = 0; j < width; ++j) {
            field |= ((bits >> (lane + j * s)) & 1u) << j;
            efield |= ((ebits >> (lane + j * s)) & 1u) << j;
          }
          const int64_t g = ((int64_t)yc << m.l2px) + xc0;
          uint2* w2 = m.base + plane_base(m, lane, phy, phz, zc) + (g >> 5);
          // the pair as one 64-bit word: opacity in the low half (.x), emission in the high half
          unsigned long long* w = reinterpret_cast<unsigned long long*>(w2);
          const int sh = (int)(g & 31);
          const uint32_t fmask = (width == 32 ? 0xFFFFFFFFu : ((1u << width) - 1u)) << sh;
          const unsigned long long set =
              (unsigned long long)(field << sh) | ((unsigned long long)(efield << sh) << 32);
          if (RC_CHK(w2, kChkMask)) {
            atomicAnd(w, ~((unsigned long long)fmask | ((unsigned long long)fmask << 32)));
            if (set) atomicOr(w, set);
          }
        }
      }
    } else if (x < Gx) {
      const int xc = x >> m.l2s;
      const int64_t g = ((int64_t)yc << m.l2px) + xc;
      uint2* w2 = m.base + plane_base(m, x & (s - 1), phy, phz, zc) + (g >> 5);
      unsigned long long* w = reinterpret_cast<unsigned long long*>(w2);
      const unsigned long long b = 1ull << (g & 31), eb = b << 32;
      if (!RC_CHK(w2, kChkMask)) continue;
      const unsigned long long set = (((bits >> lane) & 1u) ? b : 0ull) | (((ebits >> lane) & 1u) ? eb : 0ull);
      if (set != (b | eb)) atomicAnd(w, ~((b | eb) & ~set));
      if (set) atomicOr(w, set);
    }
  }
}

// Composed volume, full-resolution opacity and emissive bits, and every
// level's decimated opacity over a list of regions.  A voxel whose centre is
// inside a sphere takes the value of the last such sphere of the list, else
// its base value.  Each region tests only its own list of spheres (ascending
// indices), or all of them.
// INL: spheres, regions and lists sit in the launch's parameter block (their
// reads need no range check: the block's size bounds them by construction).
template <bool INL>
static __device__ __forceinline__ void compose_masks_body(const uint2* __restrict__ base, uint2* __restrict__ vol, uint32_t* __restrict__ occ,
                                uint32_t* __restrict__ emis, int Gx, int Gy, int Gz, int W,
                                const QSphere* __restrict__ sph, int ns, const Region* __restrict__ regs,
                                const int32_t* __restrict__ slist, const MaskSet ms) {
  const Region r = regs[blockIdx.y];
  const int nt = r.sn < 0 ? ns : r.sn;
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
    bool opaque = false, emissive = false;
    const int64_t idx = ((int64_t)z * Gy + y) * Gx + x;
    uint2 v = make_uint2(0u, 0u);
    if (x < Gx) {
      v = RC_CHK(&base[idx], kChkVolume) ? base[idx] : make_uint2(0u, 0u);
      const int64_t px = (int64_t)(2 * x + 1) * 128, py = (int64_t)(2 * y + 1) * 128, pz = (int64_t)(2 * z + 1) * 128;
      for (int k = 0; k < nt; ++k) {
        const int si = r.sn < 0 ? k : ((INL || RC_CHK(slist + r.s0 + k, kChkSpheres)) ? slist[r.s0 + k] : 0);
        if (!INL && !RC_CHK(&sph[si], kChkSpheres)) continue;
        const QSphere& S = sph[si];
        const int64_t dx = px - S.c[0], dy = py - S.c[1], dz = pz - S.c[2];
        if (dx > S.r || -dx > S.r || dy > S.r || -dy > S.r || dz > S.r || -dz > S.r) continue;
        if (dx * dx + dy * dy + dz * dz <= S.r * S.r) {
          v.x = (uint32_t)S.value.emission[0] | ((uint32_t)S.value.emission[1] << 16);
          v.y = (uint32_t)S.value.emission[2] | ((uint32_t)S.value.albedo_occ << 16);
        }
      }
      opaque = (v.y >> 31) & 1u;
      emissive = opaque && (((v.x & 0x7FFF7FFFu) | (v.y & 0x7FFFu)) != 0u);
    }
    // everything above reads only the static base and the spheres: with a
    // programmatic launch it ran while the previous frame's last kernel,
    // which reads the volume and bit planes, finished; the writes wait for it
    grid_dep_wait();
    if (x < Gx && RC_CHK(&vol[idx], kChkVolume)) vol[idx] = v;
    const unsigned bits = __ballot_sync(0xFFFFFFFFu, opaque);
    const unsigned ebits = __ballot_sync(0xFFFFFFFFu, emissive);
    if (lane == 0 && RC_CHK(&occ[((int64_t)z * Gy + y) * W + wx], kChkOccupancy) &&
        RC_CHK(&emis[((int64_t)z * Gy + y) * W + wx], kChkOccupancy)) {
      occ[((int64_t)z * Gy + y) * W + wx] = bits;
      emis[((int64_t)z * Gy + y) * W + wx] = ebits;
    }
    update_masks(ms, lane, wx, x, y, z, Gx, bits, ebits);
  }
}

static __global__ void k_compose_masks(const uint2* __restrict__ base, uint2* __restrict__ vol, uint32_t* __restrict__ occ,
                                uint32_t* __restrict__ emis, int Gx, int Gy, int Gz, int W,
                                const QSphere* __restrict__ sph, int ns, const Region* __restrict__ regs,
                                const int32_t* __restrict__ slist, const MaskSet ms) {
  compose_masks_body<false>(base, vol, occ, emis, Gx, Gy, Gz, W, sph, ns, regs, slist, ms);
}

// The same update with the spheres, regions and sphere lists carried in the
// launch's own parameters (an update small enough needs no host-to-device
// copy): spheres at byte 0, regions at reg_off, lists at list_off.
constexpr int kComposeInlineBytes = 4096;
struct ComposeInline {
  alignas(16) unsigned char b[kComposeInlineBytes];
};
static __global__ void k_compose_masks_inline(const uint2* __restrict__ base, uint2* __restrict__ vol,
                                              uint32_t* __restrict__ occ, uint32_t* __restrict__ emis, int Gx, int Gy,
                                              int Gz, int W, int ns, int reg_off, int list_off, const MaskSet ms,
                                              const __grid_constant__ ComposeInline in) {
  compose_masks_body<true>(base, vol, occ, emis, Gx, Gy, Gz, W, reinterpret_cast<const QSphere*>(in.b), ns,
                     reinterpret_cast<const Region*>(in.b + reg_off), reinterpret_cast<const int32_t*>(in.b + list_off),
                     ms);
}

// Geometry of one block's tile of probe words.
//   wide levels (Px >= 32): tile = 2 planes x 16 words; slot u -> plane u / 16,
//     word wt + u % 16.  16 words are 512/Px whole rows of the plane.
//   narrow levels (Px < 32): tile = TZ planes x TW words (TZ * TW <= 32).
struct Tile {
  int z0, w0;     // first plane, first word
  int TZ, TW;     // planes, words per plane in the tile
};

__device__ __forceinline__ Tile tile_of(const LevelArgs& a, int tile) {
  Tile t;
  if (a.l2px >= 5) {
    t.TZ = 2;
    t.TW = 16;
    const int wt = (a.wpp + 15) / 16;  // tiles per plane pair
    t.z0 = 2 * (tile / wt);
    t.w0 = 16 * (tile % wt);
  } else {
    t.TW = min(a.wpp, 32);
    t.TZ = max(1, 32 / t.TW);
    const int wt = (a.wpp + t.TW - 1) / t.TW;
    t.z0 = t.TZ * (tile / wt);
    t.w0 = t.TW * (tile % wt);
  }
  return t;
}

// Phase 1: walk the interval of direction `di` for the 32 probes of plane
// word `wl` in coarse plane `zl`; record each probe's first opaque voxel in
// hit[0..31] (every entry is written: the voxel index of an emissive hit at
// once, kBlack or kMiss for the others when the walk ends).
// The voxel sequence does not depend on what is loaded, so the walk runs in
// batches of kWalkBatch steps: the mask words of a whole batch are requested
// before the first of them is tested.  Level 0's interval is one voxel long,
// so it walks in batches of 2; the others in batches of 4.
template <int kWalkBatch>
__device__ __forceinline__ void walk_word(const LevelArgs& a, const DirInfo& di, int zl, int wl, bool test_start,
                                          uint32_t* __restrict__ hit) {
  const int s = a.spacing, l2s = a.l2s, h = s >> 1;
  const int Mx = a.M[0], My = a.M[1], Mz = a.M[2];
  const int l2px = a.l2px, Px = 1 << l2px;
  const bool wide = l2px >= 5;
  const int g0 = wl << 5;  // plane bit of this word's bit 0
  const int wy0 = g0 >> l2px, wx0 = g0 & (Px - 1);
  // probes that exist: x < Mx, y < My
  uint32_t valid;
  if (wide) {
    valid = wy0 < My ? range_bits(0, Mx - wx0) : 0u;
  } else {
    valid = range_bits(0, Mx) * a.rep;  // the row pattern replicated over the word's 32/Px rows
    valid &= range_bits(0, (My - wy0) * Px);
  }
  uint32_t done = ~valid, hits = 0u, ehits = 0u;
  const uint2* zbase = a.mask + (int64_t)zl * a.wpp;
  const int phase_stride = Mz * a.wpp;  // a level's decimated words fit 32 bits (checked on the host)
  int ax = h + di.start_off[0], ay = h + di.start_off[1], az = h + di.start_off[2];
  int tx = di.first_T[0], ty = di.first_T[1], tz = di.first_T[2];
  const int sx = di.sgn[0], sy = di.sgn[1], sz = di.sgn[2];
  const int dx = di.step_T[0], dy = di.step_T[1], dz = di.step_T[2];
  int k = di.steps;
  bool first = test_start;
  // wide rows: the in-grid probes of a cell column cx (every lane of the warp
  // walks the same offsets, so the recompute on a change of cx is uniform)
  int pcx = INT_MIN;
  uint32_t rx = 0u;
  for (; valid != 0u;) {
    int bx_[kWalkBatch], by_[kWalkBatch], bz_[kWalkBatch];
    uint2 lo_[kWalkBatch], hi_[kWalkBatch];
    bool ok_[kWalkBatch];
#pragma unroll
    for (int u = 0; u < kWalkBatch; ++u) {
      bool step_ok;
      if (first) {
        first = false;
        step_ok = true;
      } else if (k > 0) {
        --k;
        // branch-free choice of the axis with the nearest crossing (x, then y, then z on ties)
        const bool px_ = (tx <= ty) & (tx <= tz);
        const bool py_ = !px_ & (ty <= tz);
        const bool pz_ = !px_ & !py_;
        ax += px_ ? sx : 0;
        tx += px_ ? dx : 0;
        ay += py_ ? sy : 0;
        ty += py_ ? dy : 0;
        az += pz_ ? sz : 0;
        tz += pz_ ? dz : 0;
        step_ok = true;
      } else {
        step_ok = false;
      }
      bx_[u] = ax;
      by_[u] = ay;
      bz_[u] = az;
      const int zc = zl + (az >> l2s);
      const bool zin = step_ok && (unsigned)zc < (unsigned)Mz;
      ok_[u] = step_ok;
      const int phase = ((((az & (s - 1)) << l2s) + (ay & (s - 1))) << l2s) + (ax & (s - 1));
      const uint2* plane = zbase + (phase * phase_stride + (az >> l2s) * a.wpp);
      const int gs = g0 + (ay >> l2s) * Px + (ax >> l2s);
      const int q = gs >> 5;
      lo_[u] = (zin && (unsigned)q < (unsigned)a.wpp && RC_CHK(plane + q, kChkMask)) ? __ldg(plane + q)
                                                                                     : make_uint2(0u, 0u);
      hi_[u] = (zin && (unsigned)(q + 1) < (unsigned)a.wpp && RC_CHK(plane + q + 1, kChkMask)) ? __ldg(plane + q + 1)
                                                                                                 : make_uint2(0u, 0u);
    }
    // Branch-free over the batch: a step past the interval or outside the
    // grid in z (both final: the walk is monotone) loaded zeros and hits
    // nothing, and so does every step after all probes are done.
    bool stop = false;
#pragma unroll
    for (int u = 0; u < kWalkBatch; ++u) {
      const int cz = bz_[u] >> l2s, cy = by_[u] >> l2s, cx = bx_[u] >> l2s;
      stop |= !ok_[u] || (unsigned)(zl + cz) >= (unsigned)Mz;  // every probe of the word left the grid
      // probes whose cell (x + cx, y + cy) is still inside the grid
      uint32_t inr;
      if (wide) {
        if (cx != pcx) {
          pcx = cx;
          rx = range_bits(-cx - wx0, Mx - cx - wx0);
        }
        inr = ((unsigned)(wy0 + cy) < (unsigned)My) ? rx : 0u;
      } else {
        inr = range_bits(max(0, -cx), min(Mx, Mx - cx)) * a.rep;
        inr &= range_bits((-cy - wy0) * Px, (My - cy - wy0) * Px);
      }
      done |= ~inr;
      const int gs = g0 + cy * Px + cx;
      const uint32_t nw = __funnelshift_r(lo_[u].x, hi_[u].x, gs & 31) & ~done;
      done |= nw;
      hits |= nw;
      {
        uint32_t ew = __funnelshift_r(lo_[u].y, hi_[u].y, gs & 31) & nw;
        if (ew) {  // emissive hits (rare): the voxel's index
          ehits |= ew;
          const int vz = (zl << l2s) + bz_[u];
          do {
            const int b = __ffs(ew) - 1;
            ew &= ew - 1;
            const int g = g0 + b;
            const int vx = ((g & (Px - 1)) << l2s) + bx_[u], vy = ((g >> l2px) << l2s) + by_[u];
            const int64_t row = (int64_t)vz * a.G[1] + vy;
            if (RC_CHK(&hit[b], kChkShared)) hit[b] = (uint32_t)(row * a.G[0] + vx);
          } while (ew);
        }
      }
    }
    if (stop || done == 0xFFFFFFFFu) break;
  }
  // the other probes: opaque without emission, or no hit (probes that do not exist included)
#pragma unroll 8
  for (int b = 0; b < 32; ++b)
    if (!((ehits >> b) & 1u) && RC_CHK(&hit[b], kChkShared)) hit[b] = ((hits >> b) & 1u) ? kBlack : kMiss;
}


// The y blends (child rows ey = 0, 1) of one channel's three z-blended parent
// rows, then the x blend through the lanes' columns (lane l holds parent
// column (l + 1) / 2 - 1 + ...: src_near / src_far are the weight-3/4 and
// weight-1/4 columns of the lane's child).  All lanes take part.  s0, s1:
// each child's final scale, 1/64 (the three blends' factor) where its ray
// missed and 0 where it hit, so that no select follows.
__device__ __forceinline__ void yx_blend(const float zv[3], int src_near, int src_far, float s0, float s1, float& out0,
                                         float& out1) {
  const float v0 = fmaf(3.f, zv[1], zv[0]);
  const float v1 = fmaf(3.f, zv[1], zv[2]);
  const float n0 = __shfl_sync(0xFFFFFFFFu, v0, src_near), f0 = __shfl_sync(0xFFFFFFFFu, v0, src_far);
  const float n1 = __shfl_sync(0xFFFFFFFFu, v1, src_near), f1 = __shfl_sync(0xFFFFFFFFu, v1, src_far);
  out0 = fmaf(3.f, n0, f0) * s0;
  out1 = fmaf(3.f, n1, f1) * s1;
}

// Direction of block-local slot dl (0..15) in pass `pass`, or -1.
template <bool L0>
__device__ __forceinline__ int block_dir(const LevelArgs& a, int pass, int dgroup, int dl) {
  if (L0) {
    const int d = pass * kTileDirs + dl;
    return d < a.ndirs ? d : -1;
  }
  const int hn = a.n >> 1;
  const int dp = dgroup * 2 + (dl >> 2), c = dl & 3;  // two parent texels per block
  return (2 * (dp / hn) + (c >> 1)) * a.n + 2 * (dp % hn) + (c & 1);
}

// Directions staged ahead in k_level_bits_up: thread 0 issues the first
// kUpStages copies before the walk phase, once the previous level's kernel
// has completed (with a programmatic launch the other warps' walks, which
// read only the scene, run meanwhile).
constexpr int kUpStages = 4;

// Bytes of the next level's box staged per direction (3 planes x up_rows
// rows x UM[0] texels of 4 values: every channel in one copy), and its
// 128-byte aligned stride.
__host__ __device__ __forceinline__ uint32_t up_tile_bytes(int up_rows, int umx, int elem) {
  return 12u * (uint32_t)up_rows * (uint32_t)umx * (uint32_t)elem;
}
__host__ __device__ __forceinline__ uint32_t up_tile_stride(int up_rows, int umx, int elem) {
  return (up_tile_bytes(up_rows, umx, elem) + 127u) & ~127u;
}

// Bit-parallel cascade level for wide levels (>= 32 probes per row).  Block =
// one tile of 32 probe words x 8 directions (256 threads).
// Phase 1: warp = direction, lane = word: walk 32 probes per lane, record the
//   first opaque voxel of each probe (or kMiss / kBlack) in shared memory.
// Phase 2, WIDE levels (>= 32 probes per row): warp = (32 x-children x 2 y x
//   2 z block, all 8 directions).  Below the top level, missing rays take the
//   trilinear blend of the next level's child-averaged radiance: each lane
//   loads one parent column (3 x 3 values per channel), interpolates z and y
//   in registers and x through warp shuffles.
// Level 0 reduces the fluence; other levels write the 2x2-child averages.
// level_bits_block is one block's share (block index `bid`, shared memory
// s_hit of kBitsSmem bytes); CG: the next level was written during the same
// launch (see load_up).
// TM: the next level's values come from shared memory instead: per direction
// one TMA copy of the block's parent box (all UM[0] columns, up_rows rows, 3
// planes, every channel) through `tmap` into s_up (128-byte aligned,
// kUpStages stage tiles, then kUpStages "full" mbarriers the copies complete
// and kUpStages "empty" ones each warp arrives at when it is done with a
// stage; thread 0 refills a stage once every warp has arrived, so the warps
// never wait for one another at a block barrier).  Only thread 0, which
// issues the copies, waits for the launch that wrote them (grid_dep_wait);
// the block then lets the next level's launch start.
template <typename T, bool L0, bool TOP, bool CG, bool TM = false>
__device__ __forceinline__ void level_bits_block(const LevelArgs& a, int bid, uint32_t* s_hit,
                                                 const CUtensorMap* tmap = nullptr, unsigned char* s_up = nullptr,
                                                 int* err = nullptr) {
  static_assert(!TM || (!L0 && !TOP), "the staged merge serves levels between cascade 0 and the top");
  constexpr bool WIDE = true;  // narrow levels walk through the work queue (rc_walk_queue.cuh)
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tile_id = bid % a.tiles;
  const int dgroup = bid / a.tiles;
  const Tile t = tile_of(a, tile_id);
  const int Mx = a.M[0], My = a.M[1], Mz = a.M[2];
  const int npass = L0 ? (a.ndirs + kTileDirs - 1) / kTileDirs : 1;
  T* L = static_cast<T*>(a.L);
  const T* Au = static_cast<const T*>(a.A_up);

  // wide: lane's child block (x, y0 + ey, z0 + ez), ey, ez in {0, 1}.  Element
  // offsets fit 32 bits (3 * dirs * probes < 2^31 is checked on the host).
  const int unit = warp;
  const int cl2 = a.l2px - 5;
  const int c = WIDE ? (unit & ((1 << cl2) - 1)) : 0;
  const int y0 = WIDE ? ((t.w0 << 5) >> a.l2px) + 2 * (unit >> cl2) : 0;
  const int x = 32 * c + lane;
  const int p0 = (t.z0 * My + y0) * Mx + x;
  const int cstep[4] = {0, Mx, My * Mx, My * Mx + Mx};  // child i = (ez = i >> 1, ey = i & 1)
  const int slot0 = (y0 << cl2) + c - t.w0;
  unsigned okmask = 0;  // bit i = child i exists
  if (WIDE) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (x < Mx && y0 + (i & 1) < My && t.z0 + (i >> 1) < Mz) okmask |= 1u << i;
  }
  // wide: parent column of this lane (lanes 0..17 load); offsets of the 3 x 3
  // parents (z-1, z, z+1) x (y-1, y, y+1), clamped at the border
  const int qx = min(max(16 * c - 1 + lane, 0), a.UM[0] - 1);
  int aoff[9];
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int jj = 0; jj < 3; ++jj)
      aoff[k * 3 + jj] = (min(max(t.z0 / 2 - 1 + k, 0), a.UM[2] - 1) * a.UM[1] +
                          min(max(y0 / 2 - 1 + jj, 0), a.UM[1] - 1)) * a.UM[0] + qx;
  const bool ploader = lane < 18;
  // x blend from the parent columns (lane + 1) / 2 and the next one: the
  // weight-3/4 column first (the lower one for odd lanes).  Every 1D blend is
  // a + 3 b = 4 (a/4 + 3b/4); the factor 64 of the three is divided out once.
  const int src_lo = (lane + 1) >> 1;
  const int src_near = (lane & 1) ? src_lo : src_lo + 1, src_far = (lane & 1) ? src_lo + 1 : src_lo;

  // TM: the block's parent box starts at (0, ys, zs); the clamped rows and
  // planes above fall inside it (up_rows = rows of the tile / 2 + 2)
  int soff[9];
  T* up_tiles = nullptr;
  uint64_t* ubar = nullptr;
  uint32_t tstride = 0;
  if (TM) {
    const int BY = a.up_rows;
    const int y0min = (t.w0 << 5) >> a.l2px;
    const int ys = max(0, min(y0min / 2 - 1, a.UM[1] - BY));
    const int zs = max(0, min(t.z0 / 2 - 1, a.UM[2] - 3));
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int jj = 0; jj < 3; ++jj)
        soff[k * 3 + jj] = ((min(max(t.z0 / 2 - 1 + k, 0), a.UM[2] - 1) - zs) * BY +
                            (min(max(y0 / 2 - 1 + jj, 0), a.UM[1] - 1) - ys)) * a.UM[0] + qx;
    tstride = up_tile_stride(BY, a.UM[0], (int)sizeof(T));
    up_tiles = reinterpret_cast<T*>(s_up);
    ubar = reinterpret_cast<uint64_t*>(s_up + kUpStages * tstride);
    if (tid == 0) {
#pragma unroll
      for (int st = 0; st < kUpStages; ++st) {
        mbar_init(&ubar[st], 1);
        mbar_init(&ubar[kUpStages + st], kBitsThreads / 32);  // empty: one arrival per warp
      }
      mbar_fence_init();
    }
    __syncthreads();
  }
  // TM: the walk phase reads only the scene; the next level's values are
  // staged by thread 0 once the launch that wrote them has completed
  auto stage_first = [&]() {
    if (TM && tid == 0) {
      grid_dep_wait();
      const int BY = a.up_rows;
      const int ys = max(0, min(((t.w0 << 5) >> a.l2px) / 2 - 1, a.UM[1] - BY));
      const int zs = max(0, min(t.z0 / 2 - 1, a.UM[2] - 3));
      const uint32_t tbytes = up_tile_bytes(BY, a.UM[0], (int)sizeof(T));
      for (int k = 0; k < kUpStages && k < 8; ++k) {
        const int d = block_dir<L0>(a, 0, dgroup, k);
        mbar_arrive_expect_tx(&ubar[k], tbytes);
        tma_load_rgb4<T>(reinterpret_cast<unsigned char*>(up_tiles) + k * tstride, tmap, ys, d * a.UM[2] + zs,
                         &ubar[k]);
      }
    }
  };

  stage_first();  // thread 0 waits for the previous launch, the other warps start walking

  float acc[4][3];
#pragma unroll
  for (int i = 0; i < 4; ++i) acc[i][0] = acc[i][1] = acc[i][2] = 0.f;

  for (int pass = 0; pass < npass; ++pass) {
    // ---- phase 1: lane = word of the tile, warp = direction
    {
      uint32_t* hit = s_hit + (warp * kTileSlots + lane) * kHitStride;
      const int d = block_dir<L0>(a, pass, dgroup, warp);
      const int zl = t.z0 + lane / t.TW, wl = t.w0 + lane % t.TW;
      if (d >= 0 && lane < t.TZ * t.TW && zl < Mz && wl < a.wpp) {
        const DirInfo di = a.dirs[d];
        walk_word<L0 ? 2 : 4>(a, di, zl, wl, L0, hit);  // writes all 32 entries
      } else {
#pragma unroll 8
        for (int b = 0; b < 32; ++b) hit[b] = kMiss;
      }
    }
    __syncthreads();
    if (TM && pass == 0) grid_dep_release();
    // ---- phase 2
    if (WIDE) {
#pragma unroll 1
      for (int k = 0; k < 8; ++k) {
        const int dl = k;
        const int d = block_dir<L0>(a, pass, dgroup, dl);
        if (d < 0) break;
        const int ust = k % kUpStages;
        if (TM && !mbar_wait_bounded(&ubar[ust], (uint32_t)(k / kUpStages) & 1u) && lane == 0) atomicExch(err, 3);
        uint32_t rec[4];
        unsigned missm = 0, emism = 0;
        const uint32_t* hrow = s_hit + (dl * kTileSlots + slot0) * kHitStride + lane;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const uint32_t* hp = &hrow[((i >> 1) * 16 + ((i & 1) << cl2)) * kHitStride];
          rec[i] = ((okmask >> i) & 1u) && RC_CHK(hp, kChkShared) ? *hp : kBlack;
          missm |= (rec[i] == kMiss) << i;
          emism |= (rec[i] < kBlack) << i;
        }
        const bool merge = !TOP && __any_sync(0xFFFFFFFFu, missm != 0);
        const float om = L0 ? a.dirs[d].omega : 0.f;
        float val[4][3];
        float mv[3][4];  // [channel][child i = ez * 2 + ey]
        float scl[4];    // 1/64 for a child whose ray missed, else 0 (mv stays 0 without a merge)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          scl[i] = ((missm >> i) & 1u) ? (1.f / 64.f) : 0.f;
          mv[0][i] = mv[1][i] = mv[2][i] = 0.f;
        }
        if (merge && TM) {
          // staged taps (q = plane * 3 + row): every channel in one shared load;
          // per child plane the middle parent plane (weight 3/4) and plane 0 or 2
          const T* tile = reinterpret_cast<const T*>(reinterpret_cast<const unsigned char*>(up_tiles) + ust * tstride);
#pragma unroll
          for (int ez = 0; ez < 2; ++ez) {
            float3 pm[3], po[3];
#pragma unroll
            for (int jy = 0; jy < 3; ++jy) {
              pm[jy] = ploader ? lds_rgb(tile + 4 * soff[3 + jy]) : make_float3(0.f, 0.f, 0.f);
              po[jy] = ploader ? lds_rgb(tile + 4 * soff[ez == 0 ? jy : 6 + jy]) : make_float3(0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int ch = 0; ch < 3; ++ch) {
              float zv[3];
#pragma unroll
              for (int jy = 0; jy < 3; ++jy) {
                const float m = ch == 0 ? pm[jy].x : ch == 1 ? pm[jy].y : pm[jy].z;
                const float o = ch == 0 ? po[jy].x : ch == 1 ? po[jy].y : po[jy].z;
                zv[jy] = fmaf(3.f, m, o);
              }
              yx_blend(zv, src_near, src_far, scl[ez * 2], scl[ez * 2 + 1], mv[ch][ez * 2], mv[ch][ez * 2 + 1]);
            }
          }
        } else if (!TM && merge) {
          // taps from global memory, one channel at a time (value (d, probe q, ch) at Au[4 (d P_up + q) + ch])
#pragma unroll
          for (int ch = 0; ch < 3; ++ch) {
            const T* src = Au + (int64_t)d * a.P_up * 4 + ch;
            float av[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) av[q] = ploader ? load_up<T, CG>(src + 4 * aoff[q]) : 0.f;
#pragma unroll
            for (int ez = 0; ez < 2; ++ez) {
              float zv[3];
#pragma unroll
              for (int jy = 0; jy < 3; ++jy) zv[jy] = fmaf(3.f, av[3 + jy], ez == 0 ? av[jy] : av[6 + jy]);
              yx_blend(zv, src_near, src_far, scl[ez * 2], scl[ez * 2 + 1], mv[ch][ez * 2], mv[ch][ez * 2 + 1]);
            }
          }
        }
#pragma unroll
        for (int ch = 0; ch < 3; ++ch)
#pragma unroll
          for (int i = 0; i < 4; ++i) val[i][ch] = mv[ch][i];
        if (emism) {  // emissive hits are rare: patch them in
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if ((emism >> i) & 1u) voxel_emission(a.vol, rec[i], val[i]);
        }
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
          T* dst = L + (ch * a.ndirs + d) * (int)a.P + p0;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            if ((okmask >> i) & 1u) Store<T>::stream(dst + cstep[i], val[i][ch]);
            acc[i][ch] = L0 ? fmaf(om, val[i][ch], acc[i][ch]) : acc[i][ch] + val[i][ch];
          }
        }
        if (!L0 && (k & 3) == 3) {
          const int dp = dgroup * 2 + (dl >> 2);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            if ((okmask >> i) & 1u)
              store_avg<T>(a, dp, p0 + cstep[i], 0.25f * acc[i][0], 0.25f * acc[i][1], 0.25f * acc[i][2]);
            acc[i][0] = acc[i][1] = acc[i][2] = 0.f;
          }
        }
        if (TM) {
          // this warp is done with stage ust; thread 0 refills it with direction
          // k + kUpStages once every warp is
          __syncwarp();
          if (lane == 0) mbar_arrive(&ubar[kUpStages + ust]);
          if (tid == 0 && k + kUpStages < 8 &&
              !mbar_wait_bounded(&ubar[kUpStages + ust], (uint32_t)(k / kUpStages) & 1u))
            atomicExch(err, 3);
          if (tid == 0 && k + kUpStages < 8) {
            const int kn = k + kUpStages, dn = block_dir<L0>(a, pass, dgroup, kn);
            const int BY = a.up_rows;
            const int ys = max(0, min(((t.w0 << 5) >> a.l2px) / 2 - 1, a.UM[1] - BY));
            const int zs = max(0, min(t.z0 / 2 - 1, a.UM[2] - 3));
            fence_proxy_async();
            mbar_arrive_expect_tx(&ubar[ust], up_tile_bytes(BY, a.UM[0], (int)sizeof(T)));
            tma_load_rgb4<T>(reinterpret_cast<unsigned char*>(up_tiles) + ust * tstride, tmap, ys,
                             dn * a.UM[2] + zs, &ubar[ust]);
          }
        }
      }
    }
    __syncthreads();
  }
  if (TM && tid == 0) {
    // every copy was waited for above unless a wait ran out: wait (bounded)
    // for the last phase of each stage before the block's shared memory goes
    for (int st = 0; st < kUpStages && st < 8; ++st) mbar_wait_bounded(&ubar[st], (uint32_t)((7 - st) / kUpStages) & 1u);
  }

  if (L0) {
    if (WIDE) {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        if (!((okmask >> i) & 1u)) continue;
        const int64_t p = p0 + cstep[i];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch)
          if (RC_CHK(&a.fluence[p * 3 + ch], kChkFluence)) a.fluence[p * 3 + ch] = acc[i][ch];
      }
    }
  }
}

template <typename T, bool L0, bool TOP>
__global__ void __launch_bounds__(kBitsThreads, 3) k_level_bits(const __grid_constant__ LevelArgs a) {
  extern __shared__ uint32_t s_hit[];
  level_bits_block<T, L0, TOP, false>(a, blockIdx.x, s_hit);
}

// A wide level between cascade 0 and the top with the next level's values
// staged by TMA (tmap over A_up: texels of 4 values, x = UM[0], y = UM[1],
// z = direction x UM[2]; box UM[0] x up_rows x 3 texels, see tma_load_rgb4).
// Shared memory: up to 127 bytes to align, the hit records, then the stages
// and their barriers.
constexpr size_t kBitsHitBytes = (kBitsSmem + 127) & ~(size_t)127;
__host__ __device__ constexpr size_t bits_up_smem(uint32_t tile_stride) {
  return 128 + kBitsHitBytes + (size_t)kUpStages * tile_stride + 16 * kUpStages;
}

template <typename T>
__global__ void __launch_bounds__(kBitsThreads, 3)
    k_level_bits_up(const __grid_constant__ LevelArgs a, const __grid_constant__ CUtensorMap tmap, int* err) {
  extern __shared__ __align__(128) unsigned char smem_bits_up[];
  unsigned char* base = smem_bits_up + ((128u - (smem_u32(smem_bits_up) & 127u)) & 127u);
  level_bits_block<T, false, false, false, true>(a, blockIdx.x, reinterpret_cast<uint32_t*>(base), &tmap,
                                                 base + kBitsHitBytes, err);
}

}  // namespace rcx
