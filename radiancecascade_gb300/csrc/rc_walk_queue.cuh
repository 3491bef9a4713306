// rc_walk_queue.cuh -- load-balanced interval walks for the narrow cascade
// levels (fewer than 32 probes per row), and their merge kernel (sm_103a).
//
// At a narrow level one lane still walks a 32-probe word of the decimated
// opacity (see rc_walk_bits.cuh), but the level has few probes and long
// intervals, so the walks of one direction vary widely in length: a warp that
// owns a direction runs as long as its slowest word.  Here every
// (level, direction, word) is an item of one work queue over all narrow
// levels; a lane that finishes takes the next item, so lanes stay busy.  The
// walks depend only on the scene, never on another level, so all narrow
// levels walk in one launch; their first-hit records go to a small global
// buffer (L2-resident) that k_level_merge reads in the usual top-down order.
//
// Record layout of a level: rec[d][slot][32], slot = zc * wpp + word, one
// 32-bit entry per probe: the hit voxel's linear index (emissive hit), kBlack
// (opaque voxel without emission) or kMiss.
#pragma once

#include <stdlib.h>

#include <algorithm>

#include "rc_walk_bits.cuh"

namespace rcx {

struct QueueLevel {
  const uint2* mask;  // decimated (opacity, emissive) word pairs
  const DirInfo* dirs;
  uint32_t* rec;
  int64_t item_begin;  // first queue item of this level
  int32_t slots;       // M[2] * wpp words per direction
  int32_t l2s, l2px, wpp;
  int32_t M[3];
  uint32_t rep;
  int32_t test_start;  // level 0: the probe's own voxel belongs to the interval
  int32_t level;       // cascade index
  // Step tables (or null: the walk runs its own DDA): for direction d the
  // steps step_begin[d] .. step_begin[d + 1] - 1 of `steps`, each the voxel
  // offset of one walk step split as x = phase index ((pz << l2s) + py) << l2s
  // + px and y = the coarse cell (cx, cy, cz) as three signed bytes.  A table
  // ends where every probe of the level has left the grid on some axis.
  const uint2* steps;
  const int32_t* step_begin;
  // Optional selections (the learned form walks only what it needs):
  // word_on (null: every slot) -- a slot whose byte is 0 holds no walk;
  // dsel (null: every direction, items d * slots + slot) -- the level's items
  // are slot * dsel_n + k for the dsel_n directions
  // dsel[(dsel_start + k) mod dsel_len], so a warp's 32 items share a word.
  const uint8_t* word_on;
  const int32_t* dsel;
  int32_t dsel_len, dsel_start, dsel_n;
  int32_t pad;
};

// Direction and slot of item r (counted from the level's first item).
__device__ __forceinline__ void queue_item(const QueueLevel& L, int64_t r, int& d, int& slot) {
  if (L.dsel) {
    slot = (int)(r / L.dsel_n);
    int j = L.dsel_start + (int)(r - (int64_t)slot * L.dsel_n);
    if (j >= L.dsel_len) j -= L.dsel_len;
    d = __ldg(L.dsel + j);
  } else {
    d = (int)(r / L.slots);
    slot = (int)(r - (int64_t)d * L.slots);
  }
}

struct QueueArgs {
  unsigned long long* counter;  // zeroed before every launch
  int64_t total;                // items over all levels
  int32_t G[3];
  int32_t W;
  int32_t n;
  int32_t pad;
  QueueLevel lv[kMaxCascades];
};

// The records of one item when its walk ends: emissive hits already hold
// their voxel index (written at the hit); every other entry gets kBlack (hit
// without emission) or kMiss, four entries per 16-byte store.  rec is 128-byte
// aligned (32 entries per item from an aligned base); entries of probes that
// do not exist get kMiss.
__device__ __forceinline__ void write_records(uint32_t* rec, uint32_t valid, uint32_t hits, uint32_t ehits) {
  uint4* r4 = reinterpret_cast<uint4*>(rec);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    if (!((valid >> (4 * j)) & 0xFu)) continue;
    const uint32_t h4 = (hits >> (4 * j)) & 0xFu, e4 = (ehits >> (4 * j)) & 0xFu;
    uint4 old = make_uint4(0u, 0u, 0u, 0u);
    if (e4 && RC_CHK(&r4[j], kChkRecord)) old = r4[j];  // this lane's own writes
    uint4 v;
    v.x = (e4 & 1u) ? old.x : (h4 & 1u) ? kBlack : kMiss;
    v.y = (e4 & 2u) ? old.y : (h4 & 2u) ? kBlack : kMiss;
    v.z = (e4 & 4u) ? old.z : (h4 & 4u) ? kBlack : kMiss;
    v.w = (e4 & 8u) ? old.w : (h4 & 8u) ? kBlack : kMiss;
    if (RC_CHK(&r4[j], kChkRecord)) r4[j] = v;
  }
}

// One lane's walk of one queue item, advanced kBatch steps at a time.  The
// voxel offset a = (cell c, phase ph) per axis is kept split (a = c s + ph):
// a step moves one phase by +-1 and only when it wraps does the coarse cell
// change -- and with it the set of probes still inside the grid in x and y
// (inr) and whether the z plane exists (zin), which are therefore recomputed
// only then.
struct Walker {
  const uint2* mask;
  uint32_t* rec;
  int l2s, l2px, wpp, Mx, My, Mz;
  uint32_t rep;
  int zl, g0, wy0, wx0;
  uint32_t valid, done, hits, ehits;
  int ax, ay, az, tx, ty, tz, k;
  int sx, sy, sz, dx, dy, dz;
  int px, py, pz, cx, cy, cz;  // phase and coarse cell of the current offset
  uint32_t inr;                // probes whose current voxel is inside the grid in x and y
  bool zin;                    // the current z plane lies inside the grid
  bool first;

  __device__ __forceinline__ void cell_changed() {
    const int Px = 1 << l2px;
    if (l2px >= 5) {
      inr = ((unsigned)(wy0 + cy) < (unsigned)My) ? range_bits(-cx - wx0, Mx - cx - wx0) : 0u;
    } else {
      inr = range_bits(max(0, -cx), min(Mx, Mx - cx)) * rep;
      inr &= range_bits((-cy - wy0) * Px, (My - cy - wy0) * Px);
    }
    zin = (unsigned)(zl + cz) < (unsigned)Mz;
  }

  // Returns false when the item holds no probe.
  __device__ __forceinline__ bool init(const QueueArgs& q, int64_t item) {
    int li = 0;
    while (li + 1 < q.n && item >= q.lv[li + 1].item_begin) ++li;
    const QueueLevel& L = q.lv[li];
    int d, slot;
    queue_item(L, item - L.item_begin, d, slot);
    mask = L.mask;
    l2s = L.l2s;
    l2px = L.l2px;
    wpp = L.wpp;
    Mx = L.M[0];
    My = L.M[1];
    Mz = L.M[2];
    rep = L.rep;
    if (L.word_on && !__ldg(L.word_on + slot)) return false;
    zl = slot / wpp;
    const int wl = slot - zl * wpp;
    g0 = wl << 5;
    const int Px = 1 << l2px;
    wy0 = g0 >> l2px;
    wx0 = g0 & (Px - 1);
    if (l2px >= 5) {
      valid = wy0 < My ? range_bits(0, Mx - wx0) : 0u;
    } else {
      valid = range_bits(0, Mx) * rep;
      valid &= range_bits(0, (My - wy0) * Px);
    }
    if (valid == 0u) return false;
    rec = L.rec + ((int64_t)d * L.slots + slot) * 32;
    done = ~valid;
    hits = 0u;
    ehits = 0u;
    const DirInfo di = L.dirs[d];
    const int h = 1 << (l2s - 1);
    ax = h + di.start_off[0];
    ay = h + di.start_off[1];
    az = h + di.start_off[2];
    tx = di.first_T[0];
    ty = di.first_T[1];
    tz = di.first_T[2];
    sx = di.sgn[0];
    sy = di.sgn[1];
    sz = di.sgn[2];
    dx = di.step_T[0];
    dy = di.step_T[1];
    dz = di.step_T[2];
    k = di.steps;
    first = L.test_start != 0;
    const int sm = (1 << l2s) - 1;
    px = ax & sm;
    py = ay & sm;
    pz = az & sm;
    cx = ax >> l2s;
    cy = ay >> l2s;
    cz = az >> l2s;
    cell_changed();
    return true;
  }

  // Walks up to kBatch steps; returns true when the item is finished.
  template <int kBatch>
  __device__ __forceinline__ bool batch(const QueueArgs& q) {
    const int sm = (1 << l2s) - 1, Px = 1 << l2px;
    const int mzw = Mz * wpp;  // words per phase
    int bx_[kBatch], by_[kBatch], bz_[kBatch], gs_[kBatch];
    uint2 lo_[kBatch], hi_[kBatch];
    uint32_t inr_[kBatch];
    bool ok_[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      bool step_ok;
      if (first) {
        first = false;
        step_ok = true;
      } else if (k > 0) {
        --k;
        const bool px_ = (tx <= ty) & (tx <= tz);
        const bool py_ = !px_ & (ty <= tz);
        const bool pz_ = !px_ & !py_;
        const int ex = px_ ? sx : 0, ey = py_ ? sy : 0, ez = pz_ ? sz : 0;
        ax += ex;
        ay += ey;
        az += ez;
        tx += px_ ? dx : 0;
        ty += py_ ? dy : 0;
        tz += pz_ ? dz : 0;
        const int nx = px + ex, ny = py + ey, nz = pz + ez;
        const int wx = nx >> l2s, wy = ny >> l2s, wz = nz >> l2s;  // -1, 0 or +1
        px = nx & sm;
        py = ny & sm;
        pz = nz & sm;
        if ((wx | wy | wz) != 0) {  // crossed into another coarse cell (every s-th step on an axis)
          cx += wx;
          cy += wy;
          cz += wz;
          cell_changed();
        }
        step_ok = true;
      } else {
        step_ok = false;
      }
      bx_[u] = ax;
      by_[u] = ay;
      bz_[u] = az;
      ok_[u] = step_ok && zin;
      inr_[u] = step_ok ? inr : 0u;
      const int gs = g0 + cy * Px + cx;
      gs_[u] = gs;
      const int q0 = gs >> 5;
      const uint2* plane = mask + ((((pz << l2s) + py) << l2s) + px) * mzw + (zl + cz) * wpp;
      lo_[u] = (ok_[u] && (unsigned)q0 < (unsigned)wpp && RC_CHK(plane + q0, kChkMask)) ? __ldg(plane + q0)
                                                                                       : make_uint2(0u, 0u);
      hi_[u] = (ok_[u] && (unsigned)(q0 + 1) < (unsigned)wpp && RC_CHK(plane + q0 + 1, kChkMask))
                   ? __ldg(plane + q0 + 1)
                   : make_uint2(0u, 0u);
    }
    // Branch-free over the batch, as in TableWalker::batch.
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      done |= ~inr_[u];
      const uint32_t nw = __funnelshift_r(lo_[u].x, hi_[u].x, gs_[u] & 31) & ~done;
      done |= nw;
      hits |= nw;
      {
        uint32_t ew = __funnelshift_r(lo_[u].y, hi_[u].y, gs_[u] & 31) & nw;
        if (ew) {  // emissive hits (rare): the voxel's index
          ehits |= ew;
          const int vz = (zl << l2s) + bz_[u];
          do {
            const int b = __ffs(ew) - 1;
            ew &= ew - 1;
            const int g = g0 + b;
            const int vx = ((g & (Px - 1)) << l2s) + bx_[u], vy = ((g >> l2px) << l2s) + by_[u];
            const int64_t row = (int64_t)vz * q.G[1] + vy;
            if (RC_CHK(&rec[b], kChkRecord)) rec[b] = (uint32_t)(row * q.G[0] + vx);
          } while (ew);
        }
      }
    }
    return !ok_[kBatch - 1] || done == 0xFFFFFFFFu;
  }

  __device__ __forceinline__ void finish() { write_records(rec, valid, hits, ehits); }
};

// The same walk driven by a level's step table instead of its own DDA: a step
// is one 8-byte load (shared by the lanes on the same direction) and the
// per-cell state changes only when the table's coarse cell does.
struct TableWalker {
  const uint2* mask;
  uint32_t* rec;
  const uint2* st;  // next step
  int n;            // steps left
  int l2s, l2px, wpp, Mx, My, Mz, mzw;
  uint32_t rep;
  int zl, g0, wy0, wx0;
  uint32_t valid, done, hits, ehits;
  uint32_t cell;   // packed coarse cell of the current step
  int qoff;        // (zl + cz) * wpp + the first of the two words holding the probes' cells
  int sh;          // bit of that word where the word's probe 0 falls
  uint32_t inr;
  bool zin, lo_en, hi_en;  // the plane exists; and the first / second word

  __device__ __forceinline__ void set_cell(uint32_t packed) {
    cell = packed;
    const int cx = (int)(int8_t)(packed & 0xFFu), cy = (int)(int8_t)((packed >> 8) & 0xFFu),
              cz = (int)(int8_t)((packed >> 16) & 0xFFu);
    const int Px = 1 << l2px;
    if (l2px >= 5) {
      inr = ((unsigned)(wy0 + cy) < (unsigned)My) ? range_bits(-cx - wx0, Mx - cx - wx0) : 0u;
    } else {
      inr = range_bits(max(0, -cx), min(Mx, Mx - cx)) * rep;
      inr &= range_bits((-cy - wy0) * Px, (My - cy - wy0) * Px);
    }
    zin = (unsigned)(zl + cz) < (unsigned)Mz;
    const int gs = g0 + cy * Px + cx, q0 = gs >> 5;
    sh = gs & 31;
    qoff = (zl + cz) * wpp + q0;
    lo_en = zin && (unsigned)q0 < (unsigned)wpp;
    hi_en = zin && (unsigned)(q0 + 1) < (unsigned)wpp;
  }

  // Returns false when the item holds no probe.
  __device__ __forceinline__ bool init(const QueueArgs& q, int64_t item) {
    int li = 0;
    while (li + 1 < q.n && item >= q.lv[li + 1].item_begin) ++li;
    const QueueLevel& L = q.lv[li];
    int d, slot;
    queue_item(L, item - L.item_begin, d, slot);
    mask = L.mask;
    l2s = L.l2s;
    l2px = L.l2px;
    wpp = L.wpp;
    Mx = L.M[0];
    My = L.M[1];
    Mz = L.M[2];
    mzw = Mz * wpp;
    rep = L.rep;
    if (L.word_on && !__ldg(L.word_on + slot)) return false;
    zl = slot / wpp;
    const int wl = slot - zl * wpp;
    g0 = wl << 5;
    const int Px = 1 << l2px;
    wy0 = g0 >> l2px;
    wx0 = g0 & (Px - 1);
    if (l2px >= 5) {
      valid = wy0 < My ? range_bits(0, Mx - wx0) : 0u;
    } else {
      valid = range_bits(0, Mx) * rep;
      valid &= range_bits(0, (My - wy0) * Px);
    }
    if (valid == 0u) return false;
    rec = L.rec + ((int64_t)d * L.slots + slot) * 32;
    done = ~valid;
    hits = 0u;
    ehits = 0u;
    const int b0 = __ldg(L.step_begin + d);
    st = L.steps + b0;
    n = __ldg(L.step_begin + d + 1) - b0;
    set_cell(0x80808080u);  // no real cell: the first step sets it
    return true;
  }

  // Walks up to kBatch steps; returns true when the item is finished.
  template <int kBatch>
  __device__ __forceinline__ bool batch(const QueueArgs& q) {
    const int sm = (1 << l2s) - 1, Px = 1 << l2px;
    uint2 e[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) e[u] = u < n ? (RC_CHK(st + u, kChkTable) ? __ldg(st + u) : make_uint2(0u, 0u)) : make_uint2(0u, 0u);
    int gs_[kBatch];  // the shift of each step's word pair
    uint2 lo_[kBatch], hi_[kBatch];
    uint32_t inr_[kBatch];
    bool ok_[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const bool step_ok = u < n;
      if (step_ok && e[u].y != cell) set_cell(e[u].y);
      ok_[u] = step_ok && zin;
      inr_[u] = step_ok ? inr : 0u;
      gs_[u] = sh;
      const uint2* wp = mask + ((int)e[u].x * mzw + qoff);  // a level's words fit 32 bits
      lo_[u] = (step_ok && lo_en && RC_CHK(wp, kChkMask)) ? __ldg(wp) : make_uint2(0u, 0u);
      hi_[u] = (step_ok && hi_en && RC_CHK(wp + 1, kChkMask)) ? __ldg(wp + 1) : make_uint2(0u, 0u);
    }
    st += kBatch;
    n -= kBatch;
    // Branch-free over the batch: a step that is not ok (past the table's end,
    // or outside the grid in z -- both final, the walk is monotone) loaded
    // zeros and hits nothing, and steps after every probe is done hit
    // nothing either, so no step needs its own exit test.
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      done |= ~inr_[u];
      const uint32_t nw = __funnelshift_r(lo_[u].x, hi_[u].x, gs_[u] & 31) & ~done;
      done |= nw;
      hits |= nw;
      {
        uint32_t ew = __funnelshift_r(lo_[u].y, hi_[u].y, gs_[u] & 31) & nw;
        if (ew) {  // emissive hits (rare): the voxel's index, from the step's table entry
          ehits |= ew;
          const uint32_t ph = e[u].x, pc = e[u].y;
          const int bx = ((int)(int8_t)(pc & 0xFFu) << l2s) + (int)(ph & sm);
          const int by = ((int)(int8_t)((pc >> 8) & 0xFFu) << l2s) + (int)((ph >> l2s) & sm);
          const int bz = ((int)(int8_t)((pc >> 16) & 0xFFu) << l2s) + (int)(ph >> (2 * l2s));
          const int vz = (zl << l2s) + bz;
          do {
            const int b = __ffs(ew) - 1;
            ew &= ew - 1;
            const int g = g0 + b;
            const int vx = ((g & (Px - 1)) << l2s) + bx, vy = ((g >> l2px) << l2s) + by;
            const int64_t row = (int64_t)vz * q.G[1] + vy;
            if (RC_CHK(&rec[b], kChkRecord)) rec[b] = (uint32_t)(row * q.G[0] + vx);
          } while (ew);
        }
      }
    }
    return !ok_[kBatch - 1] || done == 0xFFFFFFFFu || n <= 0;
  }

  __device__ __forceinline__ void finish() { write_records(rec, valid, hits, ehits); }
};

constexpr int kQueueThreads = 256;

// ---------------------------------------------------------------------------
// Cooperative table walk: a group of G lanes walks ONE item, lane j taking
// step j of every G consecutive steps of the direction's table, so a walk of
// k steps takes k / G dependent rounds instead of k.  Along a ray a probe
// that has left the grid never comes back (the grid is convex), so the steps
// of a round can be tested independently: a probe's first hit is the lowest
// lane whose step hits it (exclusive OR-scan over the group), a probe outside
// the grid at a step has no hit at any later step, and a step outside the
// grid in z or past the table's end ends the walk.  Same records as
// TableWalker, bit for bit.
// ---------------------------------------------------------------------------
template <int G>
struct CoopWalker {
  const uint2* mask;
  uint32_t* rec;
  const uint2* st;
  int n;  // steps left
  int l2s, l2px, wpp, Mx, My, Mz, mzw;
  uint32_t rep;
  int zl, g0, wy0, wx0;
  uint32_t valid, done, hits;

  __device__ __forceinline__ bool init(const QueueArgs& q, int64_t item) {
    int li = 0;
    while (li + 1 < q.n && item >= q.lv[li + 1].item_begin) ++li;
    const QueueLevel& L = q.lv[li];
    int d, slot;
    queue_item(L, item - L.item_begin, d, slot);
    mask = L.mask;
    l2s = L.l2s;
    l2px = L.l2px;
    wpp = L.wpp;
    Mx = L.M[0];
    My = L.M[1];
    Mz = L.M[2];
    mzw = Mz * wpp;
    rep = L.rep;
    if (L.word_on && !__ldg(L.word_on + slot)) return false;
    zl = slot / wpp;
    const int wl = slot - zl * wpp;
    g0 = wl << 5;
    const int Px = 1 << l2px;
    wy0 = g0 >> l2px;
    wx0 = g0 & (Px - 1);
    if (l2px >= 5) {
      valid = wy0 < My ? range_bits(0, Mx - wx0) : 0u;
    } else {
      valid = range_bits(0, Mx) * rep;
      valid &= range_bits(0, (My - wy0) * Px);
    }
    if (valid == 0u) return false;
    rec = L.rec + ((int64_t)d * L.slots + slot) * 32;
    done = ~valid;
    hits = 0u;
    const int b0 = __ldg(L.step_begin + d);
    st = L.steps + b0;
    n = __ldg(L.step_begin + d + 1) - b0;
    return true;
  }

  // One round of G steps; every lane of the warp calls it (inactive groups
  // with active = false).  Returns true when this group's item is finished.
  __device__ __forceinline__ bool round(const QueueArgs& q, bool active, int sub) {
    uint32_t h = 0u, he = 0u, out = 0u;  // he: emissive bits of the step's voxels
    bool stop = false;
    uint32_t ph = 0u, pc = 0u;
    if (active) {
      const bool step_ok = sub < n;
      const uint2 e = (step_ok && RC_CHK(st + sub, kChkTable)) ? __ldg(st + sub) : make_uint2(0u, 0u);
      ph = e.x;
      pc = e.y;
      const int cx = (int)(int8_t)(pc & 0xFFu), cy = (int)(int8_t)((pc >> 8) & 0xFFu),
                cz = (int)(int8_t)((pc >> 16) & 0xFFu);
      const int Px = 1 << l2px;
      uint32_t inr;
      if (l2px >= 5) {
        inr = ((unsigned)(wy0 + cy) < (unsigned)My) ? range_bits(-cx - wx0, Mx - cx - wx0) : 0u;
      } else {
        inr = range_bits(max(0, -cx), min(Mx, Mx - cx)) * rep;
        inr &= range_bits((-cy - wy0) * Px, (My - cy - wy0) * Px);
      }
      const bool ok = step_ok && (unsigned)(zl + cz) < (unsigned)Mz;
      stop = !ok;
      if (ok) {
        const int gs = g0 + cy * Px + cx;
        const int q0 = gs >> 5;
        const uint2* plane = mask + (int64_t)ph * mzw + (int64_t)(zl + cz) * wpp;
        const uint2 lo =
            (unsigned)q0 < (unsigned)wpp && RC_CHK(plane + q0, kChkMask) ? __ldg(plane + q0) : make_uint2(0u, 0u);
        const uint2 hi = (unsigned)(q0 + 1) < (unsigned)wpp && RC_CHK(plane + q0 + 1, kChkMask) ? __ldg(plane + q0 + 1)
                                                                                              : make_uint2(0u, 0u);
        h = __funnelshift_r(lo.x, hi.x, gs & 31) & inr & ~done;
        he = __funnelshift_r(lo.y, hi.y, gs & 31);
        out = ~inr;
      }
    }
    // first hit per probe: the lowest lane of the group whose step hits it
    uint32_t incl = h;
#pragma unroll
    for (int o = 1; o < G; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o, G);
      if (sub >= o) incl |= y;
    }
    uint32_t before = __shfl_up_sync(0xFFFFFFFFu, incl, 1, G);
    if (sub == 0) before = 0u;
    uint32_t nw = h & ~before;
    if (nw) {
      const int sm = (1 << l2s) - 1, Px = 1 << l2px;
      const int bx = ((int)(int8_t)(pc & 0xFFu) << l2s) + (int)(ph & sm);
      const int by = ((int)(int8_t)((pc >> 8) & 0xFFu) << l2s) + (int)((ph >> l2s) & sm);
      const int bz = ((int)(int8_t)((pc >> 16) & 0xFFu) << l2s) + (int)(ph >> (2 * l2s));
      const int vz = (zl << l2s) + bz;
      do {
        const int b = __ffs(nw) - 1;
        nw &= nw - 1;
        const int g = g0 + b;
        const int vx = ((g & (Px - 1)) << l2s) + bx, vy = ((g >> l2px) << l2s) + by;
        const int64_t row = (int64_t)vz * q.G[1] + vy;
        if (RC_CHK(&rec[b], kChkRecord)) rec[b] = ((he >> b) & 1u) ? (uint32_t)(row * q.G[0] + vx) : kBlack;
      } while (nw);
    }
    // group totals: probes hit, probes out of the grid, walk ended
    uint32_t all = incl, gone = out;
    int ended = stop ? 1 : 0;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      all |= __shfl_xor_sync(0xFFFFFFFFu, all, o, G);
      gone |= __shfl_xor_sync(0xFFFFFFFFu, gone, o, G);
      ended |= __shfl_xor_sync(0xFFFFFFFFu, ended, o, G);
    }
    if (!active) return true;
    hits |= all;
    done |= all | gone;
    st += G;
    n -= G;
    return ended || n <= 0 || done == 0xFFFFFFFFu;
  }

  // Records of the probes without a hit; the group's lanes share the writes.
  __device__ __forceinline__ void finish(int sub) {
    const uint32_t m = valid & ~hits;
    for (int b = sub; b < 32; b += G)
      if (((m >> b) & 1u) && RC_CHK(&rec[b], kChkRecord)) rec[b] = kMiss;
  }
};

// Groups of G lanes per item, 32 / G items per warp at a time from *counter.
template <int G>
__device__ __forceinline__ void walk_groups_coop(const QueueArgs& q, unsigned long long* counter, int64_t end) {
  static_assert(G == 2 || G == 4 || G == 8 || G == 16 || G == 32, "group of 2, 4, 8, 16 or 32 lanes");
  const int lane = threadIdx.x & 31, sub = lane & (G - 1), grp = lane / G;
  CoopWalker<G> w;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(counter, (unsigned long long)(32 / G));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if ((int64_t)base >= end) break;
    const int64_t item = (int64_t)base + grp;
    bool active = item < end && w.init(q, item);
    while (__any_sync(0xFFFFFFFFu, active)) {
      const bool fin = w.round(q, active, sub);
      if (active && fin) {
        w.finish(sub);
        active = false;
      }
    }
  }
}

template <int G>
static __global__ void __launch_bounds__(kQueueThreads, 4) k_walk_queue_coop(const __grid_constant__ QueueArgs q) {
  grid_dep_wait();
  grid_dep_release();
  walk_groups_coop<G>(q, q.counter, q.total);
}


// Every warp takes 32 consecutive queue items at a time (from *counter, a
// global or shared counter, up to `end`) and walks them in step: lanes of one
// direction share the table entries and load neighbouring words; the warp
// takes its next 32 items when all of its lanes are done.  (Refilling lanes
// one by one instead left two thirds of the lanes idle per instruction.)
template <int kBatch, typename W>
__device__ __forceinline__ void walk_groups(const QueueArgs& q, unsigned long long* counter, int64_t end) {
  const int lane = threadIdx.x & 31;
  W w;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(counter, 32ull);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if ((int64_t)base >= end) break;
    const int64_t item = (int64_t)base + lane;
    bool active = item < end && w.init(q, item);
    while (__any_sync(0xFFFFFFFFu, active))
      if (active && w.template batch<kBatch>(q)) {
        w.finish();
        active = false;
      }
  }
}

static __global__ void __launch_bounds__(kQueueThreads) k_walk_queue(const __grid_constant__ QueueArgs q) {
  walk_groups<4, Walker>(q, q.counter, q.total);
}

// The walks of levels that all have step tables: 10 steps per load batch, so
// a lane has 20 mask loads in flight before it tests the first, at 2
// blocks/SM (124 registers, no spills) -- the walks wait on those loads, and
// more loads in flight per lane pay more than more resident warps (4
// steps at 4 blocks/SM took 134 us where this takes 116 at 256^3).  The
// walks are launched in the ordinary way (the wait returns at once) and let
// the top level's merge launch early: it waits for their records.
constexpr int kTableWalkBatch = 10;
static __global__ void __launch_bounds__(kQueueThreads, 2) k_walk_queue_tab(const __grid_constant__ QueueArgs q) {
  grid_dep_wait();
  grid_dep_release();
  walk_groups<kTableWalkBatch, TableWalker>(q, q.counter, q.total);
}

// Lanes per item of the step-table walk.  With more resident lanes than
// items, the walks' dependent steps (not the lanes) bound the launch, so G
// lanes share an item: G = the largest power of two <= resident lanes /
// items, at most 32 (1: k_walk_queue_tab, one lane per item).  RC_WALK_GROUP
// = 1, 2, 4, 8, 16 or 32 fixes it.
inline int walk_group(int64_t items, int64_t resident_blocks) {
  const char* e = getenv("RC_WALK_GROUP");
  if (e) {
    const int v = atoi(e);
    if (v == 1 || v == 2 || v == 4 || v == 8 || v == 16 || v == 32) return v;
  }
  const int64_t lanes = resident_blocks * kQueueThreads;
  int g = 1;
  while (g < 32 && (int64_t)(2 * g) * items <= lanes) g *= 2;
  return g;
}

// Blocks of the cooperative walk that fit the GPU at once (every G shares
// the launch bounds and about the same registers).
inline int64_t coop_walk_resident() {
  static const int64_t r = [] {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_queue_coop<8>, kQueueThreads, 0) != cudaSuccess) {
      (void)cudaGetLastError();
      return (int64_t)152 * 4;
    }
    return (int64_t)std::max(1, sms * per_sm);
  }();
  return r;
}

// The step-table walk of `q` (its counter already zeroed, q.total items):
// enough blocks for G lanes per item, at most the blocks that fit the GPU at
// once (`resident` for one lane per item, the cooperative kernels' own
// figure otherwise; every warp takes items until the queue is empty).
inline void launch_table_walk(const QueueArgs& q, int64_t resident, cudaStream_t s) {
  const int64_t coop_resident = coop_walk_resident();
  const int g = walk_group(q.total, coop_resident);
  const int64_t cap = g > 1 ? coop_resident : resident;
  const unsigned blocks = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((q.total * g + kQueueThreads - 1) / kQueueThreads, cap));
  switch (g) {
    case 2: k_walk_queue_coop<2><<<blocks, kQueueThreads, 0, s>>>(q); break;
    case 4: k_walk_queue_coop<4><<<blocks, kQueueThreads, 0, s>>>(q); break;
    case 8: k_walk_queue_coop<8><<<blocks, kQueueThreads, 0, s>>>(q); break;
    case 16: k_walk_queue_coop<16><<<blocks, kQueueThreads, 0, s>>>(q); break;
    case 32: k_walk_queue_coop<32><<<blocks, kQueueThreads, 0, s>>>(q); break;
    default: k_walk_queue_tab<<<blocks, kQueueThreads, 0, s>>>(q); break;
  }
}

// Merge of a narrow level from its walk records, probe p: parent texels
// 2 dpair and 2 dpair + 1 (eight child directions), or at level 0 every
// direction and the fluence.  Rays without a hit take the trilinear blend of
// the 8 nearest next-level probes of the child-averaged radiance (child index
// m sits at parent coordinate m/2 - 1/4, clamped).  CG: the records and the
// next level were written during the same launch (see load_up).
template <typename T, bool L0, bool TOP, bool CG>
__device__ __forceinline__ void merge_probe(const LevelArgs& a, const uint32_t* __restrict__ rec, int slots,
                                            int64_t p, int dpair) {
  const int Mx = a.M[0], My = a.M[1];
  // probe coordinates in 32-bit arithmetic (a level has fewer than 2^31 probes)
  const uint32_t pu = (uint32_t)p, rowi = pu / (uint32_t)Mx;
  const int mx = (int)(pu - rowi * (uint32_t)Mx), mz = (int)(rowi / (uint32_t)My), my = (int)(rowi - (uint32_t)mz * (uint32_t)My);
  const int g = (my << a.l2px) + mx;
  const int64_t rbase = (int64_t)(mz * a.wpp + (g >> 5)) * 32 + (g & 31);
  int tap_off[8];
  float tap_w[8];
  if (!TOP) {
    int qq[3][2];
    float wt[3][2];
    const int m[3] = {mx, my, mz};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      const int lo = (m[ax] - 1) >> 1;
      wt[ax][0] = (m[ax] & 1) ? 0.75f : 0.25f;
      wt[ax][1] = 1.0f - wt[ax][0];
      qq[ax][0] = min(max(lo, 0), a.UM[ax] - 1);
      qq[ax][1] = min(max(lo + 1, 0), a.UM[ax] - 1);
    }
#pragma unroll
    for (int tp = 0; tp < 8; ++tp) {
      const int ix = tp & 1, iy = (tp >> 1) & 1, iz = tp >> 2;
      tap_off[tp] = (qq[2][iz] * a.UM[1] + qq[1][iy]) * a.UM[0] + qq[0][ix];
      tap_w[tp] = wt[2][iz] * wt[1][iy] * wt[0][ix];
    }
  }
  T* L = static_cast<T*>(a.L);
  const T* Au = static_cast<const T*>(a.A_up);
  const int hn = a.n >> 1;
  float acc[3] = {0.f, 0.f, 0.f};
  auto dir_of = [&](int dl) {
    if (L0) return dl;
    const int dp = dpair * 2 + (dl >> 2), c = dl & 3;
    return (2 * (dp / hn) + (c >> 1)) * a.n + 2 * (dp % hn) + (c & 1);
  };
  auto record = [&](int d) -> uint32_t {
    const uint32_t* rp = &rec[(int64_t)d * slots * 32 + rbase];
    return !RC_CHK(rp, kChkRecord) ? kBlack : CG ? __ldca(rp) : __ldg(rp);
  };
  // Levels above cascade 0 take two directions at a time: both directions'
  // taps are requested before either's stores (loaded whatever the record,
  // which keeps the loads out of a branch; a record that is not a miss
  // replaces the blend).  Every tap lies inside the next level.
  auto gather = [&](int d, uint32_t r, float rv[3]) {
    rv[0] = rv[1] = rv[2] = 0.f;
    if (!TOP) {
#pragma unroll
      for (int tp = 0; tp < 8; ++tp) {
        const float3 v = load_rgb<T, CG>(rgb4_at(Au, d, a.P_up, tap_off[tp]));
        rv[0] = fmaf(tap_w[tp], v.x, rv[0]);
        rv[1] = fmaf(tap_w[tp], v.y, rv[1]);
        rv[2] = fmaf(tap_w[tp], v.z, rv[2]);
      }
    }
    if (r != kMiss) {
      rv[0] = rv[1] = rv[2] = 0.f;
      if (r != kBlack) voxel_emission(a.vol, r, rv);
    }
  };
  auto finish = [&](int dl, int d, const float rv[3]) {
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) Store<T>::stream(L + ((int64_t)ch * a.ndirs + d) * a.P + p, rv[ch]);
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) acc[ch] += rv[ch];
    if ((dl & 3) == 3) {
      const int dp = dpair * 2 + (dl >> 2);
      store_avg<T>(a, dp, p, 0.25f * acc[0], 0.25f * acc[1], 0.25f * acc[2]);
      acc[0] = acc[1] = acc[2] = 0.f;
    }
  };
  // cascade 0, one direction: its radiance from the record, the stores, the fluence
  auto one = [&](int d, uint32_t r) {
    float rv[3] = {0.f, 0.f, 0.f};
    if (r == kMiss) {
      if (!TOP) {
#pragma unroll
        for (int tp = 0; tp < 8; ++tp) {
          const float3 v = load_rgb<T, CG>(rgb4_at(Au, d, a.P_up, tap_off[tp]));
          rv[0] = fmaf(tap_w[tp], v.x, rv[0]);
          rv[1] = fmaf(tap_w[tp], v.y, rv[1]);
          rv[2] = fmaf(tap_w[tp], v.z, rv[2]);
        }
      }
    } else if (r != kBlack) {
      voxel_emission(a.vol, r, rv);
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) Store<T>::stream(L + ((int64_t)ch * a.ndirs + d) * a.P + p, rv[ch]);
    const float om = a.dirs[d].omega;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) acc[ch] = fmaf(om, rv[ch], acc[ch]);
  };
  if (L0) {
    // two directions per pass: their parent taps are in flight together
#pragma unroll 2
    for (int dl = 0; dl < a.ndirs; ++dl) one(dl, record(dl));
  } else {
    // the eight directions' records are requested together, then merged in order
    uint32_t r8[8];
#pragma unroll
    for (int dl = 0; dl < 8; ++dl) r8[dl] = record(dir_of(dl));
#pragma unroll
    for (int dl = 0; dl < 8; dl += 2) {
      float ra[3], rb[3];
      gather(dir_of(dl), r8[dl], ra);
      gather(dir_of(dl + 1), r8[dl + 1], rb);
      finish(dl, dir_of(dl), ra);
      finish(dl + 1, dir_of(dl + 1), rb);
    }
  }
  if (L0) {
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
      if (RC_CHK(&a.fluence[p * 3 + ch], kChkFluence)) a.fluence[p * 3 + ch] = acc[ch];
  }
}

// One thread per probe; block row blockIdx.y = pair of parent texels.
template <typename T, bool L0, bool TOP>
__global__ void __launch_bounds__(128) k_level_merge(const __grid_constant__ LevelArgs a,
                                                     const uint32_t* __restrict__ rec, int slots) {
  grid_dep_wait();  // the records and the next level's radiance
  grid_dep_release();
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.P) return;
  merge_probe<T, L0, TOP, false>(a, rec, slots, p, blockIdx.y);
}

// The top level's merge (records and emission only, no parent taps), with a
// register budget of seven blocks per SM: the compiler then keeps more of a
// thread's record loads and stores in flight (56 registers instead of the 32
// it picks unbounded; the top merge 1.3 us faster at 256^3).
template <typename T, bool L0>
__global__ void __launch_bounds__(128, 7) k_level_merge_top(const __grid_constant__ LevelArgs a,
                                                            const uint32_t* __restrict__ rec, int slots) {
  grid_dep_wait();  // the records
  grid_dep_release();
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.P) return;
  merge_probe<T, L0, true, false>(a, rec, slots, p, blockIdx.y);
}

}  // namespace rcx
