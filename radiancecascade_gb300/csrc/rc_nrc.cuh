// rc_nrc.cuh -- neural radiance cache for the far cascades (sm_103a).
//
// For a far cascade i >= F the cache stands in for the interval walk: it maps
// (probe position, direction, cascade) to the walk's result (R, T) -- the
// radiance leaving the first opaque voxel of the interval (RGB) and whether
// the ray got through (T = 1) -- and the usual top-down merge then forms
// L_i = R + T * merge(A_{i+1}).
//
// Model.  Input encoding: a multiresolution hash encoding in the manner of
// Mueller et al. 2022 ("Instant neural graphics primitives") over the query's
// probe centre, its direction texel and its cascade: 16 levels x 2 FP16
// features, 2^19 entries per level; level l quantises the probe centre
// (scaled to [0, 1]) at resolution r_l (16 .. 512, geometric) and the
// octahedral texel centre at resolution q_l (2 .. 128, geometric), and reads
// the features of that one cell (queries sit exactly on the probe and texel
// lattices, so no interpolation is needed) at hash(x, y, z, u, v, cascade) =
// x ^ 2654435761 y ^ 805459861 z ^ 0x85EBCA77 u ^ 0xC2B2AE3D v ^ 0x27D4EB2F c
// mod 2^19.  Plus 16 direction features (the texel centre u, v, sin / cos of
// pi and 2 pi times each, and a one-hot of the cascade); zero-padded to 64.
// MLP: 4 hidden layers of width 64 with ReLU, then a 16-wide linear output
// layer of which 4 are used (R, G, B scaled by radiance_scale, and T).
// Served values follow the walk's structure -- T is 0 or 1 and a ray that got
// through carries no radiance: T = [o_3 >= 1/2], R = T ? 0 : max(o / scale, 0).
// (Clamping the raw outputs instead would turn the network's zero-mean error
// on the many empty rays into a positive bias of the fluence.)
// BF16 weights and activations, FP32 accumulation in tensor memory; every
// layer is one tcgen05 M = 128 GEMM (one query per row).  Training: MSE on
// (R * scale, T), gradients through the same GEMMs (transposed operands in
// shared memory), Adam on FP32 master copies of the MLP and of the hash table.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "rc_kernels.cuh"
#include "rc_umma.cuh"
#include "rc_walk_queue.cuh"

namespace rcx {

constexpr int kNrcThreads = 128;     // one query row per thread; M = 128 per tile
constexpr int kNrcHashLevels = 16;
constexpr int kNrcPosFeat = 2 * kNrcHashLevels;  // 32
constexpr int kNrcDirFeat = 16;
constexpr int kNrcHidden = 4;

// FP32 master parameters: W_l [64 out][64 in] then b_l [64] for l = 0..3,
// then W_4 [16][64], b_4 [16].
constexpr int kNrcLayerStride = 64 * 64 + 64;
constexpr int kNrcW4 = 4 * kNrcLayerStride;
constexpr int kNrcB4 = kNrcW4 + 16 * 64;
constexpr int kNrcParams = kNrcB4 + 16;  // 17680
static_assert(kNrcParams % 4 == 0, "Adam takes the parameters four at a time");

// BF16 weight image (byte offsets), already in the K-major core layout:
//   l = 0..3:  F_l = W_l as [64 n = out][64 k = in]     at 16384 l
//              B_l = W_l^T as [64 n = in][64 k = out]   at 16384 l + 8192
//   W4F = W_4 as [16][64] at 65536,  W4B = W_4^T as [64][16] at 67584
constexpr int kImgW4F = 65536;
constexpr int kImgW4B = 67584;
constexpr int kImgBytes = 69632;

// One tile of up to 128 queries.  list = 0: directions d0 .. d0 + n - 1 of
// one probe.  list = k > 0: row r is probe `probe + r / k` with direction
// dlist[d0 + r % k] (NrcArgs.dlist), so a tile packs 128 / k probes when
// their direction lists are short; slot + r / k is the row's probe index in
// its sample phase.
struct NrcTile {
  int32_t level;
  int32_t probe;
  int32_t d0;
  int32_t n;
  int32_t slot;
  int32_t list;
};

struct NrcLevel {
  const __nv_bfloat16* denc;  // [ndirs][16] direction + cascade features
  __half* rt;                 // [4][ndirs][P]: R, G, B, T
  int64_t P;
  int32_t ndirs;
  int32_t n;                  // direction resolution (n x n texels)
  int32_t M[3];
  int32_t spacing;
  // The level's own walk records (rc_walk_queue.cuh layout rec[d][slot][32],
  // slot = z * wpp + word, bit g = y * 2^l2px + x of the probe's plane).
  const uint32_t* rec;
  int32_t slots, wpp, l2px;
  uint8_t* word_on;           // [slots] walk switch of the level's words
  const float* omega;         // [ndirs] exact texel solid angles
  uint32_t* hpos;             // [P][16] position part of the hash per hash level
  uint32_t* hdir;             // [ndirs][16] direction part of the hash per hash level
};

struct NrcHash {
  const __half* table;  // [16][T][2]
  float* grad;          // [16][T][2] (null: no scatter)
  int32_t log2T;
  int32_t res[kNrcHashLevels];   // position resolution per level
  int32_t dres[kNrcHashLevels];  // direction resolution per level
  float inv_extent;              // 1 / max grid edge
};

struct NrcArgs {
  const unsigned char* img;  // BF16 weight image
  const float* params;       // FP32 master (biases)
  NrcHash hash;
  NrcLevel lv[kMaxCascades];
  int32_t first;             // first far cascade
  int32_t nlev;
  int64_t tile0[kMaxCascades + 1];  // enumeration: first tile of each far level
  const NrcTile* tiles;      // explicit tile list (or null: enumerate the far levels)
  const int32_t* dlist;      // direction lists of the sample tiles
  int64_t ntiles;
  float* out;                // explicit tiles: raw outputs [tile][128][4]
  const float* target;       // training: [tile][128][4] (R, G, B, T)
  float* grad;               // training: FP32 gradient of the master parameters
  float* epos_grad;          // tile gradient: sum over rows of the 32 hash features' gradient
  float* loss;               // training: sum of squared errors
  float scale;               // radiance scale of the outputs
  float inv_batch;           // training: 1 / (queries in the step)
  int* err;
  // Serving (enumerated inference only): plain[level] != 0 means the level
  // runs on its walks this solve; probes whose fallback tile is flagged are
  // walked too, so their rows are not stored.
  const int32_t* plain;
  const uint8_t* flag;
  int32_t tile_shift, TX, TY;
};

__device__ __forceinline__ unsigned char* align128(unsigned char* p) {
  return reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(p) + 127) & ~(uintptr_t)127);
}

// Resolves row r of tile t: (level, probe, direction); false for an empty row.
__device__ __forceinline__ bool nrc_query(const NrcArgs& a, int64_t t, int r, int& li, int64_t& p, int& d,
                                          int& slot) {
  if (a.tiles) {
    const NrcTile tl = a.tiles[t];
    li = tl.level;
    p = tl.probe;
    slot = tl.slot;
    if (r >= tl.n) {
      d = 0;
      return false;
    }
    if (tl.list) {
      p += r / tl.list;
      slot += r / tl.list;
      d = __ldg(a.dlist + tl.d0 + r % tl.list);
    } else {
      d = tl.d0 + r;
    }
    return true;
  }
  li = a.first;
  while (li + 1 < a.nlev && t >= a.tile0[li + 1]) ++li;
  const NrcLevel& L = a.lv[li];
  // a level's queries number below 2^31 (checked when the cache is enabled)
  const uint32_t q = (uint32_t)(t - a.tile0[li]) * (uint32_t)kNrcThreads + (uint32_t)r;
  const uint32_t P = (uint32_t)L.P;
  slot = -1;
  if (q >= P * (uint32_t)L.ndirs) return false;
  const uint32_t dq = q / P;
  d = (int)dq;
  p = (int64_t)(q - dq * P);
  return true;
}

// Probe centre (voxel units) of probe p of level L, scaled to [0, 1].
__device__ __forceinline__ void nrc_probe_pos(const NrcLevel& L, int64_t p, float inv_extent, float* u) {
  const uint32_t pp = (uint32_t)p, M0 = (uint32_t)L.M[0], M1 = (uint32_t)L.M[1];
  const uint32_t row = pp / M0, mz_ = row / M1;
  const int mx = (int)(pp - row * M0), my = (int)(row - mz_ * M1), mz = (int)mz_;
  const float h = 0.5f * (float)L.spacing;
  u[0] = ((float)mx * L.spacing + h) * inv_extent;
  u[1] = ((float)my * L.spacing + h) * inv_extent;
  u[2] = ((float)mz * L.spacing + h) * inv_extent;
}

// Fallback tile (voxel cell of 2^shift edge) of probe p's centre.
__device__ __forceinline__ int64_t nrc_cell(const NrcLevel& L, int64_t p, int shift, int TX, int TY) {
  const uint32_t pp = (uint32_t)p, M0 = (uint32_t)L.M[0], M1 = (uint32_t)L.M[1];
  const uint32_t row = pp / M0, mz = row / M1;
  const int mx = (int)(pp - row * M0), my = (int)(row - mz * M1);
  const int h = L.spacing >> 1;
  return ((int64_t)(((int)mz * L.spacing + h) >> shift) * TY + ((my * L.spacing + h) >> shift)) * TX +
         ((mx * L.spacing + h) >> shift);
}

// Record index of probe p's entry for direction d: ((d * slots + slot) * 32 + bit).
__device__ __forceinline__ int64_t nrc_rec_index(const NrcLevel& L, int64_t p, int d) {
  const uint32_t pp = (uint32_t)p, M0 = (uint32_t)L.M[0], M1 = (uint32_t)L.M[1];
  const uint32_t row = pp / M0, mz = row / M1;
  const int mx = (int)(pp - row * M0), my = (int)(row - mz * M1);
  const int g = (my << L.l2px) + mx;
  return ((int64_t)d * L.slots + (int)mz * L.wpp + (g >> 5)) * 32 + (g & 31);
}

// Walk result (R, G, B, T) of one record entry: first-hit voxel (emissive),
// kBlack (opaque, no emission) or kMiss (the ray got through).
__device__ __forceinline__ void nrc_record_rt(const uint2* __restrict__ vol, uint32_t r, float* rt) {
  rt[0] = rt[1] = rt[2] = 0.f;
  rt[3] = r == kMiss ? 1.f : 0.f;
  if (r != kMiss && r != kBlack) voxel_emission(vol, r, rt);
}

// The hash of a query (see the file comment) is the XOR of a part that
// depends only on the probe's cell, x ^ y K1 ^ z K2, and a part that depends
// only on the direction texel's cell and the cascade, a K3 ^ b K4 ^ c K5.
__device__ __forceinline__ uint32_t nrc_hash_pos(const NrcHash& h, int l, const float* u) {
  const int r = h.res[l];
  const uint32_t x = (uint32_t)min((int)(u[0] * (float)r), r - 1);
  const uint32_t y = (uint32_t)min((int)(u[1] * (float)r), r - 1);
  const uint32_t z = (uint32_t)min((int)(u[2] * (float)r), r - 1);
  return x ^ (y * 2654435761u) ^ (z * 805459861u);
}
__device__ __forceinline__ uint32_t nrc_hash_dir(const NrcHash& h, int l, float du, float dv, int casc) {
  const int q = h.dres[l];
  const uint32_t a = (uint32_t)min((int)(du * (float)q), q - 1);
  const uint32_t b = (uint32_t)min((int)(dv * (float)q), q - 1);
  return (a * 0x85EBCA77u) ^ (b * 0xC2B2AE3Du) ^ ((uint32_t)casc * 0x27D4EB2Fu);
}

// Both parts for every probe and every direction of far level li, written
// once when the cache is enabled (NrcLevel.hpos, .hdir).
__global__ void k_nrc_hash_parts(const __grid_constant__ NrcArgs a, int li) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const NrcLevel& L = a.lv[li];
  if (i < L.P) {
    float u[3];
    nrc_probe_pos(L, i, a.hash.inv_extent, u);
#pragma unroll
    for (int l = 0; l < kNrcHashLevels; ++l) L.hpos[i * kNrcHashLevels + l] = nrc_hash_pos(a.hash, l, u);
  }
  if (i < L.ndirs) {
    const int d = (int)i;
    const float du = ((float)(d % L.n) + 0.5f) / (float)L.n, dv = ((float)(d / L.n) + 0.5f) / (float)L.n;
#pragma unroll
    for (int l = 0; l < kNrcHashLevels; ++l) L.hdir[i * kNrcHashLevels + l] = nrc_hash_dir(a.hash, l, du, dv, li);
  }
}

// Table rows of the 16 hash levels of query (p, d) of far level li:
// row_l = l 2^log2T + ((hpos_l ^ hdir_l) mod 2^log2T), two 64-byte loads.
__device__ __forceinline__ void nrc_rows(const NrcArgs& a, int li, int64_t p, int d, uint32_t* rows) {
  const NrcLevel& L = a.lv[li];
  const uint4* hp = reinterpret_cast<const uint4*>(L.hpos + p * kNrcHashLevels);
  const uint4* hd = reinterpret_cast<const uint4*>(L.hdir + (int64_t)d * kNrcHashLevels);
  const uint32_t T = 1u << a.hash.log2T, mask = T - 1u;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const uint4 P = RC_CHK(hp + j, kChkHash) ? __ldg(hp + j) : make_uint4(0u, 0u, 0u, 0u);
    const uint4 D = RC_CHK(hd + j, kChkHash) ? __ldg(hd + j) : make_uint4(0u, 0u, 0u, 0u);
    rows[4 * j + 0] = (4 * j + 0) * T + ((P.x ^ D.x) & mask);
    rows[4 * j + 1] = (4 * j + 1) * T + ((P.y ^ D.y) & mask);
    rows[4 * j + 2] = (4 * j + 2) * T + ((P.z ^ D.z) & mask);
    rows[4 * j + 3] = (4 * j + 3) * T + ((P.w ^ D.w) & mask);
  }
}

// Input row: 32 hash features, 16 direction features, 16 zeros.
__device__ __forceinline__ void nrc_input(const NrcArgs& a, bool valid, int li, int64_t p, int d, float* x) {
#pragma unroll
  for (int j = 0; j < 64; ++j) x[j] = 0.f;
  if (!valid) return;
  const NrcLevel& L = a.lv[li];
  uint32_t rows[kNrcHashLevels];
  nrc_rows(a, li, p, d, rows);
#pragma unroll
  for (int l = 0; l < kNrcHashLevels; ++l) {
    const __half2* hp = reinterpret_cast<const __half2*>(a.hash.table) + rows[l];
    const float2 f = RC_CHK(hp, kChkHash) ? __half22float2(__ldg(hp)) : make_float2(0.f, 0.f);
    x[2 * l] = f.x;
    x[2 * l + 1] = f.y;
  }
  const uint4* dp = reinterpret_cast<const uint4*>(L.denc + (int64_t)d * kNrcDirFeat);
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const uint4 w = __ldg(dp + j);
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&w);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float2 f = __bfloat1622float2(h[k]);
      x[32 + 8 * j + 2 * k] = f.x;
      x[32 + 8 * j + 2 * k + 1] = f.y;
    }
  }
}

__device__ __forceinline__ void copy_smem(unsigned char* dst, const unsigned char* src, int bytes) {
  for (int i = threadIdx.x * 16; i < bytes; i += blockDim.x * 16)
    *reinterpret_cast<uint4*>(dst + i) = __ldg(reinterpret_cast<const uint4*>(src + i));
}

// Waits for the MMA group committed on `bar`; every thread of the block gets
// the same answer.  On timeout *err = 3.
__device__ __forceinline__ bool nrc_wait(uint64_t* bar, uint32_t& phase, int* err) {
  const bool ok = mbar_wait_bounded(bar, phase);
  phase ^= 1u;
  const bool any_fail = __syncthreads_or(!ok);
  if (any_fail && threadIdx.x == 0) atomicExch(err, 3);
  return !any_fail;
}

// Served (R, G, B, T) from the raw outputs (see the file comment).
__device__ __host__ __forceinline__ void nrc_serve(const float* o, float scale, float* sv) {
  const bool through = o[3] >= 0.5f;
  sv[3] = through ? 1.f : 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) sv[c] = through ? 0.f : fmaxf(o[c] / scale, 0.f);
}

// The input row of a query written straight into row `row` of the K-major
// activation operand, 8 columns (16 bytes) at a time: the 32 hash features
// (16 gathers issued together), the 16 direction features (stored BF16
// already), 16 zeros.  Same values as nrc_input + store_row64_bf16.
__device__ __forceinline__ void nrc_encode_row(const NrcArgs& a, bool valid, int li, int64_t p, int d,
                                               unsigned char* XA, int row) {
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  if (!valid) {
#pragma unroll
    for (int c = 0; c < 8; ++c) *reinterpret_cast<uint4*>(XA + core_off(row, 8 * c, 64)) = zero;
    return;
  }
  uint32_t rows[kNrcHashLevels];
  nrc_rows(a, li, p, d, rows);
  __half2 f[kNrcHashLevels];
#pragma unroll
  for (int l = 0; l < kNrcHashLevels; ++l) {
    const __half2* hp = reinterpret_cast<const __half2*>(a.hash.table) + rows[l];
    f[l] = RC_CHK(hp, kChkHash) ? __ldg(hp) : __float2half2_rn(0.f);
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    __nv_bfloat162 h[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float2 v = __half22float2(f[4 * c + j]);
      h[j] = __floats2bfloat162_rn(v.x, v.y);
    }
    *reinterpret_cast<uint4*>(XA + core_off(row, 8 * c, 64)) = *reinterpret_cast<const uint4*>(h);
  }
  const uint4* dp = reinterpret_cast<const uint4*>(a.lv[li].denc + (int64_t)d * kNrcDirFeat);
  *reinterpret_cast<uint4*>(XA + core_off(row, 32, 64)) = __ldg(dp);
  *reinterpret_cast<uint4*>(XA + core_off(row, 40, 64)) = __ldg(dp + 1);
  *reinterpret_cast<uint4*>(XA + core_off(row, 48, 64)) = zero;
  *reinterpret_cast<uint4*>(XA + core_off(row, 56, 64)) = zero;
}

constexpr int kFwdGroupsMax = 2;

// Bias add and ReLU of 16 accumulator columns (c0 .. c0 + 15 of row `row`),
// stored as BF16 into the K-major operand: per column pair one packed FP32
// add and one converting ReLU (relu(round(x)) = round(relu(x)), so the values
// equal fmaxf(v + b, 0) rounded to BF16).
__device__ __forceinline__ void bias_relu_store16(unsigned char* XA, int row, int c0, const float* v,
                                                  const float* bias) {
  uint32_t hb[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float2 b = reinterpret_cast<const float2*>(bias)[j];
    asm("{\n"
        ".reg .b64 x, y, z;\n"
        ".reg .f32 lo, hi;\n"
        "mov.b64 x, {%1, %2};\n"
        "mov.b64 y, {%3, %4};\n"
        "add.rn.f32x2 z, x, y;\n"
        "mov.b64 {lo, hi}, z;\n"
        "cvt.rn.relu.bf16x2.f32 %0, hi, lo;\n"
        "}\n"
        : "=r"(hb[j])
        : "f"(v[2 * j]), "f"(v[2 * j + 1]), "f"(b.x), "f"(b.y));
  }
#pragma unroll
  for (int c = 0; c < 2; ++c)
    *reinterpret_cast<uint4*>(XA + core_off(row, c0 + 8 * c, 64)) =
        make_uint4(hb[4 * c], hb[4 * c + 1], hb[4 * c + 2], hb[4 * c + 3]);
}

// Barrier of one warpgroup (128 threads, named barrier 1 + wg; immediate ids
// so that the kernel reserves only the barriers it uses).
__device__ __forceinline__ void wg_sync(int wg) {
  if (wg == 0) asm volatile("bar.sync 1, 128;" ::: "memory");
  else asm volatile("bar.sync 2, 128;" ::: "memory");
}
// The same barrier, returning whether any of its threads passed `v`.
__device__ __forceinline__ bool wg_sync_or(int wg, bool v) {
  uint32_t r;
  if (wg == 0)
    asm volatile(
        "{\n"
        ".reg .pred p, q;\n"
        "setp.ne.u32 p, %1, 0;\n"
        "barrier.cta.red.or.pred q, 1, 128, p;\n"
        "selp.u32 %0, 1, 0, q;\n"
        "}\n"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
  else
    asm volatile(
        "{\n"
        ".reg .pred p, q;\n"
        "setp.ne.u32 p, %1, 0;\n"
        "barrier.cta.red.or.pred q, 2, 128, p;\n"
        "selp.u32 %0, 1, 0, q;\n"
        "}\n"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
  return r != 0;
}
static_assert(kFwdGroupsMax == 2, "named barriers 1 and 2 serve the two warpgroups");

// ---------------------------------------------------------------------------
// Inference.  Block = kFwdGroups warpgroups, persistent over tiles: each
// warpgroup takes its own tiles (128 queries, one per thread) through the
// five layers with its own activation operand (16 KB), tensor-memory columns
// (64) and mbarrier, so one warpgroup's epilogue runs while the other's MMAs
// and gathers are in flight; the weights (34 KB) and biases are shared.
// Epilogues read tensor memory 16 columns at a time (3 blocks/SM).
// RT: write (R, T) planes of the enumerated far levels; else raw outputs.
// ---------------------------------------------------------------------------
constexpr int kFwdGroups = kFwdGroupsMax;
constexpr int kFwdThreads = 128 * kFwdGroups;
constexpr int kFwdXA = 36864;  // activation operands start here (1024-byte aligned, after weights and biases)
constexpr int kFwdSmem = kFwdXA + kFwdGroups * 16384 + 8 * kFwdGroups + 16 + 128;
static_assert(4 * 8192 + 2048 + 272 * 4 <= kFwdXA, "weights and biases fit before the operands");

template <bool RT>
__global__ void __launch_bounds__(kFwdThreads, 3) k_nrc_forward(const __grid_constant__ NrcArgs a, int64_t ntiles) {
  extern __shared__ unsigned char sm_raw[];
  unsigned char* sm = align128(sm_raw);
  unsigned char* WF = sm;
  unsigned char* W4F = WF + 4 * 8192;
  float* sb = reinterpret_cast<float*>(W4F + 2048);
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kFwdXA + kFwdGroups * 16384);
  uint32_t* s_taddr = reinterpret_cast<uint32_t*>(bars + kFwdGroups);
  const int tid = threadIdx.x, wg = tid >> 7, row = tid & 127, warp = tid >> 5;

  for (int l = 0; l < 4; ++l) copy_smem(WF + 8192 * l, a.img + 16384 * l, 8192);
  copy_smem(W4F, a.img + kImgW4F, 2048);
  for (int j = tid; j < 272; j += blockDim.x)
    sb[j] = j < 256 ? a.params[(j >> 6) * kNrcLayerStride + 4096 + (j & 63)] : a.params[kNrcB4 + j - 256];
  if (tid == 0) {
#pragma unroll
    for (int g = 0; g < kFwdGroups; ++g) mbar_init(&bars[g], 1);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(s_taddr, 64 * kFwdGroups);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *s_taddr + 64u * (uint32_t)wg;            // this warpgroup's columns
  const uint32_t tl = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's lane quarter
  unsigned char* XA = sm + kFwdXA + wg * 16384;
  uint64_t* bar = &bars[wg];
  uint32_t phase = 0;
  bool ok = true;

  for (int64_t t = (int64_t)blockIdx.x * kFwdGroups + wg; t < ntiles && ok; t += (int64_t)gridDim.x * kFwdGroups) {
    int li, d, slot;
    int64_t p;
    bool valid = nrc_query(a, t, row, li, p, d, slot);
    if (RT) {
      // rows on the walk (the level runs plain, or the probe's tile is
      // flagged) are not served; a tile with no served row is skipped
      valid = valid && !__ldg(a.plain + li) &&
              !__ldg(a.flag + nrc_cell(a.lv[li], p, a.tile_shift, a.TX, a.TY));
      if (!wg_sync_or(wg, valid)) continue;
    }
    nrc_encode_row(a, valid, li, p, d, XA, row);
    fence_proxy_async();
    wg_sync(wg);
    float o[16];
    for (int l = 0; l < 5; ++l) {
      if (row == 0) {
        tc_fence_after();
        umma_gemm(tmem, smem_u32(XA), smem_u32(l < 4 ? WF + 8192 * l : W4F), 128, l < 4 ? 64 : 16, 64, false);
        umma_commit(bar);
      }
      const bool got = mbar_wait_bounded(bar, phase);
      phase ^= 1u;
      if (wg_sync_or(wg, !got)) {
        if (row == 0) atomicExch(a.err, 3);
        ok = false;
        break;
      }
      tc_fence_after();
      if (l < 4) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          float v[16];
          tmem_ld16(tl + 16u * q, v);
          bias_relu_store16(XA, row, 16 * q, v, sb + 64 * l + 16 * q);
        }
        tc_fence_before();
        fence_proxy_async();
        wg_sync(wg);
      } else {
        tmem_ld16(tl, o);
        tc_fence_before();
      }
    }
    if (!ok || !valid) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) o[c] += sb[256 + c];
    if (RT) {
      const NrcLevel& L = a.lv[li];
      const int64_t plane = (int64_t)L.ndirs * L.P;
      const int64_t off = (int64_t)d * L.P + p;
      float sv[4];
      nrc_serve(o, a.scale, sv);
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (RC_CHK(&L.rt[c * plane + off], kChkCache)) L.rt[c * plane + off] = __float2half_rn(sv[c]);
    } else {
      float4 r4 = make_float4(o[0], o[1], o[2], o[3]);
      float4* op = reinterpret_cast<float4*>(a.out + (t * kNrcThreads + row) * 4);
      if (RC_CHK(op, kChkCache)) *op = r4;
    }
  }
  if (!ok) mbar_wait_bounded(bar, phase ^ 1u);  // the group that timed out, if it still runs
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(*s_taddr, 64 * kFwdGroups);
}

// ---------------------------------------------------------------------------
// Training.  Block = 128 threads, persistent over training tiles (all rows of
// a tile share one probe).  Per tile: forward (keeping x_1..x_4 transposed and
// the ReLU masks), output error, then layer by layer
//   dW_l += dz_l^T x_l   (M = 128 with dz_l^T in rows 0..63, accumulated in
//                         tensor memory over the block's tiles)
//   dx_l  = dz_l W_l     (M = 128, N = 64, K = 64)
// and the probe's position-feature gradient (column sums of dx_1[:, 0:32]).
// Output layer and bias gradients: FP32 reductions in shared memory.
// Tensor memory: columns 0..63 the per-layer product, 64 + 64 l the dW_l.
// ---------------------------------------------------------------------------
constexpr int kTrWF = 0;           // 4 x 8192
constexpr int kTrWB = 32768;       // 4 x 8192
constexpr int kTrW4F = 65536;      // 2048
constexpr int kTrW4B = 67584;      // 2048
constexpr int kTrXA = 69632;       // [128][64]        16384
constexpr int kTrXT = 86016;       // 4 x [64][128]    65536
constexpr int kTrDZ = 151552;      // [128][64]        16384
constexpr int kTrDZT = 167936;     // [128][128]       32768 (rows 64..127 stay zero)
constexpr int kTrDO = 200704;      // [128][16]        4096
constexpr int kTrMisc = 204800;
// misc (floats): biases 272, dW4/db4 accumulators 4 x 64 + 4, db accumulators
// 4 x 64, output errors 128 x 4, position-gradient sums 32; then the barrier
constexpr int kTrMiscFloats = 272 + 260 + 256 + 512 + 32;
constexpr int kTrainSmem = kTrMisc + kTrMiscFloats * 4 + 16 + 128;

__global__ void __launch_bounds__(kNrcThreads) k_nrc_train(const __grid_constant__ NrcArgs a) {
  extern __shared__ unsigned char sm_raw[];
  unsigned char* sm = align128(sm_raw);
  float* sb = reinterpret_cast<float*>(sm + kTrMisc);
  float* acc4 = sb + 272;        // dW4 rows 0..3 (4 x 64), db4 (4)
  float* accb = acc4 + 260;      // db_l, l = 0..3 (4 x 64)
  float* sdo = accb + 256;       // output errors [128][4]
  float* spos = sdo + 512;       // position-gradient sums [32]
  uint64_t* bar = reinterpret_cast<uint64_t*>(spos + 32);
  uint32_t* s_taddr = reinterpret_cast<uint32_t*>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  for (int l = 0; l < 4; ++l) {
    copy_smem(sm + kTrWF + 8192 * l, a.img + 16384 * l, 8192);
    copy_smem(sm + kTrWB + 8192 * l, a.img + 16384 * l + 8192, 8192);
  }
  copy_smem(sm + kTrW4F, a.img + kImgW4F, 2048);
  copy_smem(sm + kTrW4B, a.img + kImgW4B, 2048);
  for (int j = tid; j < 272; j += blockDim.x)
    sb[j] = j < 256 ? a.params[(j >> 6) * kNrcLayerStride + 4096 + (j & 63)] : a.params[kNrcB4 + j - 256];
  for (int j = tid; j < 260 + 256 + 32; j += blockDim.x) acc4[j] = 0.f;
  for (int i = tid * 16; i < 32768; i += blockDim.x * 16)
    *reinterpret_cast<uint4*>(sm + kTrDZT + i) = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(s_taddr, 512);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *s_taddr;
  const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  bool ok = true, first = true;
  float loss = 0.f;
  unsigned char* XA = sm + kTrXA;
  unsigned char* DZ = sm + kTrDZ;
  unsigned char* DZT = sm + kTrDZT;

  for (int64_t t = blockIdx.x; t < a.ntiles && ok; t += gridDim.x) {
    int li, d, slot;
    int64_t p;
    const bool valid = nrc_query(a, t, tid, li, p, d, slot);
    uint64_t mask[4];  // ReLU masks of x_2 .. x_5 (bit j = feature j > 0)
    {
      float x[64];
      nrc_input(a, valid, li, p, d, x);
      store_row64_bf16(XA, tid, x);
#pragma unroll
      for (int j = 0; j < 64; ++j)
        reinterpret_cast<__nv_bfloat16*>(sm + kTrXT + core_off(j, tid, 128))[0] = __float2bfloat16_rn(x[j]);
    }
    fence_proxy_async();
    __syncthreads();
    // ---- forward
    float o[16];
    for (int l = 0; l < 5 && ok; ++l) {
      if (tid == 0) {
        tc_fence_after();
        umma_gemm(tmem, smem_u32(XA), smem_u32(sm + (l < 4 ? kTrWF + 8192 * l : kTrW4F)), 128, l < 4 ? 64 : 16, 64,
                  false);
        umma_commit(bar);
      }
      if (!(ok = nrc_wait(bar, phase, a.err))) break;
      tc_fence_after();
      if (l < 4) {
        float v[64];
        tmem_ld64(tl, v);
        uint64_t m = 0;
#pragma unroll
        for (int j = 0; j < 64; ++j) {
          v[j] = fmaxf(v[j] + sb[64 * l + j], 0.f);
          m |= (uint64_t)(v[j] > 0.f) << j;
        }
        mask[l] = m;
        store_row64_bf16(XA, tid, v);
        if (l < 3) {
          unsigned char* xt = sm + kTrXT + 16384 * (l + 1);
#pragma unroll
          for (int j = 0; j < 64; ++j)
            reinterpret_cast<__nv_bfloat16*>(xt + core_off(j, tid, 128))[0] = __float2bfloat16_rn(v[j]);
        }
        tc_fence_before();
        fence_proxy_async();
        __syncthreads();
      } else {
        tmem_ld16(tl, o);
        tc_fence_before();
      }
    }
    if (!ok) break;
    // ---- output error
    {
      float e[4] = {0.f, 0.f, 0.f, 0.f};
      if (valid) {
        const float4* yp = reinterpret_cast<const float4*>(a.target + (t * kNrcThreads + tid) * 4);
        const float4 y = RC_CHK(yp, kChkCache) ? *yp : make_float4(0.f, 0.f, 0.f, 0.f);
        const float yv[4] = {y.x * a.scale, y.y * a.scale, y.z * a.scale, y.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const float diff = o[c] + sb[256 + c] - yv[c];
          loss = fmaf(diff, diff, loss);
          e[c] = 2.f * diff * a.inv_batch;
        }
      }
      float eo[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) eo[c] = c < 4 ? e[c] : 0.f;
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        __nv_bfloat162 h[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(eo[8 * c + 2 * j], eo[8 * c + 2 * j + 1]);
        *reinterpret_cast<uint4*>(sm + kTrDO + core_off(tid, 8 * c, 16)) = *reinterpret_cast<const uint4*>(h);
      }
#pragma unroll
      for (int c = 0; c < 4; ++c) sdo[tid * 4 + c] = e[c];
    }
    fence_proxy_async();
    __syncthreads();
    // dx_5 = e W_4 (K = 16), issued before the FP32 reductions below
    if (tid == 0) {
      tc_fence_after();
      umma_gemm(tmem, smem_u32(sm + kTrDO), smem_u32(sm + kTrW4B), 128, 64, 16, false);
      umma_commit(bar);
    }
    {
      // dW_4 [c][k] += sum_m e[m][c] x_5[m][k]; thread: k = tid & 63, c = 2 (tid >> 6) + {0, 1}
      const int k = tid & 63, c0 = 2 * (tid >> 6);
      float s0 = 0.f, s1 = 0.f;
      for (int m = 0; m < kNrcThreads; ++m) {
        const float xv = __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(XA + core_off(m, k, 64))[0]);
        s0 = fmaf(sdo[m * 4 + c0], xv, s0);
        s1 = fmaf(sdo[m * 4 + c0 + 1], xv, s1);
      }
      acc4[c0 * 64 + k] += s0;
      acc4[(c0 + 1) * 64 + k] += s1;
      if (tid < 4) {
        float s = 0.f;
        for (int m = 0; m < kNrcThreads; ++m) s += sdo[m * 4 + tid];
        acc4[256 + tid] += s;
      }
    }
    if (!(ok = nrc_wait(bar, phase, a.err))) break;
    tc_fence_after();
    // ---- hidden layers, top down: dz_l from dx_{l+1}, then dW_l and dx_l
    for (int l = 3; l >= 0 && ok; --l) {
      {
        float v[64];
        tmem_ld64(tl, v);
#pragma unroll
        for (int j = 0; j < 64; ++j) v[j] = ((mask[l] >> j) & 1u) ? v[j] : 0.f;
        store_row64_bf16(DZ, tid, v);
#pragma unroll
        for (int j = 0; j < 64; ++j)
          reinterpret_cast<__nv_bfloat16*>(DZT + core_off(j, tid, 128))[0] = __float2bfloat16_rn(v[j]);
      }
      tc_fence_before();
      fence_proxy_async();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        umma_gemm(tmem + 64u + 64u * l, smem_u32(DZT), smem_u32(sm + kTrXT + 16384 * l), 128, 64, 128, !first);
        umma_gemm(tmem, smem_u32(DZ), smem_u32(sm + kTrWB + 8192 * l), 128, 64, 64, false);
        umma_commit(bar);
      }
      if (tid < 64) {  // db_l: column sums of dz_l
        float s = 0.f;
        for (int m = 0; m < kNrcThreads; ++m)
          s += __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(DZT + core_off(tid, m, 128))[0]);
        accb[64 * l + tid] += s;
      }
      if (!(ok = nrc_wait(bar, phase, a.err))) break;
      tc_fence_after();
    }
    if (!ok) break;
    // ---- hash-feature gradient: scattered per row into the table gradient
    {
      float v[64];
      tmem_ld64(tl, v);
      tc_fence_before();
      if (valid && a.hash.grad) {
        uint32_t rows[kNrcHashLevels];
        nrc_rows(a, li, p, d, rows);
#pragma unroll
        for (int l = 0; l < kNrcHashLevels; ++l) {
          const uint32_t row = rows[l];
          if (!RC_CHK(a.hash.grad + 2 * (size_t)row + 1, kChkHash)) continue;
          if (v[2 * l] != 0.f) atomicAdd(a.hash.grad + 2 * (size_t)row, v[2 * l]);
          if (v[2 * l + 1] != 0.f) atomicAdd(a.hash.grad + 2 * (size_t)row + 1, v[2 * l + 1]);
        }
      }
      if (a.epos_grad) {  // tile-gradient probe: row sums of the 32 features' gradient
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          float sum = v[j];
#pragma unroll
          for (int sh = 16; sh > 0; sh >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, sh);
          if (lane == 0) atomicAdd(&spos[j], sum);
        }
        __syncthreads();
        if (tid < 32) {
          atomicAdd(&a.epos_grad[tid], spos[tid]);
          spos[tid] = 0.f;
        }
      }
    }
    first = false;
    __syncthreads();
  }
  if (!ok) mbar_wait_bounded(bar, phase ^ 1u);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (ok && !first) {
    // dW_l rows (out features) sit in tensor-memory lanes 0..63: warps 0 and 1
    if (warp < 2) {
      for (int l = 0; l < 4; ++l) {
        float v[64];
        tmem_ld64(tl + 64u + 64u * l, v);
        float* g = a.grad + l * kNrcLayerStride + tid * 64;
#pragma unroll
        for (int j = 0; j < 64; ++j) atomicAdd(&g[j], v[j]);
      }
    }
    for (int j = tid; j < 256; j += blockDim.x) {
      atomicAdd(&a.grad[(j >> 6) * kNrcLayerStride + 4096 + (j & 63)], accb[j]);
      atomicAdd(&a.grad[kNrcW4 + j], acc4[j]);
    }
    if (tid < 4) atomicAdd(&a.grad[kNrcB4 + tid], acc4[256 + tid]);
  }
  // loss: one atomic per warp
#pragma unroll
  for (int sh = 16; sh > 0; sh >>= 1) loss += __shfl_xor_sync(0xFFFFFFFFu, loss, sh);
  if (lane == 0 && a.loss) atomicAdd(a.loss, loss);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// Adam (Kingma and Ba 2015) on FP32 masters; clears the gradient.  Writes the
// FP16 copy of the hash table when half_out is set.
// ---------------------------------------------------------------------------
struct AdamArgs {
  float* p;
  float* g;
  float* m;
  float* v;
  __half* half_out;
  int64_t n;
  float lr, beta1, beta2, eps;
  float c1, c2;  // bias corrections 1 - beta^t
  int32_t lazy;  // skip entries whose gradient is exactly zero (hash table)
  int32_t pad;
};

// Adam step.  With `lazy`, an entry no training sample touched this step
// (gradient exactly 0) keeps its value and moments, as Mueller et al. 2022 do
// for the hash table: a step then writes only the touched entries.
__device__ __forceinline__ float adam_one(const AdamArgs& a, float g, float& m, float& v, float p) {
  m = fmaf(a.beta1, m, (1.f - a.beta1) * g);
  v = fmaf(a.beta2, v, (1.f - a.beta2) * g * g);
  return p - a.lr * (m / a.c1) / (sqrtf(v / a.c2) + a.eps);
}

// Four entries per thread and step (16-byte loads; a.n is a multiple of 4 for
// both parameter sets, checked by the host); a lazy step skips a group whose
// four gradients are all zero without touching its moments.
__global__ void k_nrc_adam(const __grid_constant__ AdamArgs a) {
  const int64_t n4 = a.n >> 2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 g = reinterpret_cast<const float4*>(a.g)[i];
    if (a.lazy && g.x == 0.f && g.y == 0.f && g.z == 0.f && g.w == 0.f) continue;
    float4 m = reinterpret_cast<const float4*>(a.m)[i];
    float4 v = reinterpret_cast<const float4*>(a.v)[i];
    float4 p = reinterpret_cast<const float4*>(a.p)[i];
    // with `lazy`, an entry of the group whose own gradient is zero keeps its state
    if (!a.lazy || g.x != 0.f) p.x = adam_one(a, g.x, m.x, v.x, p.x);
    if (!a.lazy || g.y != 0.f) p.y = adam_one(a, g.y, m.y, v.y, p.y);
    if (!a.lazy || g.z != 0.f) p.z = adam_one(a, g.z, m.z, v.z, p.z);
    if (!a.lazy || g.w != 0.f) p.w = adam_one(a, g.w, m.w, v.w, p.w);
    reinterpret_cast<float4*>(a.m)[i] = m;
    reinterpret_cast<float4*>(a.v)[i] = v;
    reinterpret_cast<float4*>(a.p)[i] = p;
    reinterpret_cast<float4*>(a.g)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (a.half_out) {
      const __half2 lo = __floats2half2_rn(p.x, p.y), hi = __floats2half2_rn(p.z, p.w);
      uint2 h;
      h.x = *reinterpret_cast<const uint32_t*>(&lo);
      h.y = *reinterpret_cast<const uint32_t*>(&hi);
      reinterpret_cast<uint2*>(a.half_out)[i] = h;
    }
  }
}

// BF16 weight image from the FP32 masters (one thread per image element).
__global__ void k_nrc_pack(const float* __restrict__ params, unsigned char* __restrict__ img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kImgBytes / 2) return;
  const int byte = 2 * i;
  float w;
  if (byte < kImgW4F) {
    const int l = byte / 16384, part = (byte % 16384) / 8192, off = byte % 8192;
    // invert core_off for a 64 x 64 operand: off = (n/8)*1024 + (k/8)*128 + (n%8)*16 + (k%8)*2
    const int n = (off / 1024) * 8 + (off % 128) / 16, k = ((off % 1024) / 128) * 8 + (off % 16) / 2;
    const float* W = params + l * kNrcLayerStride;
    w = part == 0 ? W[n * 64 + k] : W[k * 64 + n];
  } else if (byte < kImgW4B) {
    const int off = byte - kImgW4F;  // [16 n][64 k]
    const int n = (off / 1024) * 8 + (off % 128) / 16, k = ((off % 1024) / 128) * 8 + (off % 16) / 2;
    w = params[kNrcW4 + n * 64 + k];
  } else {
    const int off = byte - kImgW4B;  // [64 n][16 k]: SBO = 256
    const int n = (off / 256) * 8 + (off % 128) / 16, k = ((off % 256) / 128) * 8 + (off % 16) / 2;
    w = params[kNrcW4 + k * 64 + n];
  }
  reinterpret_cast<__nv_bfloat16*>(img)[i] = __float2bfloat16_rn(w);
}

// ---------------------------------------------------------------------------
// Per-solve schedule kernels: which words the far levels walk, training
// targets from the walk records, the held-out error per fallback tile, the
// serve decision per level, and the merge from the network or the records.
// ---------------------------------------------------------------------------

// Sample phase of direction texel (j, k): the phases tile the octahedral map
// in a pattern of a x b texels (a * b = nph), so a phase's directions are a
// regular sub-lattice spread over the whole sphere.  Training and held-out
// samples are every probe of the far levels with the directions of phase ph
// and of phase ph + nph/2 respectively.
__host__ __device__ __forceinline__ int nrc_dir_phase(int d, int n, int nph) {
  int t = 0;
  while ((1 << t) < nph) ++t;
  const int a = 1 << ((t + 1) / 2), b = nph / a;
  const int j = d % n, k = d / n;
  return (j % a) + a * (k % b);
}

// Probe of bit b of slot `slot`, or -1 when the bit holds no probe.
__host__ __device__ __forceinline__ int64_t nrc_slot_probe(const int32_t M[3], int wpp, int l2px, int slot, int b) {
  const int z = slot / wpp, g = (slot - z * wpp) * 32 + b;
  const int x = g & ((1 << l2px) - 1), y = g >> l2px;
  if (x >= M[0] || y >= M[1] || z >= M[2]) return -1;
  return ((int64_t)z * M[1] + y) * M[0] + x;
}

struct NrcWordArgs {
  NrcLevel lv[kMaxCascades];
  int32_t first, nlev;
  const int32_t* plain;
  const uint8_t* flag;
  int32_t tile_shift, TX, TY;
  int64_t slot0[kMaxCascades + 1];  // first global slot of each far level
};

// Walk switch of every word of the far levels (one thread per level and
// slot) for the walk that follows the serve decisions: on for every word of
// a level on its walks and for the words holding a probe of a flagged tile.
__global__ void k_nrc_words(const __grid_constant__ NrcWordArgs w) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.slot0[w.nlev]) return;
  int li = w.first;
  while (li + 1 < w.nlev && i >= w.slot0[li + 1]) ++li;
  const NrcLevel& L = w.lv[li];
  const int slot = (int)(i - w.slot0[li]);
  bool on = __ldg(w.plain + li) != 0;
  for (int b = 0; b < 32 && !on; ++b) {
    const int64_t p = nrc_slot_probe(L.M, L.wpp, L.l2px, slot, b);
    if (p >= 0) on = __ldg(w.flag + nrc_cell(L, p, w.tile_shift, w.TX, w.TY)) != 0;
  }
  if (RC_CHK(&L.word_on[slot], kChkCache)) L.word_on[slot] = on;
}

// Training / held-out targets: row r of tile t is the tile's r-th direction
// of its probe, read from the level's walk records.
__global__ void k_nrc_targets(const __grid_constant__ NrcArgs a, const uint2* __restrict__ vol, int64_t ntiles,
                              float* __restrict__ target) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntiles * kNrcThreads) return;
  const NrcTile t = a.tiles[i / kNrcThreads];
  const int r = (int)(i % kNrcThreads);
  float rt[4] = {0.f, 0.f, 0.f, 0.f};
  if (r < t.n) {
    const NrcLevel& L = a.lv[t.level];
    const int64_t p = t.list ? t.probe + r / t.list : t.probe;
    const int d = t.list ? __ldg(a.dlist + t.d0 + r % t.list) : t.d0 + r;
    const uint32_t* rp = L.rec + nrc_rec_index(L, p, d);
    nrc_record_rt(vol, RC_CHK(rp, kChkRecord) ? __ldg(rp) : kBlack, rt);
  }
  float4* tp = reinterpret_cast<float4*>(target + i * 4);
  if (RC_CHK(tp, kChkCache)) *tp = make_float4(rt[0], rt[1], rt[2], rt[3]);
}

// Trilinear taps of probe p of a level into the next level's probes (child
// index m sits at parent coordinate m/2 - 1/4, clamped): offsets and weights.
__device__ __forceinline__ void merge_taps(const LevelArgs& a, int64_t p, int tap_off[8], float tap_w[8]) {
  const int Mx = a.M[0], My = a.M[1];
  // probe coordinates in 32-bit arithmetic (a level has fewer than 2^31 probes)
  const uint32_t pu = (uint32_t)p, rowi = pu / (uint32_t)Mx;
  const int mx = (int)(pu - rowi * (uint32_t)Mx), mz = (int)(rowi / (uint32_t)My), my = (int)(rowi - (uint32_t)mz * (uint32_t)My);
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

// Held-out error per fallback tile.  A held-out query (p, d) of far level i
// enters the merged radiance L_c = R_c + T M_c(p, d), M = the trilinear blend
// of the next level's child-averaged radiance (the values of the previous
// solve, which this solve's merges overwrite later; zero at the top level).
// The tile of p accumulates sum Omega_d |L^ - L|^2 (L^ from the served
// network output) and sum Omega_d |L|^2 over its held-out queries: the
// solid-angle-weighted relative L2 error of the radiance the level hands to
// the merges below.  One block = one tile; rows of one probe are contiguous,
// so a segmented warp scan sums them and the last lane of each segment adds
// the sums to the probe's cell.
struct NrcLevelArgs {
  LevelArgs lv[kMaxCascades];
};

template <typename T>
__global__ void __launch_bounds__(kNrcThreads) k_nrc_heldout(const __grid_constant__ NrcArgs a,
                                                            const __grid_constant__ NrcLevelArgs lv,
                                                            const float* __restrict__ pred,
                                                            const float* __restrict__ target,
                                                            float* __restrict__ num, float* __restrict__ den) {
  const NrcTile t = a.tiles[blockIdx.x];
  const int r = threadIdx.x, lane = r & 31;
  const int seg = t.list ? r / t.list : 0;  // row's probe within the tile
  const int64_t p = t.probe + seg;
  float e2 = 0.f, s2 = 0.f;
  if (r < t.n) {
    const int64_t i = (int64_t)blockIdx.x * kNrcThreads + r;
    const float4* pp = reinterpret_cast<const float4*>(pred + i * 4);
    const float4* yp = reinterpret_cast<const float4*>(target + i * 4);
    const float4 pr = RC_CHK(pp, kChkCache) ? *pp : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 y = RC_CHK(yp, kChkCache) ? *yp : make_float4(0.f, 0.f, 0.f, 0.f);
    const float po[4] = {pr.x, pr.y, pr.z, pr.w};
    float sv[4];
    nrc_serve(po, a.scale, sv);
    const int d = t.list ? __ldg(a.dlist + t.d0 + r % t.list) : t.d0 + r;
    const NrcLevel& L = a.lv[t.level];
    const LevelArgs& la = lv.lv[t.level];
    float M[3] = {0.f, 0.f, 0.f};
    if (t.level + 1 < a.nlev) {
      int tap_off[8];
      float tap_w[8];
      merge_taps(la, p, tap_off, tap_w);
      const T* Au = static_cast<const T*>(la.A_up);
#pragma unroll
      for (int tp = 0; tp < 8; ++tp) {
        const float3 v = load_rgb<T, false>(rgb4_at(Au, d, la.P_up, tap_off[tp]));
        M[0] = fmaf(tap_w[tp], v.x, M[0]);
        M[1] = fmaf(tap_w[tp], v.y, M[1]);
        M[2] = fmaf(tap_w[tp], v.z, M[2]);
      }
    }
    const float om = __ldg(L.omega + d);
    const float Y[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      const float lw = fmaf(Y[3], M[ch], Y[ch]), ls = fmaf(sv[3], M[ch], sv[ch]);
      e2 = fmaf(om * (ls - lw), ls - lw, e2);
      s2 = fmaf(om * lw, lw, s2);
    }
  }
  // rows past t.n belong to no probe: give them a key of their own
  const int key = r < t.n ? seg : -1 - r;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int k2 = __shfl_up_sync(0xFFFFFFFFu, key, off);
    const float ea = __shfl_up_sync(0xFFFFFFFFu, e2, off), sa = __shfl_up_sync(0xFFFFFFFFu, s2, off);
    if (lane >= off && k2 == key) {
      e2 += ea;
      s2 += sa;
    }
  }
  const int next = __shfl_down_sync(0xFFFFFFFFu, key, 1);
  if (r < t.n && (lane == 31 || next != key)) {
    const int64_t cell = nrc_cell(a.lv[t.level], p, a.tile_shift, a.TX, a.TY);
    if (!RC_CHK(&num[cell], kChkCache) || !RC_CHK(&den[cell], kChkCache)) return;
    atomicAdd(&num[cell], e2);
    // the smallest normal float marks the cell as scored this solve even where
    // no light reaches its probes
    atomicAdd(&den[cell], s2 + 1.17549435e-38f);
  }
}

// Fallback flags from the held-out sums of this solve (num, den) and of the
// last `window` solves (ring[window][2][n], this solve's sums go to row
// `slot`).  Each solve scores another sub-lattice of directions, so the
// window covers every direction of the cell.  A cell scored this solve is
// flagged when the relative error of this solve or of the window exceeds the
// threshold; cells not scored this solve keep their flag.  Clears num, den.
__global__ void k_nrc_flags(float* __restrict__ num, float* __restrict__ den, float* __restrict__ ring, int window,
                            int slot, uint8_t* __restrict__ flag, int64_t n, float thr2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float e = num[i], s = den[i];
  ring[((int64_t)slot * 2) * n + i] = e;
  ring[((int64_t)slot * 2 + 1) * n + i] = s;
  if (e > 0.f || s > 0.f) {
    float we = 0.f, ws = 0.f;
    for (int k = 0; k < window; ++k) {
      we += ring[((int64_t)k * 2) * n + i];
      ws += ring[((int64_t)k * 2 + 1) * n + i];
    }
    flag[i] = (e > thr2 * fmaxf(s, 1e-6f) || we > thr2 * fmaxf(ws, 1e-6f)) ? 1 : 0;
  }
  num[i] = 0.f;
  den[i] = 0.f;
}

// Probes of each far level that sit in fallback tiles.
__global__ void k_nrc_count(const __grid_constant__ NrcArgs a, const uint8_t* __restrict__ flag, int shift, int TX,
                            int TY, int64_t total_probes, unsigned* __restrict__ count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total_probes) return;
  int li = a.first;
  int64_t p = i;
  while (li < a.nlev && p >= a.lv[li].P) p -= a.lv[li++].P;
  if (li >= a.nlev) return;
  if (flag[nrc_cell(a.lv[li], p, shift, TX, TY)]) atomicAdd(&count[li], 1u);
}

// Serve decision per far level: a level with at least `fraction` of its
// probes in flagged tiles runs entirely on its walks (plain[level] = 1);
// served[level] counts the solves the network served the level.  Clears the
// counts for the next solve.
__global__ void k_nrc_decide(const __grid_constant__ NrcArgs a, unsigned* __restrict__ count,
                             int32_t* __restrict__ plain, unsigned long long* __restrict__ served, float fraction) {
  const int li = a.first + (int)threadIdx.x;
  if (li >= a.nlev) return;
  const int walk = (double)count[li] >= (double)fraction * (double)a.lv[li].P ? 1 : 0;
  plain[li] = walk;
  if (!walk) ++served[li];
  count[li] = 0u;
}

// ---------------------------------------------------------------------------
// Merge of a far level: per probe the interval results come from the network
// (R, T), or from the walk records when the level runs plain or the probe's
// tile is flagged; then L = R + T * trilinear(A_{i+1}) as in the plain merge.
// One thread per probe, block row = a pair of parent texels (eight child
// directions).
// ---------------------------------------------------------------------------
template <typename T, bool TOP>
__global__ void __launch_bounds__(128) k_level_merge_nrc(const __grid_constant__ LevelArgs a,
                                                         const __grid_constant__ NrcArgs n, int level) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.P) return;
  const NrcLevel& NL = n.lv[level];
  const bool walked = __ldg(n.plain + level) != 0 || __ldg(n.flag + nrc_cell(NL, p, n.tile_shift, n.TX, n.TY)) != 0;
  int tap_off[8];
  float tap_w[8];
  if (!TOP) merge_taps(a, p, tap_off, tap_w);
  T* L = static_cast<T*>(a.L);
  const T* Au = static_cast<const T*>(a.A_up);
  const int hn = a.n >> 1;
  const int64_t plane = (int64_t)a.ndirs * a.P;
  const __half* rt = NL.rt;
  float acc[3] = {0.f, 0.f, 0.f};
#pragma unroll 1
  for (int dl = 0; dl < 8; ++dl) {
    const int dp = blockIdx.y * 2 + (dl >> 2), c = dl & 3;
    const int d = (2 * (dp / hn) + (c >> 1)) * a.n + 2 * (dp % hn) + (c & 1);
    const int64_t off = (int64_t)d * a.P + p;
    float rv[4];
    if (walked) {
      const uint32_t* rp = NL.rec + nrc_rec_index(NL, p, d);
      nrc_record_rt(a.vol, RC_CHK(rp, kChkRecord) ? __ldg(rp) : kBlack, rv);
    } else {
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) rv[ch] = RC_CHK(&rt[ch * plane + off], kChkCache) ? __half2float(rt[ch * plane + off]) : 0.f;
    }
    if (!TOP && rv[3] > 0.f) {
      float sum[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int tp = 0; tp < 8; ++tp) {
        const float3 v = load_rgb<T, false>(rgb4_at(Au, d, a.P_up, tap_off[tp]));
        sum[0] = fmaf(tap_w[tp], v.x, sum[0]);
        sum[1] = fmaf(tap_w[tp], v.y, sum[1]);
        sum[2] = fmaf(tap_w[tp], v.z, sum[2]);
      }
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) rv[ch] = fmaf(rv[3], sum[ch], rv[ch]);
    }
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      Store<T>::stream(L + ((int64_t)ch * a.ndirs + d) * a.P + p, rv[ch]);
      acc[ch] += rv[ch];
    }
    if ((dl & 3) == 3) {
      store_avg<T>(a, dp, p, 0.25f * acc[0], 0.25f * acc[1], 0.25f * acc[2]);
      acc[0] = acc[1] = acc[2] = 0.f;
    }
  }
}

}  // namespace rcx
