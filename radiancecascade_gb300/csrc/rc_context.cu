// rc_context.cu -- the C ABI of include/rc.h that needs the GPU: context
// lifetime, scene upload and emitter update, the per-frame solve and result
// read-back.  One context = one scene on one GPU, ordered on one stream.
//
// Reference boundary: a GI stage implementing RenderStage (src/app.rs:3-7)
// calls rc_create/rc_destroy from resize(), rc_scene_* from update() and
// rc_solve from render(); see include/rc.h.

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "rc_ctx.h"
#include "rc_level0.cuh"
#include "rc_batch.cuh"
#include "rc_mesh.cuh"
#include "rc_shade.cuh"

using namespace rcx;

namespace rcx {

rc_status cuda_fail(cudaError_t e, const char* what) {
  rcx::set_error("%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? RC_ERR_OOM : RC_ERR_CUDA;
}

bool fault_is(const char* name) {
  const char* f = getenv("RC_FAULT");
  return f && strcmp(f, name) == 0;
}

rc_status dev_alloc(void** ptr, size_t bytes, const char* what) {
  if (fault_is("alloc")) {
    rcx::set_error("%s: injected allocation failure (RC_FAULT=alloc)", what);
    return RC_ERR_OOM;
  }
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    (void)cudaGetLastError();
    return cuda_fail(e, what);
  }
#ifdef RC_CHECKED
  check_register(*ptr, bytes);
  if ((e = check_prepare()) != cudaSuccess) return cuda_fail(e, "checked build: range upload");
#endif
  return RC_OK;
}

}  // namespace rcx

namespace {

void release(rc_context* c) {
  if (!c) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  nrc_release(c);
  if (c->flu[1]) cudaFree(c->flu[1]);
  for (void* b : c->scratch)
    if (b) cudaFree(b);
  for (int k = 0; k < 2; ++k) {
    if (c->ev_solved[k]) cudaEventDestroy(c->ev_solved[k]);
    if (c->ev_copied[k]) cudaEventDestroy(c->ev_copied[k]);
  }
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->graph) cudaGraphExecDestroy(c->graph);
  for (cudaEvent_t ev : c->tev)
    if (ev) cudaEventDestroy(ev);
  void* bufs[] = {c->err, c->recs, c->qcounter, c->base, c->vol, c->occ, c->emis, c->masks, c->dirs, c->rad, c->avg, c->flu[0], c->d_sph, c->qsteps, c->qstep_begin};  // d_reg, d_slist point into d_sph
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  if (c->ev_in) cudaEventDestroy(c->ev_in);
  if (c->ev_out) cudaEventDestroy(c->ev_out);
  for (cudaEvent_t ev : c->ev_stage)
    if (ev) cudaEventDestroy(ev);
  if (c->stream) cudaStreamDestroy(c->stream);
  cudaSetDevice(prev);
  delete c;
}

rc_status check_ctx(const rc_context* c, const char* fn) {
  if (!c) {
    rcx::set_error("%s: context is NULL", fn);
    return RC_ERR_INVALID_ARG;
  }
  return RC_OK;
}

// Sphere-list entries per sphere of capacity: the lists of one update hold at
// most this many entries per sphere, else every region tests all spheres.
constexpr int kSphereListCap = 8;

// Grow the sphere/region device buffers and the pinned staging area.
rc_status ensure_sphere_capacity(rc_context* c, int n) {
  if (n <= c->sph_cap) return RC_OK;
  int cap = std::max(64, c->sph_cap);
  while (cap < n) cap *= 2;
  for (int k = 0; k < 2; ++k)
    if (c->stage_pending[k]) {
      RC_CUDA(cudaEventSynchronize(c->ev_stage[k]), "staging wait");
      c->stage_pending[k] = false;
    }
  if (c->d_sph) cudaFree(c->d_sph);
  if (c->h_stage) cudaFreeHost(c->h_stage);
  c->d_sph = nullptr;
  c->d_reg = nullptr;
  c->d_slist = nullptr;
  c->h_stage = nullptr;
  c->sph_cap = 0;
  // one device buffer laid out as a staging slot (spheres, regions, sphere
  // lists), so that an update is one host-to-device copy
  c->slot_bytes = sizeof(QSphere) * cap + sizeof(Region) * (2 * cap + 1) + sizeof(int32_t) * kSphereListCap * cap;
  rc_status s = dev_alloc((void**)&c->d_sph, c->slot_bytes, "sphere buffer");
  if (s != RC_OK) return s;
  c->d_reg = reinterpret_cast<Region*>(reinterpret_cast<char*>(c->d_sph) + sizeof(QSphere) * cap);
  c->d_slist = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(c->d_reg) + sizeof(Region) * (2 * cap + 1));
  RC_CUDA(cudaMallocHost(&c->h_stage, 2 * c->slot_bytes), "pinned staging buffer");
  c->sph_cap = cap;
  return RC_OK;
}

// A level kernel that may start while the one before it in the stream
// finishes (programmatic stream serialization): it waits on the device
// (grid_dep_wait) before it reads what that kernel wrote.
template <typename... KArgs, typename... Args>
void launch_overlapped(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k, args...);
}

// Recompose the given regions of the volume from the base and the current
// spheres.  regions == nullptr means the whole grid.
rc_status recompose(rc_context* c, const Region* regions, int nreg) {
  RC_CUDA(check_prepare(), "checked build: range upload");
  const int n = (int)c->cur.size();
  rc_status s = ensure_sphere_capacity(c, std::max(n, 1));
  if (s != RC_OK) return s;
  // Alternate between two pinned slots; a slot is rewritten only after its
  // previous copies (issued two updates ago) have completed.
  const int k = c->slot;
  c->slot ^= 1;
  if (c->stage_pending[k]) {
    RC_CUDA(cudaEventSynchronize(c->ev_stage[k]), "staging wait");
    c->stage_pending[k] = false;
  }
  Region whole{0, c->W, 0, c->p.grid[1], 0, c->p.grid[2], 0, -1};
  if (!regions) {
    regions = &whole;
    nreg = 1;
  }
  if (nreg == 0) return RC_OK;
  {
    // a small update travels in the launch's parameters: no copy, no staging slot
    const size_t reg_off = (sizeof(QSphere) * (size_t)n + 15) & ~(size_t)15;
    const size_t list_off = reg_off + sizeof(Region) * (size_t)nreg;
    if (regions != &whole && list_off <= (size_t)kComposeInlineBytes) {
      ComposeInline in;
      if (n) memcpy(in.b, c->cur.data(), sizeof(QSphere) * n);
      Region* ireg = reinterpret_cast<Region*>(in.b + reg_off);
      memcpy(ireg, regions, sizeof(Region) * nreg);
      // per-region sphere lists where they fit (sphere_lists falls back to
      // "test every sphere" itself when they do not)
      const int64_t room = ((int64_t)kComposeInlineBytes - (int64_t)list_off) / (int64_t)sizeof(int32_t);
      if (room > 0)
        (void)sphere_lists(c->cur.data(), n, c->p.grid, ireg, nreg, reinterpret_cast<int32_t*>(in.b + list_off), room);
      else
        for (int i = 0; i < nreg; ++i) {
          ireg[i].s0 = 0;
          ireg[i].sn = -1;
        }
      int64_t words = 0;
      for (int i = 0; i < nreg; ++i)
        words = std::max<int64_t>(words, (int64_t)(regions[i].w1 - regions[i].w0) * (regions[i].y1 - regions[i].y0) *
                                             (regions[i].z1 - regions[i].z0));
      const int threads = 256;
      int64_t blocks = (words * 32 + threads - 1) / threads;
      blocks = std::min<int64_t>(std::max<int64_t>(blocks, 1), 152 * 16);
      // programmatic: the base reads and sphere tests overlap the previous
      // frame's cascade 0, the writes wait for it on the device
      launch_overlapped(k_compose_masks_inline, dim3((unsigned)blocks, (unsigned)nreg), dim3(threads), 0, c->stream,
                        (const uint2*)c->base, c->vol, c->occ, c->emis, c->p.grid[0], c->p.grid[1], c->p.grid[2],
                        c->W, n, (int)reg_off, (int)list_off, c->mset, in);
      RC_CUDA(cudaGetLastError(), "compose launch");
      return RC_OK;
    }
  }
  char* st = static_cast<char*>(c->h_stage) + k * c->slot_bytes;
  if (n) memcpy(st, c->cur.data(), sizeof(QSphere) * n);
  Region* sreg = reinterpret_cast<Region*>(st + sizeof(QSphere) * c->sph_cap);
  int32_t* slist = reinterpret_cast<int32_t*>(st + sizeof(QSphere) * c->sph_cap + sizeof(Region) * (2 * c->sph_cap + 1));
  memcpy(sreg, regions, sizeof(Region) * nreg);
  // per-region lists of the spheres whose extent meets the region (a region
  // of the whole grid, or an update whose lists would not fit, tests them all)
  const int64_t listed = sphere_lists(c->cur.data(), n, c->p.grid, sreg, nreg, slist,
                                      (int64_t)kSphereListCap * c->sph_cap);
  // spheres, regions and lists in one copy (the slot's layout is the buffer's)
  const size_t used = listed ? (size_t)(reinterpret_cast<char*>(slist + listed) - st)
                             : (size_t)(reinterpret_cast<char*>(sreg + nreg) - st);
  RC_CUDA(cudaMemcpyAsync(c->d_sph, st, used, cudaMemcpyHostToDevice, c->stream), "sphere upload");
  RC_CUDA(cudaEventRecord(c->ev_stage[k], c->stream), "event record");
  c->stage_pending[k] = true;
  int64_t words = 0;
  for (int i = 0; i < nreg; ++i)
    words = std::max<int64_t>(words, (int64_t)(regions[i].w1 - regions[i].w0) * (regions[i].y1 - regions[i].y0) *
                                         (regions[i].z1 - regions[i].z0));
  const int threads = 256;
  int64_t blocks = (words * 32 + threads - 1) / threads;
  blocks = std::min<int64_t>(std::max<int64_t>(blocks, 1), 152 * 16);
  k_compose_masks<<<dim3((unsigned)blocks, (unsigned)nreg), threads, 0, c->stream>>>(
      c->base, c->vol, c->occ, c->emis, c->p.grid[0], c->p.grid[1], c->p.grid[2], c->W, c->d_sph, n, c->d_reg,
      c->d_slist, c->mset);
  RC_CUDA(cudaGetLastError(), "compose launch");
  return RC_OK;
}

// Decimated-plane geometry of one level (see rc_walk_bits.cuh).  Levels wider
// than 256 probes per row walk with the scalar kernel.
// How a level is solved: the scalar walk (one thread per probe and direction),
// the fused bit-parallel kernel (wide levels), or the shared walk queue plus a
// merge kernel (narrow levels).
enum { kModeScalar = 0, kModeFused = 1, kModeQueue = 2, kModeDirect0 = 3, kModeTma0 = 4 };

// A level keeps decimated masks when it walks bit-parallel; the walk-free
// cascade 0 reads the full-resolution bit planes instead, so its masks are
// neither allocated nor updated.
bool needs_mask(const bool* bits_level, const int* mode, int i) {
  return bits_level[i] && !(i == 0 && (mode[0] == kModeDirect0 || mode[0] == kModeTma0));
}

struct MaskGeom {
  bool bits;
  int mode;
  int32_t l2px, wpp, tiles;
  uint32_t rep;
  int64_t words;
};

MaskGeom mask_geom(const LevelGeom& g, bool force_scalar) {
  MaskGeom m{};
  m.l2px = 0;
  while ((1 << m.l2px) < g.M[0]) ++m.l2px;
  const int64_t px = (int64_t)1 << m.l2px;
  m.wpp = (int32_t)((g.M[1] * px + 31) / 32);
  m.words = (int64_t)g.spacing * g.spacing * g.spacing * g.M[2] * m.wpp;
  // the bit-parallel kernels address a level's radiance and its decimated
  // words with 32-bit element offsets
  m.bits = !force_scalar && px <= 256 && 3 * (int64_t)g.ndirs * g.probes() < ((int64_t)1 << 31) &&
           m.words < ((int64_t)1 << 31);
  m.rep = 0;
  if (px < 32)
    for (int r = 0; r < 32 / px; ++r) m.rep |= 1u << (r * px);
  if (m.l2px >= 5) {
    m.tiles = ((g.M[2] + 1) / 2) * ((m.wpp + 15) / 16);
  } else {
    const int tw = std::min(m.wpp, 32), tz = std::max(1, 32 / tw);
    m.tiles = ((g.M[2] + tz - 1) / tz) * ((m.wpp + tw - 1) / tw);
  }
  m.mode = !m.bits ? kModeScalar : (m.l2px >= 5 ? kModeFused : kModeQueue);
  return m;
}

// Cascade 0 needs no walk when its every interval holds only the start voxel
// (see rc_level0.cuh); then k_level0_direct solves it.
bool level0_direct(const rc_params& p, const LevelGeom& g0, bool force_scalar) {
  return !force_scalar && g0.spacing == 2 && g0.M[0] % 4 == 0 && max_level_steps(g0, p.grid) == 0;
}



// cuTensorMapEncodeTiled, reached through the runtime (no libcuda link).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* ptr = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
    else
      (void)cudaGetLastError();
  }
  return fn;
}

// Cascade 0 through k_level0_tma: the walk-free cascade 0 with its parent
// tiles staged by TMA.  Needs a tensor map over cascade 1's child-averaged
// radiance viewed as [3 * dirs0 * UMz][UMy][UMx] with 16-byte aligned rows.
// Tensor map over a level's child-averaged radiance ([dir][probe][4] texels
// of es-byte values) for boxes of UMx x rows x planes texels starting at x =
// 0: FP32 as a 4-D map (channel, x, y, direction x plane) -- a texel is 16
// bytes, the smallest inner box; FP16 as a 3-D map of 8-byte texels, which
// needs an even UMx for 16-byte rows.  False when the box breaks a copy rule.
bool encode_rgb4_map(PFN_cuTensorMapEncodeTiled_v12000 enc, CUtensorMap* map, const void* A, int UMx, int UMy,
                     int64_t zplanes, int rows, int planes, size_t es) {
  if (UMx < 2 || UMx > 256 || rows > 256 || planes > 256) return false;
  CUresult r;
  if (es == 4) {
    cuuint64_t dims[4] = {4, (cuuint64_t)UMx, (cuuint64_t)UMy, (cuuint64_t)zplanes};
    cuuint64_t strides[3] = {16, (cuuint64_t)UMx * 16, (cuuint64_t)UMx * UMy * 16};
    cuuint32_t box[4] = {4, (cuuint32_t)UMx, (cuuint32_t)rows, (cuuint32_t)planes};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void*>(A), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  } else {
    if (UMx % 2 != 0) return false;
    cuuint64_t dims[3] = {(cuuint64_t)UMx, (cuuint64_t)UMy, (cuuint64_t)zplanes};
    cuuint64_t strides[2] = {(cuuint64_t)UMx * 8, (cuuint64_t)UMx * UMy * 8};
    cuuint32_t box[3] = {(cuuint32_t)UMx, (cuuint32_t)rows, (cuuint32_t)planes};
    cuuint32_t estr[3] = {1, 1, 1};
    r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void*>(A), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  }
  return r == CUDA_SUCCESS;
}

// Dynamic shared memory of one k_level0_tma block: `stages` stages of three
// 128-byte aligned channel tiles (ZC + 1 planes x rows x umx values of es
// bytes), their barriers, up to 127 bytes to align the base.
constexpr size_t level0_tma_bytes(int stages, int rows, int umx, size_t es) {
  return stages * (3 * (((size_t)(kL0Planes + 1) * rows * umx * es + 127) & ~(size_t)127)) + 16 * (size_t)stages + 128;
}
// Every instantiation fits a block's 227 KB limit, and the compiled 32- and
// 64-wide forms (five stages) still fit two blocks in an SM's 228 KB (1 KB of
// it reserved per block).
static_assert(level0_tma_bytes(l0_stages(0), kL0TileRows, 256, sizeof(float)) <= 227 * 1024, "generic cascade-0 tiles");
static_assert(level0_tma_bytes(l0_stages(128), kL0TileRows, 128, sizeof(float)) <= 227 * 1024, "128-wide cascade-0 tiles");
static_assert(2 * (level0_tma_bytes(l0_stages(64), kL0TileRows, 64, sizeof(float)) + 1024) <= 228 * 1024,
              "two blocks per SM with 64-wide cascade-0 tiles");

// The shared-memory limit of every k_level0_tma instantiation of element type
// T: the most any context can need (the generic form: rows of up to 256
// values), so that a later context never lowers it under an earlier one.
template <typename T>
cudaError_t level0_tma_smem() {
  auto set = [](auto kernel, size_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  };
  cudaError_t e = set(k_level0_tma<T, kL0Planes>, level0_tma_bytes(l0_stages(0), kL0TileRows, 256, sizeof(float)));
  if (e == cudaSuccess)
    e = set(k_level0_tma<T, kL0Planes, 32>, level0_tma_bytes(l0_stages(32), kL0TileRows, 32, sizeof(T)));
  if (e == cudaSuccess)
    e = set(k_level0_tma<T, kL0Planes, 64>, level0_tma_bytes(l0_stages(64), kL0TileRows, 64, sizeof(T)));
  if (e == cudaSuccess)
    e = set(k_level0_tma<T, kL0Planes, 128>, level0_tma_bytes(l0_stages(128), kL0TileRows, 128, sizeof(T)));
  return e;
}

bool setup_tma0(rc_context* c) {
  if (c->nlev < 2 || c->mode[0] != kModeDirect0) return false;
  const LevelArgs& a = c->args[0];
  const int UMx = a.UM[0], UMy = a.UM[1], UMz = a.UM[2];
  const size_t es = c->elem;
  if (UMx < 2 || UMx > 256 || (UMx * es) % 16 != 0) return false;
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  // cascade 1's child averages in the planar layout (set_average_layouts)
  const int py = std::min(kL0TileRows, UMy);
  cuuint64_t dims[3] = {(cuuint64_t)UMx, (cuuint64_t)UMy, (cuuint64_t)UMz * 3 * (cuuint64_t)a.ndirs};
  cuuint64_t strides[2] = {(cuuint64_t)UMx * es, (cuuint64_t)UMx * UMy * es};
  cuuint32_t box[3] = {(cuuint32_t)UMx, (cuuint32_t)py, (cuuint32_t)(kL0Planes + 1)};
  cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = enc(&c->tma0, es == 2 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                         const_cast<void*>(a.A_up), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return false;
  // The shared-memory limit is a property of the kernel, not of this context.
  cudaError_t e = es == 2 ? level0_tma_smem<__half>() : level0_tma_smem<float>();
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  c->tma0_py = py;
  c->mode[0] = kModeTma0;
  return true;
}

// Wide levels between cascade 0 and the top: stage the next level's
// child-averaged radiance by TMA where the box fits the copy rules (row pitch
// a multiple of 16 bytes, at most 256 values per row, a box inside the level).
void setup_tma_up(rc_context* c) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
  for (int i = 1; i + 1 < c->nlev; ++i) {
    if (c->mode[i] != kModeFused) continue;
    LevelArgs& a = c->args[i];
    const int UMx = a.UM[0], UMy = a.UM[1], UMz = a.UM[2];
    const int BY = (512 >> a.l2px) / 2 + 2;  // a block tile holds 512 / Px rows of each of its two planes
    const size_t es = c->elem;
    if (UMy < BY || UMz < 3) continue;
    if (!enc && !(enc = tensor_map_encoder())) return;
    if (!encode_rgb4_map(enc, &c->tmap_up[i], a.A_up, UMx, UMy, (int64_t)UMz * a.ndirs, BY, 3, es)) continue;
    // the kernel's shared-memory limit: the largest box any level can need
    // (512 / Px rows / 2 + 2 rows of Px / 2 FP32 values; largest at Px = 256)
    const int smem = (int)bits_up_smem(up_tile_stride((512 >> 8) / 2 + 2, 128, 4));
    cudaError_t e = es == 2 ? cudaFuncSetAttribute(k_level_bits_up<__half>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)
                            : cudaFuncSetAttribute(k_level_bits_up<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return;
    }
    a.up_rows = BY;
    c->tma_up[i] = true;
  }
}

// Reads and clears the device error flag; a bounded wait that ran out
// becomes RC_ERR_TIMEOUT.
rc_status check_device_error(rc_context* c, const char* fn) {
  if (!c->err) return RC_OK;
  int flag = 0;
  cudaError_t e = cudaMemcpy(&flag, c->err, sizeof flag, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, fn);
  if (flag) {
    cudaMemset(c->err, 0, sizeof(int));
    rcx::set_error("%s: a bounded device-side wait ran out (results of that solve are incomplete)", fn);
    return RC_ERR_TIMEOUT;
  }
  return RC_OK;
}

template <typename T, bool L0, bool TOP>
void launch_one(const rc_context* c, int level, cudaStream_t s) {
  const LevelArgs& a = c->args[level];
  const int threads = 128;
  switch (c->mode[level]) {
    case kModeFused: {
      const unsigned groups = L0 ? 1u : (unsigned)((a.n / 2) * (a.n / 2) / 2);  // two parent texels per block
      if (!L0 && !TOP && c->tma_up[level]) {
        const size_t smem = bits_up_smem(up_tile_stride(a.up_rows, a.UM[0], (int)sizeof(T)));
        launch_overlapped(k_level_bits_up<T>, dim3((unsigned)a.tiles * groups), dim3(kBitsThreads), smem, s, a,
                          c->tmap_up[level], c->err);
      } else {
        k_level_bits<T, L0, TOP><<<(unsigned)a.tiles * groups, kBitsThreads, kBitsSmem, s>>>(a);
      }
      break;
    }
    case kModeTma0: {
      if (L0 && !TOP) {
        const int yblocks = (a.M[1] + kL0TmaRows - 1) / kL0TmaRows;
        const unsigned blocks =
            (unsigned)(((a.M[0] + 127) / 128) * yblocks * ((a.M[2] + kL0Planes - 1) / kL0Planes));
        // the common row widths with their tile geometry (and stage count) fixed at compile time
        auto launch = [&](auto kernel, int umxc) {
          const size_t smem = level0_tma_bytes(l0_stages(umxc), c->tma0_py, a.UM[0], sizeof(T));
          launch_overlapped(kernel, dim3(blocks), dim3(kL0Threads), smem, s, a, c->tma0, c->tma0_py, c->err);
        };
        if (c->tma0_py == kL0TileRows && a.UM[0] == 32)
          launch(k_level0_tma<T, kL0Planes, 32>, 32);
        else if (c->tma0_py == kL0TileRows && a.UM[0] == 64)
          launch(k_level0_tma<T, kL0Planes, 64>, 64);
        else if (c->tma0_py == kL0TileRows && a.UM[0] == 128)
          launch(k_level0_tma<T, kL0Planes, 128>, 128);
        else
          launch(k_level0_tma<T, kL0Planes>, 0);
      }
      break;
    }
    case kModeDirect0: {
      if (L0) {
        const int64_t warps = (int64_t)((a.M[0] + 127) / 128) * a.M[1] * ((a.M[2] + 1) / 2);
        k_level0_direct<T, TOP><<<(unsigned)((warps * 32 + kL0Threads - 1) / kL0Threads), kL0Threads, 0, s>>>(a);
      }
      break;
    }
    case kModeQueue: {
      dim3 grid((unsigned)((a.P + threads - 1) / threads), L0 ? 1u : (unsigned)((a.n / 2) * (a.n / 2) / 2));
      if constexpr (TOP)
        launch_overlapped(k_level_merge_top<T, L0>, grid, dim3(threads), 0, s, a,
                          (const uint32_t*)c->rec_level[level], (int)c->rec_slots[level]);
      else
        launch_overlapped(k_level_merge<T, L0, false>, grid, dim3(threads), 0, s, a,
                          (const uint32_t*)c->rec_level[level], (int)c->rec_slots[level]);
      break;
    }
    default: {
      dim3 grid((unsigned)((a.P + threads - 1) / threads), L0 ? 1u : (unsigned)((a.n / 2) * (a.n / 2)));
      k_level_scalar<T, L0, TOP><<<grid, threads, 0, s>>>(a);
    }
  }
}

template <typename T>
void launch_level(const rc_context* c, int level, cudaStream_t s) {
  const bool top = (level == c->nlev - 1);
  if (level == 0) {
    if (top) launch_one<T, true, true>(c, level, s);
    else launch_one<T, true, false>(c, level, s);
  } else {
    if (top) launch_one<T, false, true>(c, level, s);
    else launch_one<T, false, false>(c, level, s);
  }
}

// Walks of the queued levels, except the cascades set in `skip` (bit i =
// cascade i), in one launch (they depend only on the scene).  Each level's
// records have their own place, so a subset of the levels walks in a launch
// of its own with the items renumbered.
void launch_queue_walk(const rc_context* c, cudaStream_t s, uint32_t skip = 0) {
  if (!c->queue_blocks) return;
  const QueueArgs* q = &c->qargs;
  QueueArgs sub;
  bool subset = false;
  for (int k = 0; k < c->qargs.n; ++k) subset |= ((skip >> c->qargs.lv[k].level) & 1u) != 0;
  if (subset) {
    sub = c->qargs;
    sub.n = 0;
    sub.total = 0;
    for (int k = 0; k < c->qargs.n; ++k) {
      const QueueLevel& L = c->qargs.lv[k];
      if ((skip >> L.level) & 1u) continue;
      sub.lv[sub.n] = L;
      sub.lv[sub.n].item_begin = sub.total;
      sub.total += (int64_t)L.slots * c->geom[L.level].ndirs;
      ++sub.n;
    }
    if (!sub.n) return;
    q = &sub;
  }
  // queue_blocks is already capped at one resident wave
  const int64_t blocks = std::min<int64_t>((q->total + kQueueThreads - 1) / kQueueThreads, c->queue_blocks);
  cudaMemsetAsync(q->counter, 0, sizeof(unsigned long long), s);
  if (c->qtab)
    launch_table_walk(*q, c->queue_resident, s);
  else
    k_walk_queue<<<(unsigned)blocks, kQueueThreads, 0, s>>>(*q);
}

}  // namespace

namespace rcx {
void plain_level(const rc_context* c, int level, cudaStream_t s) {
  if (c->elem == 2) launch_level<__half>(c, level, s);
  else launch_level<float>(c, level, s);
}
void plain_queue_walk(const rc_context* c, cudaStream_t s, uint32_t skip) { launch_queue_walk(c, s, skip); }
bool level_uses_queue(const rc_context* c, int level) { return c->mode[level] == kModeQueue; }
}  // namespace rcx

namespace {

// With the neural radiance cache on, the far levels (from its first level
// up) come from the cache and the walk queue runs only when a near level
// needs it.
// NVTX ranges on the enqueueing thread (RC_NVTX=1): "rc_solve", inside it
// "walks" and "cascade i" around the launches of each stage, so that a
// profiler can select a cascade's kernels (ncu --nvtx-include "rc_solve/cascade 3/").
struct NvtxRange {
  bool on;
  NvtxRange(bool enable, const char* name) : on(enable) {
    if (on) nvtxRangePushA(name);
  }
  ~NvtxRange() {
    if (on) nvtxRangePop();
  }
};
bool nvtx_enabled() {
  static const bool on = [] {
    const char* e = getenv("RC_NVTX");
    return e && e[0] == '1';
  }();
  return on;
}
const char* cascade_range_name(int i) {
  static const char* names[kMaxCascades] = {"cascade 0", "cascade 1", "cascade 2", "cascade 3", "cascade 4",
                                            "cascade 5", "cascade 6", "cascade 7", "cascade 8", "cascade 9"};
  return names[i];
}

rc_status enqueue_solve(rc_context* c, cudaStream_t s) {
  RC_CUDA(check_prepare(), "checked build: range upload");
  const bool nv = nvtx_enabled();
  NvtxRange solve_range(nv, "rc_solve");
  int near = c->nlev;
  if (c->timing) cudaEventRecord(c->tev[0], s);
  if (nrc_active(c)) {
    near = nrc_first_level(c);
    bool queue_near = false;
    for (int i = 0; i < near; ++i) queue_near |= c->mode[i] == kModeQueue;
    // the far levels' walks, where they run at all, are launched by the cache
    // (the cache's second far walk takes the near levels' walks along when
    // both use step tables: one launch balances them together)
    if (queue_near && !nrc_walks_near(c)) {
      NvtxRange r(nv, "walks");
      launch_queue_walk(c, s, ~((1u << near) - 1u));
    }
    NvtxRange r(nv, "radiance cache");
    rc_status st = nrc_enqueue_far(c, s);
    if (st != RC_OK) return st;
    // the cache's whole schedule counts under the top cascade
    if (c->timing)
      for (int i = c->nlev - 1; i >= near; --i) cudaEventRecord(c->tev[c->nlev - i], s);
  } else {
    NvtxRange r(nv, "walks");
    launch_queue_walk(c, s);
  }
  for (int i = near - 1; i >= 0; --i) {
    NvtxRange r(nv, cascade_range_name(i));
    plain_level(c, i, s);
    if (c->timing) cudaEventRecord(c->tev[c->nlev - i], s);
  }
  c->timed = c->timing;
  return RC_OK;
}

// Records size of the queue levels, and the queue arguments once `recs` and
// `counter` are placed.  Levels with the longest in-grid intervals are queued
// first so that their walks start early.
size_t queue_records_bytes(const rc_context* c) {
  size_t total = 0;
  for (int i = 0; i < c->nlev; ++i)
    if (c->mode[i] == kModeQueue) total += (size_t)c->geom[i].ndirs * c->rec_slots[i] * 32 * sizeof(uint32_t);
  return total;
}

// Step tables of the queue levels (walk_steps per direction).  Returns
// false, leaving the queue on its own DDA, when a coarse cell does not fit a
// signed byte.
bool build_step_tables(rc_context* c, const std::vector<DirInfo>& tab, std::vector<uint2>& steps,
                       std::vector<int32_t>& begin, int32_t begin_off[kMaxCascades]) {
  static_assert(sizeof(WalkStep) == sizeof(uint2), "a step table entry is a uint2 on the device");
  for (int i = 0; i < c->nlev; ++i) {
    if (c->mode[i] != kModeQueue) continue;
    const LevelGeom& g = c->geom[i];
    begin_off[i] = (int32_t)begin.size();
    for (int d = 0; d < g.ndirs; ++d) {
      if (steps.size() > (size_t)INT32_MAX / 2) return false;
      begin.push_back((int32_t)steps.size());
      const DirInfo& di = tab[c->dir_off[i] + d];
      const int64_t n = walk_steps(g, c->p.grid, di, i == 0, nullptr, 0);  // count first
      if (n < 0) return false;
      const size_t at = steps.size();
      steps.resize(at + (size_t)n);
      walk_steps(g, c->p.grid, di, i == 0, reinterpret_cast<WalkStep*>(steps.data() + at), n);
    }
    begin.push_back((int32_t)steps.size());
  }
  return true;
}

// Resident blocks of the walk kernel on the current device (SMs x blocks per SM).
int queue_resident_blocks(bool tables = false) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      (tables ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_queue_tab, kQueueThreads, 0)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_walk_queue, kQueueThreads, 0)) != cudaSuccess) {
    (void)cudaGetLastError();
    return 152 * 2;
  }
  return std::max(1, sms * per_sm);
}

void setup_queue(rc_context* c, uint32_t* recs, unsigned long long* counter) {
  QueueArgs& q = c->qargs;
  memset(&q, 0, sizeof q);
  c->qcounter = counter;
  q.counter = counter;
  for (int a = 0; a < 3; ++a) q.G[a] = c->p.grid[a];
  q.W = c->W;
  const double diag = sqrt((double)c->p.grid[0] * c->p.grid[0] + (double)c->p.grid[1] * c->p.grid[1] +
                           (double)c->p.grid[2] * c->p.grid[2]);
  int order[kMaxCascades], n = 0;
  for (int i = 0; i < c->nlev; ++i)
    if (c->mode[i] == kModeQueue) order[n++] = i;
  auto reach = [&](int i) {
    return std::min<double>((double)c->geom[i].bhi, diag) - std::min<double>((double)c->geom[i].blo, diag);
  };
  std::sort(order, order + n, [&](int x, int y) { return reach(x) > reach(y); });
  size_t off = 0;
  int64_t items = 0;
  for (int k = 0; k < n; ++k) {
    const int i = order[k];
    const LevelArgs& a = c->args[i];
    QueueLevel& L = q.lv[k];
    L.mask = a.mask;
    L.dirs = a.dirs;
    L.rec = recs + off;
    c->rec_level[i] = L.rec;
    off += (size_t)c->geom[i].ndirs * c->rec_slots[i] * 32;
    L.item_begin = items;
    items += (int64_t)c->geom[i].ndirs * c->rec_slots[i];
    L.slots = c->rec_slots[i];
    L.l2s = a.l2s;
    L.l2px = a.l2px;
    L.wpp = a.wpp;
    for (int ax = 0; ax < 3; ++ax) L.M[ax] = a.M[ax];
    L.rep = a.rep;
    L.test_start = (i == 0);
    L.level = i;
  }
  q.n = n;
  q.total = items;
  // one resident wave of blocks; every lane refills itself from the queue
  c->queue_blocks = n ? (int)std::min<int64_t>((items + kQueueThreads - 1) / kQueueThreads, queue_resident_blocks()) : 0;
}

template <typename T, bool L0, bool TOP>
cudaError_t allow_one() {
  return cudaFuncSetAttribute(k_level_bits<T, L0, TOP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBitsSmem);
}

template <typename T>
cudaError_t allow_bits_smem() {
  cudaError_t e = allow_one<T, true, true>();
  if (e == cudaSuccess) e = allow_one<T, true, false>();
  if (e == cudaSuccess) e = allow_one<T, false, true>();
  if (e == cudaSuccess) e = allow_one<T, false, false>();
  return e;
}

}  // namespace

// Creates a context.  A minimal context is a scene of a batch (solved by the
// batch's persistent kernel or by its own level launches inside the batch's
// graph).
static rc_status create_ctx(const rc_params* p, int32_t device, bool minimal, rc_context** out) {
  if (!out) {
    rcx::set_error("rc_create: out is NULL");
    return RC_ERR_INVALID_ARG;
  }
  *out = nullptr;
  char msg[256];
  if (!validate_params(p, msg, sizeof msg)) {
    rcx::set_error("rc_create: invalid rc_params: %s", msg);
    return RC_ERR_INVALID_ARG;
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    (void)cudaGetLastError();
    rcx::set_error("rc_create: no CUDA device available (%s)", e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
    return RC_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) {
    rcx::set_error("rc_create: device %d out of range (have %d)", device, ndev);
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard guard(device);
  rc_context* c = new rc_context();
  c->p = *p;
  c->device = device;
  c->nlev = p->num_cascades;
  c->elem = p->precision == RC_PRECISION_FP16 ? 2 : 4;
  level_geometry(*p, c->geom);
  c->W = (p->grid[0] + 31) / 32;

  // Direction tables (host), validated for the exact 32-bit walk.
  std::vector<DirInfo> tab;
  for (int i = 0; i < c->nlev; ++i) {
    c->dir_off[i] = tab.size();
    tab.resize(tab.size() + c->geom[i].ndirs);
    if (!build_dir_table(c->geom[i], p->grid, tab.data() + c->dir_off[i], msg, sizeof msg)) {
      rcx::set_error("rc_create: %s", msg);
      delete c;
      return RC_ERR_UNSUPPORTED;
    }
  }
  {
    std::vector<double> om((size_t)c->geom[0].ndirs);
    rc_solid_angles(c->geom[0].n, om.data());
    for (int d = 0; d < c->geom[0].ndirs; ++d) tab[c->dir_off[0] + d].omega = (float)om[d];
  }

  rc_status s = RC_OK;
  auto fail = [&](rc_status st) {
    release(c);
    return st;
  };
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(cuda_fail(e, "rc_create: stream"));
  if ((e = cudaEventCreateWithFlags(&c->ev_in, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&c->ev_out, cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&c->ev_stage[0], cudaEventDisableTiming)) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&c->ev_stage[1], cudaEventDisableTiming)) != cudaSuccess)
    return fail(cuda_fail(e, "rc_create: events"));

  const int64_t nvox = (int64_t)p->grid[0] * p->grid[1] * p->grid[2];
  if ((s = dev_alloc((void**)&c->base, nvox * 8, "scene base volume")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&c->vol, nvox * 8, "scene volume")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&c->occ, (size_t)c->W * p->grid[1] * p->grid[2] * 4, "opacity bits")) != RC_OK)
    return fail(s);
  if ((s = dev_alloc((void**)&c->emis, (size_t)c->W * p->grid[1] * p->grid[2] * 4, "emissive bits")) != RC_OK)
    return fail(s);
  {
    // Decimated opacity and emissive bits per level (bit-parallel walk).
    const bool force_scalar = getenv("RC_WALK") && strcmp(getenv("RC_WALK"), "scalar") == 0;
    int64_t total = 0;
    int64_t off[kMaxCascades];
    c->mset.n = 0;
    for (int i = 0; i < c->nlev; ++i) {
      const MaskGeom mg = mask_geom(c->geom[i], force_scalar);
      c->bits_level[i] = mg.bits;
      c->mode[i] = (i == 0 && level0_direct(*p, c->geom[0], force_scalar)) ? kModeDirect0 : mg.mode;
      c->rec_slots[i] = c->geom[i].M[2] * mg.wpp;
      off[i] = total;
      if (needs_mask(c->bits_level, c->mode, i)) total += (mg.words + 63) & ~(int64_t)63;
    }
    if (total && (s = dev_alloc((void**)&c->masks, total * 8, "decimated opacity and emission")) != RC_OK)
      return fail(s);
    if (total && (e = cudaMemset(c->masks, 0, total * 8)) != cudaSuccess) return fail(cuda_fail(e, "rc_create: memset"));
    for (int i = 0; i < c->nlev; ++i) {
      if (!needs_mask(c->bits_level, c->mode, i)) continue;
      const MaskGeom mg = mask_geom(c->geom[i], force_scalar);
      MaskLevel& m = c->mset.lv[c->mset.n++];
      const LevelGeom& g = c->geom[i];
      m.base = c->masks + off[i];
      m.l2s = 0;
      while ((1 << m.l2s) < g.spacing) ++m.l2s;
      for (int a = 0; a < 3; ++a) m.M[a] = g.M[a];
      m.l2px = mg.l2px;
      m.wpp = mg.wpp;
    }
    if ((e = allow_bits_smem<float>()) != cudaSuccess || (e = allow_bits_smem<__half>()) != cudaSuccess)
      return fail(cuda_fail(e, "rc_create: shared memory attribute"));
  }
  if ((s = dev_alloc((void**)&c->dirs, tab.size() * sizeof(DirInfo), "direction tables")) != RC_OK) return fail(s);
  e = cudaMemcpy(c->dirs, tab.data(), tab.size() * sizeof(DirInfo), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(cuda_fail(e, "rc_create: table upload"));

  size_t rad_bytes = 0, avg_bytes = 0;
  for (int i = 0; i < c->nlev; ++i) {
    const LevelGeom& g = c->geom[i];
    c->rad_off[i] = rad_bytes;
    rad_bytes += ((size_t)3 * g.ndirs * g.probes() * c->elem + 255) & ~(size_t)255;
    c->avg_off[i] = avg_bytes;
    if (i >= 1) avg_bytes += ((size_t)4 * c->geom[i - 1].ndirs * g.probes() * c->elem + 255) & ~(size_t)255;
  }
  if ((s = dev_alloc(&c->rad, rad_bytes, "cascade radiance")) != RC_OK) return fail(s);
  if (avg_bytes && (s = dev_alloc(&c->avg, avg_bytes, "child-averaged radiance")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&c->flu[0], (size_t)c->geom[0].probes() * 3 * sizeof(float), "fluence")) != RC_OK)
    return fail(s);
  c->fluence = c->flu[0];
  if ((s = ensure_sphere_capacity(c, 64)) != RC_OK) return fail(s);

  for (int i = 0; i < c->nlev; ++i) {
    LevelArgs& a = c->args[i];
    const LevelGeom& g = c->geom[i];
    memset(&a, 0, sizeof a);
    {
      const MaskGeom mg = mask_geom(g, false);
      for (int k = 0; k < c->mset.n; ++k)
        if (c->mset.lv[k].M[0] == g.M[0] && c->mset.lv[k].M[1] == g.M[1] && (1 << c->mset.lv[k].l2s) == g.spacing)
          a.mask = c->mset.lv[k].base;
      a.l2px = mg.l2px;
      a.wpp = mg.wpp;
      a.rep = mg.rep;
      a.tiles = mg.tiles;
    }
    a.l2s = 0;
    while ((1 << a.l2s) < g.spacing) ++a.l2s;
    a.emis = c->emis;
    a.occ = c->occ;
    a.vol = c->vol;
    for (int ax = 0; ax < 3; ++ax) {
      a.G[ax] = p->grid[ax];
      a.M[ax] = g.M[ax];
      a.UM[ax] = (i + 1 < c->nlev) ? c->geom[i + 1].M[ax] : 1;
    }
    a.W = c->W;
    a.dirs = c->dirs + c->dir_off[i];
    a.spacing = g.spacing;
    a.n = g.n;
    a.ndirs = g.ndirs;
    a.P = g.probes();
    a.L = static_cast<char*>(c->rad) + c->rad_off[i];
    a.A_out = i >= 1 ? static_cast<char*>(c->avg) + c->avg_off[i] : nullptr;
    a.a_out_planar = (i == 1 && (c->mode[0] == kModeDirect0 || c->mode[0] == kModeTma0)) ? 1 : 0;
    a.A_up = (i + 1 < c->nlev) ? static_cast<char*>(c->avg) + c->avg_off[i + 1] : nullptr;
    a.P_up = (i + 1 < c->nlev) ? c->geom[i + 1].probes() : 0;
    a.fluence = c->fluence;
  }
  {
    const size_t rb = queue_records_bytes(c);
    if (rb) {
      if ((s = dev_alloc((void**)&c->recs, rb, "walk records")) != RC_OK) return fail(s);
      if ((s = dev_alloc((void**)&c->qcounter, sizeof(unsigned long long), "walk queue counter")) != RC_OK)
        return fail(s);
    }
    setup_queue(c, c->recs, c->qcounter);
  }
  if (c->qargs.n > 0 && !(getenv("RC_WALK_TABLES") && strcmp(getenv("RC_WALK_TABLES"), "0") == 0)) {
    std::vector<uint2> st;
    std::vector<int32_t> begin;
    int32_t boff[kMaxCascades] = {};
    if (build_step_tables(c, tab, st, begin, boff) && !st.empty()) {
      if ((s = dev_alloc((void**)&c->qsteps, st.size() * sizeof(uint2), "walk step tables")) != RC_OK) return fail(s);
      if ((s = dev_alloc((void**)&c->qstep_begin, begin.size() * sizeof(int32_t), "walk step tables")) != RC_OK)
        return fail(s);
      if ((e = cudaMemcpy(c->qsteps, st.data(), st.size() * sizeof(uint2), cudaMemcpyHostToDevice)) != cudaSuccess ||
          (e = cudaMemcpy(c->qstep_begin, begin.data(), begin.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) !=
              cudaSuccess)
        return fail(cuda_fail(e, "rc_create: step table upload"));
      for (int k = 0; k < c->qargs.n; ++k) {
        QueueLevel& L = c->qargs.lv[k];
        L.steps = c->qsteps;
        L.step_begin = c->qstep_begin + boff[L.level];
      }
      c->qtab = true;
      c->queue_resident = queue_resident_blocks(true);
      c->queue_blocks = (int)std::min<int64_t>((c->qargs.total + kQueueThreads - 1) / kQueueThreads,
                                               c->queue_resident);
    }
  }
  if ((s = dev_alloc((void**)&c->err, sizeof(int), "error flag")) != RC_OK) return fail(s);
  if ((e = cudaMemset(c->err, 0, sizeof(int))) != cudaSuccess) return fail(cuda_fail(e, "rc_create: memset"));
  if (!(getenv("RC_TMA") && strcmp(getenv("RC_TMA"), "0") == 0)) {
    setup_tma0(c);
    setup_tma_up(c);
  }
  *out = c;
  rcx::log_message(2, "context %p: grid %dx%dx%d, %d cascades, %s, device %d%s", (void*)c, p->grid[0], p->grid[1],
                   p->grid[2], c->nlev, c->elem == 2 ? "fp16" : "fp32", device, minimal ? " (batch scene)" : "");
  return RC_OK;
}

extern "C" {

rc_status rc_create(const rc_params* p, int32_t device, rc_context** out) {
  return create_ctx(p, device, false, out);
}

rc_status rc_destroy(rc_context* ctx) {
  release(ctx);
  return RC_OK;
}

rc_status rc_get_params(const rc_context* ctx, rc_params* out) {
  if (check_ctx(ctx, "rc_get_params") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!out) {
    rcx::set_error("rc_get_params: out is NULL");
    return RC_ERR_INVALID_ARG;
  }
  *out = ctx->p;
  return RC_OK;
}

rc_status rc_scene_upload(rc_context* c, const rc_voxel* voxels, int64_t count, int32_t where) {
  if (check_ctx(c, "rc_scene_upload") != RC_OK) return RC_ERR_INVALID_ARG;
  const int64_t nvox = (int64_t)c->p.grid[0] * c->p.grid[1] * c->p.grid[2];
  if (!voxels || count != nvox || (where != RC_MEM_HOST && where != RC_MEM_DEVICE)) {
    rcx::set_error("rc_scene_upload: need %lld voxels and where = RC_MEM_HOST/RC_MEM_DEVICE", (long long)nvox);
    return RC_ERR_INVALID_ARG;
  }
  if (fault_is("upload")) {
    rcx::set_error("rc_scene_upload: injected upload failure (RC_FAULT=upload)");
    return RC_ERR_CUDA;
  }
  DeviceGuard g(c->device);
  RC_CUDA(cudaMemcpyAsync(c->base, voxels, nvox * 8,
                          where == RC_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, c->stream),
          "rc_scene_upload: copy");
  c->have_base = true;
  rc_status s = recompose(c, nullptr, 0);
  if (s != RC_OK) return s;
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_scene_upload: sync");
  return RC_OK;
}

rc_status rc_scene_set_boxes(rc_context* c, const rc_box* boxes, int32_t n) {
  if (check_ctx(c, "rc_scene_set_boxes") != RC_OK) return RC_ERR_INVALID_ARG;
  // boxes are staged in shared memory: 1536 * 32 B = 48 KB
  if (n < 0 || (n > 0 && !boxes) || n > 1536) {
    rcx::set_error("rc_scene_set_boxes: need 0 <= n <= 1536 boxes and a non-NULL array");
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(c->device);
  rc_box* d_boxes = nullptr;
  if (n) {
    rc_status s = dev_alloc((void**)&d_boxes, sizeof(rc_box) * n, "box upload");
    if (s != RC_OK) return s;
    cudaError_t e = cudaMemcpy(d_boxes, boxes, sizeof(rc_box) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(d_boxes);
      return cuda_fail(e, "rc_scene_set_boxes: copy");
    }
  }
  const int64_t nvox = (int64_t)c->p.grid[0] * c->p.grid[1] * c->p.grid[2];
  const int threads = 256;
  const int64_t blocks = std::min<int64_t>((nvox + threads - 1) / threads, 152 * 32);
  k_boxes_to_base<<<(unsigned)blocks, threads, sizeof(rc_box) * std::max(n, 1), c->stream>>>(
      c->base, c->p.grid[0], c->p.grid[1], c->p.grid[2], d_boxes, n);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (d_boxes) cudaFree(d_boxes);
  if (e != cudaSuccess) return cuda_fail(e, "rc_scene_set_boxes: voxelise");
  c->have_base = true;
  rc_status s = recompose(c, nullptr, 0);
  if (s != RC_OK) return s;
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_scene_set_boxes: sync");
  return RC_OK;
}

rc_status rc_scene_set_mesh(rc_context* c, const float* positions, int64_t nverts, const uint32_t* indices,
                            int64_t ntris, const uint16_t* tri_material, const rc_voxel* materials,
                            int32_t nmaterials) {
  if (check_ctx(c, "rc_scene_set_mesh") != RC_OK) return RC_ERR_INVALID_ARG;
  if (nverts < 0 || ntris < 0 || nverts > (1 << 26) || ntris > (1 << 26) || (nverts && !positions) ||
      (ntris && !indices) || nmaterials < 1 || !materials) {
    rcx::set_error("rc_scene_set_mesh: need vertex and index arrays, at most 2^26 of each, and >= 1 material");
    return RC_ERR_INVALID_ARG;
  }
  std::vector<int32_t> q((size_t)nverts * 3);
  for (int64_t i = 0; i < nverts * 3; ++i) {
    const double v = (double)positions[i] * 256.0;
    if (!(v >= -262144.0 && v <= 524288.0)) {
      rcx::set_error("rc_scene_set_mesh: vertex %lld lies outside [-1024, 2048] voxels", (long long)(i / 3));
      return RC_ERR_INVALID_ARG;
    }
    q[i] = (int32_t)llround(v);
  }
  for (int64_t i = 0; i < ntris * 3; ++i)
    if (indices[i] >= (uint64_t)nverts) {
      rcx::set_error("rc_scene_set_mesh: triangle %lld indexes vertex %u of %lld", (long long)(i / 3), indices[i],
                     (long long)nverts);
      return RC_ERR_INVALID_ARG;
    }
  if (tri_material)
    for (int64_t t = 0; t < ntris; ++t)
      if (tri_material[t] >= nmaterials) {
        rcx::set_error("rc_scene_set_mesh: triangle %lld uses material %u of %d", (long long)t, tri_material[t],
                       nmaterials);
        return RC_ERR_INVALID_ARG;
      }
  DeviceGuard g(c->device);
  const int64_t nvox = (int64_t)c->p.grid[0] * c->p.grid[1] * c->p.grid[2];
  int32_t* d_v = nullptr;
  uint32_t *d_i = nullptr, *d_owner = nullptr;
  uint16_t* d_m = nullptr;
  rc_voxel* d_mat = nullptr;
  auto done = [&](rc_status st) {
    void* bufs[] = {d_v, d_i, d_owner, d_m, d_mat};
    for (void* b : bufs)
      if (b) cudaFree(b);
    return st;
  };
  rc_status s;
  if ((s = dev_alloc((void**)&d_v, std::max<size_t>(1, q.size()) * 4, "mesh vertices")) != RC_OK) return done(s);
  if ((s = dev_alloc((void**)&d_i, std::max<int64_t>(1, ntris * 3) * 4, "mesh indices")) != RC_OK) return done(s);
  if ((s = dev_alloc((void**)&d_owner, nvox * 4, "voxel owners")) != RC_OK) return done(s);
  if ((s = dev_alloc((void**)&d_mat, (size_t)nmaterials * sizeof(rc_voxel), "mesh materials")) != RC_OK)
    return done(s);
  if (tri_material && (s = dev_alloc((void**)&d_m, std::max<int64_t>(1, ntris) * 2, "triangle materials")) != RC_OK)
    return done(s);
  cudaError_t e = cudaSuccess;
  if (nverts) e = cudaMemcpy(d_v, q.data(), q.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && ntris) e = cudaMemcpy(d_i, indices, (size_t)ntris * 12, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && d_m) e = cudaMemcpy(d_m, tri_material, (size_t)ntris * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_mat, materials, (size_t)nmaterials * sizeof(rc_voxel), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_owner, 0, nvox * 4, c->stream);
  if (e != cudaSuccess) return done(cuda_fail(e, "rc_scene_set_mesh: upload"));
  MeshArgs a;
  a.verts = d_v;
  a.indices = d_i;
  a.ntris = ntris;
  a.owner = d_owner;
  for (int k = 0; k < 3; ++k) a.G[k] = c->p.grid[k];
  a.pad = 0;
  if (ntris) {
    const int64_t blocks = std::min<int64_t>((ntris * 32 + 255) / 256, 152 * 16);
    k_mesh_owner<<<(unsigned)blocks, 256, 0, c->stream>>>(a);
  }
  k_mesh_materials<<<(unsigned)std::min<int64_t>((nvox + 255) / 256, 152 * 32), 256, 0, c->stream>>>(
      d_owner, d_m, d_mat, nmaterials, c->base, nvox);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return done(cuda_fail(e, "rc_scene_set_mesh: voxelise"));
  c->have_base = true;
  if ((s = recompose(c, nullptr, 0)) != RC_OK) return done(s);
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_scene_set_mesh: sync");
  return done(RC_OK);
}

rc_status rc_scene_set_spheres(rc_context* c, const rc_sphere* spheres, int32_t n) {
  if (check_ctx(c, "rc_scene_set_spheres") != RC_OK) return RC_ERR_INVALID_ARG;
  if (n < 0 || (n > 0 && !spheres) || n > 65536) {
    rcx::set_error("rc_scene_set_spheres: need 0 <= n <= 65536 and a non-NULL array");
    return RC_ERR_INVALID_ARG;
  }
  if (!c->have_base) {
    rcx::set_error("rc_scene_set_spheres: upload a scene (rc_scene_upload / rc_scene_set_boxes) first");
    return RC_ERR_STATE;
  }
  DeviceGuard g(c->device);
  std::vector<QSphere> next(n);
  for (int i = 0; i < n; ++i) quantise_sphere(spheres[i], &next[i]);
  std::vector<Region> regs;
  bool full = (int)c->cur.size() != n;
  if (!full) {
    // a sphere moving a voxel or less per frame overlaps itself: its old and
    // new extents usually become one region
    regs.resize((size_t)2 * n);
    regs.resize((size_t)update_regions(c->cur.data(), next.data(), n, c->p.grid, regs.data()));
  }
  c->cur.swap(next);
  rc_status s = ensure_sphere_capacity(c, std::max(n, 1));
  if (s != RC_OK) return s;
  return full ? recompose(c, nullptr, 0) : recompose(c, regs.data(), (int)regs.size());
}

rc_status rc_solve(rc_context* c, void* stream) {
  if (check_ctx(c, "rc_solve") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!c->have_base) {
    rcx::set_error("rc_solve: no scene uploaded");
    return RC_ERR_STATE;
  }
  DeviceGuard g(c->device);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
  if (s != c->stream) {
    RC_CUDA(cudaEventRecord(c->ev_in, c->stream), "rc_solve: event");
    RC_CUDA(cudaStreamWaitEvent(s, c->ev_in, 0), "rc_solve: wait");
  }
  if (c->flu[1]) {
    // alternate fluence buffers; wait for a read-back still copying the one reused
    const int b = c->flu_cur ^ 1;
    if (c->copy_pending[b]) RC_CUDA(cudaStreamWaitEvent(s, c->ev_copied[b], 0), "rc_solve: wait");
    c->flu_cur = b;
    c->fluence = c->flu[b];
    c->args[0].fluence = c->flu[b];
  }
  rc_status st = enqueue_solve(c, s);
  if (st != RC_OK) return st;
  RC_CUDA(cudaGetLastError(), "rc_solve: launch");
  ++c->solves;
  rcx::log_message(3, "solve %lld of context %p enqueued (grid %dx%dx%d, %d cascades%s)", (long long)c->solves,
                   (void*)c, c->p.grid[0], c->p.grid[1], c->p.grid[2], c->nlev, nrc_active(c) ? ", cache on" : "");
  if (s != c->stream) {
    RC_CUDA(cudaEventRecord(c->ev_out, s), "rc_solve: event");
    RC_CUDA(cudaStreamWaitEvent(c->stream, c->ev_out, 0), "rc_solve: wait");
  }
  return RC_OK;
}

rc_status rc_synchronize(rc_context* c) {
  if (check_ctx(c, "rc_synchronize") != RC_OK) return RC_ERR_INVALID_ARG;
  DeviceGuard g(c->device);
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_synchronize");
  if (c->copy_stream) {
    RC_CUDA(cudaStreamSynchronize(c->copy_stream), "rc_synchronize");
    c->copy_pending[0] = c->copy_pending[1] = false;
  }
  return check_device_error(c, "rc_synchronize");
}

static rc_status copy_out(rc_context* c, void* out, const void* src, size_t bytes, int32_t where, const char* fn) {
  if (where != RC_MEM_HOST && where != RC_MEM_DEVICE) {
    rcx::set_error("%s: where must be RC_MEM_HOST or RC_MEM_DEVICE", fn);
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(c->device);
  RC_CUDA(cudaMemcpyAsync(out, src, bytes, where == RC_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                          c->stream),
          fn);
  RC_CUDA(cudaStreamSynchronize(c->stream), fn);
  return check_device_error(c, fn);
}

rc_status rc_get_fluence(rc_context* c, float* out, int64_t elems, int32_t where) {
  if (check_ctx(c, "rc_get_fluence") != RC_OK) return RC_ERR_INVALID_ARG;
  const int64_t need = 3 * c->geom[0].probes();
  if (!out || elems != need) {
    rcx::set_error("rc_get_fluence: need a buffer of exactly %lld floats", (long long)need);
    return RC_ERR_INVALID_ARG;
  }
  return copy_out(c, out, c->fluence, need * sizeof(float), where, "rc_get_fluence");
}

rc_status rc_get_radiance(rc_context* c, int32_t level, void* out, int64_t bytes, int32_t where) {
  if (check_ctx(c, "rc_get_radiance") != RC_OK) return RC_ERR_INVALID_ARG;
  if (level < 0 || level >= c->nlev) {
    rcx::set_error("rc_get_radiance: level %d out of range", level);
    return RC_ERR_INVALID_ARG;
  }
  const LevelGeom& g = c->geom[level];
  const int64_t need = 3 * (int64_t)g.ndirs * g.probes() * (int64_t)c->elem;
  if (!out || bytes != need) {
    rcx::set_error("rc_get_radiance: need a buffer of exactly %lld bytes", (long long)need);
    return RC_ERR_INVALID_ARG;
  }
  return copy_out(c, out, static_cast<char*>(c->rad) + c->rad_off[level], need, where, "rc_get_radiance");
}

// Shading scratch slots of a context: 0 vertices, 1 indices, 2 triangle
// materials, 3 materials, 4 texels, 5 texture table (the mesh); 6 depth,
// 7 image, 8 bounds, 9 small list, 10 large list, 11 counts (per draw).
static rc_status shade_scratch(rc_context* c, int slot, size_t bytes, void** p) {
  bytes = std::max<size_t>(bytes, 16);
  if (c->scratch_cap[slot] < bytes) {
    if (c->scratch[slot]) cudaFree(c->scratch[slot]);
    c->scratch[slot] = nullptr;
    c->scratch_cap[slot] = 0;
    rc_status st = dev_alloc(&c->scratch[slot], bytes, "shading scratch");
    if (st != RC_OK) return st;
    c->scratch_cap[slot] = bytes;
  }
  *p = c->scratch[slot];
  return RC_OK;
}

rc_status rc_shade_set_mesh(rc_context* c, const float* vertices, int64_t nverts, const uint32_t* indices,
                            int64_t ntris, const uint16_t* tri_material, const rc_shade_material* materials,
                            int32_t nmaterials, const rc_texture* textures, int32_t ntextures) {
  if (check_ctx(c, "rc_shade_set_mesh") != RC_OK) return RC_ERR_INVALID_ARG;
  if (nverts < 0 || ntris < 0 || ntris >= ((int64_t)1 << 32) || (nverts && !vertices) || (ntris && !indices) ||
      nmaterials < 1 || !materials || ntextures < 0 || (ntextures && !textures)) {
    rcx::set_error("rc_shade_set_mesh: invalid arguments (>= 1 material, non-NULL arrays)");
    return RC_ERR_INVALID_ARG;
  }
  for (int64_t i = 0; i < ntris * 3; ++i)
    if (indices[i] >= (uint64_t)nverts) {
      rcx::set_error("rc_shade: triangle %lld indexes vertex %u of %lld", (long long)(i / 3), indices[i],
                     (long long)nverts);
      return RC_ERR_INVALID_ARG;
    }
  for (int32_t m = 0; m < nmaterials; ++m) {
    const rc_shade_material& mt = materials[m];
    if (((mt.enable_bit & 1u) && (mt.color_texture < 0 || mt.color_texture >= ntextures)) ||
        ((mt.enable_bit & 2u) && (mt.normal_texture < 0 || mt.normal_texture >= ntextures))) {
      rcx::set_error("rc_shade: material %d names a missing texture", m);
      return RC_ERR_INVALID_ARG;
    }
  }
  if (tri_material)
    for (int64_t t = 0; t < ntris; ++t)
      if (tri_material[t] >= nmaterials) {
        rcx::set_error("rc_shade: triangle %lld uses material %u of %d", (long long)t, tri_material[t], nmaterials);
        return RC_ERR_INVALID_ARG;
      }
  for (int32_t k = 0; k < ntextures; ++k)
    if (!textures[k].rgba || textures[k].width < 1 || textures[k].height < 1) {
      rcx::set_error("rc_shade: texture %d is empty", k);
      return RC_ERR_INVALID_ARG;
    }
  DeviceGuard g(c->device);
  c->shade_mesh = false;
  float* d_v = nullptr;
  uint32_t *d_i = nullptr, *d_small = nullptr, *d_big = nullptr;
  uint16_t* d_m = nullptr;
  rc_shade_material* d_mat = nullptr;
  uint8_t* d_texels = nullptr;
  ShadeTex* d_tex = nullptr;
  int4* d_bounds = nullptr;
  size_t texel_bytes = 0;
  for (int32_t k = 0; k < ntextures; ++k) texel_bytes += ((size_t)textures[k].width * textures[k].height * 4 + 15) & ~(size_t)15;
  rc_status st;
  if ((st = shade_scratch(c, 0, (size_t)nverts * kShadeVertexFloats * 4, (void**)&d_v)) != RC_OK ||
      (st = shade_scratch(c, 1, (size_t)ntris * 12, (void**)&d_i)) != RC_OK ||
      (tri_material && (st = shade_scratch(c, 2, (size_t)ntris * 2, (void**)&d_m)) != RC_OK) ||
      (st = shade_scratch(c, 3, (size_t)nmaterials * sizeof(rc_shade_material), (void**)&d_mat)) != RC_OK ||
      (st = shade_scratch(c, 4, texel_bytes, (void**)&d_texels)) != RC_OK ||
      (st = shade_scratch(c, 5, (size_t)std::max(ntextures, 1) * sizeof(ShadeTex), (void**)&d_tex)) != RC_OK ||
      (st = shade_scratch(c, 8, (size_t)ntris * sizeof(int4), (void**)&d_bounds)) != RC_OK ||
      (st = shade_scratch(c, 9, (size_t)ntris * 4, (void**)&d_small)) != RC_OK ||
      (st = shade_scratch(c, 10, (size_t)ntris * 4, (void**)&d_big)) != RC_OK)
    return st;
  cudaStream_t s = c->stream;
  std::vector<ShadeTex> tex((size_t)std::max(ntextures, 1));
  size_t off = 0;
  for (int32_t k = 0; k < ntextures; ++k) {
    const size_t bytes = (size_t)textures[k].width * textures[k].height * 4;
    RC_CUDA(cudaMemcpyAsync(d_texels + off, textures[k].rgba, bytes, cudaMemcpyHostToDevice, s), "rc_shade: upload");
    tex[k] = ShadeTex{d_texels + off, textures[k].width, textures[k].height, textures[k].srgb ? 1 : 0, 0};
    off += (bytes + 15) & ~(size_t)15;
  }
  RC_CUDA(cudaMemcpyAsync(d_tex, tex.data(), tex.size() * sizeof(ShadeTex), cudaMemcpyHostToDevice, s), "rc_shade");
  if (nverts)
    RC_CUDA(cudaMemcpyAsync(d_v, vertices, (size_t)nverts * kShadeVertexFloats * 4, cudaMemcpyHostToDevice, s),
            "rc_shade: upload");
  if (ntris) RC_CUDA(cudaMemcpyAsync(d_i, indices, (size_t)ntris * 12, cudaMemcpyHostToDevice, s), "rc_shade: upload");
  if (d_m) RC_CUDA(cudaMemcpyAsync(d_m, tri_material, (size_t)ntris * 2, cudaMemcpyHostToDevice, s), "rc_shade: upload");
  RC_CUDA(cudaMemcpyAsync(d_mat, materials, (size_t)nmaterials * sizeof(rc_shade_material), cudaMemcpyHostToDevice, s),
          "rc_shade: upload");
  // the host arrays (and the texture table above) may go once this returns
  RC_CUDA(cudaStreamSynchronize(s), "rc_shade_set_mesh");
  c->shade_ntris = ntris;
  c->shade_ntex = ntextures;
  c->shade_tmat = tri_material != nullptr;
  c->shade_mesh = true;
  return RC_OK;
}

rc_status rc_shade_draw(rc_context* c, const rc_shade_view* view, float* out, int32_t where) {
  if (check_ctx(c, "rc_shade_draw") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!view || view->width < 1 || view->height < 1 || view->width > 16384 || view->height > 16384 || !out ||
      (where != RC_MEM_HOST && where != RC_MEM_DEVICE)) {
    rcx::set_error("rc_shade_draw: invalid arguments (image 1..16384 px per side, non-NULL output)");
    return RC_ERR_INVALID_ARG;
  }
  if (!c->shade_mesh) {
    rcx::set_error("rc_shade_draw: no mesh (rc_shade_set_mesh first)");
    return RC_ERR_STATE;
  }
  if (view->gi_scale > 0.f && !c->have_base) {
    rcx::set_error("rc_shade: the GI term needs a solved scene");
    return RC_ERR_STATE;
  }
  DeviceGuard g(c->device);
  const int64_t npix = (int64_t)view->width * view->height;
  const int64_t ntris = c->shade_ntris;
  unsigned long long* d_z = nullptr;
  unsigned* d_counts = nullptr;
  float* d_out = where == RC_MEM_DEVICE ? out : nullptr;
  rc_status st;
  if ((st = shade_scratch(c, 6, (size_t)npix * 8, (void**)&d_z)) != RC_OK ||
      (!d_out && (st = shade_scratch(c, 7, (size_t)npix * 16, (void**)&d_out)) != RC_OK) ||
      (st = shade_scratch(c, 11, 2 * sizeof(unsigned), (void**)&d_counts)) != RC_OK)
    return st;
  cudaStream_t s = c->stream;
  RC_CUDA(cudaMemsetAsync(d_z, 0xFF, (size_t)npix * 8, s), "rc_shade: clear");
  RC_CUDA(cudaMemsetAsync(d_counts, 0, 2 * sizeof(unsigned), s), "rc_shade: clear");
  ShadeArgs a;
  memset(&a, 0, sizeof a);
  a.verts = static_cast<const float*>(c->scratch[0]);
  a.idx = static_cast<const uint32_t*>(c->scratch[1]);
  a.tmat = c->shade_tmat ? static_cast<const uint16_t*>(c->scratch[2]) : nullptr;
  a.mats = static_cast<const rc_shade_material*>(c->scratch[3]);
  a.tex = static_cast<const ShadeTex*>(c->scratch[5]);
  a.ntris = ntris;
  memcpy(a.vp, view->view_proj, sizeof a.vp);
  memcpy(a.eye, view->eye, sizeof a.eye);
  memcpy(a.light, view->light, sizeof a.light);
  a.W = view->width;
  a.H = view->height;
  a.zbuf = d_z;
  a.out = d_out;
  a.fluence = c->fluence;
  for (int k = 0; k < 3; ++k) a.M[k] = c->geom[0].M[k];
  a.spacing = (float)c->geom[0].spacing;
  memcpy(a.w2g, view->world_to_grid, sizeof a.w2g);
  a.gi_scale = view->gi_scale;
  a.ntex = c->shade_ntex;
  if (ntris) {
    int4* d_bounds = static_cast<int4*>(c->scratch[8]);
    uint32_t* d_small = static_cast<uint32_t*>(c->scratch[9]);
    uint32_t* d_big = static_cast<uint32_t*>(c->scratch[10]);
    k_shade_bin<<<(unsigned)((ntris + 255) / 256), 256, 0, s>>>(a, d_bounds, d_small, d_big, d_counts);
    // Both depth passes loop over the binned lists' lengths as the device
    // counted them; their grids are sized for the worst case, so the host
    // never waits between the passes.
    const int64_t blocks = std::min<int64_t>((ntris * 32 + 255) / 256, 152 * 32);
    k_shade_depth_small<<<(unsigned)blocks, 256, 0, s>>>(a, d_bounds, d_small, d_counts);
    const unsigned tiles = (unsigned)(((a.W + kShadeTile - 1) / kShadeTile) * ((a.H + kShadeTile - 1) / kShadeTile));
    k_shade_depth_big<<<dim3(tiles, (unsigned)std::min<int64_t>(ntris, kShadeBigRows)), 256, 0, s>>>(a, d_bounds,
                                                                                                    d_big, d_counts);
  }
  k_shade_pixels<<<(unsigned)((npix + 255) / 256), 256, 0, s>>>(a);
  RC_CUDA(cudaGetLastError(), "rc_shade: launch");
  if (where == RC_MEM_HOST) {
    RC_CUDA(cudaMemcpyAsync(out, d_out, (size_t)npix * 16, cudaMemcpyDeviceToHost, s), "rc_shade: read back");
    RC_CUDA(cudaStreamSynchronize(s), "rc_shade");
  }
  return RC_OK;
}

rc_status rc_shade(rc_context* c, const rc_shade_view* view, const float* vertices, int64_t nverts,
                   const uint32_t* indices, int64_t ntris, const uint16_t* tri_material,
                   const rc_shade_material* materials, int32_t nmaterials, const rc_texture* textures,
                   int32_t ntextures, float* out, int32_t where) {
  if (check_ctx(c, "rc_shade") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!view || view->width < 1 || view->height < 1 || view->width > 16384 || view->height > 16384 || nverts < 0 ||
      ntris < 0 || ntris >= ((int64_t)1 << 32) || (nverts && !vertices) || (ntris && !indices) || nmaterials < 1 ||
      !materials || ntextures < 0 || (ntextures && !textures) || !out ||
      (where != RC_MEM_HOST && where != RC_MEM_DEVICE)) {
    rcx::set_error("rc_shade: invalid arguments (image 1..16384 px per side, >= 1 material, non-NULL arrays)");
    return RC_ERR_INVALID_ARG;
  }
  if (view->gi_scale > 0.f && !c->have_base) {
    rcx::set_error("rc_shade: the GI term needs a solved scene");
    return RC_ERR_STATE;
  }
  rc_status st = rc_shade_set_mesh(c, vertices, nverts, indices, ntris, tri_material, materials, nmaterials, textures,
                                   ntextures);
  if (st != RC_OK) return st;
  st = rc_shade_draw(c, view, out, where);
  if (st != RC_OK) return st;
  DeviceGuard g(c->device);
  RC_CUDA(cudaStreamSynchronize(c->stream), "rc_shade");
  return RC_OK;
}

rc_status rc_get_volume(rc_context* c, rc_voxel* out, int64_t count, int32_t where) {
  if (check_ctx(c, "rc_get_volume") != RC_OK) return RC_ERR_INVALID_ARG;
  const int64_t need = (int64_t)c->p.grid[0] * c->p.grid[1] * c->p.grid[2];
  if (!out || count != need) {
    rcx::set_error("rc_get_volume: need a buffer of exactly %lld voxels", (long long)need);
    return RC_ERR_INVALID_ARG;
  }
  if (!c->have_base) {
    rcx::set_error("rc_get_volume: no scene uploaded");
    return RC_ERR_STATE;
  }
  return copy_out(c, out, c->vol, (size_t)need * sizeof(rc_voxel), where, "rc_get_volume");
}

rc_status rc_get_fluence_async(rc_context* c, float* out, int64_t elems) {
  if (check_ctx(c, "rc_get_fluence_async") != RC_OK) return RC_ERR_INVALID_ARG;
  const int64_t need = 3 * c->geom[0].probes();
  if (!out || elems != need) {
    rcx::set_error("rc_get_fluence_async: need a host buffer of exactly %lld floats", (long long)need);
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(c->device);
  if (!c->flu[1]) {
    rc_status s = dev_alloc((void**)&c->flu[1], (size_t)need * sizeof(float), "second fluence buffer");
    if (s != RC_OK) return s;
    RC_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking), "rc_get_fluence_async: stream");
    for (int k = 0; k < 2; ++k) {
      RC_CUDA(cudaEventCreateWithFlags(&c->ev_solved[k], cudaEventDisableTiming), "rc_get_fluence_async: event");
      RC_CUDA(cudaEventCreateWithFlags(&c->ev_copied[k], cudaEventDisableTiming), "rc_get_fluence_async: event");
    }
  }
  const int b = c->flu_cur;
  RC_CUDA(cudaEventRecord(c->ev_solved[b], c->stream), "rc_get_fluence_async: event");
  RC_CUDA(cudaStreamWaitEvent(c->copy_stream, c->ev_solved[b], 0), "rc_get_fluence_async: wait");
  RC_CUDA(cudaMemcpyAsync(out, c->flu[b], (size_t)need * sizeof(float), cudaMemcpyDeviceToHost, c->copy_stream),
          "rc_get_fluence_async: copy");
  RC_CUDA(cudaEventRecord(c->ev_copied[b], c->copy_stream), "rc_get_fluence_async: event");
  c->copy_pending[b] = true;
  return RC_OK;
}

rc_status rc_fluence_device_ptr(rc_context* c, const float** out) {
  if (check_ctx(c, "rc_fluence_device_ptr") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!out) {
    rcx::set_error("rc_fluence_device_ptr: out is NULL");
    return RC_ERR_INVALID_ARG;
  }
  *out = c->fluence;
  return RC_OK;
}

rc_status rc_radiance_device_ptr(rc_context* c, int32_t level, const void** out) {
  if (check_ctx(c, "rc_radiance_device_ptr") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!out || level < 0 || level >= c->nlev) {
    rcx::set_error("rc_radiance_device_ptr: bad level or NULL out");
    return RC_ERR_INVALID_ARG;
  }
  *out = static_cast<char*>(c->rad) + c->rad_off[level];
  return RC_OK;
}

rc_status rc_get_stream(rc_context* c, void** out) {
  if (check_ctx(c, "rc_get_stream") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!out) {
    rcx::set_error("rc_get_stream: out is NULL");
    return RC_ERR_INVALID_ARG;
  }
  *out = c->stream;
  return RC_OK;
}

rc_status rc_profile_levels(rc_context* c, int32_t iters, float* ms_out, int32_t count) {
  if (check_ctx(c, "rc_profile_levels") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!ms_out || (count != 1 + c->nlev && count != 2 + c->nlev) || iters < 1) {
    rcx::set_error("rc_profile_levels: need iters >= 1 and %d or %d output floats", 1 + c->nlev, 2 + c->nlev);
    return RC_ERR_INVALID_ARG;
  }
  if (!c->have_base) {
    rcx::set_error("rc_profile_levels: no scene uploaded");
    return RC_ERR_STATE;
  }
  DeviceGuard g(c->device);
  cudaEvent_t ev[kMaxCascades + 2];
  for (int i = 0; i < c->nlev + 2; ++i) RC_CUDA(cudaEventCreate(&ev[i]), "rc_profile_levels: event");
  double acc[kMaxCascades + 1] = {0};
  rc_status st = RC_OK;
  for (int it = 0; it < iters && st == RC_OK; ++it) {
    // a per-frame update: the current spheres' footprints are recomposed
    std::vector<Region> regs;
    for (const QSphere& q : c->cur) {
      Region r;
      if (sphere_region(q, c->p.grid, &r)) regs.push_back(r);
    }
    cudaEventRecord(ev[0], c->stream);
    if (!regs.empty()) st = recompose(c, regs.data(), (int)regs.size());
    cudaEventRecord(ev[1], c->stream);
    launch_queue_walk(c, c->stream);  // counted with the top level, which is launched next
    for (int i = c->nlev - 1, k = 2; i >= 0; --i, ++k) {
      if (c->elem == 2) launch_level<__half>(c, i, c->stream);
      else launch_level<float>(c, i, c->stream);
      cudaEventRecord(ev[k], c->stream);
    }
    cudaError_t e = cudaEventSynchronize(ev[c->nlev + 1]);
    if (e != cudaSuccess) {
      st = cuda_fail(e, "rc_profile_levels");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[0], ev[1]);
    acc[0] += ms;
    for (int i = c->nlev - 1, k = 2; i >= 0; --i, ++k) {
      cudaEventElapsedTime(&ms, ev[k - 1], ev[k]);
      acc[1 + i] += ms;
    }
  }
  // the level set as a solve launches it: events only around it
  double whole = 0.0;
  for (int it = 0; it < iters && st == RC_OK && count == 2 + c->nlev; ++it) {
    cudaEventRecord(ev[0], c->stream);
    launch_queue_walk(c, c->stream);
    for (int i = c->nlev - 1; i >= 0; --i) {
      if (c->elem == 2) launch_level<__half>(c, i, c->stream);
      else launch_level<float>(c, i, c->stream);
    }
    cudaEventRecord(ev[1], c->stream);
    cudaError_t e = cudaEventSynchronize(ev[1]);
    if (e != cudaSuccess) {
      st = cuda_fail(e, "rc_profile_levels");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[0], ev[1]);
    whole += ms;
  }
  for (int i = 0; i < c->nlev + 2; ++i) cudaEventDestroy(ev[i]);
  if (st != RC_OK) return st;
  for (int i = 0; i <= c->nlev; ++i) ms_out[i] = (float)(acc[i] / iters);
  if (count == 2 + c->nlev) ms_out[1 + c->nlev] = (float)(whole / iters);
  return RC_OK;
}

}  // extern "C"

extern "C" {

rc_status rc_check_status(int32_t device, uint64_t* first_failure, uint32_t* failures) {
#ifdef RC_CHECKED
  DeviceGuard g(device);
  unsigned long long f0 = 0, f1 = 0;
  unsigned n0 = 0, n1 = 0;
  RC_CUDA(check_read(&f0, &n0), "rc_check_status");
  RC_CUDA(nrc_check_read(&f1, &n1), "rc_check_status");
  const unsigned long long first = f0 ? f0 : f1;
  const unsigned count = n0 + n1;
  if (first_failure) *first_failure = first;
  if (failures) *failures = count;
  if (count) {
    rcx::set_error("checked build: %u out-of-range accesses skipped; the first touched %s at 0x%llx", count,
                   rcx::check_site_name((int)(first >> 56)), first & ((1ull << 56) - 1));
    return RC_ERR_STATE;
  }
  return RC_OK;
#else
  (void)device;
  if (first_failure) *first_failure = 0;
  if (failures) *failures = 0;
  rcx::set_error("rc_check_status: this library was built without RC_CHECKED (librc_checked.so has the checks)");
  return RC_ERR_UNSUPPORTED;
#endif
}

rc_status rc_set_stage_timing(rc_context* c, int32_t enable) {
  if (check_ctx(c, "rc_set_stage_timing") != RC_OK) return RC_ERR_INVALID_ARG;
  DeviceGuard g(c->device);
  if (enable && !c->tev[0])
    for (int i = 0; i <= c->nlev; ++i)
      RC_CUDA(cudaEventCreate(&c->tev[i]), "rc_set_stage_timing: events");
  c->timing = enable != 0;
  c->timed = false;
  return RC_OK;
}

rc_status rc_get_stage_ms(rc_context* c, float* ms_out, int32_t count) {
  if (check_ctx(c, "rc_get_stage_ms") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!ms_out || count < 1 + c->nlev) {
    rcx::set_error("rc_get_stage_ms: need 1 + num_cascades floats");
    return RC_ERR_INVALID_ARG;
  }
  if (!c->timed) {
    rcx::set_error("rc_get_stage_ms: no solve since rc_set_stage_timing(ctx, 1)");
    return RC_ERR_STATE;
  }
  DeviceGuard g(c->device);
  RC_CUDA(cudaEventSynchronize(c->tev[c->nlev]), "rc_get_stage_ms");
  RC_CUDA(cudaEventElapsedTime(&ms_out[0], c->tev[0], c->tev[c->nlev]), "rc_get_stage_ms");
  for (int i = 0; i < c->nlev; ++i)
    RC_CUDA(cudaEventElapsedTime(&ms_out[1 + i], c->tev[c->nlev - 1 - i], c->tev[c->nlev - i]), "rc_get_stage_ms");
  return RC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// rc_solve_noalloc: the same kernels as rc_solve, with every piece of working
// memory carved out of one file-scope device array instead of cudaMalloc.
// ---------------------------------------------------------------------------
namespace {

// Working memory shared by every rc_solve_noalloc call in the process.
__device__ __align__(256) unsigned char g_noalloc_scratch[RC_NOALLOC_SCRATCH_BYTES];

constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_scratch_ptr[kNoallocMaxDevices] = {};

// Host staging of the walk tables (built under the mutex below).
constexpr size_t kNoallocMaxDirs = RC_NOALLOC_SCRATCH_BYTES / sizeof(DirInfo);
DirInfo g_noalloc_tab[kNoallocMaxDirs];
double g_noalloc_omega[kNoallocMaxDirs];

// The tables reach the scratch as kernel arguments, in chunks of 640 entries
// (30,720 bytes; kernel arguments may take up to 32,764 bytes).  A launch
// copies its arguments when it is made, so no work left on the stream reads
// the host staging above, which the next call rewrites.
constexpr int kTabChunk = 640;
struct DirChunk {
  DirInfo d[kTabChunk];
};
static_assert(sizeof(DirChunk) + 16 <= 32764, "walk-table chunk fits the kernel-argument limit");

__global__ void k_put_dirs(DirInfo* __restrict__ dst, int n, const __grid_constant__ DirChunk c) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = c.d[i];
}

// Opacity bits and decimated opacity of a caller-owned volume (the volume is
// only read).
__global__ void k_masks_from_volume(const uint2* __restrict__ vol, uint32_t* __restrict__ occ,
                                    uint32_t* __restrict__ emis, int Gx, int Gy, int Gz, int W, const MaskSet ms) {
  const int64_t words = (int64_t)W * Gy * Gz;
  const int lane = threadIdx.x & 31;
  const int64_t warp0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t wstride = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = warp0; w < words; w += wstride) {
    const int wx = (int)(w % W);
    const int y = (int)((w / W) % Gy);
    const int z = (int)(w / ((int64_t)W * Gy));
    const int x = wx * 32 + lane;
    bool opaque = false, emissive = false;
    if (x < Gx) {
      const uint2 v = __ldg(&vol[((int64_t)z * Gy + y) * Gx + x]);
      opaque = (v.y >> 31) & 1u;
      emissive = opaque && (((v.x & 0x7FFF7FFFu) | (v.y & 0x7FFFu)) != 0u);
    }
    const unsigned bits = __ballot_sync(0xFFFFFFFFu, opaque);
    const unsigned ebits = __ballot_sync(0xFFFFFFFFu, emissive);
    if (lane == 0) {
      occ[((int64_t)z * Gy + y) * W + wx] = bits;
      emis[((int64_t)z * Gy + y) * W + wx] = ebits;
    }
    update_masks(ms, lane, wx, x, y, z, Gx, bits, ebits);
  }
}

size_t carve(size_t& off, size_t bytes) {
  const size_t at = off;
  off = (off + bytes + 255) & ~(size_t)255;
  return at;
}

}  // namespace

extern "C" rc_status rc_solve_noalloc(const rc_params* p, const rc_voxel* voxels, float* fluence, void* radiance,
                                      void* stream) {
  char msg[256];
  if (!validate_params(p, msg, sizeof msg)) {
    rcx::set_error("rc_solve_noalloc: invalid rc_params: %s", msg);
    return RC_ERR_INVALID_ARG;
  }
  if (!voxels || !fluence || !radiance) {
    rcx::set_error("rc_solve_noalloc: voxels, fluence and radiance must be device pointers, not NULL");
    return RC_ERR_INVALID_ARG;
  }
  // The kernels read and write these buffers with 16-byte vector accesses.
  if ((reinterpret_cast<uintptr_t>(voxels) | reinterpret_cast<uintptr_t>(fluence) |
       reinterpret_cast<uintptr_t>(radiance)) & 15u) {
    rcx::set_error("rc_solve_noalloc: voxels, fluence and radiance must be 16-byte aligned");
    return RC_ERR_INVALID_ARG;
  }
  int dev = 0;
  RC_CUDA(cudaGetDevice(&dev), "rc_solve_noalloc: current device");
  if (dev < 0 || dev >= kNoallocMaxDevices) {
    rcx::set_error("rc_solve_noalloc: device %d beyond the %d supported", dev, kNoallocMaxDevices);
    return RC_ERR_UNSUPPORTED;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  // A context view that owns nothing: geometry and launch arguments only.
  rc_context v;
  v.p = *p;
  v.device = dev;
  v.nlev = p->num_cascades;
  v.elem = p->precision == RC_PRECISION_FP16 ? 2 : 4;
  level_geometry(*p, v.geom);
  v.W = (p->grid[0] + 31) / 32;

  // Scratch layout, checked against the static maximum before any GPU work.
  const bool force_scalar = getenv("RC_WALK") && strcmp(getenv("RC_WALK"), "scalar") == 0;
  const int64_t full_words = (int64_t)v.W * p->grid[1] * p->grid[2];
  size_t off = 0;
  const size_t occ_off = carve(off, (size_t)full_words * 4);
  const size_t emis_off = carve(off, (size_t)full_words * 4);
  size_t mask_off[kMaxCascades] = {}, mask_bytes = 0, mask_begin = off;
  MaskGeom mgs[kMaxCascades];
  for (int i = 0; i < v.nlev; ++i) {
    mgs[i] = mask_geom(v.geom[i], force_scalar);
    v.bits_level[i] = mgs[i].bits;
    v.mode[i] = (i == 0 && level0_direct(*p, v.geom[0], force_scalar)) ? kModeDirect0 : mgs[i].mode;
    v.rec_slots[i] = v.geom[i].M[2] * mgs[i].wpp;
    if (needs_mask(v.bits_level, v.mode, i)) mask_off[i] = carve(off, (size_t)mgs[i].words * 8);
  }
  mask_bytes = off - mask_begin;
  size_t avg_off[kMaxCascades] = {};
  for (int i = 1; i < v.nlev; ++i)
    avg_off[i] = carve(off, (size_t)4 * v.geom[i - 1].ndirs * v.geom[i].probes() * v.elem);
  size_t ndirs_total = 0;
  for (int i = 0; i < v.nlev; ++i) ndirs_total += (size_t)v.geom[i].ndirs;
  const size_t dirs_off = carve(off, ndirs_total * sizeof(DirInfo));
  const size_t rec_off = carve(off, queue_records_bytes(&v));
  const size_t counter_off = carve(off, sizeof(unsigned long long));
  if (off > RC_NOALLOC_SCRATCH_BYTES || ndirs_total > kNoallocMaxDirs) {
    rcx::set_error("rc_solve_noalloc: these parameters need %zu bytes of scratch; the static maximum is %u bytes",
                   off, (unsigned)RC_NOALLOC_SCRATCH_BYTES);
    return RC_ERR_UNSUPPORTED;
  }

  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  // Once per device, with that device current: the array's device address
  // and the shared-memory opt-in of the bit-parallel kernel.
  if (!g_noalloc_scratch_ptr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "rc_solve_noalloc: scratch address");
    if ((e = allow_bits_smem<float>()) != cudaSuccess || (e = allow_bits_smem<__half>()) != cudaSuccess)
      return cuda_fail(e, "rc_solve_noalloc: shared memory attribute");
    g_noalloc_scratch_ptr[dev] = ptr;
#ifdef RC_CHECKED
    check_register(ptr, RC_NOALLOC_SCRATCH_BYTES);
#endif
  }
#ifdef RC_CHECKED
  {
    // the caller's buffers are the kernels' to read and write
    size_t rb = 0;
    for (int i = 0; i < v.nlev; ++i) rb += (size_t)3 * v.geom[i].ndirs * v.geom[i].probes() * v.elem;
    check_register(voxels, (size_t)p->grid[0] * p->grid[1] * p->grid[2] * sizeof(rc_voxel));
    check_register(fluence, (size_t)v.geom[0].probes() * 3 * sizeof(float));
    check_register(radiance, rb);
    RC_CUDA(check_prepare(), "checked build: range upload");
  }
#endif
  char* scratch = static_cast<char*>(g_noalloc_scratch_ptr[dev]);

  // Walk tables, built on the host and copied into the scratch.
  size_t t = 0;
  size_t dir_off[kMaxCascades] = {};
  for (int i = 0; i < v.nlev; ++i) {
    dir_off[i] = t;
    if (!build_dir_table(v.geom[i], p->grid, g_noalloc_tab + t, msg, sizeof msg)) {
      rcx::set_error("rc_solve_noalloc: %s", msg);
      return RC_ERR_UNSUPPORTED;
    }
    t += (size_t)v.geom[i].ndirs;
  }
  rc_solid_angles(v.geom[0].n, g_noalloc_omega);
  for (int d = 0; d < v.geom[0].ndirs; ++d) g_noalloc_tab[d].omega = (float)g_noalloc_omega[d];
  DirInfo* dirs = reinterpret_cast<DirInfo*>(scratch + dirs_off);
  for (size_t c0 = 0; c0 < ndirs_total; c0 += kTabChunk) {
    const int cnt = (int)std::min<size_t>(kTabChunk, ndirs_total - c0);
    DirChunk chunk;
    memcpy(chunk.d, g_noalloc_tab + c0, (size_t)cnt * sizeof(DirInfo));
    k_put_dirs<<<1, 256, 0, st>>>(dirs + c0, cnt, chunk);
    RC_CUDA(cudaGetLastError(), "rc_solve_noalloc: table upload");
  }
  // Decimated opacity keeps unused padding bits at zero; the previous call's
  // contents are cleared.  Everything else is fully rewritten below.
  if (mask_bytes) RC_CUDA(cudaMemsetAsync(scratch + mask_begin, 0, mask_bytes, st), "rc_solve_noalloc: clear");

  uint32_t* occ = reinterpret_cast<uint32_t*>(scratch + occ_off);
  uint32_t* emis = reinterpret_cast<uint32_t*>(scratch + emis_off);
  v.emis = emis;
  v.mset.n = 0;
  size_t rad_off = 0;
  for (int i = 0; i < v.nlev; ++i) {
    const LevelGeom& g = v.geom[i];
    LevelArgs& a = v.args[i];
    memset(&a, 0, sizeof a);
    int l2s = 0;
    while ((1 << l2s) < g.spacing) ++l2s;
    if (needs_mask(v.bits_level, v.mode, i)) {
      MaskLevel& m = v.mset.lv[v.mset.n++];
      m.base = reinterpret_cast<uint2*>(scratch + mask_off[i]);
      m.l2s = l2s;
      for (int ax = 0; ax < 3; ++ax) m.M[ax] = g.M[ax];
      m.l2px = mgs[i].l2px;
      m.wpp = mgs[i].wpp;
      a.mask = m.base;
    }
    a.l2s = l2s;
    a.l2px = mgs[i].l2px;
    a.wpp = mgs[i].wpp;
    a.rep = mgs[i].rep;
    a.tiles = mgs[i].tiles;
    a.emis = emis;
    a.occ = occ;
    a.vol = reinterpret_cast<const uint2*>(voxels);
    for (int ax = 0; ax < 3; ++ax) {
      a.G[ax] = p->grid[ax];
      a.M[ax] = g.M[ax];
      a.UM[ax] = (i + 1 < v.nlev) ? v.geom[i + 1].M[ax] : 1;
    }
    a.W = v.W;
    a.dirs = dirs + dir_off[i];
    a.spacing = g.spacing;
    a.n = g.n;
    a.ndirs = g.ndirs;
    a.P = g.probes();
    a.L = static_cast<char*>(radiance) + rad_off;
    rad_off += (size_t)3 * g.ndirs * g.probes() * v.elem;
    a.A_out = i >= 1 ? scratch + avg_off[i] : nullptr;
    a.a_out_planar = (i == 1 && (v.mode[0] == kModeDirect0 || v.mode[0] == kModeTma0)) ? 1 : 0;
    a.A_up = (i + 1 < v.nlev) ? scratch + avg_off[i + 1] : nullptr;
    a.P_up = (i + 1 < v.nlev) ? v.geom[i + 1].probes() : 0;
    a.fluence = fluence;
  }
  const int threads = 256;
  const int64_t blocks = std::min<int64_t>(std::max<int64_t>((full_words * 32 + threads - 1) / threads, 1), 152 * 16);
  k_masks_from_volume<<<(unsigned)blocks, threads, 0, st>>>(reinterpret_cast<const uint2*>(voxels), occ, emis,
                                                             p->grid[0], p->grid[1], p->grid[2], v.W, v.mset);
  RC_CUDA(cudaGetLastError(), "rc_solve_noalloc: opacity launch");
  setup_queue(&v, reinterpret_cast<uint32_t*>(scratch + rec_off),
              reinterpret_cast<unsigned long long*>(scratch + counter_off));
  rc_status es = enqueue_solve(&v, st);
  if (es != RC_OK) return es;
  RC_CUDA(cudaGetLastError(), "rc_solve_noalloc: cascade launch");
  return RC_OK;
}

// ---------------------------------------------------------------------------
// Batched solve: many scenes, one persistent launch in a CUDA graph.
// ---------------------------------------------------------------------------
// One scene's share of the batch's gathered fluence: n floats from src to
// offset off of the staging buffer.
struct FluSeg {
  const float* src;
  int64_t off;
  int64_t n;
};

struct rc_batch {
  int device = 0;
  int n = 0;
  std::vector<rc_context*> scenes;
  cudaStream_t stream = nullptr;
  BatchLevel* d_levels = nullptr;
  BatchItem* d_items = nullptr;
  QueueArgs* d_qargs = nullptr;  // per scene: its narrow-level walk queue
  unsigned* d_next = nullptr;
  unsigned* d_done = nullptr;
  int* d_err = nullptr;
  size_t levels_cap = 0, items_cap = 0;
  int nlevels = 0, nitems = 0;
  BatchTiles tiles{256, 4, 1, 1024};
  int blocks = 0;
  bool fp16 = false;
  // per_scene: the solve is every scene's own level launches, as parallel
  // branches of the graph (side streams while capturing), instead of the
  // persistent kernel; the scenes' error flags are gathered into d_err
  bool per_scene = false;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  // scene-launch form: emitter updates run on the side streams, each after
  // the batch stream's work so far (ev_batch), and the next solve waits for
  // the side streams used since the last one (pending)
  cudaEvent_t ev_batch = nullptr;
  std::vector<cudaEvent_t> ev_side;
  std::vector<char> pending;
  int** d_errs = nullptr;
  cudaGraphExec_t graph = nullptr;
  // Asynchronous read-back: every scene's fluence is gathered into one
  // device buffer on the batch stream (the solves after it may then start),
  // and copied to the host from there on copy_stream; the next gather waits
  // for that copy (ev_copied).
  float* flu_stage = nullptr;
  FluSeg* d_flu_seg = nullptr;
  int64_t flu_max_seg = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_gathered = nullptr, ev_copied = nullptr;
  bool copy_pending = false;
};

namespace {

void batch_free_graph(rc_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
}

bool tiles_valid(const rc_batch_tiles* t) {
  auto ok = [](int32_t v) { return v >= 1 && v <= 65536; };
  return t && ok(t->probes_per_item) && ok(t->dirs_per_item) && ok(t->blocks_per_item) && ok(t->walks_per_item);
}

// Level table and item queue for tile shape `ts`: every scene's walk tasks
// first, then the levels top first across scenes.
rc_status batch_build(rc_batch* b, const BatchTiles& ts) {
  std::vector<BatchLevel> lv;
  std::vector<int> first(b->n), walk(b->n, -1);
  int maxN = 0;
  for (int k = 0; k < b->n; ++k) {
    rc_context* c = b->scenes[k];
    maxN = std::max(maxN, c->nlev);
    if (c->qargs.total > 0) {
      BatchLevel W;
      memset(&W, 0, sizeof W);
      W.mode = kBatchWalk;
      W.q = b->d_qargs + k;
      W.up = W.dep2 = -1;
      W.ntiles = (int)((c->qargs.total + ts.wpi - 1) / ts.wpi);
      walk[k] = (int)lv.size();
      lv.push_back(W);
    }
    first[k] = (int)lv.size();
    for (int i = 0; i < c->nlev; ++i) {
      BatchLevel L;
      memset(&L, 0, sizeof L);
      const LevelArgs& a = c->args[i];
      L.a = a;
      L.up = (i + 1 < c->nlev) ? first[k] + i + 1 : -1;
      L.dep2 = -1;
      L.is_l0 = (i == 0);
      L.is_top = (i == c->nlev - 1);
      const int64_t npar = (i == 0) ? 1 : c->geom[i - 1].ndirs;
      if (c->mode[i] == kModeFused) {
        L.mode = kBatchBits;
        L.units = a.tiles * (i == 0 ? 1 : (a.n / 2) * (a.n / 2) / 2);
        L.ntiles = (L.units + ts.upi - 1) / ts.upi;
      } else if (c->mode[i] == kModeDirect0 || c->mode[i] == kModeTma0) {  // the walk-free form either way
        L.mode = kBatchDirect0;
        const int64_t warps = (int64_t)((a.M[0] + 127) / 128) * a.M[1] * ((a.M[2] + 1) / 2);
        L.units = (int)((warps + 7) / 8);
        L.ntiles = (L.units + ts.upi - 1) / ts.upi;
      } else {
        const bool merge = c->mode[i] == kModeQueue;
        L.mode = merge ? kBatchMerge : kBatchScalar;
        if (merge) {
          L.rec = c->rec_level[i];
          L.slots = c->rec_slots[i];
          L.dep2 = walk[k];
        }
        const int64_t groups = (i == 0) ? 1 : (merge ? npar / 2 : npar);
        L.ptiles = (int)((a.P + ts.ppi - 1) / ts.ppi);
        L.ntiles = (int)(L.ptiles * ((groups + ts.qpi - 1) / ts.qpi));
      }
      lv.push_back(L);
    }
  }
  std::vector<BatchItem> items;
  for (int k = 0; k < b->n; ++k)
    if (walk[k] >= 0)
      for (int t = 0; t < lv[walk[k]].ntiles; ++t) items.push_back(BatchItem{walk[k], t});
  for (int t = 0; t < maxN; ++t)
    for (int k = 0; k < b->n; ++k) {
      const int N = b->scenes[k]->nlev;
      if (t >= N) continue;
      const int li = first[k] + N - 1 - t;
      for (int tile = 0; tile < lv[li].ntiles; ++tile) items.push_back(BatchItem{li, tile});
    }
  // Fault injection for tests: one level waits for a tile that never comes.
  if (fault_is("timeout")) lv[first[0] + b->scenes[0]->nlev - 1].ntiles += 1;
  DeviceGuard g(b->device);
  if (lv.size() > b->levels_cap) {
    if (b->d_levels) cudaFree(b->d_levels);
    if (b->d_done) cudaFree(b->d_done);
    b->d_levels = nullptr;
    b->d_done = nullptr;
    rc_status s = dev_alloc((void**)&b->d_levels, lv.size() * sizeof(BatchLevel), "batch level table");
    if (s != RC_OK) return s;
    if ((s = dev_alloc((void**)&b->d_done, lv.size() * sizeof(unsigned), "batch counters")) != RC_OK) return s;
    b->levels_cap = lv.size();
  }
  if (items.size() > b->items_cap) {
    if (b->d_items) cudaFree(b->d_items);
    b->d_items = nullptr;
    rc_status s = dev_alloc((void**)&b->d_items, items.size() * sizeof(BatchItem), "batch items");
    if (s != RC_OK) return s;
    b->items_cap = items.size();
  }
  RC_CUDA(cudaMemcpy(b->d_levels, lv.data(), lv.size() * sizeof(BatchLevel), cudaMemcpyHostToDevice), "batch upload");
  RC_CUDA(cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice),
          "batch upload");
  b->nlevels = (int)lv.size();
  b->nitems = (int)items.size();
  b->tiles = ts;
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  if (b->fp16)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_persistent<__half>, kBatchThreads, kBitsSmem);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_persistent<float>, kBatchThreads, kBitsSmem);
  (void)cudaGetLastError();
  b->blocks = std::max(1, std::min(b->nitems, std::max(1, sms * std::max(per_sm, 1))));
  batch_free_graph(b);
  return RC_OK;
}

void batch_enqueue(rc_batch* b, cudaStream_t s) {
  cudaMemsetAsync(b->d_next, 0, sizeof(unsigned), s);
  cudaMemsetAsync(b->d_done, 0, (size_t)b->nlevels * sizeof(unsigned), s);
  if (b->fp16)
    k_batch_persistent<__half><<<b->blocks, kBatchThreads, kBitsSmem, s>>>(b->d_levels, b->d_items, b->nitems,
                                                                           b->tiles, b->d_next, b->d_done, b->d_err);
  else
    k_batch_persistent<float><<<b->blocks, kBatchThreads, kBitsSmem, s>>>(b->d_levels, b->d_items, b->nitems,
                                                                          b->tiles, b->d_next, b->d_done, b->d_err);
}

// Every scene's fluence into one contiguous buffer: block row blockIdx.y
// copies segment blockIdx.y (n floats from src to dst + off).
__global__ void k_gather_fluence(const FluSeg* __restrict__ seg, float* __restrict__ dst) {
  const FluSeg g = seg[blockIdx.y];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.n; i += (int64_t)gridDim.x * blockDim.x)
    dst[g.off + i] = __ldcs(g.src + i);
}

// A scene's bounded waits report into its own flag: after a per-scene solve
// the flags are moved into the batch's.
__global__ void k_gather_errors(int* const* errs, int n, int* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int f = *errs[i];
    if (f) {
      atomicMax(out, f);
      *errs[i] = 0;
    }
  }
}

// Every scene's solve on its own branch: fork from the batch stream, one side
// stream per scene (up to 64, reused round robin), join, gather the flags.
void batch_enqueue_scenes(rc_batch* b, cudaStream_t s) {
  cudaEventRecord(b->fork, s);
  const int ns = (int)b->side.size();
  for (int k = 0; k < b->n; ++k) {
    cudaStream_t sk = b->side[k % ns];
    if (k < ns) cudaStreamWaitEvent(sk, b->fork, 0);
    (void)enqueue_solve(b->scenes[k], sk);
  }
  for (int j = 0; j < ns; ++j) {
    cudaEventRecord(b->joins[j], b->side[j]);
    cudaStreamWaitEvent(s, b->joins[j], 0);
  }
  k_gather_errors<<<1, 256, 0, s>>>(b->d_errs, b->n, b->d_err);
}

rc_status batch_side_streams(rc_batch* b) {
  if (!b->side.empty()) return RC_OK;
  const int ns = std::min(b->n, 64);
  RC_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "batch fork event");
  RC_CUDA(cudaEventCreateWithFlags(&b->ev_batch, cudaEventDisableTiming), "batch event");
  for (int j = 0; j < ns; ++j) {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr, es = nullptr;
    RC_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "batch side stream");
    b->side.push_back(st);
    RC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "batch join event");
    b->joins.push_back(ev);
    RC_CUDA(cudaEventCreateWithFlags(&es, cudaEventDisableTiming), "batch side event");
    b->ev_side.push_back(es);
  }
  b->pending.assign((size_t)ns, 0);
  return RC_OK;
}

// Before work on the batch stream that reads what emitter updates on side
// streams wrote: the batch stream waits for every side stream used since.
rc_status batch_join_updates(rc_batch* b) {
  for (size_t j = 0; j < b->pending.size(); ++j) {
    if (!b->pending[j]) continue;
    RC_CUDA(cudaEventRecord(b->ev_side[j], b->side[j]), "batch update join");
    RC_CUDA(cudaStreamWaitEvent(b->stream, b->ev_side[j], 0), "batch update join");
    b->pending[j] = 0;
  }
  return RC_OK;
}

// The whole batch solve as one CUDA graph: two counter resets + the
// persistent launch, or the scenes' own launches in parallel branches.
rc_status batch_graph(rc_batch* b) {
  if (b->graph) return RC_OK;
  if (b->per_scene) {
    rc_status s = batch_side_streams(b);
    if (s != RC_OK) return s;
  }
  cudaGraph_t graph = nullptr;
  RC_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "batch capture");
  if (b->per_scene)
    batch_enqueue_scenes(b, b->stream);
  else
    batch_enqueue(b, b->stream);
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  if (e != cudaSuccess) return cuda_fail(e, "batch capture");
  e = cudaGraphInstantiate(&b->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    b->graph = nullptr;
    return cuda_fail(e, "batch graph instantiate");
  }
  return RC_OK;
}

rc_status batch_check(const rc_batch* b, const char* fn) {
  if (!b) {
    rcx::set_error("%s: batch is NULL", fn);
    return RC_ERR_INVALID_ARG;
  }
  return RC_OK;
}

rc_status batch_error_flag(rc_batch* b, const char* fn) {
  int flag = 0;
  RC_CUDA(cudaMemcpy(&flag, b->d_err, sizeof flag, cudaMemcpyDeviceToHost), fn);
  if (flag) {
    cudaMemset(b->d_err, 0, sizeof(int));
    rcx::set_error("%s: a level waited longer than its bound for the level above (batch results incomplete)", fn);
    return RC_ERR_TIMEOUT;
  }
  return RC_OK;
}

}  // namespace

extern "C" {

rc_status rc_batch_create(const rc_params* params, int32_t nscenes, int32_t device, rc_batch** out) {
  if (!out || !params || nscenes < 1 || nscenes > 4096) {
    rcx::set_error("rc_batch_create: need 1..4096 scene parameter blocks and a non-NULL out");
    return RC_ERR_INVALID_ARG;
  }
  *out = nullptr;
  for (int k = 0; k < nscenes; ++k) {
    char msg[256];
    if (!validate_params(&params[k], msg, sizeof msg)) {
      rcx::set_error("rc_batch_create: scene %d: %s", k, msg);
      return RC_ERR_INVALID_ARG;
    }
    if (params[k].precision != params[0].precision) {
      rcx::set_error("rc_batch_create: every scene must use the same precision");
      return RC_ERR_INVALID_ARG;
    }
  }
  rc_batch* b = new rc_batch();
  b->device = device;
  b->n = nscenes;
  b->fp16 = params[0].precision == RC_PRECISION_FP16;
  auto fail = [&](rc_status st) {
    rc_batch_destroy(b);
    return st;
  };
  for (int k = 0; k < nscenes; ++k) {
    rc_context* c = nullptr;
    rc_status s = create_ctx(&params[k], device, true, &c);
    if (s != RC_OK) return fail(s);
    b->scenes.push_back(c);
  }
  DeviceGuard g(device);
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail(cuda_fail(e, "rc_batch_create: stream"));
  rc_status s;
  if ((s = dev_alloc((void**)&b->d_next, sizeof(unsigned), "batch queue")) != RC_OK) return fail(s);
  if ((s = dev_alloc((void**)&b->d_err, sizeof(int), "batch error flag")) != RC_OK) return fail(s);
  if ((e = cudaMemset(b->d_err, 0, sizeof(int))) != cudaSuccess) return fail(cuda_fail(e, "rc_batch_create"));
  if ((s = dev_alloc((void**)&b->d_qargs, (size_t)nscenes * sizeof(QueueArgs), "batch walk queues")) != RC_OK)
    return fail(s);
  {
    std::vector<QueueArgs> qa((size_t)nscenes);
    for (int k = 0; k < nscenes; ++k) qa[k] = b->scenes[k]->qargs;
    if ((e = cudaMemcpy(b->d_qargs, qa.data(), qa.size() * sizeof(QueueArgs), cudaMemcpyHostToDevice)) != cudaSuccess)
      return fail(cuda_fail(e, "rc_batch_create: upload"));
  }
  {
    std::vector<int*> errs((size_t)nscenes);
    for (int k = 0; k < nscenes; ++k) errs[k] = b->scenes[k]->err;
    if ((s = dev_alloc((void**)&b->d_errs, errs.size() * sizeof(int*), "batch scene flags")) != RC_OK) return fail(s);
    if ((e = cudaMemcpy(b->d_errs, errs.data(), errs.size() * sizeof(int*), cudaMemcpyHostToDevice)) != cudaSuccess)
      return fail(cuda_fail(e, "rc_batch_create: upload"));
  }
  if ((s = batch_build(b, b->tiles)) != RC_OK) return fail(s);
  // RC_BATCH_MODE=scenes / persistent fixes the form (the autotuner then keeps it)
  if (const char* m = getenv("RC_BATCH_MODE")) b->per_scene = strcmp(m, "scenes") == 0;
  *out = b;
  return RC_OK;
}

rc_status rc_batch_destroy(rc_batch* b) {
  if (!b) return RC_OK;
  {
    DeviceGuard g(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_free_graph(b);
    if (b->copy_stream) cudaStreamSynchronize(b->copy_stream);
    void* bufs[] = {b->d_levels, b->d_items, b->d_qargs, b->d_next, b->d_done, b->d_err, b->d_errs,
                    b->flu_stage, b->d_flu_seg};
    for (void* x : bufs)
      if (x) cudaFree(x);
    if (b->ev_gathered) cudaEventDestroy(b->ev_gathered);
    if (b->ev_copied) cudaEventDestroy(b->ev_copied);
    if (b->copy_stream) cudaStreamDestroy(b->copy_stream);
    for (cudaStream_t st : b->side) cudaStreamSynchronize(st);
    for (cudaStream_t st : b->side) cudaStreamDestroy(st);
    for (cudaEvent_t ev : b->joins) cudaEventDestroy(ev);
    for (cudaEvent_t ev : b->ev_side) cudaEventDestroy(ev);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->ev_batch) cudaEventDestroy(b->ev_batch);
    if (b->stream) cudaStreamDestroy(b->stream);
  }
  for (rc_context* c : b->scenes) release(c);
  delete b;
  return RC_OK;
}

rc_status rc_batch_scene_set(rc_batch* b, int32_t scene, const rc_box* boxes, int32_t nboxes,
                             const rc_sphere* spheres, int32_t nspheres) {
  if (batch_check(b, "rc_batch_scene_set") != RC_OK) return RC_ERR_INVALID_ARG;
  if (scene < 0 || scene >= b->n) {
    rcx::set_error("rc_batch_scene_set: scene %d out of range", scene);
    return RC_ERR_INVALID_ARG;
  }
  {
    // the scene's volume must not change under a solve or an update in flight
    DeviceGuard g(b->device);
    rc_status s0 = batch_join_updates(b);
    if (s0 != RC_OK) return s0;
    RC_CUDA(cudaStreamSynchronize(b->stream), "rc_batch_scene_set");
  }
  rc_status s = rc_scene_set_boxes(b->scenes[scene], boxes, nboxes);
  if (s != RC_OK) return s;
  s = rc_scene_set_spheres(b->scenes[scene], spheres, nspheres);
  if (s != RC_OK) return s;
  return rc_synchronize(b->scenes[scene]);
}

rc_status rc_batch_solve(rc_batch* b, void* stream) {
  if (batch_check(b, "rc_batch_solve") != RC_OK) return RC_ERR_INVALID_ARG;
  {
    DeviceGuard g(b->device);
    RC_CUDA(check_prepare(), "checked build: range upload");
  }
  for (int k = 0; k < b->n; ++k)
    if (!b->scenes[k]->have_base) {
      rcx::set_error("rc_batch_solve: scene %d has no scene data", k);
      return RC_ERR_STATE;
    }
  DeviceGuard g(b->device);
  rc_status s = batch_graph(b);
  if (s != RC_OK) return s;
  if ((s = batch_join_updates(b)) != RC_OK) return s;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : b->stream;
  cudaEvent_t ev = nullptr;
  if (st != b->stream) {
    // the caller's stream first waits for the batch stream's work (emitter
    // updates), then the batch stream for the solve
    RC_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "rc_batch_solve: event");
    cudaEventRecord(ev, b->stream);
    cudaStreamWaitEvent(st, ev, 0);
  }
  RC_CUDA(cudaGraphLaunch(b->graph, st), "rc_batch_solve: graph launch");
  if (st != b->stream) {
    cudaEventRecord(ev, st);
    cudaStreamWaitEvent(b->stream, ev, 0);
    cudaEventDestroy(ev);
  }
  return RC_OK;
}

rc_status rc_batch_synchronize(rc_batch* b) {
  if (batch_check(b, "rc_batch_synchronize") != RC_OK) return RC_ERR_INVALID_ARG;
  DeviceGuard g(b->device);
  rc_status s = batch_join_updates(b);  // emitter updates still on side streams
  if (s != RC_OK) return s;
  RC_CUDA(cudaStreamSynchronize(b->stream), "rc_batch_synchronize");
  if (b->copy_stream) {
    RC_CUDA(cudaStreamSynchronize(b->copy_stream), "rc_batch_synchronize");
    b->copy_pending = false;
  }
  return batch_error_flag(b, "rc_batch_synchronize");
}

rc_status rc_batch_get_fluence(rc_batch* b, int32_t scene, float* out, int64_t elems, int32_t where) {
  if (batch_check(b, "rc_batch_get_fluence") != RC_OK) return RC_ERR_INVALID_ARG;
  if (scene < 0 || scene >= b->n) {
    rcx::set_error("rc_batch_get_fluence: scene %d out of range", scene);
    return RC_ERR_INVALID_ARG;
  }
  rc_status s = rc_batch_synchronize(b);
  if (s != RC_OK) return s;
  return rc_get_fluence(b->scenes[scene], out, elems, where);
}

rc_status rc_batch_set_spheres(rc_batch* b, int32_t scene, const rc_sphere* spheres, int32_t n) {
  if (batch_check(b, "rc_batch_set_spheres") != RC_OK) return RC_ERR_INVALID_ARG;
  if (scene < 0 || scene >= b->n) {
    rcx::set_error("rc_batch_set_spheres: scene %d out of range", scene);
    return RC_ERR_INVALID_ARG;
  }
  // The scene's emitter update (sphere upload + re-voxelisation of the voxels
  // the old and new spheres cover) goes on the batch stream, in order with
  // the solves: the solve in flight reads the old volume, the next the new.
  rc_context* c = b->scenes[scene];
  DeviceGuard g(b->device);
  cudaStream_t own = c->stream;
  cudaStream_t st = b->stream;
  if (b->per_scene) {
    // the scene-launch form: the update runs on the scene's side stream,
    // after everything enqueued on the batch stream so far (the solve that
    // reads the old volume); the next solve waits for it
    rc_status s0 = batch_side_streams(b);
    if (s0 != RC_OK) return s0;
    const size_t j = (size_t)scene % b->side.size();
    RC_CUDA(cudaEventRecord(b->ev_batch, b->stream), "rc_batch_set_spheres: event");
    RC_CUDA(cudaStreamWaitEvent(b->side[j], b->ev_batch, 0), "rc_batch_set_spheres: wait");
    st = b->side[j];
    b->pending[j] = 1;
  }
  c->stream = st;
  const rc_status s = rc_scene_set_spheres(c, spheres, n);  // its message names the failing check
  c->stream = own;
  return s;
}

rc_status rc_batch_get_fluence_all(rc_batch* b, float* out, int64_t elems, int32_t where) {
  if (batch_check(b, "rc_batch_get_fluence_all") != RC_OK) return RC_ERR_INVALID_ARG;
  int64_t need = 0;
  for (int k = 0; k < b->n; ++k) need += b->scenes[k]->geom[0].probes() * 3;
  if (!out || elems != need || (where != RC_MEM_HOST && where != RC_MEM_DEVICE)) {
    rcx::set_error("rc_batch_get_fluence_all: need a non-NULL buffer of exactly %lld floats", (long long)need);
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(b->device);
  const cudaMemcpyKind kind = where == RC_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  int64_t off = 0;
  for (int k = 0; k < b->n; ++k) {
    const rc_context* c = b->scenes[k];
    const size_t bytes = (size_t)c->geom[0].probes() * 3 * sizeof(float);
    RC_CUDA(cudaMemcpyAsync(out + off, c->fluence, bytes, kind, b->stream), "rc_batch_get_fluence_all");
    off += c->geom[0].probes() * 3;
  }
  return rc_batch_synchronize(b);
}

rc_status rc_batch_get_fluence_all_async(rc_batch* b, float* out, int64_t elems) {
  if (batch_check(b, "rc_batch_get_fluence_all_async") != RC_OK) return RC_ERR_INVALID_ARG;
  int64_t need = 0;
  for (int k = 0; k < b->n; ++k) need += b->scenes[k]->geom[0].probes() * 3;
  if (!out || elems != need) {
    rcx::set_error("rc_batch_get_fluence_all_async: need a non-NULL host buffer of exactly %lld floats",
                   (long long)need);
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(b->device);
  if (!b->flu_stage) {
    // first read: the staging buffer, its segment table, the copy stream
    std::vector<FluSeg> seg((size_t)b->n);
    int64_t off = 0;
    for (int k = 0; k < b->n; ++k) {
      const int64_t nk = b->scenes[k]->geom[0].probes() * 3;
      seg[(size_t)k] = FluSeg{b->scenes[k]->fluence, off, nk};
      b->flu_max_seg = std::max(b->flu_max_seg, nk);
      off += nk;
    }
    rc_status s = dev_alloc((void**)&b->flu_stage, (size_t)need * sizeof(float), "batch fluence staging");
    if (s == RC_OK) s = dev_alloc((void**)&b->d_flu_seg, seg.size() * sizeof(FluSeg), "batch fluence segments");
    if (s != RC_OK) return s;
    RC_CUDA(cudaMemcpy(b->d_flu_seg, seg.data(), seg.size() * sizeof(FluSeg), cudaMemcpyHostToDevice),
            "rc_batch_get_fluence_all_async: segments");
    RC_CUDA(cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking), "rc_batch_get_fluence_all_async");
    RC_CUDA(cudaEventCreateWithFlags(&b->ev_gathered, cudaEventDisableTiming), "rc_batch_get_fluence_all_async");
    RC_CUDA(cudaEventCreateWithFlags(&b->ev_copied, cudaEventDisableTiming), "rc_batch_get_fluence_all_async");
  }
  // the staging buffer is free once the previous read's copy is done
  if (b->copy_pending) RC_CUDA(cudaStreamWaitEvent(b->stream, b->ev_copied, 0), "rc_batch_get_fluence_all_async");
  const unsigned bx = (unsigned)std::min<int64_t>((b->flu_max_seg + 1023) / 1024, 64);
  k_gather_fluence<<<dim3(bx, (unsigned)b->n), 256, 0, b->stream>>>(b->d_flu_seg, b->flu_stage);
  RC_CUDA(cudaGetLastError(), "rc_batch_get_fluence_all_async: gather");
  RC_CUDA(cudaEventRecord(b->ev_gathered, b->stream), "rc_batch_get_fluence_all_async");
  RC_CUDA(cudaStreamWaitEvent(b->copy_stream, b->ev_gathered, 0), "rc_batch_get_fluence_all_async");
  RC_CUDA(cudaMemcpyAsync(out, b->flu_stage, (size_t)need * sizeof(float), cudaMemcpyDeviceToHost, b->copy_stream),
          "rc_batch_get_fluence_all_async: copy");
  RC_CUDA(cudaEventRecord(b->ev_copied, b->copy_stream), "rc_batch_get_fluence_all_async");
  b->copy_pending = true;
  return RC_OK;
}

rc_status rc_batch_get_radiance(rc_batch* b, int32_t scene, int32_t level, void* out, int64_t bytes, int32_t where) {
  if (batch_check(b, "rc_batch_get_radiance") != RC_OK) return RC_ERR_INVALID_ARG;
  if (scene < 0 || scene >= b->n) {
    rcx::set_error("rc_batch_get_radiance: scene %d out of range", scene);
    return RC_ERR_INVALID_ARG;
  }
  rc_status s = rc_batch_synchronize(b);
  if (s != RC_OK) return s;
  return rc_get_radiance(b->scenes[scene], level, out, bytes, where);
}

rc_status rc_batch_set_tiles(rc_batch* b, const rc_batch_tiles* tiles) {
  if (batch_check(b, "rc_batch_set_tiles") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!tiles_valid(tiles)) {
    rcx::set_error("rc_batch_set_tiles: every tile size must be in [1, 65536]");
    return RC_ERR_INVALID_ARG;
  }
  DeviceGuard g(b->device);
  RC_CUDA(cudaStreamSynchronize(b->stream), "rc_batch_set_tiles");
  const BatchTiles ts{tiles->probes_per_item, tiles->dirs_per_item, tiles->blocks_per_item, tiles->walks_per_item};
  if (!getenv("RC_BATCH_MODE")) b->per_scene = false;  // tiles shape the persistent kernel
  return batch_build(b, ts);
}

rc_status rc_batch_get_tiles(const rc_batch* b, rc_batch_tiles* out) {
  if (batch_check(b, "rc_batch_get_tiles") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!out) {
    rcx::set_error("rc_batch_get_tiles: out is NULL");
    return RC_ERR_INVALID_ARG;
  }
  out->probes_per_item = b->tiles.ppi;
  out->dirs_per_item = b->tiles.qpi;
  out->blocks_per_item = b->tiles.upi;
  out->walks_per_item = b->tiles.wpi;
  return RC_OK;
}

rc_status rc_batch_get_form(const rc_batch* b, int32_t* scene_launches) {
  if (batch_check(b, "rc_batch_get_form") != RC_OK) return RC_ERR_INVALID_ARG;
  if (!scene_launches) {
    rcx::set_error("rc_batch_get_form: out is NULL");
    return RC_ERR_INVALID_ARG;
  }
  *scene_launches = b->per_scene ? 1 : 0;
  return RC_OK;
}

// Coordinate descent over the tile shape: each parameter in turn over its
// candidates with the others held, two sweeps, every candidate timed over
// `iters` graph launches after one warm-up launch; then the scenes' own
// launches as parallel graph branches, kept when faster (RC_BATCH_MODE fixes
// the form instead).
rc_status rc_batch_tune(rc_batch* b, int32_t iters, rc_batch_tiles* best_out, float* best_ms) {
  if (batch_check(b, "rc_batch_tune") != RC_OK) return RC_ERR_INVALID_ARG;
  if (iters < 1) {
    rcx::set_error("rc_batch_tune: iters must be >= 1");
    return RC_ERR_INVALID_ARG;
  }
  static const int kCand[4][4] = {{64, 128, 256, 512}, {1, 2, 4, 16}, {1, 2, 4, 8}, {256, 1024, 4096, 16384}};
  DeviceGuard g(b->device);
  cudaEvent_t e0, e1;
  RC_CUDA(cudaEventCreate(&e0), "rc_batch_tune: event");
  RC_CUDA(cudaEventCreate(&e1), "rc_batch_tune: event");
  BatchTiles best = b->tiles;
  float best_t = 3.4e38f;
  rc_status st = RC_OK;
  const bool fixed = getenv("RC_BATCH_MODE") != nullptr;
  const bool scenes_only = fixed && b->per_scene;
  if (!scenes_only) b->per_scene = false;
  auto time_shape = [&](const BatchTiles& ts, float* ms) -> rc_status {
    rc_status r;
    if ((r = batch_build(b, ts)) != RC_OK) return r;
    if ((r = rc_batch_solve(b, nullptr)) != RC_OK) return r;  // warm-up (builds the graph)
    cudaEventRecord(e0, b->stream);
    for (int i = 0; i < iters; ++i)
      if ((r = rc_batch_solve(b, nullptr)) != RC_OK) return r;
    cudaEventRecord(e1, b->stream);
    if ((r = rc_batch_synchronize(b)) != RC_OK) return r;
    cudaEventElapsedTime(ms, e0, e1);
    *ms /= iters;
    return RC_OK;
  };
  st = time_shape(best, &best_t);
  for (int sweep = 0; sweep < 2 && st == RC_OK && !scenes_only; ++sweep)
    for (int dim = 0; dim < 4 && st == RC_OK; ++dim)
      for (int ci = 0; ci < 4 && st == RC_OK; ++ci) {
        BatchTiles ts = best;
        int* f[4] = {&ts.ppi, &ts.qpi, &ts.upi, &ts.wpi};
        if (*f[dim] == kCand[dim][ci]) continue;
        *f[dim] = kCand[dim][ci];
        float ms = 0.f;
        if ((st = time_shape(ts, &ms)) != RC_OK) break;
        if (ms < best_t) {
          best_t = ms;
          best = ts;
        }
      }
  if (st == RC_OK && !fixed) {
    // the scenes' own launches, in parallel graph branches
    b->per_scene = true;
    float ms = 0.f;
    st = time_shape(best, &ms);
    if (st == RC_OK && ms < best_t)
      best_t = ms;
    else
      b->per_scene = false;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != RC_OK) return st;
  if ((st = batch_build(b, best)) != RC_OK) return st;
  if (best_out) {
    best_out->probes_per_item = best.ppi;
    best_out->dirs_per_item = best.qpi;
    best_out->blocks_per_item = best.upi;
    best_out->walks_per_item = best.wpi;
  }
  if (best_ms) *best_ms = best_t;
  return RC_OK;
}

}  // extern "C"
