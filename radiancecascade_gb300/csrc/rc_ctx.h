// rc_ctx.h -- the context object behind the C ABI and the helpers the CUDA
// translation units share (rc_context.cu: cascades; rc_nrc.cu: the neural
// radiance cache).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <vector>

#include "rc_internal.h"
#include "rc_kernels.cuh"
#include "rc_walk_bits.cuh"
#include "rc_walk_queue.cuh"

namespace rcx {
struct NrcState;
}

struct rc_context {
  rc_params p{};
  int device = 0;
  int nlev = 0;
  rcx::LevelGeom geom[rcx::kMaxCascades]{};
  size_t elem = 4;  // bytes per stored radiance value
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaEvent_t ev_stage[2] = {nullptr, nullptr};  // staging slot copies done
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;

  uint2* base = nullptr;     // static volume (boxes / upload)
  uint2* vol = nullptr;      // composed volume
  uint32_t* occ = nullptr;   // opacity bits
  uint32_t* emis = nullptr;  // emissive bits (opaque with nonzero emission)
  int W = 0;                 // words per x row
  uint2* masks = nullptr;    // decimated (opacity, emissive) bits of the levels that walk bit-parallel
  rcx::MaskSet mset{};
  bool bits_level[rcx::kMaxCascades]{};   // level has decimated opacity
  int mode[rcx::kMaxCascades]{};          // how the level is solved (kMode*)
  uint32_t* recs = nullptr;               // walk records of the queue-walked levels
  unsigned long long* qcounter = nullptr;
  // step tables of the queue levels (k_walk_queue_tab); qtab: every queue level has one
  uint2* qsteps = nullptr;
  int32_t* qstep_begin = nullptr;
  bool qtab = false;
  rcx::QueueArgs qargs{};
  int queue_blocks = 0;
  int queue_resident = 0;  // blocks of the step-table walk that fit the GPU at once
  int rec_slots[rcx::kMaxCascades]{};
  const uint32_t* rec_level[rcx::kMaxCascades]{};
  CUtensorMap tma0{};                // cascade 1's child-averaged radiance, for k_level0_tma
  // wide levels between cascade 0 and the top: the next level's child-averaged
  // radiance staged by TMA (k_level_bits_up)
  bool tma_up[rcx::kMaxCascades]{};
  CUtensorMap tmap_up[rcx::kMaxCascades]{};
  int tma0_py = 0;
  int* err = nullptr;                // device error flag set by bounded waits
  rcx::DirInfo* dirs = nullptr;      // all levels, concatenated
  size_t dir_off[rcx::kMaxCascades]{};
  void* rad = nullptr;               // L_i for all levels
  size_t rad_off[rcx::kMaxCascades]{};  // bytes
  void* avg = nullptr;               // A_i for levels >= 1
  size_t avg_off[rcx::kMaxCascades]{};  // bytes
  float* fluence = nullptr;          // written by the last solve
  // asynchronous read-back (rc_get_fluence_async): two device fluence
  // buffers used alternately, copies on their own stream
  float* flu[2] = {nullptr, nullptr};
  int flu_cur = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_solved[2] = {nullptr, nullptr};
  cudaEvent_t ev_copied[2] = {nullptr, nullptr};
  bool copy_pending[2] = {false, false};

  // dynamic spheres
  rcx::QSphere* d_sph = nullptr;
  rcx::Region* d_reg = nullptr;
  int32_t* d_slist = nullptr;  // per-region sphere lists
  int sph_cap = 0;
  void* h_stage = nullptr;  // pinned, two slots of (spheres, regions)
  size_t slot_bytes = 0;
  int slot = 0;
  bool stage_pending[2] = {false, false};
  std::vector<rcx::QSphere> cur;
  bool have_base = false;
  rcx::LevelArgs args[rcx::kMaxCascades]{};

  rcx::NrcState* nrc = nullptr;  // neural radiance cache (rc_nrc_enable), or null

  // per-solve stage timing (rc_set_stage_timing): tev[0] before the solve,
  // tev[nlev - i] after cascade i
  bool timing = false;
  bool timed = false;  // a solve has recorded the events
  cudaEvent_t tev[rcx::kMaxCascades + 1] = {};
  int64_t solves = 0;

  // device scratch of the shading pass, grown on demand and kept
  void* scratch[12] = {};
  size_t scratch_cap[12] = {};
  // the mesh rc_shade_set_mesh left on the device for rc_shade_draw
  bool shade_mesh = false;
  int64_t shade_ntris = 0;
  int32_t shade_ntex = 0;
  bool shade_tmat = false;
};

namespace rcx {

rc_status cuda_fail(cudaError_t e, const char* what);
bool fault_is(const char* name);
rc_status dev_alloc(void** ptr, size_t bytes, const char* what);

#define RC_CUDA(call, what)                                 \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return ::rcx::cuda_fail(e_, what); \
  } while (0)

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

// Plain solve of one level (its usual kernel), the walk queue of the narrow
// levels, and whether a level reads walk records (rc_context.cu).
void plain_level(const rc_context* c, int level, cudaStream_t s);
// Walks of the queued levels except those set in `skip` (bit i = cascade i).
void plain_queue_walk(const rc_context* c, cudaStream_t s, uint32_t skip);
bool level_uses_queue(const rc_context* c, int level);

// Neural radiance cache hooks (rc_nrc.cu).
bool nrc_active(const rc_context* c);
int nrc_first_level(const rc_context* c);  // first cascade the cache serves
// Whether the cache's far walk also walks the near levels that use the walk
// queue (both use step tables); then the solve launches no near walk.
bool nrc_walks_near(const rc_context* c);
// Checked build: the radiance-cache translation unit's failure words (read
// and cleared; zeros in the ordinary build).
cudaError_t nrc_check_read(unsigned long long* first, unsigned* count);
// Enqueues the cache's per-frame work for the far cascades (training-sample
// walks, refit, inference, fallback walks) and their merges, top level down to
// the first far level.  Called from the solve before the near levels.
rc_status nrc_enqueue_far(rc_context* c, cudaStream_t s);
void nrc_release(rc_context* c);

}  // namespace rcx
