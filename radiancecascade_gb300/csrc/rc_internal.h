// rc_internal.h -- types shared by the host side and the CUDA kernels of the
// radiance-cascade engine.  Not part of the public ABI (include/rc.h is).
#pragma once

#include <stdint.h>

#include <vector>

#include "../../include/rc.h"

#ifdef __CUDACC__
#define RC_HD __host__ __device__ __forceinline__
#else
#define RC_HD inline
#endif

namespace rcx {

constexpr int kMaxCascades = 10;

// Per (cascade level, direction) constants of the exact integer voxel walk.
//
// The ray from a probe centre O (a lattice point) has integer direction D.
// Its k-th crossing of an axis-a voxel plane happens at ray parameter
// t = k / |D_a|; scaled by P = prod over nonzero |D_b| it is the integer
// T = k * P / |D_a| = k * step_T[a].  The walk always crosses the axis with
// the smallest next T (x before y before z on ties), so every probe of a
// level shares the same sequence of voxel offsets for a given direction.
//
// A level covers the distances [b_lo, b_hi).  start_off is the offset of the
// last voxel entered before b_lo (the first voxel itself for b_lo = 0),
// first_T the T of the next crossing on each axis and steps the number of
// crossings whose distance lies in [b_lo, b_hi).
struct alignas(16) DirInfo {
  int32_t step_T[3];   // T increment per crossing; 0 = axis never crossed
  int32_t first_T[3];  // T of the first crossing inside the interval; INT32_MAX if never
  int16_t start_off[3];
  int8_t sgn[3];       // -1, 0, +1
  int8_t pad0[3];
  int32_t steps;
  float omega;         // solid angle of the texel (steradians)
  int32_t pad1;
};
static_assert(sizeof(DirInfo) == 48, "DirInfo layout");

struct LevelGeom {
  int32_t M[3];      // probes per axis
  int32_t spacing;   // voxels
  int32_t n;         // direction resolution (n*n directions)
  int32_t ndirs;
  int64_t blo, bhi;  // interval in voxels
  int64_t probes() const { return (int64_t)M[0] * M[1] * M[2]; }
};

// Quantised sphere as the voxeliser uses it: centre and radius in 1/256 voxel.
struct QSphere {
  int64_t c[3];
  int64_t r;
  rc_voxel value;
  int32_t pad[2];
};

// Region of whole 32-voxel x-words, inclusive-exclusive, for partial rebuilds.
struct Region {
  int32_t w0, w1;  // x words
  int32_t y0, y1;
  int32_t z0, z1;
  int32_t s0, sn;  // spheres that may cover the region: list[s0 .. s0 + sn), or all when sn < 0
};

}  // namespace rcx

// ---- host helpers implemented in rc_host.cpp ------------------------------
namespace rcx {
bool validate_params(const rc_params* p, char* msg, size_t cap);
void level_geometry(const rc_params& p, LevelGeom* out);  // out[num_cascades]
// Fills the direction table of one level; returns false (with msg) when the
// integer walk would leave the exact 32-bit range.
bool build_dir_table(const LevelGeom& g, const int32_t grid[3], DirInfo* out, char* msg, size_t cap);

// One step of a walk as the queue kernel replays it: the voxel offset from
// the probe's cell origin split into the decimated-plane phase index
// ((pz << l2s) + py) << l2s + px and the coarse cell (cx, cy, cz) as three
// signed bytes (cx in bits 0-7).  Same layout as the device's uint2.
struct WalkStep {
  uint32_t phase;
  uint32_t cell;
};
// Appends to `out` the steps of direction `di` of level `g` (the start voxel
// first when `test_start`), replayed with the walk's own rule (the axis with
// the smallest next T; x before y before z on ties) and cut where every probe
// of the level has left the grid on some axis.  Returns the number of steps,
// or -1 when a coarse cell does not fit a signed byte.
int64_t walk_steps(const LevelGeom& g, const int32_t grid[3], const DirInfo& di, bool test_start, WalkStep* out,
                   int64_t cap);
// Largest number of voxel crossings any direction of the level takes.
int64_t max_level_steps(const LevelGeom& g, const int32_t grid[3]);
void quantise_sphere(const rc_sphere& s, QSphere* q);
// Bounding region (whole x-words, clipped to the grid) of a quantised sphere.
bool sphere_region(const QSphere& q, const int32_t grid[3], Region* r);
// Regions an emitter update recomposes, appended to `out` (at most 2 per
// sphere): for each sphere the box around its old and new extents when that
// box is no larger than the two apart, else both.  Returns the count added.
int update_regions(const QSphere* old_sph, const QSphere* new_sph, int n, const int32_t grid[3], Region* out);
// For each region, the spheres whose extent meets it (ascending indices)
// into list[regs[r].s0 .. + regs[r].sn).  When the lists would exceed `cap`
// entries or `nreg * n` tests exceed 2^22, every region gets sn = -1 (test all
// spheres).  Returns the number of list entries.
int64_t sphere_lists(const QSphere* sph, int n, const int32_t grid[3], Region* regs, int nreg, int32_t* list,
                     int64_t cap);
void set_error(const char* fmt, ...);

// Device ranges the checked build's kernels may touch (rc_check.cuh):
// registered by dev_alloc and by the entry points that borrow caller
// buffers; check_ranges returns a copy and a version that changes with
// every registration.  No-ops' worth of bookkeeping in the ordinary build.
struct CheckRange {
  uint64_t lo, hi;
};
void check_register(const void* p, size_t bytes);
std::vector<CheckRange> check_ranges(uint64_t* version);
const char* check_site_name(int site);
// Diagnostics on stderr by the RC_LOG environment variable (read once):
// 0 or unset = silent, 1 = every error as it is set, 2 = also context
// lifetime and configuration, 3 = also one line per solve.
int log_level();
void log_message(int level, const char* fmt, ...);
}  // namespace rcx
