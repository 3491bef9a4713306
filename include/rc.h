/*
 * rc.h -- C ABI of the GB300 radiance-cascade global-illumination engine.
 *
 * The reference renderer's only extension point is the RenderStage trait
 * (reference: src/app.rs:3-7): update() receives per-frame state and uploads it
 * (src/window/app.rs:112-132, src/renderer.rs:620-631), render() records GPU
 * work into the frame (src/window/app.rs:246-248, src/renderer.rs:559-613),
 * resize() rebuilds size-dependent resources (src/window/app.rs:104-110).
 * A GI pass is a RenderStage implementation; this header is the foreign
 * function interface such a stage calls:
 *
 *   RenderStage::resize  ->  rc_create / rc_destroy            (grid + cascade shape)
 *   RenderStage::update  ->  rc_scene_upload, rc_scene_set_spheres (scene volume, emitters)
 *   RenderStage::render  ->  rc_solve                            (all cascades + fluence)
 *   consumer binding     ->  rc_get_fluence / rc_get_radiance / rc_fluence_device_ptr
 *
 * Conventions
 *   - Every entry point returns an rc_status; nothing aborts or throws across
 *     the boundary.  rc_last_error() gives a message for the calling thread.
 *   - The context owns its device memory.  Caller buffers are borrowed for the
 *     duration of the call only.
 *   - Calls on one context must be serialised by the caller.  GPU work is
 *     ordered on the stream passed to rc_solve (or the context's own stream
 *     when NULL).  rc_solve is asynchronous; rc_get_* synchronise.
 *   - Only plain C types cross this boundary; no CUDA or framework types.
 *     Streams are passed as void* (a cudaStream_t).
 */
#ifndef RC_H_
#define RC_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RC_ABI_VERSION 1

typedef enum rc_status {
  RC_OK = 0,
  RC_ERR_INVALID_ARG = 1,  /* bad pointer, size, dimension or parameter      */
  RC_ERR_OOM = 2,          /* a device or pinned-host allocation failed       */
  RC_ERR_CUDA = 3,         /* a CUDA runtime call failed (incl. no device)    */
  RC_ERR_TIMEOUT = 4,      /* a bounded device-side wait ran out              */
  RC_ERR_UNSUPPORTED = 5,  /* parameters outside the exact-arithmetic range   */
  RC_ERR_STATE = 6         /* call out of order (e.g. solve before upload)    */
} rc_status;

enum { RC_PRECISION_FP32 = 0, RC_PRECISION_FP16 = 1 };
enum { RC_MEM_HOST = 0, RC_MEM_DEVICE = 1 };

/* Cascade parameters.  Grid edges are in voxels.  Cascade i (0-based) has
 * probe spacing s_i = probe_spacing0 * 2^i voxels with probe centres at
 * (m + 1/2) * s_i, (dir_res0 * 2^i)^2 octahedral directions, and covers the
 * distance interval [b_i, b_{i+1}) with b_0 = 0, b_1 = interval0 and
 * b_{i+1} = interval_ratio * b_i + interval0.  Every grid edge must be a
 * multiple of the top cascade's spacing. */
typedef struct rc_params {
  int32_t grid[3];
  int32_t num_cascades;   /* >= 1                                    */
  int32_t probe_spacing0; /* power of two, >= 2       (default 2)     */
  int32_t dir_res0;       /* even, >= 2, top level <= 256 (default 4) */
  int32_t interval0;      /* >= 1                     (default 1)     */
  int32_t interval_ratio; /* >= 2                     (default 4)     */
  int32_t precision;      /* RC_PRECISION_FP32 / RC_PRECISION_FP16    */
  int32_t reserved[7];    /* must be zero                             */
} rc_params;

/* One voxel of the scene volume, 8 bytes.
 *   emission:   RGB radiance leaving the voxel, IEEE-754 binary16 bits
 *   albedo_occ: bit 15 = opaque; bits 10..14 / 5..9 / 0..4 = albedo R/G/B as
 *               5-bit unorm.
 * A non-opaque voxel is empty space: its emission and albedo are ignored. */
typedef struct rc_voxel {
  uint16_t emission[3];
  uint16_t albedo_occ;
} rc_voxel;

#define RC_VOXEL_OPAQUE 0x8000u

/* Axis-aligned box covering voxels lo <= v < hi (clipped to the grid). */
typedef struct rc_box {
  int32_t lo[3];
  int32_t hi[3];
  rc_voxel value;
} rc_box;

/* Sphere emitter.  Centre and radius are in voxel units and are quantised to
 * 1/256 voxel when voxelised; a voxel belongs to the sphere when its centre
 * lies within the radius.  velocity is in voxels per frame. */
typedef struct rc_sphere {
  double centre[3];
  double radius;
  double velocity[3];
  rc_voxel value;
  uint32_t pad[2];
} rc_sphere;  /* 72 bytes */

/* Seeded synthetic scene description (boxes, then spheres). */
typedef struct rc_scene_spec {
  int32_t grid[3];
  int32_t num_boxes;
  int32_t box_edge_min, box_edge_max;  /* integer edges, inclusive range  */
  int32_t num_spheres;
  int32_t reserved;
  double albedo_min, albedo_max;       /* per channel                     */
  double radius_min, radius_max;       /* voxels                          */
  double emission_min, emission_max;   /* per channel                     */
  double speed;                        /* voxels per frame                */
} rc_scene_spec;

/* Shape of one cascade level as laid out in device memory. */
typedef struct rc_level_info {
  int32_t probes[3];      /* probes per axis                            */
  int32_t spacing;        /* voxels between probe centres               */
  int32_t dir_res;        /* n: the level has n*n directions            */
  int32_t num_dirs;
  int32_t interval_lo;    /* b_i, voxels                                */
  int32_t interval_hi;    /* b_{i+1}, voxels                            */
  int64_t radiance_elems; /* 3 * num_dirs * probes (planar RGB)         */
  int64_t radiance_bytes; /* radiance_elems * element size              */
} rc_level_info;

typedef struct rc_context rc_context;

/* ---- errors --------------------------------------------------------- */
const char* rc_status_string(rc_status s);
/* Message of the last failing call on this thread (never NULL). */
const char* rc_last_error(void);
int rc_abi_version(void);

/* ---- host-only helpers (no GPU needed) ------------------------------- */
rc_status rc_params_default(rc_params* p, int32_t grid_edge, int32_t num_cascades);
rc_status rc_params_validate(const rc_params* p);
rc_status rc_level_info_get(const rc_params* p, int32_t level, rc_level_info* out);
/* Elements of the cascade-0 fluence buffer: 3 * probes0 (RGB interleaved). */
int64_t rc_fluence_elems(const rc_params* p);
/* Seeded scene generator: writes spec->num_boxes boxes and
 * spec->num_spheres spheres. */
rc_status rc_scene_generate(const rc_scene_spec* spec, uint64_t seed,
                            rc_box* boxes, rc_sphere* spheres);
/* Advance spheres by `frames` frames: centre += velocity, reflected so that
 * the whole sphere stays inside the grid. */
rc_status rc_spheres_advance(rc_sphere* spheres, int32_t n,
                             const int32_t grid[3], int32_t frames);
/* Voxelise boxes then spheres (later objects win) into a host volume of
 * grid[0]*grid[1]*grid[2] voxels, x fastest. */
rc_status rc_voxelise_host(const int32_t grid[3], const rc_box* boxes,
                           int32_t nboxes, const rc_sphere* spheres,
                           int32_t nspheres, rc_voxel* out);
/* Octahedral direction table of resolution n: n*n integer vectors (x,y,z)
 * with |x|+|y|+|z| = n, texel (j,k) at index k*n + j. */
rc_status rc_directions(int32_t n, int32_t* out_xyz);
/* Exact solid angle (steradians) of every octahedral texel at resolution n. */
rc_status rc_solid_angles(int32_t n, double* out);

/* ---- context -------------------------------------------------------- */
rc_status rc_create(const rc_params* p, int32_t device, rc_context** out);
rc_status rc_destroy(rc_context* ctx);  /* NULL is accepted */
rc_status rc_get_params(const rc_context* ctx, rc_params* out);

/* Static scene volume (x fastest).  where = RC_MEM_HOST or RC_MEM_DEVICE.
 * Replaces the base volume; dynamic spheres are re-applied on top. */
rc_status rc_scene_upload(rc_context* ctx, const rc_voxel* voxels,
                          int64_t count, int32_t where);
/* Voxelise up to 1536 boxes on the device into the base volume (later
 * boxes win). */
rc_status rc_scene_set_boxes(rc_context* ctx, const rc_box* boxes,
                             int32_t n);
/* Voxelises a triangle mesh into the static scene, replacing boxes or an
 * earlier mesh (spheres are composed on top as usual).  positions: nverts x 3
 * floats in grid units (voxel (x, y, z) covers [x, x+1) x ...), each within
 * [-1024, 2048]; indices: ntris x 3; tri_material: ntris indices into
 * materials (NULL: material 0 everywhere).  Positions are rounded to 1/256
 * voxel and a voxel is set when a triangle touches its closed box (exact
 * integer separating-axis test), so walls are watertight; where triangles
 * overlap, the later triangle wins. */
rc_status rc_scene_set_mesh(rc_context* ctx, const float* positions,
                            int64_t nverts, const uint32_t* indices,
                            int64_t ntris, const uint16_t* tri_material,
                            const rc_voxel* materials, int32_t nmaterials);

/* Dynamic emitters drawn over the base volume (later spheres win).  Only
 * the voxels under the previous and the new spheres are rewritten. */
rc_status rc_scene_set_spheres(rc_context* ctx, const rc_sphere* spheres,
                               int32_t n);

/* Solve all cascades top-down and the cascade-0 fluence.  stream may be
 * NULL (context stream).  Asynchronous. */
rc_status rc_solve(rc_context* ctx, void* stream);
rc_status rc_synchronize(rc_context* ctx);

/* Cascade-0 fluence, RGB interleaved float32, probe order x fastest. */
rc_status rc_get_fluence(rc_context* ctx, float* out, int64_t elems,
                         int32_t where);
/* Merged radiance of one level, planar [3][num_dirs][pz][py][px], float32
 * or binary16 according to params.precision. */
rc_status rc_get_radiance(rc_context* ctx, int32_t level, void* out,
                          int64_t bytes, int32_t where);
/* Device pointer of the fluence written by the last solve (context-owned,
 * valid until destroy; once rc_get_fluence_async is in use, solves alternate
 * between two buffers, so ask again after each solve). */
rc_status rc_fluence_device_ptr(rc_context* ctx, const float** out);
/* The composed scene volume (static scene + spheres), count = grid voxels. */
rc_status rc_get_volume(rc_context* ctx, rc_voxel* out, int64_t count,
                        int32_t where);
/* Starts copying the last solve's fluence into host memory `out` (pinned
 * memory overlaps; pageable memory works but copies synchronously) on the
 * context's copy stream and returns; the copy overlaps the next solve, which
 * writes the other of two device fluence buffers.  `out` is complete after
 * rc_synchronize. */
rc_status rc_get_fluence_async(rc_context* ctx, float* out, int64_t elems);
rc_status rc_radiance_device_ptr(rc_context* ctx, int32_t level,
                                 const void** out);
/* The context's own stream (a cudaStream_t), for ordering consumer work
 * after rc_solve and for timing. */
rc_status rc_get_stream(rc_context* ctx, void** out);

/* ---- profiling ------------------------------------------------------ */
/* Runs `iters` frames on the context stream with CUDA events around every
 * kernel and writes the mean milliseconds per launch: ms_out[0] = scene
 * recomposition under the current spheres (the per-frame emitter update),
 * ms_out[1 + i] = cascade level i (the top level's figure includes the one
 * launch that walks every level with fewer than 32 probes per row).  Needs
 * 1 + num_cascades floats; with 2 + num_cascades, ms_out[1 + num_cascades]
 * is the whole level set of a frame timed without events between its
 * kernels (as rc_solve runs it: each level kernel may start while the one
 * before it finishes), from another `iters` frames.  Synchronises. */
rc_status rc_profile_levels(rc_context* ctx, int32_t iters, float* ms_out,
                            int32_t count);
/* Per-solve stage timing.  With timing on, every rc_solve records CUDA
 * events between its stages on the solve's stream (no host wait);
 * rc_get_stage_ms then waits for the last solve and writes ms_out[0] = the
 * whole solve and ms_out[1 + i] = cascade i (the top cascade's figure holds
 * the walk launch of the narrow cascades and, with the radiance cache on,
 * the cache's whole schedule).  Needs 1 + num_cascades floats.  Diagnostics:
 * the RC_LOG environment variable prints every error (1), also context
 * lifetime (2), also one line per solve (3) on stderr; RC_NVTX=1 wraps every
 * solve's launches in NVTX ranges "rc_solve" / "walks", "cascade i",
 * "radiance cache" for profilers. */
rc_status rc_set_stage_timing(rc_context* ctx, int32_t enable);
rc_status rc_get_stage_ms(rc_context* ctx, float* ms_out, int32_t count);

/* ---- checked build ---------------------------------------------------- */
/* librc_checked.so (the same sources built with RC_CHECKED) tests the
 * kernels' buffer accesses before making them: global accesses against the
 * library's allocations and borrowed caller buffers, shared accesses against
 * the block's shared memory.  An access that fails is skipped, counted, and
 * the first one's site and address kept; no kernel traps.  This call waits
 * for `device`, reads and clears those words: RC_OK when no access failed,
 * RC_ERR_STATE (message: count, site, address) otherwise; in the ordinary
 * library RC_ERR_UNSUPPORTED. */
rc_status rc_check_status(int32_t device, uint64_t* first_failure,
                          uint32_t* failures);

/* ---- batched solve --------------------------------------------------- */
/* Many independent scenes (each with its own rc_params: grid, cascades)
 * solved together.  rc_batch_solve launches one CUDA graph holding either one
 * persistent kernel that takes (scene, level, tile) items from a queue, top
 * level first, a level waiting (bounded) for the level above of its own
 * scene; or every scene's own level launches as parallel branches (see
 * rc_batch_tune for which).  Every scene must use the same precision. */
typedef struct rc_batch rc_batch;
rc_status rc_batch_create(const rc_params* params, int32_t nscenes,
                          int32_t device, rc_batch** out);
rc_status rc_batch_destroy(rc_batch* b);  /* NULL is accepted */
/* Voxelises boxes then spheres into scene `scene` (synchronises). */
rc_status rc_batch_scene_set(rc_batch* b, int32_t scene, const rc_box* boxes,
                             int32_t nboxes, const rc_sphere* spheres,
                             int32_t nspheres);
rc_status rc_batch_solve(rc_batch* b, void* stream);  /* asynchronous */
/* Synchronises; RC_ERR_TIMEOUT when a bounded wait ran out (the batch stays
 * usable). */
rc_status rc_batch_synchronize(rc_batch* b);
rc_status rc_batch_get_fluence(rc_batch* b, int32_t scene, float* out,
                               int64_t elems, int32_t where);
rc_status rc_batch_get_radiance(rc_batch* b, int32_t scene, int32_t level,
                                void* out, int64_t bytes, int32_t where);
/* Replaces the emitters of scene `scene` (the static scene stays): only the
 * voxels under the previous and the new spheres are rewritten, on the batch's
 * stream, so the update is ordered after the solves already enqueued and
 * before the next one, with no host wait (the host array may be freed on
 * return).  The scene must have been set with rc_batch_scene_set. */
rc_status rc_batch_set_spheres(rc_batch* b, int32_t scene,
                               const rc_sphere* spheres, int32_t n);
/* Every scene's cascade-0 fluence, scene after scene (each RGB interleaved,
 * rc_fluence_elems of its params), in one buffer of exactly their total
 * size; one synchronisation for the whole batch.  Pinned host memory lets
 * the copies run at full speed. */
rc_status rc_batch_get_fluence_all(rc_batch* b, float* out, int64_t elems,
                                   int32_t where);
/* The same read started after the solves enqueued so far, without
 * waiting: `out` (host memory of the same size; pinned memory overlaps,
 * pageable memory copies synchronously) is complete after
 * rc_batch_synchronize or any later call that synchronises.  The fluences
 * are first gathered into one device buffer on the batch stream (the first
 * call allocates it: the total size of the batch's fluence), then copied to
 * `out` on the batch's own copy stream; emitter updates and solves enqueued
 * afterwards wait only for the gather, so the copy to the host overlaps the
 * next solve, and the next read waits for this one's copy.  A caller that
 * alternates two output buffers overlaps its next frame's host work with
 * this frame's solve and read-back. */
rc_status rc_batch_get_fluence_all_async(rc_batch* b, float* out, int64_t elems);
/* Tile shape of the batch's queue items. */
typedef struct rc_batch_tiles {
  int32_t probes_per_item;  /* narrow levels: probes per item               */
  int32_t dirs_per_item;    /* narrow levels: parent texels (or pairs) per item */
  int32_t blocks_per_item;  /* wide levels, cascade 0: kernel blocks per item */
  int32_t walks_per_item;   /* walk-queue tasks (32-probe walks) per item    */
} rc_batch_tiles;
/* Every field in [1, 65536]; rebuilds the queue (synchronises). */
rc_status rc_batch_set_tiles(rc_batch* b, const rc_batch_tiles* tiles);
rc_status rc_batch_get_tiles(const rc_batch* b, rc_batch_tiles* out);
/* The form rc_batch_solve uses: *scene_launches = 1 for the scenes' own
 * level launches as parallel graph branches, 0 for the persistent kernel. */
rc_status rc_batch_get_form(const rc_batch* b, int32_t* scene_launches);
/* Autotuner: coordinate descent over the tile shape of the persistent
 * kernel, each candidate timed over `iters` solves of the current scenes;
 * then one more candidate, the scenes' own level launches as parallel
 * branches of the batch's graph.  Keeps the fastest form and reports it (the
 * tiles are the persistent kernel's best; outputs may be NULL).  The
 * environment variable RC_BATCH_MODE=persistent or =scenes, read when the
 * batch is created, fixes the form instead (the tuner then times only it);
 * rc_batch_set_tiles selects the persistent kernel. */
rc_status rc_batch_tune(rc_batch* b, int32_t iters, rc_batch_tiles* best,
                        float* best_ms);

/* ---- headless raster + Blinn-Phong shading --------------------------- */
/* The reference renderer's forward pass (src/shader.wgsl:30-43, 76-100;
 * pipeline state src/renderer.rs:330-358) for one triangle list into an RGBA
 * float image, plus an optional global-illumination term from the context's
 * last fluence: gi_scale / (4 pi) x fluence at the fragment (trilinear
 * between cascade-0 probes) joins the light colour.  gi_scale = 0 is the
 * reference shading exactly. */
typedef struct rc_shade_material {
  float ambient[4];   /* rgb, w = 1 when the material defines it (0: absent) */
  float diffuse[4];
  float specular[4];
  float shininess;
  uint32_t enable_bit;      /* bit 0 colour texture, bit 1 normal map        */
  int32_t color_texture;    /* index into the texture list (when bit 0)     */
  int32_t normal_texture;   /* index into the texture list (when bit 1)     */
} rc_shade_material;

typedef struct rc_texture {
  const uint8_t* rgba;  /* host RGBA8 rows, width x height                 */
  int32_t width, height;
  int32_t srgb;         /* 1: colour texture (sRGB-encoded), 0: normal map */
  int32_t pad;
} rc_texture;

typedef struct rc_shade_view {
  float view_proj[16];     /* column-major: clip = view_proj * (p, 1)      */
  float eye[3];            /* camera position (view_position)              */
  float light[3];          /* point light position                         */
  int32_t width, height;   /* image size in pixels                         */
  float world_to_grid[12]; /* grid = A p + b, row-major 3 x 4 (GI lookup)   */
  float gi_scale;          /* 0: no GI term                                */
  int32_t pad;
} rc_shade_view;

/* vertices: nverts x 17 floats (position, colour, normal, tangent,
 * bitangent, uv -- src/renderer.rs:370-410); indices: ntris x 3;
 * tri_material: ntris indices (NULL: material 0).  Pixels no triangle
 * covers are (0, 0, 0, 1).  out: width x height x 4 floats, row 0 at the
 * top, host or device (where). */
rc_status rc_shade(rc_context* ctx, const rc_shade_view* view,
                   const float* vertices, int64_t nverts,
                   const uint32_t* indices, int64_t ntris,
                   const uint16_t* tri_material,
                   const rc_shade_material* materials, int32_t nmaterials,
                   const rc_texture* textures, int32_t ntextures,
                   float* out, int32_t where);

/* rc_shade in two parts, as the reference builds its vertex, index and
 * material buffers once (src/renderer.rs:411-490) and renders every frame
 * from them (src/renderer.rs:559, src/app.rs:4-6): rc_shade_set_mesh
 * uploads the mesh, materials and textures (same arguments and checks as
 * rc_shade; the host arrays may be freed on return); rc_shade_draw shades
 * one view of the last uploaded mesh with the context's current fluence.
 * With where = RC_MEM_HOST the draw returns when the image is in `out`; with
 * RC_MEM_DEVICE it returns once the work is queued on the context's stream
 * (rc_synchronize waits for it).  rc_shade = set_mesh + draw + synchronize. */
rc_status rc_shade_set_mesh(rc_context* ctx, const float* vertices, int64_t nverts,
                            const uint32_t* indices, int64_t ntris,
                            const uint16_t* tri_material,
                            const rc_shade_material* materials, int32_t nmaterials,
                            const rc_texture* textures, int32_t ntextures);
rc_status rc_shade_draw(rc_context* ctx, const rc_shade_view* view, float* out, int32_t where);

/* ---- neural radiance cache ------------------------------------------ */
/* With the cache enabled, rc_solve serves the far cascades (first_level and
 * up) from a small network instead of walking their intervals: it predicts
 * each (probe, direction)'s interval result (R = radiance of the first
 * opaque voxel, T = 1 when the ray got through) from a multiresolution hash
 * grid of the probe position and the direction.  Every solve walks
 * 1/2^train_fraction_log2 of the directions of every far probe (a regular
 * sub-lattice of the octahedral map, another one each solve) as training
 * samples and a second such slice as held-out samples.  The held-out samples
 * score the network per voxel tile of fallback_tile^3: the solid-angle
 * weighted relative L2 error of the merged radiance (R + T x the next
 * cascade's radiance) the tile's far probes hand to the cascades below, over
 * this solve and over the last 2^train_fraction_log2 solves.  A tile above
 * fallback_threshold on either walks its probes instead of serving them; a
 * far cascade with at least plain_level_fraction of its probes in such tiles
 * walks entirely.  The network then serves the other probes with the weights
 * just scored, and one Adam step on the training samples prepares the next
 * solve.  Every decision is taken on the device: rc_solve does not wait. */
typedef struct rc_nrc_params {
  int32_t first_level;          /* first cascade served (default 2)          */
  int32_t hash_log2_entries;    /* entries per hash level, log2 (19)        */
  int32_t base_resolution;      /* coarsest hash grid (16)                  */
  int32_t max_resolution;       /* finest hash grid (512)                   */
  float learning_rate;          /* Adam step (1e-2)                         */
  float beta1, beta2, epsilon;  /* Adam (0.9, 0.99, 1e-10)                  */
  int32_t train_fraction_log2;  /* samples: 1/2^k of the far directions (4)  */
  int32_t steps_per_solve;      /* Adam steps per solve (1)                 */
  float fallback_threshold;     /* held-out relative L2 error (0.01)        */
  int32_t fallback_tile;        /* voxel tile edge, power of two (8)        */
  float radiance_scale;         /* network predicts R * scale (1/4)         */
  float plain_level_fraction;   /* a far cascade with at least this share of
                                   its probes in fallback tiles walks
                                   entirely (0.5)                           */
  uint64_t seed;                /* initial weights                          */
} rc_nrc_params;

#define RC_MAX_CASCADES 10

typedef struct rc_nrc_stats {
  int64_t solves;          /* solves served by the cache                     */
  int64_t steps;           /* Adam steps taken                               */
  float last_loss;         /* mean squared error of the last step            */
  int32_t served_levels;   /* bit i: the network served cascade i (its
                              probes outside flagged tiles) in the last
                              solve; else the whole cascade walked          */
  int64_t fallback_tiles;  /* of `tiles`, those on the plain walk now       */
  int64_t tiles;           /* fallback tiles that hold a far-cascade probe  */
  int64_t served_solves[RC_MAX_CASCADES]; /* per cascade: solves since
                              rc_nrc_enable in which the network served it  */
} rc_nrc_stats;

rc_status rc_nrc_params_default(rc_nrc_params* out);
/* Allocates and initialises the cache (all tiles start on the plain walk).
 * Every far cascade must have the bit-parallel walk (RC_ERR_UNSUPPORTED
 * otherwise, e.g. with RC_WALK=scalar). */
rc_status rc_nrc_enable(rc_context* ctx, const rc_nrc_params* params);
rc_status rc_nrc_disable(rc_context* ctx);
/* Serialises the parameters (MLP and hash grid, FP32).  With out == NULL or
 * bytes too small, writes the size needed to *needed and returns
 * RC_ERR_INVALID_ARG for a short buffer (RC_OK for NULL). */
rc_status rc_nrc_save(rc_context* ctx, void* out, int64_t bytes, int64_t* needed);
/* Loads parameters saved by rc_nrc_save with the same rc_nrc_params and
 * geometry; resets the optimiser state. */
rc_status rc_nrc_load(rc_context* ctx, const void* in, int64_t bytes);
rc_status rc_nrc_get_stats(rc_context* ctx, rc_nrc_stats* out);
/* The cache's (R, G, B, T) for n queries of far cascade `level` (host
 * arrays): out[4 i .. 4 i + 3] for probe probes[i], direction dirs[i]. */
rc_status rc_nrc_query(rc_context* ctx, int32_t level, const int32_t* probes,
                       const int32_t* dirs, int64_t n, float* out);
/* Gradient of sum((y - f(x))^2) / n over directions d0 .. d0 + n - 1 of one
 * probe (n <= 128) with targets (R, G, B, T) in `targets` [n][4]: the MLP
 * parameters' gradient (rc_nrc_param_count() floats, layout as rc_nrc_save's
 * MLP block) and the probe's 32 position features' gradient.  No update. */
rc_status rc_nrc_tile_gradient(rc_context* ctx, int32_t level, int32_t probe,
                               int32_t d0, int32_t n, const float* targets,
                               float* param_grad, float* pos_grad);
int32_t rc_nrc_param_count(void);

/* ---- allocation-free solve ------------------------------------------ */
/* No counterpart in the reference.
 *
 * Solves one frame of a static scene into buffers the caller owns, without
 * allocating any memory.  It exists for callers that cannot call cudaMalloc:
 * a renderer that reserves its whole device-memory budget at start-up and
 * forbids growth inside the frame loop (a cudaMalloc can also synchronise the
 * device and stall the frame), or a plugin host that hands each stage fixed
 * buffers and owns every allocation itself.
 *
 *   voxels    device pointer, grid[0]*grid[1]*grid[2] rc_voxel (x fastest)
 *   fluence   device pointer, rc_fluence_elems(p) floats (RGB interleaved)
 *   radiance  device pointer, every level's merged radiance back to back in
 *             level order, each laid out as rc_get_radiance describes
 *             (sum of rc_level_info.radiance_bytes)
 *   stream    cudaStream_t or NULL (legacy default stream)
 *
 * All three buffers must be 16-byte aligned (cudaMalloc's 256-byte alignment
 * is ample); a misaligned pointer returns RC_ERR_INVALID_ARG before any GPU
 * work.
 *
 * Its working memory (opacity bits, the per-level decimated opacity, the
 * child-averaged radiance and the walk tables) lives in one statically sized
 * device array of RC_NOALLOC_SCRATCH_BYTES (8 MiB, enough for grids up to 64^3
 * with the default cascade shape) that every GPU loading the library holds
 * until the process exits.  Parameters that need more return
 * RC_ERR_UNSUPPORTED with the required size in rc_last_error().
 *
 * The first call on a device looks up that array's device address (set-up
 * done once per device), so make the first call before any stream capture.
 * All calls share the array: calls whose GPU work overlaps (different
 * streams, or other host threads) race on it and must be serialised by the
 * caller.  The call is asynchronous on `stream`. */
#define RC_NOALLOC_SCRATCH_BYTES (8u << 20)
rc_status rc_solve_noalloc(const rc_params* p, const rc_voxel* voxels,
                           float* fluence, void* radiance, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* RC_H_ */
