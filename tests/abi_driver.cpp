// abi_driver.cpp -- drives the C ABI of include/rc.h from C++, the way a
// native renderer (the reference's Rust stage, through its extern "C"
// block) would.  Built and run by tests/test_host_abi.py ("host": no GPU
// calls) and tests/test_gpu_abi.py ("gpu": one solve, fluence written to a
// file for comparison with the Python binding).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "rc.h"

#define CHECK(cond)                                                      \
  do {                                                                   \
    if (!(cond)) {                                                       \
      std::fprintf(stderr, "FAILED %s:%d: %s (%s)\n", __FILE__, __LINE__, #cond, rc_last_error()); \
      return 1;                                                          \
    }                                                                    \
  } while (0)

static int host_checks() {
  CHECK(rc_abi_version() >= 1);
  CHECK(std::strlen(rc_status_string(RC_ERR_TIMEOUT)) > 0);
  rc_params p;
  CHECK(rc_params_default(&p, 64, 5) == RC_OK);
  CHECK(rc_params_validate(&p) == RC_OK);
  rc_params bad = p;
  bad.grid[0] = 63;  // not a multiple of the top spacing
  CHECK(rc_params_validate(&bad) == RC_ERR_INVALID_ARG);
  CHECK(std::strlen(rc_last_error()) > 0);
  CHECK(rc_params_validate(nullptr) == RC_ERR_INVALID_ARG);
  rc_level_info li;
  CHECK(rc_level_info_get(&p, 0, &li) == RC_OK && li.probes[0] == 32 && li.num_dirs == 16);
  CHECK(rc_level_info_get(&p, 5, &li) == RC_ERR_INVALID_ARG);
  CHECK(rc_fluence_elems(&p) == 3LL * 32 * 32 * 32);
  // directions and solid angles
  std::vector<int32_t> d(3 * 64);
  CHECK(rc_directions(8, d.data()) == RC_OK);
  for (int k = 0; k < 64; ++k) CHECK(std::abs(d[3 * k]) + std::abs(d[3 * k + 1]) + std::abs(d[3 * k + 2]) == 8);
  std::vector<double> om(64);
  CHECK(rc_solid_angles(8, om.data()) == RC_OK);
  double sum = 0;
  for (double w : om) sum += w;
  CHECK(std::fabs(sum - 4 * M_PI) < 1e-9);
  // generator + host voxeliser
  rc_scene_spec spec;
  std::memset(&spec, 0, sizeof spec);
  spec.grid[0] = spec.grid[1] = spec.grid[2] = 32;
  spec.num_boxes = 5;
  spec.box_edge_min = 3;
  spec.box_edge_max = 9;
  spec.num_spheres = 2;
  spec.albedo_min = 0.2;
  spec.albedo_max = 0.9;
  spec.radius_min = 2.0;
  spec.radius_max = 4.0;
  spec.emission_min = 1.0;
  spec.emission_max = 20.0;
  spec.speed = 0.5;
  std::vector<rc_box> boxes(5);
  std::vector<rc_sphere> spheres(2);
  CHECK(rc_scene_generate(&spec, 7, boxes.data(), spheres.data()) == RC_OK);
  std::vector<rc_voxel> vox(32 * 32 * 32);
  CHECK(rc_voxelise_host(spec.grid, boxes.data(), 5, spheres.data(), 2, vox.data()) == RC_OK);
  int occupied = 0;
  for (const rc_voxel& v : vox) occupied += (v.albedo_occ & 0x8000) != 0;
  CHECK(occupied > 0);
  CHECK(rc_spheres_advance(spheres.data(), 2, spec.grid, 3) == RC_OK);
  // NULL handling never aborts
  CHECK(rc_destroy(nullptr) == RC_OK);
  CHECK(rc_solve(nullptr, nullptr) == RC_ERR_INVALID_ARG);
  CHECK(rc_get_fluence(nullptr, nullptr, 0, RC_MEM_HOST) == RC_ERR_INVALID_ARG);
  CHECK(rc_create(&p, 0, nullptr) == RC_ERR_INVALID_ARG);
  CHECK(rc_batch_destroy(nullptr) == RC_OK);
  CHECK(rc_batch_solve(nullptr, nullptr) == RC_ERR_INVALID_ARG);
  CHECK(rc_get_fluence_async(nullptr, nullptr, 0) == RC_ERR_INVALID_ARG);
  CHECK(rc_shade_set_mesh(nullptr, nullptr, 0, nullptr, 0, nullptr, nullptr, 0, nullptr, 0) == RC_ERR_INVALID_ARG);
  rc_shade_view view;
  std::memset(&view, 0, sizeof view);
  CHECK(rc_shade_draw(nullptr, &view, nullptr, RC_MEM_HOST) == RC_ERR_INVALID_ARG);
  CHECK(rc_nrc_enable(nullptr, nullptr) == RC_ERR_INVALID_ARG);
  std::printf("host ok\n");
  return 0;
}

static int gpu_solve(const char* out_path) {
  rc_params p;
  CHECK(rc_params_default(&p, 32, 4) == RC_OK);
  rc_context* ctx = nullptr;
  CHECK(rc_create(&p, 0, &ctx) == RC_OK && ctx);
  rc_scene_spec spec;
  std::memset(&spec, 0, sizeof spec);
  spec.grid[0] = spec.grid[1] = spec.grid[2] = 32;
  spec.num_boxes = 6;
  spec.box_edge_min = 3;
  spec.box_edge_max = 10;
  spec.num_spheres = 3;
  spec.albedo_min = 0.2;
  spec.albedo_max = 0.9;
  spec.radius_min = 1.5;
  spec.radius_max = 4.0;
  spec.emission_min = 1.0;
  spec.emission_max = 20.0;
  spec.speed = 0.5;
  std::vector<rc_box> boxes(6);
  std::vector<rc_sphere> spheres(3);
  CHECK(rc_scene_generate(&spec, 77, boxes.data(), spheres.data()) == RC_OK);
  CHECK(rc_solve(ctx, nullptr) == RC_ERR_STATE);  // no scene yet
  CHECK(rc_scene_set_boxes(ctx, boxes.data(), 6) == RC_OK);
  CHECK(rc_scene_set_spheres(ctx, spheres.data(), 3) == RC_OK);
  CHECK(rc_solve(ctx, nullptr) == RC_OK);
  const int64_t n = rc_fluence_elems(&p);
  std::vector<float> flu((size_t)n);
  CHECK(rc_get_fluence(ctx, flu.data(), n - 1, RC_MEM_HOST) == RC_ERR_INVALID_ARG);
  CHECK(rc_get_fluence(ctx, flu.data(), n, RC_MEM_HOST) == RC_OK);
  CHECK(rc_get_radiance(ctx, 9, flu.data(), 4, RC_MEM_HOST) == RC_ERR_INVALID_ARG);
  CHECK(rc_synchronize(ctx) == RC_OK);
  CHECK(rc_destroy(ctx) == RC_OK);
  std::FILE* f = std::fopen(out_path, "wb");
  CHECK(f != nullptr);
  CHECK(std::fwrite(flu.data(), sizeof(float), flu.size(), f) == flu.size());
  std::fclose(f);
  std::printf("gpu ok\n");
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 2 && std::strcmp(argv[1], "host") == 0) return host_checks();
  if (argc >= 3 && std::strcmp(argv[1], "gpu") == 0) return gpu_solve(argv[2]);
  std::fprintf(stderr, "usage: abi_driver host | gpu <fluence.bin>\n");
  return 2;
}
