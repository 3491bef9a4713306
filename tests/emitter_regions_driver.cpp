// emitter_regions_driver.cpp -- runs the emitter update's host logic
// (rcx::update_regions and rcx::sphere_lists from rc_host.cpp) on spheres
// read from stdin, for tests/test_emitter_regions.py.
//   stdin: gx gy gz n, then n lines "cx cy cz r" (old) and n lines (new), 1/256 voxel units
//   stdout: the regions "w0 w1 y0 y1 z0 z1 s0 sn", then the list entries
#include <cstdio>
#include <vector>

#include "rc_internal.h"

int main() {
  int32_t grid[3];
  int n = 0;
  if (std::scanf("%d %d %d %d", &grid[0], &grid[1], &grid[2], &n) != 4) return 2;
  std::vector<rcx::QSphere> old_sph((size_t)n), new_sph((size_t)n);
  for (int pass = 0; pass < 2; ++pass)
    for (int i = 0; i < n; ++i) {
      rcx::QSphere& q = pass ? new_sph[(size_t)i] : old_sph[(size_t)i];
      long long c0, c1, c2, r;
      if (std::scanf("%lld %lld %lld %lld", &c0, &c1, &c2, &r) != 4) return 3;
      q = rcx::QSphere{};
      q.c[0] = c0;
      q.c[1] = c1;
      q.c[2] = c2;
      q.r = r;
    }
  std::vector<rcx::Region> regs((size_t)2 * n + 1);
  const int nreg = rcx::update_regions(old_sph.data(), new_sph.data(), n, grid, regs.data());
  std::vector<int32_t> list((size_t)8 * n + 8);
  const int64_t listed = rcx::sphere_lists(new_sph.data(), n, grid, regs.data(), nreg, list.data(), (int64_t)list.size());
  std::printf("%d %lld\n", nreg, (long long)listed);
  for (int r = 0; r < nreg; ++r)
    std::printf("%d %d %d %d %d %d %d %d\n", regs[r].w0, regs[r].w1, regs[r].y0, regs[r].y1, regs[r].z0, regs[r].z1,
                regs[r].s0, regs[r].sn);
  for (int64_t k = 0; k < listed; ++k) std::printf("%d\n", list[(size_t)k]);
  return 0;
}
