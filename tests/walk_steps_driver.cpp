// walk_steps_driver.cpp -- prints the walk step tables of one cascade level
// as the engine's host code builds them (rcx::build_dir_table and
// rcx::walk_steps from rc_host.cpp), for tests/test_walk_steps.py.
//   walk_steps_driver gx gy gz num_cascades level
// Output: per direction "d n", then n lines "phase cell".
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "rc_internal.h"

int main(int argc, char** argv) {
  if (argc != 6) return 2;
  rc_params p;
  if (rc_params_default(&p, std::atoi(argv[1]), std::atoi(argv[4])) != RC_OK) return 3;
  for (int a = 0; a < 3; ++a) p.grid[a] = std::atoi(argv[1 + a]);
  if (rc_params_validate(&p) != RC_OK) return 4;
  const int level = std::atoi(argv[5]);
  rcx::LevelGeom geom[rcx::kMaxCascades];
  rcx::level_geometry(p, geom);
  const rcx::LevelGeom& g = geom[level];
  std::vector<rcx::DirInfo> tab((size_t)g.ndirs);
  char msg[256];
  if (!rcx::build_dir_table(g, p.grid, tab.data(), msg, sizeof msg)) return 5;
  for (int d = 0; d < g.ndirs; ++d) {
    const int64_t n = rcx::walk_steps(g, p.grid, tab[d], level == 0, nullptr, 0);
    if (n < 0) return 6;
    std::vector<rcx::WalkStep> st((size_t)n);
    rcx::walk_steps(g, p.grid, tab[d], level == 0, st.data(), n);
    std::printf("%d %lld\n", d, (long long)n);
    for (const rcx::WalkStep& w : st) std::printf("%u %u\n", w.phase, w.cell);
  }
  return 0;
}
