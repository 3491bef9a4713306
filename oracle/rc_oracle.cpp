// rc_oracle.cpp -- CPU oracle for the radiance-cascade hot path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product (radiancecascade_gb300/)
// links, imports or calls this file.  It is used by tests/, by the smoke
// check and by bench.py's CPU baseline leg.
//
// Parity status: the reference repository (jw910731/RadianceCascade) holds no
// radiance-cascade implementation, no tests and no golden vectors for this
// path -- its only GPU programs are a forward raster pass (src/shader.wgsl,
// src/light.wgsl) and its only extension point is RenderStage
// (src/app.rs:3-7).  Parity with the reference is therefore UNPINNED.  This
// oracle restates the published method instead:
//   - radiance cascades: Sannikov, "Radiance Cascades: A Novel Approach to
//     Calculating Global Illumination" (2023) -- per-cascade interval rays,
//     top-down merge R + T * (merged far field), fluence = sum_d omega_d L_0;
//   - voxel traversal: Amanatides & Woo, "A Fast Voxel Traversal Algorithm for
//     Ray Tracing" (1987), done here in exact integer arithmetic;
//   - octahedral direction map: Engelhardt & Dachsbacher (2008);
//   - solid angle of a planar triangle: Van Oosterom & Strackee (1983).
// It is pinned by a second, independent Python restatement
// (oracle/oracle_np.py) and by known-answer tests derived from the physics
// (empty scene, furnace = 4*pi*E, occluders, symmetry).
//
// Two marching strategies are provided.  The FP64 oracle walks every ray
// from its probe centre and classifies each voxel entry by its exact distance
// (independent of the product's "jump to the interval start" logic); the
// jump strategy computes the interval start directly and is what the timed
// FP32 CPU baseline uses.  Both make identical discrete decisions.
//
// Build: oracle/build_oracle.py (g++ -O2 -fopenmp -ffp-contract=off).

#include "../include/rc.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Deterministic generator: splitmix64 (Steele, Lea & Flood 2014).
// ---------------------------------------------------------------------------
inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Rng {
  uint64_t s;
  Rng(uint64_t seed, uint64_t stream)
      : s(mix64(seed ^ mix64(stream ^ 0xD1B54A32D192ED03ull))) {}
  uint64_t next() {
    s += 0x9E3779B97F4A7C15ull;
    return mix64(s);
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
};

// binary16 decode (exact) and round-to-nearest-even encode.
double half_to_double(uint16_t h) {
  int sign = h >> 15, e = (h >> 10) & 31, m = h & 1023;
  double v;
  if (e == 0) v = std::ldexp((double)m, -24);
  else if (e == 31) v = m ? NAN : INFINITY;
  else v = std::ldexp(1024.0 + m, e - 25);
  return sign ? -v : v;
}

uint16_t float_to_half(float f) {
  double v = std::fabs((double)f);
  uint16_t sign = std::signbit(f) ? 0x8000 : 0;
  if (std::isnan(f)) return sign | 0x7E00;
  if (v >= 65520.0) return sign | 0x7C00;
  if (v < std::ldexp(1.0, -14)) {  // subnormal range: multiples of 2^-24
    double q = std::nearbyint(v * std::ldexp(1.0, 24));
    return sign | (uint16_t)q;  // q == 1024 encodes the smallest normal
  }
  int e;
  std::frexp(v, &e);  // v = f * 2^e, f in [0.5, 1)
  e -= 1;             // v in [2^e, 2^(e+1))
  double q = std::nearbyint(v * std::ldexp(1.0, 10 - e));  // [1024, 2048]
  if (q >= 2048.0) { q = 1024.0; e += 1; }
  if (e + 15 >= 31) return sign | 0x7C00;
  return sign | (uint16_t)(((e + 15) << 10) | ((int)q - 1024));
}

inline bool is_opaque(const rc_voxel& v) { return (v.albedo_occ & RC_VOXEL_OPAQUE) != 0; }

// ---------------------------------------------------------------------------
// Geometry shared by both marching strategies.
// ---------------------------------------------------------------------------
struct Dir {
  int64_t D[3];   // integer direction, |x|+|y|+|z| = n
  int64_t S;      // |D|^2
};

// Octahedral texel (j,k) of an n x n map: u = (2j+1)/n - 1, v = (2k+1)/n - 1;
// upper hemisphere (|u|+|v| <= 1): (u, v, 1-|u|-|v|); lower: the folded
// (sgn u (1-|v|), sgn v (1-|u|), 1-|u|-|v|).  Scaled by n to integers.
std::vector<Dir> make_dirs(int n) {
  std::vector<Dir> out((size_t)n * n);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) {
      int64_t U = 2 * j + 1 - n, V = 2 * k + 1 - n;
      int64_t au = U < 0 ? -U : U, av = V < 0 ? -V : V;
      Dir d;
      if (au + av <= n) {
        d.D[0] = U; d.D[1] = V; d.D[2] = n - au - av;
      } else {
        d.D[0] = (U < 0 ? -1 : 1) * (n - av);
        d.D[1] = (V < 0 ? -1 : 1) * (n - au);
        d.D[2] = n - au - av;
      }
      d.S = d.D[0] * d.D[0] + d.D[1] * d.D[1] + d.D[2] * d.D[2];
      out[(size_t)k * n + j] = d;
    }
  return out;
}

// Number of positive integers k with k * sqrt(S) < b * |Da|: the count of
// axis-a plane crossings closer to the probe centre than distance b.
int64_t crossings_before(int64_t b, int64_t Da, int64_t S) {
  int64_t a = Da < 0 ? -Da : Da;
  if (b <= 0 || a == 0) return 0;
  int64_t rhs = b * b * a * a;
  int64_t k = (int64_t)std::floor((double)b * (double)a / std::sqrt((double)S));
  while (k > 0 && k * k * S >= rhs) --k;
  while ((k + 1) * (k + 1) * S < rhs) ++k;
  return k;
}

struct LevelShape {
  int M[3];       // probes per axis
  int s;          // spacing
  int n;          // direction resolution
  int64_t blo, bhi;
  size_t probes() const { return (size_t)M[0] * M[1] * M[2]; }
};

std::vector<LevelShape> make_levels(const rc_params& p) {
  std::vector<LevelShape> L(p.num_cascades);
  int64_t b = 0;
  for (int i = 0; i < p.num_cascades; ++i) {
    LevelShape& l = L[i];
    l.s = p.probe_spacing0 << i;
    for (int a = 0; a < 3; ++a) l.M[a] = p.grid[a] / l.s;
    l.n = p.dir_res0 << i;
    l.blo = b;
    b = (i == 0) ? p.interval0 : b * p.interval_ratio + p.interval0;
    l.bhi = b;
  }
  return L;
}

struct Volume {
  int G[3];
  const rc_voxel* v;
  bool inside(const int64_t V[3]) const {
    return V[0] >= 0 && V[1] >= 0 && V[2] >= 0 && V[0] < G[0] && V[1] < G[1] && V[2] < G[2];
  }
  const rc_voxel& at(const int64_t V[3]) const {
    return v[((size_t)V[2] * G[1] + V[1]) * G[0] + V[0]];
  }
};

// March from the probe centre O (a lattice point).  The ray starts in the
// voxel it enters first (O - 1 on axes where D < 0).  Each step crosses the
// nearest voxel plane; on equal crossing distance x steps before y before z.
// A voxel belongs to interval [blo, bhi) when the distance at which the ray
// enters it lies in that range (the starting voxel is entered at 0).  Returns
// the first opaque voxel of the interval inside the grid, if any.
bool march_from_origin(const Volume& vol, const int64_t O[3], const Dir& d,
                       int64_t blo, int64_t bhi, int64_t hit[3]) {
  int64_t V[3], k[3] = {0, 0, 0}, ad[3];
  for (int a = 0; a < 3; ++a) {
    V[a] = O[a] - (d.D[a] < 0 ? 1 : 0);
    ad[a] = d.D[a] < 0 ? -d.D[a] : d.D[a];
  }
  if (blo == 0 && is_opaque(vol.at(V))) {
    std::memcpy(hit, V, sizeof V);
    return true;
  }
  for (;;) {
    int best = -1;
    for (int a = 0; a < 3; ++a) {
      if (ad[a] == 0) continue;
      // crossing times (k+1)/|D_a|, compared by cross-multiplication
      if (best < 0 || (k[a] + 1) * ad[best] < (k[best] + 1) * ad[a]) best = a;
    }
    k[best] += 1;
    V[best] += d.D[best] < 0 ? -1 : 1;
    int64_t lhs = k[best] * k[best] * d.S;
    if (lhs >= bhi * bhi * ad[best] * ad[best]) return false;  // entered at >= bhi
    if (!vol.inside(V)) return false;                           // left the grid
    if (lhs >= blo * blo * ad[best] * ad[best] && is_opaque(vol.at(V))) {
      std::memcpy(hit, V, sizeof V);
      return true;
    }
  }
}

// Same decisions, starting directly at the interval: skip the crossings that
// lie before blo on each axis, then take exactly the crossings in [blo, bhi).
bool march_jump(const Volume& vol, const int64_t O[3], const Dir& d,
                int64_t blo, int64_t bhi, int64_t hit[3]) {
  int64_t V[3], k[3], ad[3], steps = 0;
  for (int a = 0; a < 3; ++a) {
    ad[a] = d.D[a] < 0 ? -d.D[a] : d.D[a];
    k[a] = crossings_before(blo, ad[a], d.S);
    int sg = d.D[a] < 0 ? -1 : 1;
    V[a] = O[a] - (d.D[a] < 0 ? 1 : 0) + sg * k[a];
    steps += crossings_before(bhi, ad[a], d.S) - k[a];
  }
  if (blo == 0 && is_opaque(vol.at(V))) {
    std::memcpy(hit, V, sizeof V);
    return true;
  }
  for (int64_t s = 0; s < steps; ++s) {
    int best = -1;
    for (int a = 0; a < 3; ++a) {
      if (ad[a] == 0) continue;
      if (best < 0 || (k[a] + 1) * ad[best] < (k[best] + 1) * ad[a]) best = a;
    }
    k[best] += 1;
    V[best] += d.D[best] < 0 ? -1 : 1;
    if (!vol.inside(V)) return false;
    if (is_opaque(vol.at(V))) {
      std::memcpy(hit, V, sizeof V);
      return true;
    }
  }
  return false;
}

// ---------------------------------------------------------------------------
// Solid angles: a texel of the octahedral map is a planar polygon on the
// octahedron |x|+|y|+|z| = 1 (split along |u|+|v| = 1 into an upper and a
// lower piece); its solid angle is the sum over a triangle fan of
// Van Oosterom & Strackee's formula.
// ---------------------------------------------------------------------------
double tri_solid_angle(const double a[3], const double b[3], const double c[3]) {
  auto dot = [](const double* x, const double* y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; };
  double bc[3] = {b[1] * c[2] - b[2] * c[1], b[2] * c[0] - b[0] * c[2], b[0] * c[1] - b[1] * c[0]};
  double det = dot(a, bc);
  double la = std::sqrt(dot(a, a)), lb = std::sqrt(dot(b, b)), lc = std::sqrt(dot(c, c));
  double den = la * lb * lc + dot(a, b) * lc + dot(a, c) * lb + dot(b, c) * la;
  return 2.0 * std::atan2(std::fabs(det), den);
}

// Clip a convex polygon (in (a,c) = (|u|,|v|) coordinates) to a*sx + c*sx <= lim*sx.
std::vector<std::pair<double, double>> clip(const std::vector<std::pair<double, double>>& P, bool keep_below) {
  std::vector<std::pair<double, double>> out;
  auto f = [&](const std::pair<double, double>& q) {
    double v = q.first + q.second - 1.0;
    return keep_below ? -v : v;  // >= 0 inside
  };
  for (size_t i = 0; i < P.size(); ++i) {
    const auto& A = P[i];
    const auto& B = P[(i + 1) % P.size()];
    double fa = f(A), fb = f(B);
    if (fa >= 0) out.push_back(A);
    if ((fa > 0 && fb < 0) || (fa < 0 && fb > 0)) {
      double t = fa / (fa - fb);
      out.push_back({A.first + t * (B.first - A.first), A.second + t * (B.second - A.second)});
    }
  }
  return out;
}

double texel_solid_angle(int n, int j, int k) {
  double u0 = 2.0 * j / n - 1.0, u1 = 2.0 * (j + 1) / n - 1.0;
  double v0 = 2.0 * k / n - 1.0, v1 = 2.0 * (k + 1) / n - 1.0;
  double a0 = std::min(std::fabs(u0), std::fabs(u1)), a1 = std::max(std::fabs(u0), std::fabs(u1));
  double c0 = std::min(std::fabs(v0), std::fabs(v1)), c1 = std::max(std::fabs(v0), std::fabs(v1));
  std::vector<std::pair<double, double>> sq = {{a0, c0}, {a1, c0}, {a1, c1}, {a0, c1}};
  double total = 0.0;
  for (int lower = 0; lower < 2; ++lower) {
    auto P = clip(sq, lower == 0);
    if (P.size() < 3) continue;
    std::vector<std::array<double, 3>> Q;
    for (auto& q : P) {
      double a = q.first, c = q.second;
      if (!lower) Q.push_back({a, c, 1.0 - a - c});
      else Q.push_back({1.0 - c, 1.0 - a, 1.0 - a - c});
    }
    for (size_t t = 1; t + 1 < Q.size(); ++t) total += tri_solid_angle(Q[0].data(), Q[t].data(), Q[t + 1].data());
  }
  return total;
}

// ---------------------------------------------------------------------------
// The solver.
// ---------------------------------------------------------------------------
template <typename Real>
int solve(const rc_params& p, const rc_voxel* voxels, Real* fluence, Real* radiance, int nthreads, bool jump) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const auto levels = make_levels(p);
  const int N = p.num_cascades;
  Volume vol{{p.grid[0], p.grid[1], p.grid[2]}, voxels};

  // Per-level merged radiance L_i (planar [3][dirs][probes]) and the
  // direction-averaged A_i (planar [3][dirs of level i-1][probes of level i]).
  std::vector<std::vector<Real>> L(N), A(N);
  for (int i = N - 1; i >= 0; --i) {
    const LevelShape& lv = levels[i];
    const auto dirs = make_dirs(lv.n);
    const size_t P = lv.probes(), ND = dirs.size();
    L[i].assign(3 * ND * P, Real(0));
    const bool top = (i == N - 1);
    const LevelShape* up = top ? nullptr : &levels[i + 1];
    const std::vector<Real>* Aup = top ? nullptr : &A[i + 1];

#pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (long long d = 0; d < (long long)ND; ++d)
      for (int mz = 0; mz < lv.M[2]; ++mz)
        for (int my = 0; my < lv.M[1]; ++my)
          for (int mx = 0; mx < lv.M[0]; ++mx) {
            const int64_t O[3] = {(int64_t)(2 * mx + 1) * lv.s / 2, (int64_t)(2 * my + 1) * lv.s / 2,
                                  (int64_t)(2 * mz + 1) * lv.s / 2};
            int64_t hv[3];
            bool hit = jump ? march_jump(vol, O, dirs[d], lv.blo, lv.bhi, hv)
                            : march_from_origin(vol, O, dirs[d], lv.blo, lv.bhi, hv);
            Real out[3];
            if (hit) {
              const rc_voxel& v = vol.at(hv);
              for (int c = 0; c < 3; ++c) out[c] = (Real)half_to_double(v.emission[c]);
            } else if (top) {
              out[0] = out[1] = out[2] = Real(0);
            } else {
              // Trilinear interpolation over the 8 parent probes of the next
              // cascade: child index m sits at parent coordinate m/2 - 1/4.
              int q[3][2];
              Real w[3][2];
              const int m[3] = {mx, my, mz};
              for (int a = 0; a < 3; ++a) {
                int lo = (m[a] - 1) >> 1;
                bool even = (m[a] & 1) == 0;
                w[a][0] = even ? Real(0.25) : Real(0.75);
                w[a][1] = Real(1) - w[a][0];
                q[a][0] = std::min(std::max(lo, 0), up->M[a] - 1);
                q[a][1] = std::min(std::max(lo + 1, 0), up->M[a] - 1);
              }
              const size_t UP = up->probes();
              for (int c = 0; c < 3; ++c) {
                Real acc = Real(0);
                for (int tz = 0; tz < 2; ++tz)
                  for (int ty = 0; ty < 2; ++ty)
                    for (int tx = 0; tx < 2; ++tx) {
                      size_t qi = ((size_t)q[2][tz] * up->M[1] + q[1][ty]) * up->M[0] + q[0][tx];
                      acc += w[2][tz] * w[1][ty] * w[0][tx] * (*Aup)[((size_t)c * ND + d) * UP + qi];
                    }
                out[c] = acc;
              }
            }
            size_t pi = ((size_t)mz * lv.M[1] + my) * lv.M[0] + mx;
            for (int c = 0; c < 3; ++c) L[i][((size_t)c * ND + d) * P + pi] = out[c];
          }

    if (i >= 1) {
      // A_i(q, dp) = 1/4 sum of L_i over the 2x2 child texels of parent texel dp.
      const int np = levels[i - 1].n, nc = lv.n;
      const size_t NDP = (size_t)np * np;
      A[i].assign(3 * NDP * P, Real(0));
#pragma omp parallel for
      for (long long dp = 0; dp < (long long)NDP; ++dp) {
        int jp = (int)(dp % np), kp = (int)(dp / np);
        for (int c = 0; c < 3; ++c)
          for (size_t pi = 0; pi < P; ++pi) {
            Real s = Real(0);
            for (int b = 0; b < 2; ++b)
              for (int a = 0; a < 2; ++a) {
                size_t dc = (size_t)(2 * kp + b) * nc + (2 * jp + a);
                s += L[i][((size_t)c * ND + dc) * P + pi];
              }
            A[i][((size_t)c * NDP + dp) * P + pi] = Real(0.25) * s;
          }
      }
    }
    if (i + 1 < N) { A[i + 1].clear(); A[i + 1].shrink_to_fit(); }
  }

  // Fluence phi(p) = sum_d omega_d L_0(p, d), RGB interleaved.
  const LevelShape& l0 = levels[0];
  const size_t P0 = l0.probes(), ND0 = (size_t)l0.n * l0.n;
  std::vector<Real> omega(ND0);
  for (int k = 0; k < l0.n; ++k)
    for (int j = 0; j < l0.n; ++j) omega[(size_t)k * l0.n + j] = (Real)texel_solid_angle(l0.n, j, k);
  if (fluence) {
#pragma omp parallel for
    for (long long pi = 0; pi < (long long)P0; ++pi)
      for (int c = 0; c < 3; ++c) {
        Real s = Real(0);
        for (size_t d = 0; d < ND0; ++d) s += omega[d] * L[0][((size_t)c * ND0 + d) * P0 + pi];
        fluence[(size_t)pi * 3 + c] = s;
      }
  }
  if (radiance) {
    size_t off = 0;
    for (int i = 0; i < N; ++i) {
      std::memcpy(radiance + off, L[i].data(), L[i].size() * sizeof(Real));
      off += L[i].size();
    }
  }
  return 0;
}

bool params_ok(const rc_params* p) {
  if (!p || p->num_cascades < 1 || p->num_cascades > 10) return false;
  if (p->probe_spacing0 < 2 || (p->probe_spacing0 & (p->probe_spacing0 - 1))) return false;
  if (p->dir_res0 < 2 || (p->dir_res0 & 1)) return false;
  if (p->interval0 < 1 || p->interval_ratio < 2) return false;
  int top = p->probe_spacing0 << (p->num_cascades - 1);
  for (int a = 0; a < 3; ++a)
    if (p->grid[a] < top || p->grid[a] % top) return false;
  return true;
}

}  // namespace

extern "C" {

// Total radiance elements over all levels (3 * dirs * probes per level).
int64_t rco_radiance_elems(const rc_params* p) {
  if (!params_ok(p)) return -1;
  int64_t t = 0;
  for (auto& l : make_levels(*p)) t += 3 * (int64_t)l.n * l.n * (int64_t)l.probes();
  return t;
}

int rco_solve_f64(const rc_params* p, const rc_voxel* vol, double* fluence, double* radiance, int nthreads,
                  int jump) {
  if (!params_ok(p) || !vol) return 1;
  return solve<double>(*p, vol, fluence, radiance, nthreads, jump != 0);
}

int rco_solve_f32(const rc_params* p, const rc_voxel* vol, float* fluence, float* radiance, int nthreads,
                  int jump) {
  if (!params_ok(p) || !vol) return 1;
  return solve<float>(*p, vol, fluence, radiance, nthreads, jump != 0);
}

int rco_directions(int n, int32_t* out) {
  if (n < 2 || (n & 1)) return 1;
  auto d = make_dirs(n);
  for (size_t i = 0; i < d.size(); ++i)
    for (int a = 0; a < 3; ++a) out[3 * i + a] = (int32_t)d[i].D[a];
  return 0;
}

int rco_solid_angles(int n, double* out) {
  if (n < 2 || (n & 1)) return 1;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) out[(size_t)k * n + j] = texel_solid_angle(n, j, k);
  return 0;
}

int64_t rco_crossings_before(int64_t b, int64_t Da, int64_t S) { return crossings_before(b, Da, S); }

uint16_t rco_float_to_half(float f) { return float_to_half(f); }
double rco_half_to_double(uint16_t h) { return half_to_double(h); }

// Seeded scene: box k draws (edge xyz, lo xyz, albedo rgb) from stream k;
// sphere k draws (radius, centre xyz, emission rgb, then a direction by
// rejection in the unit ball) from stream 2^32 + k.
int rco_scene_generate(const rc_scene_spec* sp, uint64_t seed, rc_box* boxes, rc_sphere* spheres) {
  if (!sp) return 1;
  for (int b = 0; b < sp->num_boxes; ++b) {
    Rng r(seed, (uint64_t)b);
    int e[3], lo[3];
    for (int a = 0; a < 3; ++a) {
      int span = sp->box_edge_max - sp->box_edge_min + 1;
      e[a] = sp->box_edge_min + (int)std::floor(r.uniform() * span);
      if (e[a] > sp->box_edge_max) e[a] = sp->box_edge_max;
      if (e[a] > sp->grid[a]) e[a] = sp->grid[a];
    }
    for (int a = 0; a < 3; ++a) {
      lo[a] = (int)std::floor(r.uniform() * (sp->grid[a] - e[a] + 1));
      if (lo[a] > sp->grid[a] - e[a]) lo[a] = sp->grid[a] - e[a];
    }
    int alb[3];
    for (int c = 0; c < 3; ++c) {
      double x = sp->albedo_min + r.uniform() * (sp->albedo_max - sp->albedo_min);
      int q = (int)std::floor(x * 31.0 + 0.5);
      alb[c] = std::min(std::max(q, 0), 31);
    }
    rc_box& B = boxes[b];
    for (int a = 0; a < 3; ++a) { B.lo[a] = lo[a]; B.hi[a] = lo[a] + e[a]; }
    B.value.emission[0] = B.value.emission[1] = B.value.emission[2] = 0;
    B.value.albedo_occ = (uint16_t)(RC_VOXEL_OPAQUE | (alb[0] << 10) | (alb[1] << 5) | alb[2]);
  }
  for (int s = 0; s < sp->num_spheres; ++s) {
    Rng r(seed, (1ull << 32) + (uint64_t)s);
    rc_sphere& S = spheres[s];
    std::memset(&S, 0, sizeof S);
    double rad = sp->radius_min + r.uniform() * (sp->radius_max - sp->radius_min);
    S.radius = rad;
    for (int a = 0; a < 3; ++a) {
      double u = r.uniform();
      S.centre[a] = (sp->grid[a] >= 2.0 * rad) ? rad + u * (sp->grid[a] - 2.0 * rad) : 0.5 * sp->grid[a];
    }
    for (int c = 0; c < 3; ++c) {
      float e = (float)(sp->emission_min + r.uniform() * (sp->emission_max - sp->emission_min));
      S.value.emission[c] = float_to_half(e);
    }
    S.value.albedo_occ = RC_VOXEL_OPAQUE;
    double v[3], q;
    for (;;) {
      for (int a = 0; a < 3; ++a) v[a] = 2.0 * r.uniform() - 1.0;
      q = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      if (q > 1e-6 && q <= 1.0) break;
    }
    double inv = sp->speed / std::sqrt(q);
    for (int a = 0; a < 3; ++a) S.velocity[a] = v[a] * inv;
  }
  return 0;
}

void rco_spheres_advance(rc_sphere* sp, int n, const int32_t grid[3], int frames) {
  for (int f = 0; f < frames; ++f)
    for (int s = 0; s < n; ++s)
      for (int a = 0; a < 3; ++a) {
        double lo = sp[s].radius, hi = grid[a] - sp[s].radius;
        if (hi < lo) { sp[s].centre[a] = 0.5 * grid[a]; continue; }
        double c = sp[s].centre[a] + sp[s].velocity[a];
        if (c < lo) { c = 2.0 * lo - c; sp[s].velocity[a] = -sp[s].velocity[a]; }
        else if (c > hi) { c = 2.0 * hi - c; sp[s].velocity[a] = -sp[s].velocity[a]; }
        sp[s].centre[a] = c;
      }
}

// Boxes in order, then spheres in order; a later object overwrites.
int rco_voxelise(const int32_t grid[3], const rc_box* boxes, int nb, const rc_sphere* spheres, int ns,
                 rc_voxel* out) {
  const size_t G0 = grid[0], G1 = grid[1], G2 = grid[2];
  std::memset(out, 0, G0 * G1 * G2 * sizeof(rc_voxel));
  for (int b = 0; b < nb; ++b) {
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::max(boxes[b].lo[a], 0);
      hi[a] = std::min(boxes[b].hi[a], grid[a]);
    }
    for (int z = lo[2]; z < hi[2]; ++z)
      for (int y = lo[1]; y < hi[1]; ++y)
        for (int x = lo[0]; x < hi[0]; ++x) out[((size_t)z * G1 + y) * G0 + x] = boxes[b].value;
  }
  for (int s = 0; s < ns; ++s) {
    int64_t cq[3], rq = std::llround(spheres[s].radius * 256.0);
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      cq[a] = std::llround(spheres[s].centre[a] * 256.0);
      lo[a] = std::max(0, (int)std::floor((double)(cq[a] - rq) / 256.0) - 1);
      hi[a] = std::min(grid[a], (int)std::ceil((double)(cq[a] + rq) / 256.0) + 1);
    }
    for (int z = lo[2]; z < hi[2]; ++z)
      for (int y = lo[1]; y < hi[1]; ++y)
        for (int x = lo[0]; x < hi[0]; ++x) {
          int64_t dx = (int64_t)(2 * x + 1) * 128 - cq[0];
          int64_t dy = (int64_t)(2 * y + 1) * 128 - cq[1];
          int64_t dz = (int64_t)(2 * z + 1) * 128 - cq[2];
          if (dx * dx + dy * dy + dz * dz <= rq * rq) out[((size_t)z * G1 + y) * G0 + x] = spheres[s].value;
        }
  }
  return 0;
}

// Triangle mesh voxelisation.  Positions in grid units are rounded to 1/256
// voxel; voxel (x, y, z) is the closed box [256x, 256x+256] x ... in those
// units.  A voxel belongs to a triangle when no separating axis exists among
// the box normals, the triangle normal and the nine cross products of the
// triangle edges with the box normals (Akenine-Moeller 2001), with touching
// counted as overlap.  Triangles in order, a later triangle overwrites.
// Every quantity is an exact 64-bit integer.
static bool separated(const int64_t q[3][3], const int64_t axis[3], int64_t half) {
  int64_t pmin = 0, pmax = 0, radius = 0;
  for (int k = 0; k < 3; ++k) {
    const int64_t proj = axis[0] * q[k][0] + axis[1] * q[k][1] + axis[2] * q[k][2];
    pmin = k ? std::min(pmin, proj) : proj;
    pmax = k ? std::max(pmax, proj) : proj;
  }
  for (int c = 0; c < 3; ++c) radius += half * (axis[c] < 0 ? -axis[c] : axis[c]);
  return pmin > radius || pmax < -radius;
}

int rco_voxelise_mesh(const int32_t grid[3], const float* positions, int64_t nverts, const uint32_t* indices,
                      int64_t ntris, const uint16_t* tri_material, const rc_voxel* materials, int nmaterials,
                      rc_voxel* out) {
  const size_t G0 = grid[0], G1 = grid[1], G2 = grid[2];
  std::memset(out, 0, G0 * G1 * G2 * sizeof(rc_voxel));
  std::vector<int64_t> qv((size_t)nverts * 3);
  for (int64_t i = 0; i < nverts * 3; ++i) qv[i] = std::llround((double)positions[i] * 256.0);
  for (int64_t t = 0; t < ntris; ++t) {
    int64_t tri[3][3];
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) tri[k][c] = qv[(size_t)indices[3 * t + k] * 3 + c];
    int lo[3], hi[3];
    for (int c = 0; c < 3; ++c) {
      const int64_t mn = std::min(tri[0][c], std::min(tri[1][c], tri[2][c]));
      const int64_t mx = std::max(tri[0][c], std::max(tri[1][c], tri[2][c]));
      // voxels whose closed extent [256 x, 256 x + 256] meets [mn, mx]
      const int64_t first = (int64_t)std::ceil((double)(mn - 256) / 256.0);
      const int64_t last = (int64_t)std::floor((double)mx / 256.0);
      lo[c] = (int)std::max<int64_t>(first, 0);
      hi[c] = (int)std::min<int64_t>(last, grid[c] - 1);
    }
    int m = tri_material ? tri_material[t] : 0;
    if (m >= nmaterials) m = nmaterials - 1;
    const int64_t e[3][3] = {{tri[1][0] - tri[0][0], tri[1][1] - tri[0][1], tri[1][2] - tri[0][2]},
                             {tri[2][0] - tri[1][0], tri[2][1] - tri[1][1], tri[2][2] - tri[1][2]},
                             {tri[0][0] - tri[2][0], tri[0][1] - tri[2][1], tri[0][2] - tri[2][2]}};
    std::vector<std::array<int64_t, 3>> axes;
    for (int c = 0; c < 3; ++c) {
      std::array<int64_t, 3> u = {0, 0, 0};
      u[c] = 1;
      axes.push_back(u);
    }
    axes.push_back({e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
                    e[0][0] * e[1][1] - e[0][1] * e[1][0]});
    for (int i = 0; i < 3; ++i)
      for (int c = 0; c < 3; ++c) {
        // e_i x unit(c)
        std::array<int64_t, 3> a = {0, 0, 0};
        const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
        a[c1] = e[i][c2];
        a[c2] = -e[i][c1];
        axes.push_back(a);
      }
    for (int z = lo[2]; z <= hi[2]; ++z)
      for (int y = lo[1]; y <= hi[1]; ++y)
        for (int x = lo[0]; x <= hi[0]; ++x) {
          const int64_t centre[3] = {256 * (int64_t)x + 128, 256 * (int64_t)y + 128, 256 * (int64_t)z + 128};
          int64_t q[3][3];
          for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) q[k][c] = tri[k][c] - centre[c];
          bool hit = true;
          for (const auto& ax : axes)
            if (separated(q, ax.data(), 128)) {
              hit = false;
              break;
            }
          if (hit) out[((size_t)z * G1 + y) * G0 + x] = materials[m];
        }
  }
  return 0;
}

// Headless forward pass of the reference renderer (src/shader.wgsl:30-43,
// 76-100; src/renderer.rs:330-358): homogeneous rasterisation, depth Less,
// nearest then earlier triangle, Blinn-Phong fragment shading, optional
// fluence term (gi_scale / 4 pi x trilinear fluence between cascade-0
// probes).  FP32 throughout, written independently of the product.
namespace {
struct Tex {
  const uint8_t* p;
  int w, h, srgb;
};
float s2l(float c) { return c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f); }
void texel(const Tex& t, int x, int y, float* o) {
  const uint8_t* q = t.p + ((size_t)y * t.w + x) * 4;
  for (int k = 0; k < 4; ++k) o[k] = q[k] / 255.f;
  if (t.srgb)
    for (int k = 0; k < 3; ++k) o[k] = s2l(o[k]);
}
float mirror(float u) {
  float f = u - 2.f * std::floor(u * 0.5f);
  return f > 1.f ? 2.f - f : f;
}
void sample(const Tex& t, float u, float v, bool linear, float* o) {
  const float mu = mirror(u) * t.w, mv = mirror(v) * t.h;
  auto cx = [&](int x) { return std::min(std::max(x, 0), t.w - 1); };
  auto cy = [&](int y) { return std::min(std::max(y, 0), t.h - 1); };
  if (!linear) {
    texel(t, cx((int)std::floor(mu)), cy((int)std::floor(mv)), o);
    return;
  }
  const float fx = mu - 0.5f, fy = mv - 0.5f;
  const int xi = (int)std::floor(fx), yi = (int)std::floor(fy);
  const float ax = fx - xi, ay = fy - yi;
  float a[4], b[4], c[4], d[4];
  texel(t, cx(xi), cy(yi), a);
  texel(t, cx(xi + 1), cy(yi), b);
  texel(t, cx(xi), cy(yi + 1), c);
  texel(t, cx(xi + 1), cy(yi + 1), d);
  for (int k = 0; k < 4; ++k) o[k] = (a[k] * (1 - ax) + b[k] * ax) * (1 - ay) + (c[k] * (1 - ax) + d[k] * ax) * ay;
}
void norm(float* v) {
  const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  for (int k = 0; k < 3; ++k) v[k] /= l;
}
struct TriSetup {
  float clip[3][4];
  float inv[3][3];
  bool ok;
};
TriSetup setup_tri(const float* vp, const float* verts, const uint32_t* idx, int64_t t) {
  TriSetup s{};
  for (int k = 0; k < 3; ++k) {
    const float* p = verts + (size_t)idx[3 * t + k] * 17;
    for (int r = 0; r < 4; ++r) s.clip[k][r] = vp[r] * p[0] + vp[4 + r] * p[1] + vp[8 + r] * p[2] + vp[12 + r];
  }
  // M = rows (x, y, w) of the three vertices as columns; inverse via the adjugate
  const float m[3][3] = {{s.clip[0][0], s.clip[1][0], s.clip[2][0]},
                         {s.clip[0][1], s.clip[1][1], s.clip[2][1]},
                         {s.clip[0][3], s.clip[1][3], s.clip[2][3]}};
  float adj[3][3];
  adj[0][0] = m[1][1] * m[2][2] - m[1][2] * m[2][1];
  adj[0][1] = m[0][2] * m[2][1] - m[0][1] * m[2][2];
  adj[0][2] = m[0][1] * m[1][2] - m[0][2] * m[1][1];
  adj[1][0] = m[1][2] * m[2][0] - m[1][0] * m[2][2];
  adj[1][1] = m[0][0] * m[2][2] - m[0][2] * m[2][0];
  adj[1][2] = m[0][2] * m[1][0] - m[0][0] * m[1][2];
  adj[2][0] = m[1][0] * m[2][1] - m[1][1] * m[2][0];
  adj[2][1] = m[0][1] * m[2][0] - m[0][0] * m[2][1];
  adj[2][2] = m[0][0] * m[1][1] - m[0][1] * m[1][0];
  const float det = m[0][0] * adj[0][0] + m[0][1] * adj[1][0] + m[0][2] * adj[2][0];
  s.ok = std::fabs(det) > 1e-30f;
  if (s.ok)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) s.inv[i][j] = adj[i][j] * (1.f / det);
  return s;
}
void bary(const TriSetup& s, float px, float py, float* g) {
  for (int k = 0; k < 3; ++k) g[k] = s.inv[k][0] * px + s.inv[k][1] * py + s.inv[k][2];
}
void attrs(const TriSetup& s, const float* verts, const uint32_t* idx, int64_t t, float px, float py, float* at) {
  float g[3];
  bary(s, px, py, g);
  const float w = 1.f / (g[0] + g[1] + g[2]);
  for (int j = 0; j < 17; ++j) at[j] = 0.f;
  for (int k = 0; k < 3; ++k) {
    const float* v = verts + (size_t)idx[3 * t + k] * 17;
    const float b = g[k] * w;
    for (int j = 0; j < 17; ++j) at[j] += b * v[j];
  }
}
}  // namespace

int rco_shade(const rc_shade_view* view, const float* verts, int64_t nverts, const uint32_t* idx, int64_t ntris,
              const uint16_t* tmat, const rc_shade_material* mats, const rc_texture* textures, int ntex,
              const float* fluence, const int32_t probes[3], int spacing, float* out) {
  (void)nverts;
  const int W = view->width, H = view->height;
  std::vector<Tex> tex;
  for (int k = 0; k < ntex; ++k) tex.push_back(Tex{textures[k].rgba, textures[k].width, textures[k].height, textures[k].srgb});
  std::vector<uint64_t> zb((size_t)W * H, ~0ull);
  std::vector<TriSetup> su((size_t)ntris);
  for (int64_t t = 0; t < ntris; ++t) su[t] = setup_tri(view->view_proj, verts, idx, t);
  for (int64_t t = 0; t < ntris; ++t) {
    if (!su[t].ok) continue;
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const float px = (2.f * ((float)x + 0.5f)) / (float)W - 1.f;
        const float py = 1.f - (2.f * ((float)y + 0.5f)) / (float)H;
        float g[3];
        bary(su[t], px, py, g);
        if (!(g[0] >= 0.f && g[1] >= 0.f && g[2] >= 0.f) || g[0] + g[1] + g[2] <= 0.f) continue;
        const float z = g[0] * su[t].clip[0][2] + g[1] * su[t].clip[1][2] + g[2] * su[t].clip[2][2];
        if (!(z >= 0.f && z < 1.f)) continue;
        uint32_t zb32;
        std::memcpy(&zb32, &z, 4);
        const uint64_t key = ((uint64_t)zb32 << 32) | (uint64_t)t;
        uint64_t& cur = zb[(size_t)y * W + x];
        if (key < cur) cur = key;
      }
  }
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      float* o = out + ((size_t)y * W + x) * 4;
      o[0] = o[1] = o[2] = 0.f;
      o[3] = 1.f;
      const uint64_t key = zb[(size_t)y * W + x];
      if (key == ~0ull) continue;
      const int64_t t = (int64_t)(key & 0xFFFFFFFFull);
      const float px = (2.f * ((float)x + 0.5f)) / (float)W - 1.f;
      const float py = 1.f - (2.f * ((float)y + 0.5f)) / (float)H;
      float at[17], ax[17], ay[17];
      attrs(su[t], verts, idx, t, px, py, at);
      const rc_shade_material& m = mats[tmat ? tmat[t] : 0];
      const uint32_t eb = m.enable_bit;
      float du[2] = {0, 0}, dv[2] = {0, 0};
      if (eb & 3u) {
        attrs(su[t], verts, idx, t, px + 2.f / W, py, ax);
        attrs(su[t], verts, idx, t, px, py - 2.f / H, ay);
        du[0] = ax[15] - at[15];
        dv[0] = ax[16] - at[16];
        du[1] = ay[15] - at[15];
        dv[1] = ay[16] - at[16];
      }
      auto mag = [&](const Tex& tt) {
        const float x2 = du[0] * tt.w * du[0] * tt.w + dv[0] * tt.h * dv[0] * tt.h;
        const float y2 = du[1] * tt.w * du[1] * tt.w + dv[1] * tt.h * dv[1] * tt.h;
        return std::max(x2, y2) <= 1.f;
      };
      const float u = at[15], v = 1.f - at[16];
      float col[3] = {at[3], at[4], at[5]};
      if (eb & 1u) {
        float s4[4];
        sample(tex[m.color_texture], u, v, mag(tex[m.color_texture]), s4);
        for (int k = 0; k < 3; ++k) col[k] = s4[k];
      }
      float lc[3];
      for (int k = 0; k < 3; ++k) lc[k] = m.ambient[k] * 0.05f * m.ambient[3];
      float n[3] = {at[6], at[7], at[8]};
      if (eb & 2u) {
        float s4[4];
        sample(tex[m.normal_texture], u, v, mag(tex[m.normal_texture]), s4);
        float tg[3] = {at[9], at[10], at[11]}, bt[3] = {at[12], at[13], at[14]};
        norm(tg);
        norm(bt);
        const float cf[3] = {s4[0] * 2.f - 1.f, s4[1] * 2.f - 1.f, s4[2] * 2.f - 1.f};
        for (int k = 0; k < 3; ++k) n[k] = cf[0] * tg[k] + cf[1] * bt[k] + cf[2] * at[6 + k];
      }
      norm(n);
      float vd[3] = {view->eye[0] - at[0], view->eye[1] - at[1], view->eye[2] - at[2]};
      norm(vd);
      const float ndv = vd[0] * n[0] + vd[1] * n[1] + vd[2] * n[2];
      if (ndv < 0.f)
        for (int k = 0; k < 3; ++k) n[k] = -n[k];
      float ld[3] = {view->light[0] - at[0], view->light[1] - at[1], view->light[2] - at[2]};
      norm(ld);
      const float ndl = std::max(ld[0] * n[0] + ld[1] * n[1] + ld[2] * n[2], 0.f);
      for (int k = 0; k < 3; ++k) lc[k] += m.diffuse[k] * 0.7f * ndl * m.diffuse[3];
      float hd[3] = {vd[0] + ld[0], vd[1] + ld[1], vd[2] + ld[2]};
      norm(hd);
      const float st = std::pow(std::max(n[0] * hd[0] + n[1] * hd[1] + n[2] * hd[2], 0.f), m.shininess);
      const float on = ndv > 1e-6f ? 1.f : 0.f;
      for (int k = 0; k < 3; ++k) lc[k] += m.specular[k] * st * 1.f * m.specular[3] * on;
      if (view->gi_scale > 0.f && fluence) {
        float gp[3];
        for (int r = 0; r < 3; ++r)
          gp[r] = view->world_to_grid[4 * r] * at[0] + view->world_to_grid[4 * r + 1] * at[1] +
                  view->world_to_grid[4 * r + 2] * at[2] + view->world_to_grid[4 * r + 3];
        int i0[3], i1[3];
        float w1[3];
        for (int k = 0; k < 3; ++k) {
          const float mm = gp[k] / (float)spacing - 0.5f, fl = std::floor(mm);
          w1[k] = mm - fl;
          i0[k] = std::min(std::max((int)fl, 0), probes[k] - 1);
          i1[k] = std::min(std::max((int)fl + 1, 0), probes[k] - 1);
        }
        float f[3] = {0, 0, 0};
        for (int k = 0; k < 8; ++k) {
          const int xx = (k & 1) ? i1[0] : i0[0], yy = (k & 2) ? i1[1] : i0[1], zz = (k & 4) ? i1[2] : i0[2];
          const float w = ((k & 1) ? w1[0] : 1.f - w1[0]) * ((k & 2) ? w1[1] : 1.f - w1[1]) *
                          ((k & 4) ? w1[2] : 1.f - w1[2]);
          const float* sp = fluence + (((size_t)zz * probes[1] + yy) * probes[0] + xx) * 3;
          for (int c = 0; c < 3; ++c) f[c] += w * sp[c];
        }
        const float sc = view->gi_scale * 0.0795774715f;
        for (int k = 0; k < 3; ++k) lc[k] += sc * f[k];
      }
      float pr[3];
      for (int k = 0; k < 3; ++k) pr[k] = (m.ambient[k] - 1e-5f) + (m.diffuse[k] - 1e-5f) + (m.specular[k] - 1e-5f);
      const float none = (pr[0] + pr[1] + pr[2]) <= 0.f ? 1.f : 0.f;
      for (int k = 0; k < 3; ++k) o[k] = (lc[k] + none) * col[k];
    }
  return 0;
}

}  // extern "C"
