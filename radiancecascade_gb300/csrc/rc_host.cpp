// rc_host.cpp -- host-side logic of the radiance-cascade engine that needs no
// GPU: parameter validation, cascade geometry, the exact integer walk tables,
// solid angles, the seeded scene generator, emitter motion and a host
// voxeliser.  Compiled with -ffp-contract=off so that its double arithmetic
// gives the same bits on x86_64 and aarch64.
//
// The reference has no cascade code (its only GPU programs are the forward
// raster pass in src/shader.wgsl and the debug light in src/light.wgsl); the
// method follows Sannikov's radiance cascades (2023), Amanatides & Woo voxel
// traversal (1987) and the Engelhardt & Dachsbacher octahedral map (2008).

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <vector>

#include "rc_internal.h"

namespace rcx {

static thread_local char g_last_error[512] = "no error";

int log_level() {
  static const int level = [] {
    const char* e = getenv("RC_LOG");
    return e ? atoi(e) : 0;
  }();
  return level;
}

void log_message(int level, const char* fmt, ...) {
  if (log_level() < level) return;
  char buf[640];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  fprintf(stderr, "rc[%s] %s\n", level <= 1 ? "error" : level == 2 ? "info" : "frame", buf);
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
  va_end(ap);
  log_message(1, "%s", g_last_error);
}

static std::mutex g_check_mutex;
static std::vector<CheckRange> g_check;
static uint64_t g_check_version = 0;

void check_register(const void* p, size_t bytes) {
  if (!p || !bytes) return;
  std::lock_guard<std::mutex> lock(g_check_mutex);
  const uint64_t lo = (uint64_t)(uintptr_t)p, hi = lo + bytes;
  for (const CheckRange& r : g_check)
    if (r.lo == lo && r.hi == hi) return;
  g_check.push_back(CheckRange{lo, hi});
  ++g_check_version;
}

std::vector<CheckRange> check_ranges(uint64_t* version) {
  std::lock_guard<std::mutex> lock(g_check_mutex);
  if (version) *version = g_check_version;
  return g_check;
}

const char* check_site_name(int site) {
  static const char* names[] = {"unknown",           "radiance",      "voxel volume",     "opacity bits",
                                "decimated opacity", "walk records",  "walk tables",      "fluence",
                                "shared memory",     "hash table",    "cache buffers",    "emitter regions"};
  return (site >= 0 && site < (int)(sizeof names / sizeof names[0])) ? names[site] : "unknown";
}

static bool fail(char* msg, size_t cap, const char* text) {
  if (msg && cap) snprintf(msg, cap, "%s", text);
  return false;
}

bool validate_params(const rc_params* p, char* msg, size_t cap) {
  if (!p) return fail(msg, cap, "params is NULL");
  if (p->num_cascades < 1 || p->num_cascades > kMaxCascades)
    return fail(msg, cap, "num_cascades must be in [1, 10]");
  if (p->probe_spacing0 < 2 || (p->probe_spacing0 & (p->probe_spacing0 - 1)))
    return fail(msg, cap, "probe_spacing0 must be a power of two >= 2");
  if (p->dir_res0 < 2 || (p->dir_res0 & 1)) return fail(msg, cap, "dir_res0 must be even and >= 2");
  if (p->interval0 < 1) return fail(msg, cap, "interval0 must be >= 1");
  if (p->interval_ratio < 2) return fail(msg, cap, "interval_ratio must be >= 2");
  if (p->precision != RC_PRECISION_FP32 && p->precision != RC_PRECISION_FP16)
    return fail(msg, cap, "precision must be RC_PRECISION_FP32 or RC_PRECISION_FP16");
  for (int i = 0; i < 7; ++i)
    if (p->reserved[i]) return fail(msg, cap, "reserved fields must be zero");
  int64_t top = (int64_t)p->probe_spacing0 << (p->num_cascades - 1);
  for (int a = 0; a < 3; ++a) {
    if (p->grid[a] < 1 || p->grid[a] > 1024) return fail(msg, cap, "grid edges must be in [1, 1024]");
    if (p->grid[a] % top)
      return fail(msg, cap, "every grid edge must be a multiple of the top cascade's probe spacing");
  }
  // level i >= 1 launches one block row per parent texel: (n_i / 2)^2 <= 65535
  if ((int64_t)p->dir_res0 << (p->num_cascades - 1) > 256)
    return fail(msg, cap, "top cascade direction resolution exceeds 256");
  return true;
}

void level_geometry(const rc_params& p, LevelGeom* out) {
  int64_t b = 0;
  for (int i = 0; i < p.num_cascades; ++i) {
    LevelGeom& g = out[i];
    g.spacing = p.probe_spacing0 << i;
    for (int a = 0; a < 3; ++a) g.M[a] = p.grid[a] / g.spacing;
    g.n = p.dir_res0 << i;
    g.ndirs = g.n * g.n;
    g.blo = b;
    b = (i == 0) ? (int64_t)p.interval0 : b * p.interval_ratio + p.interval0;
    g.bhi = b;
  }
}

// Integer octahedral direction of texel (j, k) at resolution n, scaled so
// that |x| + |y| + |z| = n.
static void oct_dir(int n, int j, int k, int64_t D[3]) {
  const int64_t u = 2 * j + 1 - n, v = 2 * k + 1 - n;
  const int64_t au = u < 0 ? -u : u, av = v < 0 ? -v : v;
  const int64_t z = n - au - av;
  if (z >= 0) {
    D[0] = u;
    D[1] = v;
  } else {
    D[0] = u < 0 ? -(n - av) : (n - av);
    D[1] = v < 0 ? -(n - au) : (n - au);
  }
  D[2] = z;
}

// Crossings of one axis strictly closer than distance b: the largest k with
// k^2 * S < b^2 * Da^2 (Da = |D_a|, S = |D|^2).
static int64_t crossings(int64_t b, int64_t Da, int64_t S) {
  if (b <= 0 || Da == 0) return 0;
  const int64_t lim = b * b * Da * Da;
  int64_t k = (int64_t)(sqrt((double)lim / (double)S));
  while (k > 0 && k * k * S >= lim) --k;
  while ((k + 1) * (k + 1) * S < lim) ++k;
  return k;
}

int64_t walk_steps(const LevelGeom& g, const int32_t grid[3], const DirInfo& di, bool test_start, WalkStep* out,
                   int64_t cap) {
  int l2s = 0;
  while ((1 << l2s) < g.spacing) ++l2s;
  const int s = 1 << l2s, h = s >> 1;
  int64_t a[3], t[3], n = 0;
  for (int ax = 0; ax < 3; ++ax) {
    a[ax] = h + di.start_off[ax];
    t[ax] = di.first_T[ax];
  }
  // 1 stored, 0 every probe out of the grid, -1 cell out of range
  auto push = [&]() -> int {
    uint32_t ph = 0, pc = 0;
    for (int ax = 2; ax >= 0; --ax) {
      if (a[ax] >= grid[ax] || a[ax] + (int64_t)(g.M[ax] - 1) * s < 0) return 0;
      const int64_t cell = a[ax] >> l2s;  // floor division
      if (cell < -127 || cell > 127) return -1;
      ph = (ph << l2s) | (uint32_t)(a[ax] & (s - 1));
      pc |= ((uint32_t)cell & 0xFFu) << (8 * ax);
    }
    if (n < cap) out[n] = WalkStep{ph, pc};
    ++n;
    return 1;
  };
  int r = test_start ? push() : 1;
  for (int k = 0; k < di.steps && r == 1; ++k) {
    const int ax = (t[0] <= t[1] && t[0] <= t[2]) ? 0 : (t[1] <= t[2] ? 1 : 2);
    a[ax] += di.sgn[ax];
    t[ax] += di.step_T[ax];
    r = push();
  }
  return r < 0 ? -1 : n;
}

bool build_dir_table(const LevelGeom& g, const int32_t grid[3], DirInfo* out, char* msg, size_t cap) {
  // A ray from a probe inside the grid is outside it beyond the grid diagonal,
  // so the walk never needs crossings farther away than that.
  const double diag = sqrt((double)grid[0] * grid[0] + (double)grid[1] * grid[1] + (double)grid[2] * grid[2]);
  const int64_t reach = (int64_t)ceil(diag) + 1;
  const int64_t blo = std::min<int64_t>(g.blo, reach), bhi = std::min<int64_t>(g.bhi, reach);
  for (int k = 0; k < g.n; ++k)
    for (int j = 0; j < g.n; ++j) {
      int64_t D[3];
      oct_dir(g.n, j, k, D);
      const int64_t A[3] = {D[0] < 0 ? -D[0] : D[0], D[1] < 0 ? -D[1] : D[1], D[2] < 0 ? -D[2] : D[2]};
      const int64_t S = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
      int64_t P = 1;
      for (int a = 0; a < 3; ++a)
        if (A[a]) P *= A[a];
      DirInfo& di = out[(size_t)k * g.n + j];
      memset(&di, 0, sizeof di);
      int64_t steps = 0;
      for (int a = 0; a < 3; ++a) {
        const int64_t klo = crossings(blo, A[a], S), khi = crossings(bhi, A[a], S);
        const int sg = D[a] > 0 ? 1 : (D[a] < 0 ? -1 : 0);
        di.sgn[a] = (int8_t)sg;
        const int64_t off = (D[a] < 0 ? -1 : 0) + sg * klo;
        if (off < INT16_MIN || off > INT16_MAX) return fail(msg, cap, "interval start offset exceeds 16 bits");
        di.start_off[a] = (int16_t)off;
        if (A[a]) {
          const int64_t st = P / A[a];
          // the walk reaches T = (khi + 1) * st and adds st once more at most
          if ((khi + 2) * st >= (int64_t)INT32_MAX)
            return fail(msg, cap, "cascade intervals exceed the exact 32-bit walk range");
          di.step_T[a] = (int32_t)st;
          di.first_T[a] = (int32_t)((klo + 1) * st);
        } else {
          di.step_T[a] = 0;
          di.first_T[a] = INT32_MAX;
        }
        steps += khi - klo;
      }
      di.steps = (int32_t)steps;
    }
  return true;
}

int64_t max_level_steps(const LevelGeom& g, const int32_t grid[3]) {
  const double diag = sqrt((double)grid[0] * grid[0] + (double)grid[1] * grid[1] + (double)grid[2] * grid[2]);
  const int64_t reach = (int64_t)ceil(diag) + 1;
  const int64_t blo = std::min<int64_t>(g.blo, reach), bhi = std::min<int64_t>(g.bhi, reach);
  int64_t best = 0;
  for (int k = 0; k < g.n; ++k)
    for (int j = 0; j < g.n; ++j) {
      int64_t D[3];
      oct_dir(g.n, j, k, D);
      const int64_t A[3] = {D[0] < 0 ? -D[0] : D[0], D[1] < 0 ? -D[1] : D[1], D[2] < 0 ? -D[2] : D[2]};
      const int64_t S = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
      int64_t steps = 0;
      for (int a = 0; a < 3; ++a) steps += crossings(bhi, A[a], S) - crossings(blo, A[a], S);
      best = std::max(best, steps);
    }
  return best;
}

void quantise_sphere(const rc_sphere& s, QSphere* q) {
  memset(q, 0, sizeof *q);
  for (int a = 0; a < 3; ++a) q->c[a] = llround(s.centre[a] * 256.0);
  q->r = llround(s.radius * 256.0);
  q->value = s.value;
}

static int64_t floor_div(int64_t a, int64_t b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

bool sphere_region(const QSphere& q, const int32_t grid[3], Region* r) {
  // voxel x is inside when |(2x+1)*128 - c| <= r, i.e. x in [(c-r)/256 - 1/2, (c+r)/256 - 1/2]
  int64_t lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = std::max<int64_t>(0, floor_div(q.c[a] - q.r, 256) - 1);
    hi[a] = std::min<int64_t>(grid[a], floor_div(q.c[a] + q.r, 256) + 2);
    if (hi[a] <= lo[a]) return false;
  }
  r->w0 = (int32_t)(lo[0] >> 5);
  r->w1 = (int32_t)((hi[0] + 31) >> 5);
  r->y0 = (int32_t)lo[1];
  r->y1 = (int32_t)hi[1];
  r->z0 = (int32_t)lo[2];
  r->z1 = (int32_t)hi[2];
  r->s0 = 0;
  r->sn = -1;
  return true;
}

int update_regions(const QSphere* old_sph, const QSphere* new_sph, int n, const int32_t grid[3], Region* out) {
  auto words = [](const Region& r) { return (int64_t)(r.w1 - r.w0) * (r.y1 - r.y0) * (r.z1 - r.z0); };
  int k = 0;
  for (int i = 0; i < n; ++i) {
    Region a, b;
    const bool ha = sphere_region(old_sph[i], grid, &a), hb = sphere_region(new_sph[i], grid, &b);
    if (ha && hb) {
      Region u = a;
      u.w0 = std::min(a.w0, b.w0);
      u.w1 = std::max(a.w1, b.w1);
      u.y0 = std::min(a.y0, b.y0);
      u.y1 = std::max(a.y1, b.y1);
      u.z0 = std::min(a.z0, b.z0);
      u.z1 = std::max(a.z1, b.z1);
      if (words(u) <= words(a) + words(b)) {
        out[k++] = u;
      } else {
        out[k++] = a;
        out[k++] = b;
      }
    } else if (ha) {
      out[k++] = a;
    } else if (hb) {
      out[k++] = b;
    }
  }
  return k;
}

int64_t sphere_lists(const QSphere* sph, int n, const int32_t grid[3], Region* regs, int nreg, int32_t* list,
                     int64_t cap) {
  int64_t listed = 0;
  bool ok = n > 0 && (int64_t)nreg * n <= (int64_t)1 << 22;
  std::vector<Region> ext;
  if (ok) {
    ext.resize((size_t)n);
    for (int i = 0; i < n; ++i)
      if (!sphere_region(sph[i], grid, &ext[(size_t)i])) ext[(size_t)i].w1 = ext[(size_t)i].w0;  // meets nothing
  }
  for (int r = 0; r < nreg && ok; ++r) {
    Region& g = regs[r];
    g.s0 = (int32_t)listed;
    g.sn = 0;
    for (int i = 0; i < n; ++i) {
      const Region& e = ext[(size_t)i];
      if (e.w0 < g.w1 && g.w0 < e.w1 && e.y0 < g.y1 && g.y0 < e.y1 && e.z0 < g.z1 && g.z0 < e.z1) {
        if (listed == cap) {
          ok = false;
          break;
        }
        list[listed++] = i;
        ++g.sn;
      }
    }
  }
  if (!ok) {
    listed = 0;
    for (int r = 0; r < nreg; ++r) {
      regs[r].s0 = 0;
      regs[r].sn = -1;
    }
  }
  return listed;
}

// ---------------------------------------------------------------------------
// Solid angle of an octahedral texel.  Each texel is a square in (|u|,|v|);
// the line |u|+|v| = 1 splits it into an upper and a lower planar piece on
// the octahedron.  The solid angle of each convex piece is a fan of
// triangles, each from tan(Omega/2) = |a.(b x c)| / (1 + a.b + b.c + c.a)
// with unit vectors a, b, c (Eriksson 1990).
// ---------------------------------------------------------------------------
struct V3 {
  double x, y, z;
};

static V3 unit(V3 p) {
  double l = sqrt(p.x * p.x + p.y * p.y + p.z * p.z);
  return {p.x / l, p.y / l, p.z / l};
}

static double tri_omega(V3 a, V3 b, V3 c) {
  a = unit(a);
  b = unit(b);
  c = unit(c);
  const double det = a.x * (b.y * c.z - b.z * c.y) - a.y * (b.x * c.z - b.z * c.x) + a.z * (b.x * c.y - b.y * c.x);
  const double den = 1.0 + (a.x * b.x + a.y * b.y + a.z * b.z) + (b.x * c.x + b.y * c.y + b.z * c.z) +
                     (c.x * a.x + c.y * a.y + c.z * a.z);
  return 2.0 * atan2(fabs(det), den);
}

static double texel_omega(int n, int j, int k) {
  double ua = fabs(2.0 * j / n - 1.0), ub = fabs(2.0 * (j + 1) / n - 1.0);
  double va = fabs(2.0 * k / n - 1.0), vb = fabs(2.0 * (k + 1) / n - 1.0);
  const double a0 = std::min(ua, ub), a1 = std::max(ua, ub), c0 = std::min(va, vb), c1 = std::max(va, vb);
  const double sq[4][2] = {{a0, c0}, {a1, c0}, {a1, c1}, {a0, c1}};
  double total = 0.0;
  for (int piece = 0; piece < 2; ++piece) {
    // keep points with (a + c - 1) <= 0 for the upper piece, >= 0 for the lower
    double poly[8][2];
    int m = 0;
    for (int i = 0; i < 4; ++i) {
      const double* p = sq[i];
      const double* q = sq[(i + 1) & 3];
      double fp = p[0] + p[1] - 1.0, fq = q[0] + q[1] - 1.0;
      if (piece) {
        fp = -fp;
        fq = -fq;
      }
      if (fp <= 0) {
        poly[m][0] = p[0];
        poly[m][1] = p[1];
        ++m;
      }
      if ((fp < 0 && fq > 0) || (fp > 0 && fq < 0)) {
        const double t = fp / (fp - fq);
        poly[m][0] = p[0] + t * (q[0] - p[0]);
        poly[m][1] = p[1] + t * (q[1] - p[1]);
        ++m;
      }
    }
    if (m < 3) continue;
    V3 P[8];
    for (int i = 0; i < m; ++i) {
      const double a = poly[i][0], c = poly[i][1];
      P[i] = piece == 0 ? V3{a, c, 1.0 - a - c} : V3{1.0 - c, 1.0 - a, 1.0 - a - c};
    }
    for (int i = 1; i + 1 < m; ++i) total += tri_omega(P[0], P[i], P[i + 1]);
  }
  return total;
}

// ---------------------------------------------------------------------------
// Seeded generator: splitmix64 streams (Steele, Lea & Flood 2014).
// ---------------------------------------------------------------------------
static inline uint64_t sm64_mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Stream {
  uint64_t state;
  Stream(uint64_t seed, uint64_t id) : state(sm64_mix(seed ^ sm64_mix(id ^ 0xD1B54A32D192ED03ull))) {}
  double next01() {
    state += 0x9E3779B97F4A7C15ull;
    return (double)(sm64_mix(state) >> 11) * (1.0 / 9007199254740992.0);
  }
};

// float -> binary16, round to nearest even, by integer manipulation.
static uint16_t to_half(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  const uint16_t sign = (uint16_t)((x >> 16) & 0x8000u);
  x &= 0x7FFFFFFFu;
  if (x >= 0x7F800000u) return sign | (x > 0x7F800000u ? 0x7E00 : 0x7C00);
  if (x >= 0x477FF000u) return sign | 0x7C00;  // rounds to infinity
  if (x < 0x38800000u) {                        // below the smallest normal half
    const uint32_t e = x >> 23, m = (x & 0x7FFFFFu) | (e ? 0x800000u : 0);
    const int s = 126 - (int)e;
    if (e == 0 || s > 24) return sign;
    uint32_t q = m >> s;
    const uint32_t rem = m & ((1u << s) - 1), halfway = 1u << (s - 1);
    if (rem > halfway || (rem == halfway && (q & 1))) ++q;
    return sign | (uint16_t)q;
  }
  uint32_t q = ((((x >> 23) - 112) << 10) | ((x & 0x7FFFFFu) >> 13));
  const uint32_t rem = x & 0x1FFFu;
  if (rem > 0x1000u || (rem == 0x1000u && (q & 1))) ++q;
  return sign | (uint16_t)q;
}

}  // namespace rcx

using namespace rcx;

extern "C" {

const char* rc_status_string(rc_status s) {
  switch (s) {
    case RC_OK: return "RC_OK";
    case RC_ERR_INVALID_ARG: return "RC_ERR_INVALID_ARG";
    case RC_ERR_OOM: return "RC_ERR_OOM";
    case RC_ERR_CUDA: return "RC_ERR_CUDA";
    case RC_ERR_TIMEOUT: return "RC_ERR_TIMEOUT";
    case RC_ERR_UNSUPPORTED: return "RC_ERR_UNSUPPORTED";
    case RC_ERR_STATE: return "RC_ERR_STATE";
  }
  return "RC_ERR_UNKNOWN";
}

const char* rc_last_error(void) { return g_last_error; }

int rc_abi_version(void) { return RC_ABI_VERSION; }

rc_status rc_params_default(rc_params* p, int32_t grid_edge, int32_t num_cascades) {
  if (!p) {
    set_error("rc_params_default: p is NULL");
    return RC_ERR_INVALID_ARG;
  }
  memset(p, 0, sizeof *p);
  p->grid[0] = p->grid[1] = p->grid[2] = grid_edge;
  p->num_cascades = num_cascades;
  p->probe_spacing0 = 2;
  p->dir_res0 = 4;
  p->interval0 = 1;
  p->interval_ratio = 4;
  p->precision = RC_PRECISION_FP32;
  return RC_OK;
}

rc_status rc_params_validate(const rc_params* p) {
  char msg[256];
  if (!validate_params(p, msg, sizeof msg)) {
    set_error("invalid rc_params: %s", msg);
    return RC_ERR_INVALID_ARG;
  }
  return RC_OK;
}

rc_status rc_level_info_get(const rc_params* p, int32_t level, rc_level_info* out) {
  if (rc_params_validate(p) != RC_OK) return RC_ERR_INVALID_ARG;
  if (!out || level < 0 || level >= p->num_cascades) {
    set_error("rc_level_info_get: bad level or NULL output");
    return RC_ERR_INVALID_ARG;
  }
  LevelGeom g[kMaxCascades];
  level_geometry(*p, g);
  const LevelGeom& l = g[level];
  for (int a = 0; a < 3; ++a) out->probes[a] = l.M[a];
  out->spacing = l.spacing;
  out->dir_res = l.n;
  out->num_dirs = l.ndirs;
  out->interval_lo = (int32_t)l.blo;
  out->interval_hi = (int32_t)std::min<int64_t>(l.bhi, INT32_MAX);
  out->radiance_elems = 3 * (int64_t)l.ndirs * l.probes();
  out->radiance_bytes = out->radiance_elems * (p->precision == RC_PRECISION_FP16 ? 2 : 4);
  return RC_OK;
}

int64_t rc_fluence_elems(const rc_params* p) {
  if (rc_params_validate(p) != RC_OK) return -1;
  LevelGeom g[kMaxCascades];
  level_geometry(*p, g);
  return 3 * g[0].probes();
}

rc_status rc_directions(int32_t n, int32_t* out_xyz) {
  if (n < 2 || (n & 1) || n > 4096 || !out_xyz) {
    set_error("rc_directions: n must be even in [2, 4096] and out non-NULL");
    return RC_ERR_INVALID_ARG;
  }
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) {
      int64_t D[3];
      oct_dir(n, j, k, D);
      for (int a = 0; a < 3; ++a) out_xyz[3 * ((size_t)k * n + j) + a] = (int32_t)D[a];
    }
  return RC_OK;
}

rc_status rc_solid_angles(int32_t n, double* out) {
  if (n < 2 || (n & 1) || n > 4096 || !out) {
    set_error("rc_solid_angles: n must be even in [2, 4096] and out non-NULL");
    return RC_ERR_INVALID_ARG;
  }
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j) out[(size_t)k * n + j] = texel_omega(n, j, k);
  return RC_OK;
}

rc_status rc_scene_generate(const rc_scene_spec* sp, uint64_t seed, rc_box* boxes, rc_sphere* spheres) {
  if (!sp || sp->num_boxes < 0 || sp->num_spheres < 0 || (sp->num_boxes && !boxes) ||
      (sp->num_spheres && !spheres) || sp->box_edge_min < 1 || sp->box_edge_max < sp->box_edge_min) {
    set_error("rc_scene_generate: bad spec or NULL output");
    return RC_ERR_INVALID_ARG;
  }
  for (int a = 0; a < 3; ++a)
    if (sp->grid[a] < 1) {
      set_error("rc_scene_generate: grid edges must be positive");
      return RC_ERR_INVALID_ARG;
    }
  const int span = sp->box_edge_max - sp->box_edge_min + 1;
  for (int b = 0; b < sp->num_boxes; ++b) {
    Stream r(seed, (uint64_t)b);
    int edge[3];
    for (int a = 0; a < 3; ++a) {
      int e = sp->box_edge_min + (int)floor(r.next01() * span);
      e = std::min(e, sp->box_edge_max);
      edge[a] = std::min(e, sp->grid[a]);
    }
    rc_box& B = boxes[b];
    for (int a = 0; a < 3; ++a) {
      int lo = (int)floor(r.next01() * (sp->grid[a] - edge[a] + 1));
      lo = std::min(lo, sp->grid[a] - edge[a]);
      B.lo[a] = lo;
      B.hi[a] = lo + edge[a];
    }
    int q[3];
    for (int c = 0; c < 3; ++c) {
      const double x = sp->albedo_min + r.next01() * (sp->albedo_max - sp->albedo_min);
      q[c] = std::min(std::max((int)floor(x * 31.0 + 0.5), 0), 31);
    }
    B.value.emission[0] = B.value.emission[1] = B.value.emission[2] = 0;
    B.value.albedo_occ = (uint16_t)(RC_VOXEL_OPAQUE | (q[0] << 10) | (q[1] << 5) | q[2]);
  }
  for (int s = 0; s < sp->num_spheres; ++s) {
    Stream r(seed, (1ull << 32) + (uint64_t)s);
    rc_sphere& S = spheres[s];
    memset(&S, 0, sizeof S);
    S.radius = sp->radius_min + r.next01() * (sp->radius_max - sp->radius_min);
    for (int a = 0; a < 3; ++a) {
      const double u = r.next01();
      S.centre[a] = (sp->grid[a] >= 2.0 * S.radius) ? S.radius + u * (sp->grid[a] - 2.0 * S.radius)
                                                     : 0.5 * sp->grid[a];
    }
    for (int c = 0; c < 3; ++c) {
      const float e = (float)(sp->emission_min + r.next01() * (sp->emission_max - sp->emission_min));
      S.value.emission[c] = to_half(e);
    }
    S.value.albedo_occ = RC_VOXEL_OPAQUE;
    double v[3], q2;
    do {
      for (int a = 0; a < 3; ++a) v[a] = 2.0 * r.next01() - 1.0;
      q2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    } while (!(q2 > 1e-6 && q2 <= 1.0));
    const double scale = sp->speed / sqrt(q2);
    for (int a = 0; a < 3; ++a) S.velocity[a] = v[a] * scale;
  }
  return RC_OK;
}

rc_status rc_spheres_advance(rc_sphere* sp, int32_t n, const int32_t grid[3], int32_t frames) {
  if ((n && !sp) || n < 0 || !grid || frames < 0) {
    set_error("rc_spheres_advance: bad arguments");
    return RC_ERR_INVALID_ARG;
  }
  for (int f = 0; f < frames; ++f)
    for (int s = 0; s < n; ++s)
      for (int a = 0; a < 3; ++a) {
        const double lo = sp[s].radius, hi = grid[a] - sp[s].radius;
        if (hi < lo) {
          sp[s].centre[a] = 0.5 * grid[a];
          continue;
        }
        double c = sp[s].centre[a] + sp[s].velocity[a];
        if (c < lo) {
          c = 2.0 * lo - c;
          sp[s].velocity[a] = -sp[s].velocity[a];
        } else if (c > hi) {
          c = 2.0 * hi - c;
          sp[s].velocity[a] = -sp[s].velocity[a];
        }
        sp[s].centre[a] = c;
      }
  return RC_OK;
}

rc_status rc_voxelise_host(const int32_t grid[3], const rc_box* boxes, int32_t nboxes, const rc_sphere* spheres,
                           int32_t nspheres, rc_voxel* out) {
  if (!grid || !out || nboxes < 0 || nspheres < 0 || (nboxes && !boxes) || (nspheres && !spheres)) {
    set_error("rc_voxelise_host: bad arguments");
    return RC_ERR_INVALID_ARG;
  }
  const int64_t gx = grid[0], gy = grid[1], gz = grid[2];
  if (gx < 1 || gy < 1 || gz < 1) {
    set_error("rc_voxelise_host: grid edges must be positive");
    return RC_ERR_INVALID_ARG;
  }
  memset(out, 0, (size_t)(gx * gy * gz) * sizeof(rc_voxel));
  for (int b = 0; b < nboxes; ++b) {
    const int64_t x0 = std::max<int64_t>(boxes[b].lo[0], 0), x1 = std::min<int64_t>(boxes[b].hi[0], gx);
    const int64_t y0 = std::max<int64_t>(boxes[b].lo[1], 0), y1 = std::min<int64_t>(boxes[b].hi[1], gy);
    const int64_t z0 = std::max<int64_t>(boxes[b].lo[2], 0), z1 = std::min<int64_t>(boxes[b].hi[2], gz);
    for (int64_t z = z0; z < z1; ++z)
      for (int64_t y = y0; y < y1; ++y)
        for (int64_t x = x0; x < x1; ++x) out[(z * gy + y) * gx + x] = boxes[b].value;
  }
  for (int s = 0; s < nspheres; ++s) {
    QSphere q;
    quantise_sphere(spheres[s], &q);
    Region r;
    if (!sphere_region(q, grid, &r)) continue;
    const int64_t x0 = (int64_t)r.w0 * 32, x1 = std::min<int64_t>((int64_t)r.w1 * 32, gx);
    for (int64_t z = r.z0; z < r.z1; ++z)
      for (int64_t y = r.y0; y < r.y1; ++y)
        for (int64_t x = x0; x < x1; ++x) {
          const int64_t dx = (2 * x + 1) * 128 - q.c[0], dy = (2 * y + 1) * 128 - q.c[1],
                        dz = (2 * z + 1) * 128 - q.c[2];
          if (dx * dx + dy * dy + dz * dz <= q.r * q.r) out[(z * gy + y) * gx + x] = q.value;
        }
  }
  return RC_OK;
}

}  // extern "C"
