// rc_shade.cuh -- headless raster + Blinn-Phong shading that consumes the
// cascade-0 fluence (sm_103a).
//
// Restates the reference renderer's forward pass for a triangle list:
//   vertex stage (src/shader.wgsl:30-43): clip = view_proj * (position, 1);
//   fragment stage (src/shader.wgsl:76-100): texture / vertex colour by
//     enable_bit bit 0, optional normal map through the TBN (bit 1), view-facing
//     normal flip, ambient 0.05, diffuse 0.7 N.L, specular (N.H)^shininess when
//     N.V > 1e-6, and the "no material" predicate;
//   pipeline state (src/renderer.rs:330-358): no culling, depth test Less
//     against a buffer cleared to 1, colour cleared to (0, 0, 0, 1).
// Added on top (gi_scale > 0): the fluence of the cascades, trilinear between
// cascade-0 probes at the fragment's grid position, scaled by the surface
// colour and gi_scale / (4 pi), joins the light colour -- the step after the
// GI solve.
//
// Rasterisation is homogeneous (Olano and Greer 1997): for a pixel at NDC
// (px, py) the perspective-correct barycentrics are g = M^-1 (px, py, 1),
// M = [x_i; y_i; w_i] of the clip-space vertices; the pixel is covered when
// every g_i >= 0 (behind-the-eye intersections give all g_i <= 0), so no
// near-plane clipping is needed, and z_ndc = sum g_i z_i.  Pass 1 resolves
// visibility per pixel with a 64-bit atomicMin of (depth bits, triangle) --
// nearest first, then the earlier triangle, as a Less depth test with
// in-order submission; pass 2 shades each covered pixel once.
#pragma once

#include <math.h>
#include <stdint.h>

#include "rc_internal.h"

namespace rcx {

constexpr int kShadeVertexFloats = 17;  // position, colour, normal, tangent, bitangent, uv

struct ShadeTex {
  const uint8_t* texels;  // RGBA8 rows
  int32_t w, h;
  int32_t srgb;           // colour textures are sRGB-encoded, normal maps linear
  int32_t pad;
};

struct ShadeArgs {
  const float* verts;      // [nverts][17]
  const uint32_t* idx;     // [ntris][3]
  const uint16_t* tmat;    // [ntris] material of each triangle (or null: 0)
  const rc_shade_material* mats;
  const ShadeTex* tex;     // textures referenced by the materials
  int64_t ntris;
  float vp[16];            // column-major view_proj
  float eye[3];
  float light[3];
  int32_t W, H;
  unsigned long long* zbuf;  // [H][W]: (depth bits << 32) | triangle, ~0 = empty
  float* out;              // [H][W][4]
  // fluence (gi_scale > 0)
  const float* fluence;    // [Mz][My][Mx][3]
  int32_t M[3];
  float spacing;
  float w2g[12];           // grid = A world + b, row-major 3 x 4
  float gi_scale;
  int32_t ntex;
};

// clip = vp * (p, 1)
__device__ __forceinline__ void shade_clip(const float* vp, const float* p, float* c) {
#pragma unroll
  for (int r = 0; r < 4; ++r) c[r] = vp[r] * p[0] + vp[4 + r] * p[1] + vp[8 + r] * p[2] + vp[12 + r];
}

// Rows of M^-1 (up to the common factor 1/det, folded in): g = R (px, py, 1).
// Returns false for a triangle seen edge-on (det ~ 0).
__device__ __forceinline__ bool shade_setup(const float c[3][4], float R[3][3]) {
  // M = [x0 x1 x2; y0 y1 y2; w0 w1 w2]
  const float a = c[0][0], b = c[1][0], d = c[2][0];
  const float e = c[0][1], f = c[1][1], g = c[2][1];
  const float h = c[0][3], i = c[1][3], j = c[2][3];
  const float A0 = f * j - g * i, A1 = d * i - b * j, A2 = b * g - d * f;
  const float B0 = g * h - e * j, B1 = a * j - d * h, B2 = d * e - a * g;
  const float C0 = e * i - f * h, C1 = b * h - a * i, C2 = a * f - b * e;
  const float det = a * A0 + b * B0 + d * C0;
  if (!(fabsf(det) > 1e-30f)) return false;
  const float s = 1.f / det;
  // inverse = adj / det; row k of the inverse gives g_k
  R[0][0] = A0 * s; R[0][1] = A1 * s; R[0][2] = A2 * s;
  R[1][0] = B0 * s; R[1][1] = B1 * s; R[1][2] = B2 * s;
  R[2][0] = C0 * s; R[2][1] = C1 * s; R[2][2] = C2 * s;
  return true;
}

__device__ __forceinline__ void shade_load_tri(const ShadeArgs& a, int64_t t, float c[3][4]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float* v = a.verts + (int64_t)__ldg(&a.idx[t * 3 + k]) * kShadeVertexFloats;
    const float p[3] = {__ldg(v), __ldg(v + 1), __ldg(v + 2)};
    shade_clip(a.vp, p, c[k]);
  }
}

// Screen bounds of triangle t (the whole image when a vertex is at or behind
// the eye); false when it covers nothing.
__device__ __forceinline__ bool shade_bounds(const ShadeArgs& a, const float c[3][4], int4& b) {
  b = make_int4(0, 0, a.W - 1, a.H - 1);
  if (c[0][3] > 0.f && c[1][3] > 0.f && c[2][3] > 0.f) {
    float lx = 1e30f, hx = -1e30f, ly = 1e30f, hy = -1e30f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float sx = (c[k][0] / c[k][3] + 1.f) * 0.5f * a.W, sy = (1.f - c[k][1] / c[k][3]) * 0.5f * a.H;
      lx = fminf(lx, sx); hx = fmaxf(hx, sx); ly = fminf(ly, sy); hy = fmaxf(hy, sy);
    }
    // clamp in float first: a vertex near the eye plane projects far away
    lx = fmaxf(lx - 1.f, 0.f); ly = fmaxf(ly - 1.f, 0.f);
    hx = fminf(hx + 1.f, (float)(a.W - 1)); hy = fminf(hy + 1.f, (float)(a.H - 1));
    if (!(lx <= hx && ly <= hy)) return false;
    b = make_int4((int)floorf(lx), (int)floorf(ly), (int)ceilf(hx), (int)ceilf(hy));
  }
  return true;
}

// Depth test of triangle t at pixel (x, y).
__device__ __forceinline__ void shade_fragment(const ShadeArgs& a, int64_t t, const float c[3][4],
                                               const float R[3][3], int x, int y) {
  const float px = (2.f * ((float)x + 0.5f)) / (float)a.W - 1.f;
  const float py = 1.f - (2.f * ((float)y + 0.5f)) / (float)a.H;
  float g[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) g[k] = R[k][0] * px + R[k][1] * py + R[k][2];
  if (!(g[0] >= 0.f && g[1] >= 0.f && g[2] >= 0.f) || g[0] + g[1] + g[2] <= 0.f) return;
  const float z = g[0] * c[0][2] + g[1] * c[1][2] + g[2] * c[2][2];
  if (!(z >= 0.f && z < 1.f)) return;
  const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | (unsigned long long)t;
  atomicMin(&a.zbuf[(int64_t)y * a.W + x], key);
}

constexpr int kShadeTile = 64;          // pixels per side of a large triangle's tile
constexpr int kShadeBigRows = 32;       // blocks per tile that share the large triangles
constexpr int kShadeSmallArea = 4096;   // bounds of at most this many pixels: one warp per triangle

// Pass 0: bounds of every triangle, split into small ones (a warp each) and
// large ones (a block per 64 x 64 tile of their bounds).
static __global__ void k_shade_bin(const __grid_constant__ ShadeArgs a, int4* __restrict__ bounds,
                                   uint32_t* __restrict__ small, uint32_t* __restrict__ big,
                                   unsigned* __restrict__ counts) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.ntris) return;
  float c[3][4], R[3][3];
  shade_load_tri(a, t, c);
  int4 b;
  if (!shade_setup(c, R) || !shade_bounds(a, c, b)) return;
  bounds[t] = b;
  const int64_t area = (int64_t)(b.z - b.x + 1) * (b.w - b.y + 1);
  if (area <= kShadeSmallArea) small[atomicAdd(&counts[0], 1u)] = (uint32_t)t;
  else big[atomicAdd(&counts[1], 1u)] = (uint32_t)t;
}

// Pass 1a: one warp per small triangle, lanes over the pixels of its bounds.
static __global__ void k_shade_depth_small(const __grid_constant__ ShadeArgs a, const int4* __restrict__ bounds,
                                           const uint32_t* __restrict__ list, const unsigned* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t n = counts[0];
  for (int64_t k = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < n; k += warps) {
    const int64_t t = list[k];
    float c[3][4], R[3][3];
    shade_load_tri(a, t, c);
    shade_setup(c, R);
    const int4 b = bounds[t];
    const int nx = b.z - b.x + 1;
    const int count = nx * (b.w - b.y + 1);
    for (int q = lane; q < count; q += 32) shade_fragment(a, t, c, R, b.x + q % nx, b.y + q / nx);
  }
}

// Pass 1b: block (tile, large triangle), threads over the tile's pixels.
static __global__ void k_shade_depth_big(const __grid_constant__ ShadeArgs a, const int4* __restrict__ bounds,
                                         const uint32_t* __restrict__ list, const unsigned* __restrict__ counts) {
  const int tiles_x = (a.W + kShadeTile - 1) / kShadeTile;
  const int tx = (int)(blockIdx.x % tiles_x), ty = (int)(blockIdx.x / tiles_x);
  for (int64_t k = blockIdx.y; k < (int64_t)counts[1]; k += gridDim.y) {
    const int64_t t = list[k];
    const int4 b = bounds[t];
    const int x0 = max(b.x, tx * kShadeTile), x1 = min(b.z, tx * kShadeTile + kShadeTile - 1);
    const int y0 = max(b.y, ty * kShadeTile), y1 = min(b.w, ty * kShadeTile + kShadeTile - 1);
    if (x0 > x1 || y0 > y1) continue;
    float c[3][4], R[3][3];
    shade_load_tri(a, t, c);
    shade_setup(c, R);
    const int nx = x1 - x0 + 1;
    const int count = nx * (y1 - y0 + 1);
    for (int q = threadIdx.x; q < count; q += blockDim.x) shade_fragment(a, t, c, R, x0 + q % nx, y0 + q / nx);
  }
}

__device__ __forceinline__ float srgb_to_linear(float c) {
  return c <= 0.04045f ? c / 12.92f : powf((c + 0.055f) / 1.055f, 2.4f);
}

__device__ __forceinline__ float mirror_repeat(float u) {
  // MirrorRepeat: period 2, reflected on odd periods
  const float f = u - 2.f * floorf(u * 0.5f);
  return f > 1.f ? 2.f - f : f;
}

__device__ __forceinline__ float4 texel(const ShadeTex& t, int x, int y) {
  const uint8_t* p = t.texels + ((int64_t)y * t.w + x) * 4;
  float4 v = make_float4(p[0] / 255.f, p[1] / 255.f, p[2] / 255.f, p[3] / 255.f);
  if (t.srgb) {
    v.x = srgb_to_linear(v.x);
    v.y = srgb_to_linear(v.y);
    v.z = srgb_to_linear(v.z);
  }
  return v;
}

// Sample with MirrorRepeat addressing; `linear` selects the magnification
// (bilinear) filter, else the minification (nearest) filter.
__device__ __forceinline__ float4 shade_sample(const ShadeTex& t, float u, float v, bool linear) {
  const float mu = mirror_repeat(u) * t.w, mv = mirror_repeat(v) * t.h;
  if (!linear) {
    const int x = min(max((int)floorf(mu), 0), t.w - 1), y = min(max((int)floorf(mv), 0), t.h - 1);
    return texel(t, x, y);
  }
  const float fx = mu - 0.5f, fy = mv - 0.5f;
  const int xi = (int)floorf(fx), yi = (int)floorf(fy);
  const float ax = fx - xi, ay = fy - yi;
  auto clampx = [&](int x) { return min(max(x, 0), t.w - 1); };
  auto clampy = [&](int y) { return min(max(y, 0), t.h - 1); };
  const float4 t00 = texel(t, clampx(xi), clampy(yi)), t10 = texel(t, clampx(xi + 1), clampy(yi));
  const float4 t01 = texel(t, clampx(xi), clampy(yi + 1)), t11 = texel(t, clampx(xi + 1), clampy(yi + 1));
  float4 r;
  r.x = (t00.x * (1 - ax) + t10.x * ax) * (1 - ay) + (t01.x * (1 - ax) + t11.x * ax) * ay;
  r.y = (t00.y * (1 - ax) + t10.y * ax) * (1 - ay) + (t01.y * (1 - ax) + t11.y * ax) * ay;
  r.z = (t00.z * (1 - ax) + t10.z * ax) * (1 - ay) + (t01.z * (1 - ax) + t11.z * ax) * ay;
  r.w = (t00.w * (1 - ax) + t10.w * ax) * (1 - ay) + (t01.w * (1 - ax) + t11.w * ax) * ay;
  return r;
}

__device__ __forceinline__ void nrm3(float* v) {
  const float l = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= l;
  v[1] /= l;
  v[2] /= l;
}

__device__ __forceinline__ float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Trilinear fluence between cascade-0 probe centres (clamped at the border).
__device__ __forceinline__ void shade_fluence(const ShadeArgs& a, const float* wp, float* f) {
  float gp[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) gp[r] = a.w2g[4 * r] * wp[0] + a.w2g[4 * r + 1] * wp[1] + a.w2g[4 * r + 2] * wp[2] + a.w2g[4 * r + 3];
  int i0[3], i1[3];
  float w1[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float m = gp[k] / a.spacing - 0.5f;  // probe m sits at (m + 1/2) spacing
    const float fl = floorf(m);
    w1[k] = m - fl;
    i0[k] = min(max((int)fl, 0), a.M[k] - 1);
    i1[k] = min(max((int)fl + 1, 0), a.M[k] - 1);
  }
  f[0] = f[1] = f[2] = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int x = (k & 1) ? i1[0] : i0[0], y = (k & 2) ? i1[1] : i0[1], z = (k & 4) ? i1[2] : i0[2];
    const float w = ((k & 1) ? w1[0] : 1.f - w1[0]) * ((k & 2) ? w1[1] : 1.f - w1[1]) * ((k & 4) ? w1[2] : 1.f - w1[2]);
    const float* s = a.fluence + (((int64_t)z * a.M[1] + y) * a.M[0] + x) * 3;
    f[0] += w * s[0];
    f[1] += w * s[1];
    f[2] += w * s[2];
  }
}

// Perspective-correct attributes of triangle t at pixel (x, y).
__device__ __forceinline__ void shade_attrs(const ShadeArgs& a, int64_t t, float px, float py, float* at) {
  float c[3][4], R[3][3];
  shade_load_tri(a, t, c);
  shade_setup(c, R);
  float g[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) g[k] = R[k][0] * px + R[k][1] * py + R[k][2];
  const float s = 1.f / (g[0] + g[1] + g[2]);
#pragma unroll
  for (int j = 0; j < kShadeVertexFloats; ++j) at[j] = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float* v = a.verts + (int64_t)__ldg(&a.idx[t * 3 + k]) * kShadeVertexFloats;
    const float b = g[k] * s;
#pragma unroll
    for (int j = 0; j < kShadeVertexFloats; ++j) at[j] += b * __ldg(v + j);
  }
}

// Pass 2: one thread per pixel.
static __global__ void k_shade_pixels(const __grid_constant__ ShadeArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)a.W * a.H) return;
  const int x = (int)(i % a.W), y = (int)(i / a.W);
  const unsigned long long key = a.zbuf[i];
  float4 outc = make_float4(0.f, 0.f, 0.f, 1.f);
  if (key != ~0ull) {
    const int64_t t = (int64_t)(key & 0xFFFFFFFFull);
    const float px = (2.f * ((float)x + 0.5f)) / (float)a.W - 1.f;
    const float py = 1.f - (2.f * ((float)y + 0.5f)) / (float)a.H;
    float at[kShadeVertexFloats];
    shade_attrs(a, t, px, py, at);
    const float* wp = at;           // world position
    const float* vcol = at + 3;
    float nin[3] = {at[6], at[7], at[8]};
    float tan_[3] = {at[9], at[10], at[11]};
    float bit_[3] = {at[12], at[13], at[14]};
    const float u = at[15], v = 1.f - at[16];
    const rc_shade_material m = a.mats[a.tmat ? a.tmat[t] : 0];
    const uint32_t eb = m.enable_bit;
    // Level of detail from the texture coordinate's rate between this pixel and
    // its right and lower neighbours on the same triangle plane: at most one
    // texel per pixel magnifies (bilinear), more minifies (nearest).
    float du[2] = {0.f, 0.f}, dv[2] = {0.f, 0.f};
    if (eb & 3u) {
      float ax_[kShadeVertexFloats], ay_[kShadeVertexFloats];
      shade_attrs(a, t, px + 2.f / a.W, py, ax_);
      shade_attrs(a, t, px, py - 2.f / a.H, ay_);
      du[0] = ax_[15] - at[15];
      dv[0] = ax_[16] - at[16];
      du[1] = ay_[15] - at[15];
      dv[1] = ay_[16] - at[16];
    }
    auto magnifies = [&](const ShadeTex& tt) {
      const float x2 = du[0] * tt.w * du[0] * tt.w + dv[0] * tt.h * dv[0] * tt.h;
      const float y2 = du[1] * tt.w * du[1] * tt.w + dv[1] * tt.h * dv[1] * tt.h;
      return fmaxf(x2, y2) <= 1.f;
    };
    float col[3];
    if (eb & 1u) {
      const ShadeTex& ct = a.tex[m.color_texture];
      const float4 s = shade_sample(ct, u, v, magnifies(ct));
      col[0] = s.x; col[1] = s.y; col[2] = s.z;
    } else {
      col[0] = vcol[0]; col[1] = vcol[1]; col[2] = vcol[2];
    }
    float lc[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) lc[k] = m.ambient[k] * 0.05f * m.ambient[3];
    float n[3];
    if (eb & 2u) {
      const ShadeTex& nt = a.tex[m.normal_texture];
      const float4 s = shade_sample(nt, u, v, magnifies(nt));
      const float cf[3] = {s.x * 2.f - 1.f, s.y * 2.f - 1.f, s.z * 2.f - 1.f};
      nrm3(tan_);
      nrm3(bit_);
#pragma unroll
      for (int k = 0; k < 3; ++k) n[k] = cf[0] * tan_[k] + cf[1] * bit_[k] + cf[2] * nin[k];
      nrm3(n);
    } else {
      n[0] = nin[0]; n[1] = nin[1]; n[2] = nin[2];
      nrm3(n);
    }
    float vd[3] = {a.eye[0] - wp[0], a.eye[1] - wp[1], a.eye[2] - wp[2]};
    nrm3(vd);
    const float ndv = dot3(vd, n);
    const float flip = ndv < 0.f ? -1.f : 1.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) n[k] *= flip;
    float ld[3] = {a.light[0] - wp[0], a.light[1] - wp[1], a.light[2] - wp[2]};
    nrm3(ld);
    const float ndl = fmaxf(dot3(ld, n), 0.f);
#pragma unroll
    for (int k = 0; k < 3; ++k) lc[k] += m.diffuse[k] * 0.7f * ndl * m.diffuse[3];
    float hd[3] = {vd[0] + ld[0], vd[1] + ld[1], vd[2] + ld[2]};
    nrm3(hd);
    const float strength = powf(fmaxf(dot3(n, hd), 0.f), m.shininess);
    const float spec_on = ndv > 1e-6f ? 1.f : 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) lc[k] += m.specular[k] * strength * 1.f * m.specular[3] * spec_on;
    if (a.gi_scale > 0.f && a.fluence) {
      float fl[3];
      shade_fluence(a, wp, fl);
      const float s = a.gi_scale * 0.0795774715f;  // 1 / (4 pi)
#pragma unroll
      for (int k = 0; k < 3; ++k) lc[k] += s * fl[k];
    }
    const float pred = (m.ambient[0] - 1e-5f) + (m.diffuse[0] - 1e-5f) + (m.specular[0] - 1e-5f);
    const float pg = (m.ambient[1] - 1e-5f) + (m.diffuse[1] - 1e-5f) + (m.specular[1] - 1e-5f);
    const float pb = (m.ambient[2] - 1e-5f) + (m.diffuse[2] - 1e-5f) + (m.specular[2] - 1e-5f);
    const float none = (pred + pg + pb) <= 0.f ? 1.f : 0.f;
    outc = make_float4((lc[0] + none) * col[0], (lc[1] + none) * col[1], (lc[2] + none) * col[2], 1.f);
  }
  reinterpret_cast<float4*>(a.out)[i] = outc;
}

}  // namespace rcx
