"""Python host side of the radiance-cascade engine, above the C ABI.

`Engine` owns one rc_context (one scene on one GPU).  `GiStage` mirrors the
reference renderer's plugin interface RenderStage<T> (src/app.rs:3-7):
resize() rebuilds the size-dependent context, update() uploads per-frame
scene changes (the light upload it parallels is src/window/app.rs:124-131),
render() enqueues the cascade solve on a stream.  Errors raise RCError with
the library's status and message instead of panicking.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _ffi as F
from ._ffi import BOX_DT, SPHERE_DT, VOXEL_DT, RCError  # noqa: F401  (re-exported)


def make_params(grid, num_cascades: int, precision: str = "fp32", spacing0: int = 2, dir_res0: int = 4,
                interval0: int = 1, ratio: int = 4) -> F.Params:
    g = (grid,) * 3 if isinstance(grid, int) else tuple(grid)
    p = F.Params()
    F.check(F.lib().rc_params_default(C.byref(p), g[0], num_cascades))
    p.grid[:] = g
    p.probe_spacing0, p.dir_res0, p.interval0, p.interval_ratio = spacing0, dir_res0, interval0, ratio
    p.precision = {"fp32": F.RC_PRECISION_FP32, "fp16": F.RC_PRECISION_FP16}[precision]
    F.check(F.lib().rc_params_validate(C.byref(p)))
    return p


def level_info(p: F.Params, level: int) -> F.LevelInfo:
    info = F.LevelInfo()
    F.check(F.lib().rc_level_info_get(C.byref(p), level, C.byref(info)))
    return info


def scene_spec(grid, num_boxes, edge, num_spheres, radius, emission, albedo=(0.2, 0.9),
               speed=0.5) -> F.SceneSpec:
    s = F.SceneSpec()
    s.grid[:] = (grid,) * 3 if isinstance(grid, int) else tuple(grid)
    s.num_boxes, s.box_edge_min, s.box_edge_max = num_boxes, edge[0], edge[1]
    s.num_spheres = num_spheres
    s.albedo_min, s.albedo_max = albedo
    s.radius_min, s.radius_max = radius
    s.emission_min, s.emission_max = emission
    s.speed = speed
    return s


def generate_scene(spec: F.SceneSpec, seed: int):
    boxes = np.zeros(spec.num_boxes, BOX_DT)
    spheres = np.zeros(spec.num_spheres, SPHERE_DT)
    F.check(F.lib().rc_scene_generate(C.byref(spec), seed, F.ptr(boxes), F.ptr(spheres)))
    return boxes, spheres


def advance_spheres(spheres: np.ndarray, grid, frames: int = 1) -> None:
    g = (C.c_int32 * 3)(*((grid,) * 3 if isinstance(grid, int) else grid))
    F.check(F.lib().rc_spheres_advance(F.ptr(spheres), len(spheres), g, frames))


def voxelise_host(grid, boxes: np.ndarray, spheres: np.ndarray) -> np.ndarray:
    g3 = (grid,) * 3 if isinstance(grid, int) else tuple(grid)
    out = np.zeros(g3[0] * g3[1] * g3[2], VOXEL_DT)
    g = (C.c_int32 * 3)(*g3)
    F.check(F.lib().rc_voxelise_host(g, F.ptr(boxes), len(boxes), F.ptr(spheres), len(spheres), F.ptr(out)))
    return out


def directions(n: int) -> np.ndarray:
    out = np.zeros((n * n, 3), np.int32)
    F.check(F.lib().rc_directions(n, F.ptr(out)))
    return out


def solid_angles(n: int) -> np.ndarray:
    out = np.zeros(n * n, np.float64)
    F.check(F.lib().rc_solid_angles(n, F.ptr(out)))
    return out


# Benchmark workloads: seeded synthetic scenes.
#   c64:  64^3 voxels, 24 boxes (edges 4..20, albedo 0.2..0.9), 4 emissive spheres
#         (radius 2..5, emission 1..20), 5 cascades, seed 1001
#   c256: 256^3 voxels, 400 boxes (edges 4..48), 32 spheres (radius 2..8,
#         emission 1..50), 6 cascades, seed 1002, spheres moving 0.5 voxel/frame
WORKLOADS = {
    "c64": dict(grid=64, cascades=5, boxes=24, edge=(4, 20), spheres=4, radius=(2.0, 5.0),
                emission=(1.0, 20.0), seed=1001),
    "c256": dict(grid=256, cascades=6, boxes=400, edge=(4, 48), spheres=32, radius=(2.0, 8.0),
                 emission=(1.0, 50.0), seed=1002),
}


# ---- triangle meshes ----------------------------------------------------------
def load_obj(path: str) -> dict:
    """Wavefront OBJ (+ its MTL library) as the reference renderer loads it
    (src/primitives.rs:104-175 through tobj with triangulate + single_index):
    polygons fan-triangulated, triangle winding reversed (src/primitives.rs:
    369-376), per-triangle material, and the light position -- the centroid of
    the positions of the first object whose material is named "Light"
    (src/renderer.rs:176, src/primitives.rs:133-155), or None.
    -> dict(positions [n,3] f32, indices [m,3] u32, tri_material [m] u16,
            materials [{name, Ka, Kd, Ks, Ke, Ns}], light)"""
    base = os.path.dirname(path)
    verts, tris, tri_mat, objects = [], [], [], []
    mat_index, materials = {}, []
    cur_mat = -1

    def material_id(name):
        if name not in mat_index:
            mat_index[name] = len(materials)
            materials.append({"name": name, "Ka": None, "Kd": None, "Ks": None, "Ke": None, "Ns": None})
        return mat_index[name]

    def load_mtl(fn):
        cur = None
        try:
            with open(os.path.join(base, fn), errors="replace") as f:
                for line in f:
                    t = line.split()
                    if not t:
                        continue
                    if t[0] == "newmtl":
                        cur = materials[material_id(" ".join(t[1:]))]
                    elif cur is not None and t[0] in ("Ka", "Kd", "Ks", "Ke") and len(t) >= 4:
                        cur[t[0]] = [float(x) for x in t[1:4]]
                    elif cur is not None and t[0] == "Ns":
                        cur["Ns"] = float(t[1])
        except OSError:
            pass

    obj_start = 0
    with open(path, errors="replace") as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                verts.append([float(x) for x in t[1:4]])
            elif t[0] == "mtllib":
                load_mtl(" ".join(t[1:]))
            elif t[0] == "usemtl":
                cur_mat = material_id(" ".join(t[1:]))
            elif t[0] in ("o", "g"):
                objects.append((obj_start, len(tris)))
                obj_start = len(tris)
            elif t[0] == "f":
                ids = []
                for v in t[1:]:
                    k = int(v.split("/")[0])
                    ids.append(k - 1 if k > 0 else len(verts) + k)
                for i in range(1, len(ids) - 1):
                    tris.append([ids[i + 1], ids[i], ids[0]])  # fan, winding reversed
                    tri_mat.append(max(cur_mat, 0))
    objects.append((obj_start, len(tris)))
    positions = np.asarray(verts, np.float32).reshape(-1, 3)
    indices = np.asarray(tris, np.uint32).reshape(-1, 3)
    tri_material = np.asarray(tri_mat, np.uint16)
    light = None
    for a, b in objects:
        if b > a and materials and materials[tri_material[a]]["name"] == "Light":
            used = np.unique(indices[a:b])
            light = positions[used].mean(0)
            break
    if not materials:
        materials.append({"name": "default", "Ka": None, "Kd": None, "Ks": None, "Ke": None, "Ns": None})
    return dict(positions=positions, indices=indices, tri_material=tri_material, materials=materials, light=light)


def mesh_to_grid(positions: np.ndarray, grid, margin: float = 1.0) -> np.ndarray:
    """Uniform scale + offset placing the mesh's bounding box inside the grid."""
    g = np.asarray((grid,) * 3 if isinstance(grid, int) else grid, np.float64)
    p = np.asarray(positions, np.float64)
    lo, hi = p.min(0), p.max(0)
    scale = float(np.min((g - 2 * margin) / np.maximum(hi - lo, 1e-12)))
    return ((p - (lo + hi) / 2) * scale + g / 2).astype(np.float32)


def mesh_materials(materials, emission_scale: float = 1.0, light_emission=(10.0, 10.0, 10.0)) -> np.ndarray:
    """rc_voxel per material: albedo from Kd, emission from Ke (times
    emission_scale), and `light_emission` for a material named "Light"."""
    out = np.zeros(len(materials), VOXEL_DT)
    for i, m in enumerate(materials):
        kd = m["Kd"] if m["Kd"] is not None else [0.8, 0.8, 0.8]
        ke = m["Ke"] if m["Ke"] is not None else [0.0, 0.0, 0.0]
        if m["name"] == "Light":
            ke = list(light_emission)
            emission_scale_i = 1.0
        else:
            emission_scale_i = emission_scale
        a = [min(31, max(0, int(round(float(c) * 31)))) for c in kd]
        out[i]["albedo_occ"] = 0x8000 | (a[0] << 10) | (a[1] << 5) | a[2]
        out[i]["emission"] = [int(np.float16(float(c) * emission_scale_i).view(np.uint16)) for c in ke]
    return out


def room_mesh(grid: int, boxes: int = 6, seed: int = 7):
    """Procedural test mesh in grid units: a closed room (6 walls, inward),
    axis-aligned blocks and a tessellated sphere (material 2, emissive),
    -> positions, indices, tri_material, materials (3 rc_voxels)."""
    rng = np.random.default_rng(seed)
    P, I, M = [], [], []

    def quad(a, b, c, d, m):
        k = sum(len(x) for x in P)
        P.append(np.array([a, b, c, d], np.float32))
        I.extend([[k, k + 1, k + 2], [k, k + 2, k + 3]])
        M.extend([m, m])

    def block(lo, hi, m):
        x0, y0, z0 = lo
        x1, y1, z1 = hi
        quad((x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0), m)
        quad((x0, y0, z1), (x0, y1, z1), (x1, y1, z1), (x1, y0, z1), m)
        quad((x0, y0, z0), (x0, y1, z0), (x0, y1, z1), (x0, y0, z1), m)
        quad((x1, y0, z0), (x1, y0, z1), (x1, y1, z1), (x1, y1, z0), m)
        quad((x0, y0, z0), (x0, y0, z1), (x1, y0, z1), (x1, y0, z0), m)
        quad((x0, y1, z0), (x1, y1, z0), (x1, y1, z1), (x0, y1, z1), m)

    e = grid - 0.5
    block((0.5, 0.5, 0.5), (e, e, e), 0)
    for _ in range(boxes):
        lo = rng.uniform(2, grid - 10, 3)
        block(tuple(lo), tuple(lo + rng.uniform(2, grid / 4, 3)), 1)
    # UV sphere
    c = rng.uniform(grid * 0.3, grid * 0.7, 3)
    r = grid * 0.08
    nu, nv = 16, 8
    k0 = sum(len(x) for x in P)
    sp = []
    for j in range(nv + 1):
        th = np.pi * j / nv
        for i in range(nu):
            ph = 2 * np.pi * i / nu
            sp.append(c + r * np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)]))
    P.append(np.asarray(sp, np.float32))
    for j in range(nv):
        for i in range(nu):
            a, b = k0 + j * nu + i, k0 + j * nu + (i + 1) % nu
            I.extend([[a, b + nu, b], [a, a + nu, b + nu]])
            M.extend([2, 2])
    mats = np.zeros(3, VOXEL_DT)
    mats["albedo_occ"] = [0x8000 | (20 << 10) | (20 << 5) | 20, 0x8000 | (25 << 10) | (12 << 5) | 8,
                          0x8000 | (31 << 10) | (31 << 5) | 31]
    mats[2]["emission"] = [int(np.float16(v).view(np.uint16)) for v in (12.0, 9.0, 4.0)]
    return (np.concatenate(P).astype(np.float32), np.asarray(I, np.uint32), np.asarray(M, np.uint16), mats)


# ---- shading pass helpers ----------------------------------------------------
def perspective_rh(fovy_rad: float, aspect: float, znear: float, zfar: float) -> np.ndarray:
    """Right-handed perspective with depth in [0, 1] (the reference's
    Projection::calc_matrix, src/camera.rs:77-79), column-major 4x4."""
    h = np.cos(0.5 * fovy_rad) / np.sin(0.5 * fovy_rad)
    w = h / aspect
    r = zfar / (znear - zfar)
    m = np.zeros((4, 4))  # m[col][row]
    m[0, 0], m[1, 1], m[2, 2], m[2, 3], m[3, 2] = w, h, r, -1.0, r * znear
    return m


def look_to_rh(eye, direction, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """Right-handed view matrix looking along `direction`, column-major 4x4."""
    f = np.asarray(direction, np.float64)
    f = f / np.linalg.norm(f)
    s = np.cross(f, up)
    s = s / np.linalg.norm(s)
    u = np.cross(s, f)
    e = np.asarray(eye, np.float64)
    m = np.zeros((4, 4))
    m[0] = (s[0], u[0], -f[0], 0.0)
    m[1] = (s[1], u[1], -f[1], 0.0)
    m[2] = (s[2], u[2], -f[2], 0.0)
    m[3] = (-e.dot(s), -e.dot(u), e.dot(f), 1.0)
    return m


def camera_view_proj(eye, yaw: float, pitch: float, width: int, height: int, fovy_deg: float = 45.0,
                     znear: float = 0.1, zfar: float = 100.0) -> np.ndarray:
    """projection * view as the reference's camera builds it (src/camera.rs:20,
    43-52: direction (cos pitch cos yaw, sin pitch, cos pitch sin yaw), up +Y);
    -> 16 floats, column-major."""
    d = (np.cos(pitch) * np.cos(yaw), np.sin(pitch), np.cos(pitch) * np.sin(yaw))
    p = perspective_rh(np.radians(fovy_deg), width / height, znear, zfar)
    v = look_to_rh(eye, d)
    # column-major product: (P V)[col] = P applied to V's columns
    pv = (p.T @ v.T).T
    return pv.astype(np.float32).reshape(-1)


def mesh_tbn(positions: np.ndarray, indices: np.ndarray, texcoords: Optional[np.ndarray]):
    """Per-vertex tangent, bitangent and normal as the reference derives them
    (src/primitives.rs:245-354): per triangle, the UV deltas scaled by 2^11,
    T and B from the inverse of [duv1 duv2], N = B x T; accumulated over the
    triangles without NaN, averaged and normalised (X, Y, Z where none)."""
    p = np.asarray(positions, np.float32)
    n = len(p)
    uv = np.zeros((n, 2), np.float32) if texcoords is None or len(texcoords) != n else np.asarray(texcoords, np.float32)
    T = np.zeros((n, 3), np.float32)
    B = np.zeros((n, 3), np.float32)
    N = np.zeros((n, 3), np.float32)
    cnt = np.zeros(n, np.int64)
    with np.errstate(all="ignore"):
        for c in np.asarray(indices, np.int64).reshape(-1, 3):
            dp1, dp2 = p[c[1]] - p[c[0]], p[c[2]] - p[c[0]]
            d1 = (uv[c[1]] - uv[c[0]]) * np.float32(2.0 ** 11)
            d2 = (uv[c[2]] - uv[c[0]]) * np.float32(2.0 ** 11)
            det = np.float32(d1[0] * d2[1] - d2[0] * d1[1])
            inv_det = np.float32(1.0) / det
            col0 = np.array([d2[1], -d1[1]], np.float32) * inv_det
            col1 = np.array([-d2[0], d1[0]], np.float32) * inv_det
            t = col0[0] * dp1 - col0[1] * dp2
            b = -col1[0] * dp1 + col1[1] * dp2
            nn = np.cross(b, t)
            nn = nn / np.linalg.norm(nn)
            if np.isnan(t).any() or np.isnan(b).any() or np.isnan(nn).any():
                continue
            for k in c:
                T[k] += t
                B[k] += b
                N[k] += nn
                cnt[k] += 1
    out = []
    for acc, dflt in ((T, (1, 0, 0)), (B, (0, 1, 0)), (N, (0, 0, 1))):
        r = np.tile(np.asarray(dflt, np.float32), (n, 1))
        m = cnt > 0
        with np.errstate(all="ignore"):
            v = acc[m] / cnt[m, None]
            r[m] = v / np.linalg.norm(v, axis=1, keepdims=True)
        out.append(r)
    return out


def shade_vertices(positions, indices, colors=None, normals=None, texcoords=None) -> np.ndarray:
    """The 17-float vertex records the reference builds (src/renderer.rs:
    370-410): position, colour (default 1), normal (the mesh's, else the TBN
    normal), tangent, bitangent, uv (default 0)."""
    p = np.asarray(positions, np.float32)
    n = len(p)
    t, b, tn = mesh_tbn(p, indices, texcoords)
    v = np.zeros((n, 17), np.float32)
    v[:, 0:3] = p
    v[:, 3:6] = 1.0 if colors is None else colors
    v[:, 6:9] = tn if normals is None else normals
    v[:, 9:12] = t
    v[:, 12:15] = b
    if texcoords is not None and len(texcoords) == n:
        v[:, 15:17] = texcoords
    return v


def shade_material(ambient=None, diffuse=None, specular=None, shininess=None, color_texture=-1,
                   normal_texture=-1) -> F.ShadeMaterial:
    """UniformMaterial (src/primitives.rs:39-73): an absent component is (0, 0, 0, 0),
    a present one (rgb, 1); shininess defaults to 1."""
    m = F.ShadeMaterial()
    for name, v in (("ambient", ambient), ("diffuse", diffuse), ("specular", specular)):
        getattr(m, name)[:] = (0.0, 0.0, 0.0, 0.0) if v is None else (v[0], v[1], v[2], 1.0)
    m.shininess = 1.0 if shininess is None else shininess
    m.enable_bit = (1 if color_texture >= 0 else 0) | (2 if normal_texture >= 0 else 0)
    m.color_texture = max(color_texture, 0)
    m.normal_texture = max(normal_texture, 0)
    return m


# Batched workload: `count` cubic scenes, scene k seeded 2000 + k, edge drawn
# uniformly from BATCH_EDGES by splitmix64(seed); the 64^3 workload's box and
# sphere density per voxel (24 boxes and 4 spheres per 64^3, edges 4..20,
# radius 2..5, emission 1..20, at least one of each); cascade count by edge.
BATCH_EDGES = (32, 48, 64, 96, 128, 192)
BATCH_CASCADES = {32: 4, 48: 4, 64: 5, 96: 5, 128: 6, 192: 6}


def _splitmix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return x ^ (x >> 31)


def batch_workload(count: int = 64, base_seed: int = 2000):
    """-> [(edge, cascades, boxes, spheres)] for the batched workload."""
    out = []
    for k in range(count):
        seed = base_seed + k
        edge = BATCH_EDGES[_splitmix64(seed) % len(BATCH_EDGES)]
        scale = (edge / 64.0) ** 3
        nb, ns = max(1, round(24 * scale)), max(1, round(4 * scale))
        spec = scene_spec(edge, nb, (4, 20), ns, (2.0, 5.0), (1.0, 20.0))
        boxes, spheres = generate_scene(spec, seed)
        out.append((edge, BATCH_CASCADES[edge], boxes, spheres))
    return out


def workload_scene(name: str, frame: int = 0):
    w = WORKLOADS[name]
    spec = scene_spec(w["grid"], w["boxes"], w["edge"], w["spheres"], w["radius"], w["emission"])
    boxes, spheres = generate_scene(spec, w["seed"])
    if frame:
        advance_spheres(spheres, w["grid"], frame)
    return boxes, spheres


class Engine:
    """One radiance-cascade context: a scene volume and its cascades on one GPU."""

    def __init__(self, params: F.Params, device: int = 0):
        self._lib = F.lib()
        self.params = params
        h = C.c_void_p()
        F.check(self._lib.rc_create(C.byref(params), device, C.byref(h)))
        self._h = h
        self.levels = [level_info(params, i) for i in range(params.num_cascades)]
        self.probes0 = tuple(self.levels[0].probes)

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise RCError(F.RC_ERR_STATE, "engine is closed")
        return self._h

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self._lib.rc_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- scene -------------------------------------------------------
    def upload(self, voxels: np.ndarray) -> None:
        v = np.ascontiguousarray(voxels, dtype=VOXEL_DT).reshape(-1)
        F.check(self._lib.rc_scene_upload(self.handle, F.ptr(v), v.size, F.RC_MEM_HOST))

    def upload_device(self, dev_ptr: int, count: int) -> None:
        F.check(self._lib.rc_scene_upload(self.handle, C.c_void_p(dev_ptr), count, F.RC_MEM_DEVICE))

    def set_boxes(self, boxes: np.ndarray) -> None:
        b = np.ascontiguousarray(boxes, dtype=BOX_DT)
        F.check(self._lib.rc_scene_set_boxes(self.handle, F.ptr(b), len(b)))

    def set_mesh(self, positions: np.ndarray, indices: np.ndarray, materials: np.ndarray,
                 tri_material: Optional[np.ndarray] = None) -> None:
        """Voxelise a triangle mesh (positions in grid units) as the static scene."""
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
        mats = np.ascontiguousarray(materials, VOXEL_DT).reshape(-1)
        tm = None if tri_material is None else np.ascontiguousarray(tri_material, np.uint16)
        F.check(self._lib.rc_scene_set_mesh(self.handle, F.ptr(pos), len(pos), F.ptr(idx), len(idx),
                                            None if tm is None else F.ptr(tm), F.ptr(mats), len(mats)))

    def set_spheres(self, spheres: np.ndarray) -> None:
        s = np.ascontiguousarray(spheres, dtype=SPHERE_DT)
        F.check(self._lib.rc_scene_set_spheres(self.handle, F.ptr(s), len(s)))

    # ---- solve -------------------------------------------------------
    def solve(self, stream: Optional[int] = None) -> None:
        F.check(self._lib.rc_solve(self.handle, C.c_void_p(stream) if stream else None))

    def synchronize(self) -> None:
        F.check(self._lib.rc_synchronize(self.handle))

    # ---- results -----------------------------------------------------
    def fluence(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        n = 3 * int(np.prod(self.probes0))
        if out is None:
            out = np.empty(n, np.float32)
        F.check(self._lib.rc_get_fluence(self.handle, F.ptr(out), n, F.RC_MEM_HOST))
        return out.reshape(-1, 3)

    @staticmethod
    def _shade_mesh_args(vertices, indices, materials, tri_material, textures):
        v = np.ascontiguousarray(vertices, np.float32)
        i = np.ascontiguousarray(indices, np.uint32)
        tm = None if tri_material is None else np.ascontiguousarray(tri_material, np.uint16)
        mats = (F.ShadeMaterial * len(materials))(*materials)
        keep = [np.ascontiguousarray(t["rgba"], np.uint8) for t in textures]
        tex = (F.Texture * max(len(textures), 1))()
        for k, t in enumerate(textures):
            tex[k].rgba = keep[k].ctypes.data
            tex[k].width, tex[k].height, tex[k].srgb = keep[k].shape[1], keep[k].shape[0], int(t.get("srgb", 1))
        return (F.ptr(v), len(v), F.ptr(i), len(i), None if tm is None else F.ptr(tm), mats, len(materials), tex,
                len(textures)), (v, i, tm, keep)

    def shade(self, view: F.ShadeView, vertices: np.ndarray, indices: np.ndarray, materials,
              tri_material: Optional[np.ndarray] = None, textures=()) -> np.ndarray:
        """Raster + shade into an (H, W, 4) float32 image (see rc_shade)."""
        args, _keep = self._shade_mesh_args(vertices, indices, materials, tri_material, textures)
        out = np.zeros((view.height, view.width, 4), np.float32)
        F.check(self._lib.rc_shade(self.handle, C.byref(view), *args, F.ptr(out), F.RC_MEM_HOST))
        return out

    def shade_set_mesh(self, vertices: np.ndarray, indices: np.ndarray, materials,
                       tri_material: Optional[np.ndarray] = None, textures=()) -> None:
        """Uploads the mesh that shade_draw renders (rc_shade_set_mesh)."""
        args, _keep = self._shade_mesh_args(vertices, indices, materials, tri_material, textures)
        F.check(self._lib.rc_shade_set_mesh(self.handle, *args))

    def shade_draw(self, view: F.ShadeView, out=None):
        """Shades one view of the uploaded mesh (rc_shade_draw).  `out`: None
        (a new host array), a C-contiguous (H, W, 4) float32 host array, or a
        CUDA tensor of that shape (the draw is then only queued on the
        context's stream)."""
        if out is None:
            out = np.zeros((view.height, view.width, 4), np.float32)
        if isinstance(out, np.ndarray):
            if out.dtype != np.float32 or out.shape != (view.height, view.width, 4) or not out.flags.c_contiguous:
                raise ValueError("shade_draw: out must be a C-contiguous (H, W, 4) float32 array")
            F.check(self._lib.rc_shade_draw(self.handle, C.byref(view), F.ptr(out), F.RC_MEM_HOST))
            return out
        if tuple(out.shape) != (view.height, view.width, 4) or not out.is_cuda or not out.is_contiguous() \
                or str(out.dtype) != "torch.float32":
            raise ValueError("shade_draw: out must be a contiguous (H, W, 4) float32 CUDA tensor")
        F.check(self._lib.rc_shade_draw(self.handle, C.byref(view), C.c_void_p(out.data_ptr()), F.RC_MEM_DEVICE))
        return out

    def volume(self) -> np.ndarray:
        """The composed scene volume (rc_voxel per voxel, x fastest)."""
        g = self.params.grid
        out = np.zeros(g[0] * g[1] * g[2], VOXEL_DT)
        F.check(self._lib.rc_get_volume(self.handle, F.ptr(out), out.size, F.RC_MEM_HOST))
        return out

    def fluence_async(self, out: np.ndarray) -> None:
        """Starts the read-back of the last solve's fluence into `out` (float32,
        3 x probes; pinned memory overlaps the next solve); complete after
        synchronize()."""
        if out.dtype != np.float32 or not out.flags.c_contiguous or out.size != 3 * int(np.prod(self.probes0)):
            raise ValueError("out must be a contiguous float32 array of 3 x cascade-0 probes")
        F.check(self._lib.rc_get_fluence_async(self.handle, F.ptr(out), out.size))

    def radiance(self, level: int) -> np.ndarray:
        info = self.levels[level]
        dt = np.float16 if self.params.precision == F.RC_PRECISION_FP16 else np.float32
        out = np.empty(info.radiance_elems, dt)
        F.check(self._lib.rc_get_radiance(self.handle, level, F.ptr(out), info.radiance_bytes, F.RC_MEM_HOST))
        px, py, pz = info.probes
        return out.reshape(3, info.num_dirs, pz, py, px)

    def fluence_device_ptr(self) -> int:
        p = C.c_void_p()
        F.check(self._lib.rc_fluence_device_ptr(self.handle, C.byref(p)))
        return p.value

    def stream(self) -> int:
        p = C.c_void_p()
        F.check(self._lib.rc_get_stream(self.handle, C.byref(p)))
        return p.value or 0

    def profile_levels(self, iters: int = 5, whole: bool = False) -> np.ndarray:
        """Mean ms per launch: [compose, level 0, level 1, ...] (CUDA events);
        with whole=True one more entry: the frame's level set timed without
        events between its kernels (they overlap as in a solve)."""
        out = np.zeros(1 + self.params.num_cascades + (1 if whole else 0), np.float32)
        F.check(self._lib.rc_profile_levels(self.handle, iters, F.ptr(out), out.size))
        return out

    def set_stage_timing(self, enable: bool = True) -> None:
        """CUDA events between the stages of every solve (no host wait)."""
        F.check(self._lib.rc_set_stage_timing(self.handle, 1 if enable else 0))

    def stage_ms(self) -> np.ndarray:
        """[whole solve, cascade 0, cascade 1, ...] ms of the last solve (waits for it)."""
        out = np.zeros(1 + self.params.num_cascades, np.float32)
        F.check(self._lib.rc_get_stage_ms(self.handle, F.ptr(out), out.size))
        return out

    def radiance_device_ptr(self, level: int) -> int:
        p = C.c_void_p()
        F.check(self._lib.rc_radiance_device_ptr(self.handle, level, C.byref(p)))
        return p.value

    # ---- neural radiance cache ----------------------------------------
    @staticmethod
    def nrc_params(**kw) -> F.NrcParams:
        p = F.NrcParams()
        F.check(F.lib().rc_nrc_params_default(C.byref(p)))
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def nrc_enable(self, params: Optional[F.NrcParams] = None, **kw) -> None:
        p = params if params is not None else self.nrc_params(**kw)
        F.check(self._lib.rc_nrc_enable(self.handle, C.byref(p)))
        self._nrc_on = True

    def nrc_disable(self) -> None:
        F.check(self._lib.rc_nrc_disable(self.handle))
        self._nrc_on = False

    @property
    def nrc_on(self) -> bool:
        """Whether the radiance cache serves the far cascades."""
        return getattr(self, "_nrc_on", False)

    def nrc_stats(self) -> dict:
        st = F.NrcStats()
        F.check(self._lib.rc_nrc_get_stats(self.handle, C.byref(st)))
        out = {k: getattr(st, k) for k, _ in st._fields_ if k != "pad"}
        out["served_solves"] = list(st.served_solves)
        return out

    def nrc_save(self) -> bytes:
        need = C.c_int64()
        F.check(self._lib.rc_nrc_save(self.handle, None, 0, C.byref(need)))
        buf = (C.c_char * need.value)()
        F.check(self._lib.rc_nrc_save(self.handle, buf, need.value, C.byref(need)))
        return bytes(buf)

    def nrc_load(self, blob: bytes) -> None:
        buf = (C.c_char * len(blob)).from_buffer_copy(blob)
        F.check(self._lib.rc_nrc_load(self.handle, buf, len(blob)))

    def nrc_query(self, level: int, probes, dirs) -> np.ndarray:
        pr = np.ascontiguousarray(probes, np.int32)
        di = np.ascontiguousarray(dirs, np.int32)
        out = np.zeros((len(pr), 4), np.float32)
        F.check(self._lib.rc_nrc_query(self.handle, level, F.ptr(pr), F.ptr(di), len(pr), F.ptr(out)))
        return out

    def nrc_tile_gradient(self, level: int, probe: int, d0: int, targets: np.ndarray):
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 4)
        pg = np.zeros(F.lib().rc_nrc_param_count(), np.float32)
        eg = np.zeros(32, np.float32)
        F.check(self._lib.rc_nrc_tile_gradient(self.handle, level, probe, d0, len(t), F.ptr(t), F.ptr(pg), F.ptr(eg)))
        return pg, eg


class Batch:
    """Many independent scenes solved by one persistent launch (a CUDA graph).

    Each scene has its own ``rc_params`` (grid, cascade count); all share one
    precision.  ``solve()`` is asynchronous; the results calls synchronise.
    """

    def __init__(self, params_list, device: int = 0):
        self._lib = F.lib()
        arr = (F.Params * len(params_list))(*params_list)
        self.params = list(params_list)
        h = C.c_void_p()
        F.check(self._lib.rc_batch_create(arr, len(params_list), device, C.byref(h)))
        self._h = h

    @property
    def handle(self) -> C.c_void_p:
        if self._h is None:
            raise RCError(F.RC_ERR_STATE, "batch is closed")
        return self._h

    def __len__(self) -> int:
        return len(self.params)

    def close(self) -> None:
        if getattr(self, "_h", None) is not None:
            self._lib.rc_batch_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_scene(self, k: int, boxes: np.ndarray, spheres: np.ndarray) -> None:
        b = np.ascontiguousarray(boxes, dtype=BOX_DT)
        s = np.ascontiguousarray(spheres, dtype=SPHERE_DT)
        F.check(self._lib.rc_batch_scene_set(self.handle, k, F.ptr(b), len(b), F.ptr(s), len(s)))

    def set_spheres(self, k: int, spheres: np.ndarray) -> None:
        """Scene k's emitters for the next solve (asynchronous, incremental)."""
        s = np.ascontiguousarray(spheres, dtype=SPHERE_DT)
        F.check(self._lib.rc_batch_set_spheres(self.handle, k, F.ptr(s), len(s)))

    def fluence_elems(self) -> int:
        return sum(3 * int(np.prod(level_info(p, 0).probes)) for p in self.params)

    def fluence_all(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Every scene's fluence, scene after scene, flat float32 (one synchronisation);
        `out` may be a preallocated (pinned) array of fluence_elems() floats."""
        n = self.fluence_elems()
        if out is None:
            out = np.empty(n, np.float32)
        F.check(self._lib.rc_batch_get_fluence_all(self.handle, F.ptr(out), n, F.RC_MEM_HOST))
        return out

    def fluence_all_async(self, out: np.ndarray) -> None:
        """Starts reading every scene's fluence into `out` (a pinned array of
        fluence_elems() floats) after the solves enqueued so far; complete
        after synchronize()."""
        F.check(self._lib.rc_batch_get_fluence_all_async(self.handle, F.ptr(out), out.size))

    def solve(self, stream: Optional[int] = None) -> None:
        F.check(self._lib.rc_batch_solve(self.handle, C.c_void_p(stream) if stream else None))

    def synchronize(self) -> None:
        F.check(self._lib.rc_batch_synchronize(self.handle))

    def fluence(self, k: int) -> np.ndarray:
        probes0 = level_info(self.params[k], 0).probes
        n = 3 * int(np.prod(probes0))
        out = np.empty(n, np.float32)
        F.check(self._lib.rc_batch_get_fluence(self.handle, k, F.ptr(out), n, F.RC_MEM_HOST))
        return out.reshape(-1, 3)

    def radiance(self, k: int, level: int) -> np.ndarray:
        info = level_info(self.params[k], level)
        dt = np.float16 if self.params[k].precision == F.RC_PRECISION_FP16 else np.float32
        out = np.empty(info.radiance_elems, dt)
        F.check(self._lib.rc_batch_get_radiance(self.handle, k, level, F.ptr(out), info.radiance_bytes,
                                                F.RC_MEM_HOST))
        px, py, pz = info.probes
        return out.reshape(3, info.num_dirs, pz, py, px)

    def set_tiles(self, probes_per_item: int, dirs_per_item: int, blocks_per_item: int = 1,
                  walks_per_item: int = 1024) -> None:
        t = F.BatchTiles(probes_per_item, dirs_per_item, blocks_per_item, walks_per_item)
        F.check(self._lib.rc_batch_set_tiles(self.handle, C.byref(t)))

    def tiles(self) -> dict:
        t = F.BatchTiles()
        F.check(self._lib.rc_batch_get_tiles(self.handle, C.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    def form(self) -> str:
        """"scenes" (every scene's own launches as parallel graph branches) or
        "persistent" (one persistent kernel over a queue of tiles)."""
        v = C.c_int32()
        F.check(self._lib.rc_batch_get_form(self.handle, C.byref(v)))
        return "scenes" if v.value else "persistent"

    def tune(self, iters: int = 3):
        """Autotunes the tile shape; -> (tiles dict, ms per solve of the best)."""
        t, ms = F.BatchTiles(), C.c_float()
        F.check(self._lib.rc_batch_tune(self.handle, iters, C.byref(t), C.byref(ms)))
        return {k: getattr(t, k) for k, _ in t._fields_}, ms.value


@dataclass
class GiState:
    """Per-frame state a GI stage reads in update(): the emitters."""
    spheres: np.ndarray = field(default_factory=lambda: np.zeros(0, SPHERE_DT))
    frame: int = 0


class GiStage:
    """RenderStage<GiState> analogue (reference: src/app.rs:3-7).

    resize(params)  -- (re)create the context for a new grid / cascade shape
    update(state)   -- upload the frame's emitters (only what changed is rewritten)
    render(stream)  -- enqueue every cascade and the fluence on `stream`
    """

    def __init__(self, params: F.Params, boxes: Optional[np.ndarray] = None,
                 voxels: Optional[np.ndarray] = None, device: int = 0):
        self.device = device
        self._boxes, self._voxels = boxes, voxels
        self.engine: Optional[Engine] = None
        self.resize(params)

    def resize(self, params: F.Params) -> None:
        if self.engine is not None:
            self.engine.close()
        self.engine = Engine(params, self.device)
        if self._voxels is not None:
            self.engine.upload(self._voxels)
        else:
            self.engine.set_boxes(self._boxes if self._boxes is not None else np.zeros(0, BOX_DT))

    def update(self, state: GiState) -> None:
        self.engine.set_spheres(state.spheres)

    def render(self, stream: Optional[int] = None) -> None:
        self.engine.solve(stream)

    def fluence(self) -> np.ndarray:
        return self.engine.fluence()

    def close(self) -> None:
        if self.engine is not None:
            self.engine.close()
            self.engine = None


def frames(stage: GiStage, spheres: np.ndarray, grid, count: int, start: int = 0):
    """Drive `count` frames of moving emitters through a stage (generator of frame indices)."""
    sph = spheres.copy()
    if start:
        advance_spheres(sph, grid, start)
    for f in range(start, start + count):
        stage.update(GiState(spheres=sph, frame=f))
        stage.render()
        yield f
        advance_spheres(sph, grid, 1)


__all__ = ["Engine", "GiStage", "GiState", "make_params", "level_info", "scene_spec", "generate_scene",
           "advance_spheres", "voxelise_host", "directions", "solid_angles", "WORKLOADS", "workload_scene",
           "frames", "RCError", "VOXEL_DT", "BOX_DT", "SPHERE_DT"]


class FrameLog:
    """Per-frame metrics as JSON lines: frame, ms of the whole solve and of each
    cascade (the engine's stage timing), algorithmic GB/s of the solve, the
    radiance cache's loss and fallback-tile fraction when it is on, and any
    extra fields the caller adds (e.g. the fluence error against an oracle).

        log = FrameLog("frames.jsonl", engine, algorithmic_bytes=B)
        for f in range(n):
            engine.set_spheres(spheres); engine.solve()
            log.write(f, fluence_rel_l2=...)
    """

    def __init__(self, path_or_file, engine: "Engine", algorithmic_bytes: Optional[float] = None):
        import json  # noqa: F401  (used in write)
        self._own = isinstance(path_or_file, (str, os.PathLike))
        self._f = open(path_or_file, "w") if self._own else path_or_file
        self._eng = engine
        self._bytes = algorithmic_bytes
        engine.set_stage_timing(True)

    def record(self, frame: int, **extra) -> dict:
        ms = self._eng.stage_ms()
        rec = {"frame": int(frame), "solve_ms": round(float(ms[0]), 5),
               "cascade_ms": [round(float(x), 5) for x in ms[1:]]}
        if self._bytes:
            rec["algorithmic_gb_per_s"] = round(self._bytes / (float(ms[0]) / 1000.0) / 1e9, 2)
        if self._eng.nrc_on:
            st = self._eng.nrc_stats()
            rec["nrc_loss"] = float(st["last_loss"])
            rec["nrc_fallback_fraction"] = float(st["fallback_tiles"]) / max(1, int(st["tiles"]))
            rec["nrc_served_levels"] = int(st["served_levels"])
        rec.update(extra)
        return rec

    def write(self, frame: int, **extra) -> dict:
        import json
        rec = self.record(frame, **extra)
        self._f.write(json.dumps(rec) + "\n")
        self._f.flush()
        return rec

    def close(self) -> None:
        self._eng.set_stage_timing(False)
        if self._own:
            self._f.close()
