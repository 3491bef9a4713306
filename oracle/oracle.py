"""ctypes front end of the C++ oracle (oracle/rc_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by
bench.py's CPU baseline.  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None

VOXEL_DT = np.dtype([("emission", "<u2", (3,)), ("albedo_occ", "<u2")])
BOX_DT = np.dtype([("lo", "<i4", (3,)), ("hi", "<i4", (3,)), ("value", VOXEL_DT)])
SPHERE_DT = np.dtype([("centre", "<f8", (3,)), ("radius", "<f8"), ("velocity", "<f8", (3,)),
                      ("value", VOXEL_DT), ("pad", "<u4", (2,))])
assert VOXEL_DT.itemsize == 8 and BOX_DT.itemsize == 32 and SPHERE_DT.itemsize == 72


class Params(C.Structure):
    _fields_ = [("grid", C.c_int32 * 3), ("num_cascades", C.c_int32), ("probe_spacing0", C.c_int32),
                ("dir_res0", C.c_int32), ("interval0", C.c_int32), ("interval_ratio", C.c_int32),
                ("precision", C.c_int32), ("reserved", C.c_int32 * 7)]


class SceneSpec(C.Structure):
    _fields_ = [("grid", C.c_int32 * 3), ("num_boxes", C.c_int32), ("box_edge_min", C.c_int32),
                ("box_edge_max", C.c_int32), ("num_spheres", C.c_int32), ("reserved", C.c_int32),
                ("albedo_min", C.c_double), ("albedo_max", C.c_double), ("radius_min", C.c_double),
                ("radius_max", C.c_double), ("emission_min", C.c_double), ("emission_max", C.c_double),
                ("speed", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.rco_radiance_elems.restype = C.c_int64
        L.rco_radiance_elems.argtypes = [P]
        for name in ("rco_solve_f64", "rco_solve_f32"):
            getattr(L, name).argtypes = [P, P, P, P, C.c_int, C.c_int]
            getattr(L, name).restype = C.c_int
        L.rco_directions.argtypes = [C.c_int, P]
        L.rco_solid_angles.argtypes = [C.c_int, P]
        L.rco_crossings_before.argtypes = [C.c_int64, C.c_int64, C.c_int64]
        L.rco_crossings_before.restype = C.c_int64
        L.rco_float_to_half.argtypes = [C.c_float]
        L.rco_float_to_half.restype = C.c_uint16
        L.rco_scene_generate.argtypes = [P, C.c_uint64, P, P]
        L.rco_spheres_advance.argtypes = [P, C.c_int, P, C.c_int]
        L.rco_spheres_advance.restype = None
        L.rco_voxelise.argtypes = [P, P, C.c_int, P, C.c_int, P]
        L.rco_voxelise_mesh.argtypes = [P, P, C.c_int64, P, C.c_int64, P, P, C.c_int, P]
        L.rco_shade.argtypes = [P, P, C.c_int64, P, C.c_int64, P, P, P, C.c_int, P, P, C.c_int, P]
        _lib = L
    return _lib


def params(grid, num_cascades, spacing0=2, dir_res0=4, interval0=1, ratio=4, precision=0) -> Params:
    g = (grid,) * 3 if isinstance(grid, int) else tuple(grid)
    p = Params()
    p.grid[:] = g
    p.num_cascades, p.probe_spacing0, p.dir_res0 = num_cascades, spacing0, dir_res0
    p.interval0, p.interval_ratio, p.precision = interval0, ratio, precision
    return p


def level_shapes(p: Params):
    out, b = [], 0
    for i in range(p.num_cascades):
        s = p.probe_spacing0 << i
        n = p.dir_res0 << i
        blo = b
        b = p.interval0 if i == 0 else b * p.interval_ratio + p.interval0
        out.append(dict(spacing=s, probes=tuple(p.grid[a] // s for a in range(3)), n=n, dirs=n * n,
                        blo=blo, bhi=b))
    return out


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def solve(p: Params, voxels: np.ndarray, dtype=np.float64, nthreads=0, jump=False):
    """-> (fluence[P0,3], [L_i arrays shaped (3, dirs, Mz, My, Mx)])."""
    L = lib()
    voxels = np.ascontiguousarray(voxels, dtype=VOXEL_DT)
    shapes = level_shapes(p)
    P0 = int(np.prod(shapes[0]["probes"]))
    flu = np.zeros((P0, 3), dtype)
    rad = np.zeros(L.rco_radiance_elems(C.byref(p)), dtype)
    fn = L.rco_solve_f64 if dtype == np.float64 else L.rco_solve_f32
    rc = fn(C.byref(p), _ptr(voxels), _ptr(flu), _ptr(rad), nthreads, 1 if jump else 0)
    if rc != 0:
        raise ValueError("oracle rejected the parameters")
    levels, off = [], 0
    for sh in shapes:
        Mx, My, Mz = sh["probes"]
        cnt = 3 * sh["dirs"] * Mx * My * Mz
        levels.append(rad[off:off + cnt].reshape(3, sh["dirs"], Mz, My, Mx))
        off += cnt
    return flu, levels


def scene_spec(grid, num_boxes, edge_min, edge_max, num_spheres, rmin, rmax, emin, emax,
               albedo=(0.2, 0.9), speed=0.5) -> SceneSpec:
    s = SceneSpec()
    s.grid[:] = (grid,) * 3 if isinstance(grid, int) else tuple(grid)
    s.num_boxes, s.box_edge_min, s.box_edge_max, s.num_spheres = num_boxes, edge_min, edge_max, num_spheres
    s.albedo_min, s.albedo_max = albedo
    s.radius_min, s.radius_max, s.emission_min, s.emission_max, s.speed = rmin, rmax, emin, emax, speed
    return s


def generate(spec: SceneSpec, seed: int):
    boxes = np.zeros(spec.num_boxes, BOX_DT)
    spheres = np.zeros(spec.num_spheres, SPHERE_DT)
    lib().rco_scene_generate(C.byref(spec), seed, _ptr(boxes), _ptr(spheres))
    return boxes, spheres


def advance(spheres: np.ndarray, grid, frames: int):
    g = (C.c_int32 * 3)(*((grid,) * 3 if isinstance(grid, int) else grid))
    lib().rco_spheres_advance(_ptr(spheres), len(spheres), g, frames)


def voxelise_mesh(grid, positions, indices, tri_material, materials):
    """Triangle mesh (positions in grid units) -> rc_voxel volume, later triangles win."""
    g3 = (grid,) * 3 if isinstance(grid, int) else tuple(grid)
    out = np.zeros(g3[0] * g3[1] * g3[2], VOXEL_DT)
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices, np.uint32).reshape(-1, 3)
    mats = np.ascontiguousarray(materials, VOXEL_DT)
    tm = None if tri_material is None else np.ascontiguousarray(tri_material, np.uint16)
    g = (C.c_int32 * 3)(*g3)
    lib().rco_voxelise_mesh(g, _ptr(pos), len(pos), _ptr(idx), len(idx), None if tm is None else _ptr(tm),
                            _ptr(mats), len(mats), _ptr(out))
    return out


def shade(view, vertices, indices, tri_material, materials, textures, fluence=None, probes=(1, 1, 1), spacing=2):
    """CPU restatement of the shading pass -> (H, W, 4) float32 image.  view,
    materials, textures: the ctypes structures of the C ABI."""
    out = np.zeros((view.height, view.width, 4), np.float32)
    v = np.ascontiguousarray(vertices, np.float32)
    i = np.ascontiguousarray(indices, np.uint32)
    tm = None if tri_material is None else np.ascontiguousarray(tri_material, np.uint16)
    fl = None if fluence is None else np.ascontiguousarray(fluence, np.float32)
    pr = (C.c_int32 * 3)(*probes)
    lib().rco_shade(C.byref(view), _ptr(v), len(v), _ptr(i), len(i), None if tm is None else _ptr(tm),
                    materials, textures, len(textures) if textures else 0,
                    None if fl is None else _ptr(fl), pr, spacing, _ptr(out))
    return out


def voxelise(grid, boxes, spheres):
    g3 = (grid,) * 3 if isinstance(grid, int) else tuple(grid)
    out = np.zeros(g3[0] * g3[1] * g3[2], VOXEL_DT)
    g = (C.c_int32 * 3)(*g3)
    lib().rco_voxelise(g, _ptr(boxes), len(boxes), _ptr(spheres), len(spheres), _ptr(out))
    return out


def directions(n: int) -> np.ndarray:
    out = np.zeros((n * n, 3), np.int32)
    lib().rco_directions(n, _ptr(out))
    return out


def solid_angles(n: int) -> np.ndarray:
    out = np.zeros(n * n, np.float64)
    lib().rco_solid_angles(n, _ptr(out))
    return out


def crossings_before(b: int, Da: int, S: int) -> int:
    return lib().rco_crossings_before(b, Da, S)


def float_to_half(x: float) -> int:
    return lib().rco_float_to_half(x)


# Workload definitions: seeded scenes of the benchmark configurations.
CONFIGS = {
    # 64^3, 24 boxes (edges 4..20), 4 spheres (r 2..5, emission 1..20), 5 cascades
    "c64": dict(grid=64, cascades=5, boxes=24, edge=(4, 20), spheres=4, radius=(2.0, 5.0),
                emission=(1.0, 20.0), seed=1001),
    # 256^3, 400 boxes (edges 4..48), 32 spheres (r 2..8, emission 1..50), 6 cascades
    "c256": dict(grid=256, cascades=6, boxes=400, edge=(4, 48), spheres=32, radius=(2.0, 8.0),
                 emission=(1.0, 50.0), seed=1002),
}


def config_scene(name: str, frame: int = 0, grid=None):
    c = CONFIGS[name]
    g = grid or c["grid"]
    spec = scene_spec(g, c["boxes"], c["edge"][0], c["edge"][1], c["spheres"], c["radius"][0],
                      c["radius"][1], c["emission"][0], c["emission"][1])
    boxes, spheres = generate(spec, c["seed"])
    if frame:
        advance(spheres, g, frame)
    return boxes, spheres


if __name__ == "__main__":  # pragma: no cover
    print(os.path.basename(build_oracle.build()))
