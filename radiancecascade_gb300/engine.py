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

    def profile_levels(self, iters: int = 5) -> np.ndarray:
        """Mean ms per launch: [compose, level 0, level 1, ...] (CUDA events)."""
        out = np.zeros(1 + self.params.num_cascades, np.float32)
        F.check(self._lib.rc_profile_levels(self.handle, iters, F.ptr(out), out.size))
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

    def nrc_disable(self) -> None:
        F.check(self._lib.rc_nrc_disable(self.handle))

    def nrc_stats(self) -> dict:
        st = F.NrcStats()
        F.check(self._lib.rc_nrc_get_stats(self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_ if k != "pad"}

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
