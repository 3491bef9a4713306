#!/usr/bin/env python
"""Frames/s of the radiance-cascade solve on the 256^3 moving-emitter workload.

A step is one frame: the 32 emissive spheres advance 0.5 voxel, the volume
under the old and new spheres is recomposed on the device, and all 6
cascades plus the cascade-0 fluence are solved.

  value  frames/s with the scene resident in HBM, CUDA events on the
         context stream (per-frame working set ~1.3 GB >> L2)
  e2e    frames/s through the public C ABI with host buffers: each step
         copies the frame's sphere array host->device and reads the fluence
         back into pinned host memory
  roofline   level kernels: algorithmic bytes per frame / their event time
  cpu_baseline   the FP32 CPU port of the method, all host threads
  learned    the learned+FP16 form on the same workload (FP16 radiance, far
             cascades from the neural radiance cache): frames/s, speed-up over
             the plain FP32 value, fluence error against the FP64 oracle

--workload batch64 measures the batched form instead (64 uneven scenes, one
persistent launch), in scenes/s.

--impl reference times the CPU implementation of the same path (the oracle
port, FP32, all host threads) on the same workload: the reference project
has no cascade code of its own and its wgpu path cannot run headless here.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "c256"
WORKLOAD_DESC = ("256^3 voxels, 400 seeded opaque boxes (edges 4-48), 32 emissive spheres (radius 2-8, "
                 "emission 1-50) moving 0.5 voxel/frame; 6 cascades: 128^3 probes x 16 dirs at cascade 0, "
                 "x4 dirs and /2 probes per axis per level, intervals 0,1,5,21,85,341,1365")


def init_replicas(world: int, local: int):
    """One process per GPU: the process group (NCCL on GPUs, gloo on CPU) when
    world > 1, else None.  Rendezvous from MASTER_ADDR / MASTER_PORT."""
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return dist


def max_over_ranks(value: float, dist) -> float:
    """The slowest rank's figure (wall or event time): the job is done when it is."""
    if dist is None:
        return value
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_first_frame(rank: int, steps: int, warmup: int) -> int:
    """Replicas solve disjoint frame ranges of the moving-emitter workload."""
    return rank * (steps + warmup)


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def algorithmic_bytes(levels, grid, elem_bytes):
    """Bytes per frame: N_c * S + sum_i W_i + sum_{i>=1} W_i + F (scene 8 B/voxel read once per
    cascade, merged radiance written once and read once by the level below, fluence written)."""
    S = 8 * grid ** 3
    W = [3 * elem_bytes * l.num_dirs * l.probes[0] * l.probes[1] * l.probes[2] for l in levels]
    F = 12 * levels[0].probes[0] * levels[0].probes[1] * levels[0].probes[2]
    per_launch = []
    for i in range(len(levels)):
        b = S + W[i] + (W[i + 1] if i + 1 < len(levels) else 0) + (F if i == 0 else 0)
        per_launch.append(b)
    return sum(per_launch), per_launch


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms; start()
    returns once the first sample is written, so that the samples cover the
    timed region that follows."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="rc_clocks_", suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 5.0 and self.proc.poll() is None and os.path.getsize(self.path) == 0:
                time.sleep(0.02)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak_gbs():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic_per_launch():
    """DRAM bytes per level-kernel launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "frame_c256_launch_list.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1].strip().split()[0])
    except Exception:
        pass
    return None


def cpu_port_frames_per_s(frames: int, threads: int, precision=np.float32):
    """Times the FP32 CPU port of the path on `frames` frames of the workload."""
    from oracle import oracle as O
    boxes, spheres = O.config_scene(WORKLOAD)
    p = O.params(256, 6)
    t_total = 0.0
    for f in range(frames):
        t0 = time.perf_counter()
        vox = O.voxelise(256, boxes, spheres)
        O.solve(p, vox, dtype=precision, jump=True, nthreads=threads)
        t_total += time.perf_counter() - t0
        O.advance(spheres, 256, 1)
    return frames / t_total, t_total


def timed_frames(eng, R, sph, frames, local):
    """Event-timed frames (set emitters + solve) on the engine's stream; -> (ms, spheres of the last frame)."""
    import torch
    stream = torch.cuda.ExternalStream(eng.stream(), device=local)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    last = sph.copy()
    for _ in range(frames):
        last = sph.copy()
        eng.set_spheres(sph)
        eng.solve()
        R.advance_spheres(sph, 256, 1)
    t1.record(stream)
    t1.synchronize()
    return t0.elapsed_time(t1), last


def learned_form(args, R, local, boxes, spheres, plain_fps):
    """The learned+FP16 form of the same moving-emitter workload: FP16 radiance,
    the far cascades (from --learned-first-level, default 4) from the neural
    radiance cache, refit every frame on 1/16 of the walked directions of every
    far probe, per-8^3-tile fallback at 1% held-out error.  The cache first
    learns for `learned_warmup` frames; the timed frames follow."""
    import torch

    from oracle import oracle as O
    out = {}
    eng = R.Engine(R.make_params(256, 6, precision="fp16"), device=local)
    eng.set_boxes(boxes)
    sph = spheres.copy()
    for _ in range(3):
        eng.set_spheres(sph)
        eng.solve()
    eng.synchronize()
    ms, _ = timed_frames(eng, R, sph.copy(), args.steps, local)
    out["plain_fp16_frames_per_s"] = round(args.steps / (ms / 1000.0), 3)
    eng.nrc_enable(first_level=args.learned_first_level, fallback_threshold=args.learned_threshold,
                   plain_level_fraction=args.learned_plain_fraction)
    for _ in range(args.learned_warmup):
        eng.set_spheres(sph)
        eng.solve()
        R.advance_spheres(sph, 256, 1)
    eng.synchronize()
    before = eng.nrc_stats()["served_solves"]
    torch.cuda.nvtx.range_push("learned_timed")  # launch lists of the learned frames select this range
    ms, last = timed_frames(eng, R, sph, args.steps, local)
    torch.cuda.nvtx.range_pop()
    fps = args.steps / (ms / 1000.0)
    g = eng.fluence().astype(np.float64)
    st = eng.nrc_stats()
    served = [(st["served_solves"][i] - before[i]) / args.steps for i in range(6)]
    eng.close()
    ref, _ = O.solve(O.params(256, 6), O.voxelise(256, boxes, last), jump=True)
    out.update({
        "frames_per_s": round(fps, 3), "ms_per_frame": round(ms / args.steps, 4),
        "speedup_vs_plain_fp32": round(fps / plain_fps, 4),
        "fluence_rel_l2_vs_fp64": float(np.linalg.norm(g - ref) / np.linalg.norm(ref)),
        "fluence_max_abs_vs_fp64": float(np.abs(g - ref).max()),
        "fallback_tiles": int(st["fallback_tiles"]), "tiles": int(st["tiles"]),
        "cascades_from_network": [i for i in range(6) if (st["served_levels"] >> i) & 1],
        "served_fraction_of_timed_frames": {str(i): round(served[i], 4) for i in range(args.learned_first_level, 6)},
        "frames_learned_before_timing": args.learned_warmup, "frames_timed": args.steps,
        "first_level": args.learned_first_level, "fallback_threshold": args.learned_threshold,
        "plain_level_fraction": args.learned_plain_fraction,
        "storage": "radiance f16, network bf16 with f32 accumulation",
    })
    return out


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    sys.path.insert(0, ROOT)
    from oracle import build_oracle
    build_oracle.build()
    for _ in range(args.warmup):
        cpu_port_frames_per_s(1, threads)
    value, secs = cpu_port_frames_per_s(args.steps, threads)
    line = {
        "impl": "reference", "metric": "frames/s at 256^3 (radiance cascades, fluence + per-probe radiance)",
        "value": round(value, 4), "unit": "frames/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000.0 * secs / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD_DESC, "precision": "fp32"},
        "cpu_baseline": {"value": round(value, 4), "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": "%d consecutive frames of the 256^3 workload, full frame each "
                                   "(voxelise + 6 cascades + fluence)" % args.steps},
        "e2e": {"value": round(value, 4), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference repository holds no radiance-cascade implementation (only a wgpu forward "
                 "raster pass); this arm times the CPU restatement of the method on all host threads"),
    }
    print(json.dumps(line), flush=True)
    return 0


BATCH_DESC = ("64 cubic scenes (seed 2000+k), edges uniform over {32,48,64,96,128,192}, 64^3 workload's "
              "box/sphere density, 4-6 cascades by edge; one CUDA graph per solve: the persistent kernel "
              "(autotuned tile shape) or every scene's own level launches as parallel branches, whichever "
              "the autotuner measures faster")


def batch_bytes(batch_items, elem_bytes):
    """Algorithmic bytes of one batch solve: the per-frame formula summed over scenes."""
    import radiancecascade_gb300 as R
    total = 0
    for edge, N, _, _ in batch_items:
        p = R.make_params(edge, N)
        total += algorithmic_bytes([R.level_info(p, i) for i in range(N)], edge, elem_bytes)[0]
    return total


def cpu_port_batch_scenes_per_s(items, threads, budget_s=20.0):
    """Oracle FP32 on the batch's scenes in order until `budget_s` has passed;
    scenes/s extrapolated by voxel count to the whole batch."""
    from oracle import oracle as O
    t_total, vox_done, done = 0.0, 0, 0
    for edge, N, boxes, spheres in items:
        t0 = time.perf_counter()
        O.solve(O.params(edge, N), O.voxelise(edge, boxes, spheres), dtype=np.float32, jump=True,
                nthreads=threads)
        t_total += time.perf_counter() - t0
        vox_done += edge ** 3
        done += 1
        if t_total >= budget_s:
            break
    vox_all = sum(e ** 3 for e, _, _, _ in items)
    batch_s = t_total * vox_all / vox_done
    return len(items) / batch_s, done, t_total


def batch_measure(args, R, local, dist, world, steps):
    """The batched workload on this rank: scenes/s of the graph-launched
    persistent solve with the scenes resident, the same scenes as one context
    each back to back, and e2e through the public API (per step every scene's
    emitters move one frame and are uploaded from host arrays, one solve, every
    fluence read back into pinned host memory with one synchronisation)."""
    import torch
    items = R.batch_workload()
    prec = args.precision
    b = R.Batch([R.make_params(e, N, precision=prec) for e, N, _, _ in items], device=local)
    for k, (_, _, boxes, spheres) in enumerate(items):
        b.set_scene(k, boxes, spheres)
    tiles, tune_ms = b.tune(iters=2)
    stream = torch.cuda.Stream(local)
    sp = stream.cuda_stream
    for _ in range(args.warmup):
        b.solve(sp)
    b.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(steps):
        b.solve(sp)
    t1.record(stream)
    t1.synchronize()
    b.synchronize()
    torch.cuda.synchronize()
    clock_info = clocks.stop()
    ms = max_over_ranks(t0.elapsed_time(t1), dist)
    value = world * len(items) * steps / (ms / 1000.0)

    # the same scenes as separate contexts (fastest per-level kernels), one after another
    engines = []
    for e, N, boxes, spheres in items:
        g = R.Engine(R.make_params(e, N, precision=prec), device=local)
        g.set_boxes(boxes)
        g.set_spheres(spheres)
        engines.append(g)
    for _ in range(2):
        for g in engines:
            g.solve(sp)
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(steps):
        for g in engines:
            g.solve(sp)
    s1.record(stream)
    s1.synchronize()
    seq_ms = s0.elapsed_time(s1) / steps
    for g in engines:
        g.close()

    # e2e: per step every scene's spheres advance one frame and are uploaded
    # (incremental re-voxelisation on the batch stream), one solve, one read of
    # every fluence into pinned host memory -- started without waiting, into
    # one of two buffers in turn, so the next step's host work overlaps this
    # step's solve and read-back (every read is complete at the final wait)
    sph = [sx.copy() for _, _, _, sx in items]
    nbytes_in = sum(int(sx.nbytes) for sx in sph)
    flats = [torch.empty(b.fluence_elems(), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    nbytes_out = int(flats[0].nbytes)

    def e2e_step(f):
        for k, (edge, _, _, _) in enumerate(items):
            R.advance_spheres(sph[k], edge, 1)
            b.set_spheres(k, sph[k])
        b.solve()
        b.fluence_all_async(flats[f & 1])

    for f in range(2):
        e2e_step(f)
    b.synchronize()
    if dist:
        dist.barrier()
    e2e_steps = max(3, min(steps, 50))
    w0 = time.perf_counter()
    for f in range(e2e_steps):
        e2e_step(f)
    b.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - w0, dist)
    e2e_value = world * len(items) * e2e_steps / e2e_s

    # the form the tuner chose, and the persistent kernel timed on its own
    # (its best tile shape) when the tuner chose the scenes' own launches
    form = b.form()
    persistent_ms = None
    if form == "scenes":
        b.set_tiles(**{k: tiles[k] for k in ("probes_per_item", "dirs_per_item", "blocks_per_item",
                                             "walks_per_item")})
        for _ in range(2):
            b.solve(sp)
        b.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(steps):
            b.solve(sp)
        p1.record(stream)
        p1.synchronize()
        b.synchronize()
        persistent_ms = p0.elapsed_time(p1) / steps

    elem = 2 if prec == "fp16" else 4
    B = batch_bytes(items, elem)
    achieved = B / (ms / steps / 1000.0) / 1e9
    peak, peak_kind = measured_peak_gbs()
    b.close()
    return {
        "items": items, "value": value, "ms_per_step": ms / steps, "clock_info": clock_info,
        "tile": dict(tiles, tune_ms=round(tune_ms, 4)), "seq_ms": seq_ms, "B": B, "form": form,
        "persistent_ms": persistent_ms,
        "e2e": {"value": round(e2e_value, 3), "unit": "scenes/s", "h2d_bytes_per_step": nbytes_in,
                "d2h_bytes_per_step": nbytes_out, "steps": e2e_steps},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind, "traffic": None,
                     "kernel": ("every scene's level kernels, parallel graph branches" if form == "scenes"
                                else "k_batch_persistent"), "algorithmic_bytes_per_step": B},
    }


def run_batch(args, rank, world):
    """Scenes/s of the batched workload (replicas: every rank solves its own copy)."""
    import torch
    import radiancecascade_gb300 as R

    local = _env_int("LOCAL_RANK", 0)
    dist = init_replicas(world, local)
    torch.cuda.set_device(local)
    m = batch_measure(args, R, local, dist, world, args.steps)
    items, B = m["items"], m["B"]
    prec = args.precision
    line = {
        "metric": "scenes/s, batched uneven scenes in one graph launch",
        "value": round(m["value"], 3), "unit": "scenes/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(m["ms_per_step"], 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f16" if prec == "fp16" else "f32",
        "data": "synthetic",
        "config": {"workload": BATCH_DESC, "scenes": len(items), "precision": prec, "tile": m["tile"],
                   "parallelism": "replicas" if world > 1 else "single-gpu",
                   "l2": "inputs larger than L2 (%.1f GB of scene + radiance)" % (B / 1e9)},
        "e2e": m["e2e"],
        "gpu_launches": args.steps,
        "per_scene_contexts_ms_per_batch": round(m["seq_ms"], 4),
        "form": m["form"],
        "persistent_kernel_ms_per_batch": (round(m["persistent_ms"], 4) if m["persistent_ms"] else None),
        "roofline": m["roofline"],
    }
    if m["clock_info"]:
        line["clocks"] = m["clock_info"]
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, done, secs = cpu_port_batch_scenes_per_s(items, threads)
        line["cpu_baseline"] = {"value": round(v, 4), "unit": "scenes/s", "cores": threads, "kind": "port",
                                "sample": "first %d scenes of the batch (%.1f s, FP32, OpenMP), scaled to the "
                                          "batch by voxel count" % (done, secs)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def fp16_report(R, local, frames=6):
    """The FP16 storage form of the 64^3 workload: per frame (emitters moving
    one step per frame) the fluence relative L2 and max-abs error against the
    FP64 oracle and against the plain FP32 path; and frame 0 at 256^3."""
    from oracle import oracle as O

    def err(a, b):
        a = np.asarray(a, np.float64)
        b = np.asarray(b, np.float64)
        return float(np.linalg.norm(a - b) / np.linalg.norm(b)), float(np.abs(a - b).max())

    out = {"workload": "64^3 c64 scene (24 boxes, 4 spheres), 5 cascades; spheres advance one frame per row",
           "frames": []}
    boxes, sph = R.workload_scene("c64")
    sph = sph.copy()
    e16 = R.Engine(R.make_params(64, 5, precision="fp16"), device=local)
    e32 = R.Engine(R.make_params(64, 5), device=local)
    for e in (e16, e32):
        e.set_boxes(boxes)
    for f in range(frames):
        for e in (e16, e32):
            e.set_spheres(sph)
            e.solve()
        g16, g32 = e16.fluence(), e32.fluence()
        ref, _ = O.solve(O.params(64, 5), O.voxelise(64, boxes, sph))
        r64, m64 = err(g16, ref)
        r32, m32 = err(g16, g32)
        out["frames"].append({"frame": f, "rel_l2_vs_fp64": r64, "max_abs_vs_fp64": m64,
                              "rel_l2_vs_fp32": r32, "max_abs_vs_fp32": m32,
                              "fp32_rel_l2_vs_fp64": err(g32, ref)[0]})
        R.advance_spheres(sph, 64, 1)
    e16.close()
    e32.close()
    b256, s256 = R.workload_scene(WORKLOAD)
    e = R.Engine(R.make_params(256, 6, precision="fp16"), device=local)
    e.set_boxes(b256)
    e.set_spheres(s256)
    e.solve()
    g16 = e.fluence()
    e.close()
    e = R.Engine(R.make_params(256, 6), device=local)
    e.set_boxes(b256)
    e.set_spheres(s256)
    e.solve()
    g32 = e.fluence()
    e.close()
    ref, _ = O.solve(O.params(256, 6), O.voxelise(256, b256, s256), jump=True)
    r64, m64 = err(g16, ref)
    r32, m32 = err(g16, g32)
    out["c256_frame0"] = {"rel_l2_vs_fp64": r64, "max_abs_vs_fp64": m64, "rel_l2_vs_fp32": r32,
                          "max_abs_vs_fp32": m32}
    out["storage"] = "radiance f16, transmittance decisions exact, merge accumulation f32"
    return out


RENDER_DESC = ("256^3 procedural room mesh (walls, 40 blocks, a 131k-triangle sphere) voxelised on the GPU, "
               "32 emissive spheres moving 0.5 voxel/frame, 6 cascades; per frame: emitter update, GI solve, "
               "1920x1080 raster + Blinn-Phong shading with the fluence term")


def run_render(args, rank, world):
    """Frames/s of the whole renderer frame on a mesh scene (secondary workload)."""
    import torch
    import radiancecascade_gb300 as R
    from radiancecascade_gb300 import _ffi as F

    local = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    g, W, H = 256, 1920, 1080
    pos, idx, tm, vox_mats = R.room_mesh(g, boxes=40, seed=5)
    # a finely tessellated sphere (2 x 256 x 256 triangles)
    nu, nv, c, r = 256, 256, np.array([160.0, 96.0, 150.0]), 30.0
    th, ph = np.meshgrid(np.linspace(0, np.pi, nv + 1), np.linspace(0, 2 * np.pi, nu, endpoint=False), indexing="ij")
    sp = (c + r * np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], -1)).reshape(-1, 3)
    j, i = np.meshgrid(np.arange(nv), np.arange(nu), indexing="ij")
    a = (j * nu + i).ravel() + len(pos)
    b = (j * nu + (i + 1) % nu).ravel() + len(pos)
    sph_idx = np.concatenate([np.stack([a, b + nu, b], 1), np.stack([a, a + nu, b + nu], 1)])
    pos = np.concatenate([pos, sp.astype(np.float32)])
    idx = np.concatenate([idx, sph_idx.astype(np.uint32)])
    tm = np.concatenate([tm, np.ones(len(sph_idx), np.uint16)])
    uv = np.stack([pos[:, 0] / g + pos[:, 2] / (2 * g), pos[:, 1] / g], 1).astype(np.float32)
    verts = R.shade_vertices(pos, idx, texcoords=uv)
    mats = [R.shade_material(ambient=(1, 1, 1), diffuse=(0.6, 0.6, 0.6), specular=(0.4, 0.4, 0.4), shininess=32),
            R.shade_material(ambient=(1, 1, 1), diffuse=(0.8, 0.7, 0.6), specular=(0.2, 0.2, 0.2), shininess=8),
            R.shade_material(ambient=(1, 1, 1), diffuse=(1, 1, 1), specular=(0, 0, 0), shininess=1)]
    spec = R.scene_spec(g, 0, (4, 8), 32, (2.0, 8.0), (1.0, 50.0))
    _, spheres = R.generate_scene(spec, 1002)
    eng = R.Engine(R.make_params(g, 6), device=local)
    t0 = time.perf_counter()
    eng.set_mesh(pos, idx, vox_mats, tm)
    vox_s = time.perf_counter() - t0
    view = F.ShadeView()
    view.view_proj[:] = R.camera_view_proj((128.0, 140.0, 8.0), np.pi / 2, -0.15, W, H, fovy_deg=75, znear=0.5,
                                           zfar=600.0)
    view.eye[:] = (128.0, 140.0, 8.0)
    view.light[:] = (80.0, 220.0, 120.0)
    view.width, view.height = W, H
    view.world_to_grid[:] = [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0]
    view.gi_scale = 1.0
    sph = spheres.copy()
    steps = max(1, min(args.steps, 60))
    # the mesh is uploaded once (rc_shade_set_mesh), as the reference builds its buffers once
    t0 = time.perf_counter()
    eng.shade_set_mesh(verts, idx, mats, tm)
    upload_s = time.perf_counter() - t0
    dimg = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    himg = torch.empty((H, W, 4), dtype=torch.float32, pin_memory=True).numpy()
    st = torch.cuda.ExternalStream(eng.stream())

    def frame(out):
        eng.set_spheres(sph)
        eng.solve()
        eng.shade_draw(view, out)
        R.advance_spheres(sph, g, 1)

    # value: image left in device memory, CUDA events on the context's stream
    for _ in range(args.warmup):
        frame(dimg)
    eng.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps):
        frame(dimg)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # e2e: the image read back into pinned host memory every frame, host clock
    for _ in range(args.warmup):
        frame(himg)
    t0 = time.perf_counter()
    for _ in range(steps):
        frame(himg)
    e2e_s = (time.perf_counter() - t0) / steps
    # the one-call form: rc_shade uploads the mesh and writes a new pageable array every frame
    t0 = time.perf_counter()
    for _ in range(min(steps, 10)):
        eng.set_spheres(sph)
        eng.solve()
        img = eng.shade(view, verts, idx, mats, tm)
        R.advance_spheres(sph, g, 1)
    one_call_s = (time.perf_counter() - t0) / min(steps, 10)
    line = {
        "metric": "renderer frames/s (GI solve + 1080p shading) on a mesh scene", "value": round(1000.0 / ms, 3),
        "unit": "frames/s", "n_gpus": 1, "steps": steps, "warmup": args.warmup,
        "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": RENDER_DESC, "triangles": int(len(idx)), "image": [W, H],
                   "timing": "CUDA events on the context's stream, image left in device memory"},
        "e2e": {"value": round(1.0 / e2e_s, 3), "unit": "frames/s", "h2d_bytes_per_step": int(sph.nbytes),
                "d2h_bytes_per_step": int(himg.nbytes)},
        "one_call_frames_per_s": round(1.0 / one_call_s, 3),
        "one_call_note": "rc_shade per frame: mesh upload from pageable memory + image into a new pageable array",
        "mesh_upload_s": round(upload_s, 4),
        "voxelise_s": round(vox_s, 4), "voxelise_triangles_per_s": round(len(idx) / vox_s, 1),
        "lit_pixels": float((img[..., :3] > 0).any(-1).mean()),
    }
    eng.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp16"])
    ap.add_argument("--cpu-frames", type=int, default=2, help="frames of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--learned-warmup", type=int, default=48,
                    help="frames the radiance cache learns before the learned form is timed")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned+FP16 form")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched workload's figures")
    ap.add_argument("--learned-first-level", type=int, default=4, help="first cascade the radiance cache serves")
    ap.add_argument("--learned-threshold", type=float, default=0.01,
                    help="held-out relative error above which a tile falls back to the plain walk")
    ap.add_argument("--learned-plain-fraction", type=float, default=0.5,
                    help="a cascade runs its plain kernels when this fraction of its probes is in fallback tiles")
    ap.add_argument("--workload", default="c256", choices=["c256", "batch64", "render"],
                    help="c256: the 256^3 moving-emitter frame (default); batch64: 64 uneven scenes")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank, world, local = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1), _env_int("LOCAL_RANK", 0)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "batch64":
        return run_batch(args, rank, world)
    if args.workload == "render":
        return run_render(args, rank, world)

    import torch
    import radiancecascade_gb300 as R

    dist = init_replicas(world, local)
    torch.cuda.set_device(local)

    boxes, spheres = R.workload_scene(WORKLOAD)
    params = R.make_params(256, 6, precision=args.precision)
    eng = R.Engine(params, device=local)
    eng.set_boxes(boxes)
    levels = eng.levels
    # replicas: rank r starts at frame r * steps so the ranks solve different frames
    sph = spheres.copy()
    if rank:
        R.advance_spheres(sph, 256, replica_first_frame(rank, args.steps, args.warmup))
    stream = torch.cuda.ExternalStream(eng.stream(), device=local)

    for _ in range(args.warmup):
        eng.set_spheres(sph)
        eng.solve()
        R.advance_spheres(sph, 256, 1)
    eng.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for _ in range(args.steps):
        eng.set_spheres(sph)
        eng.solve()
        R.advance_spheres(sph, 256, 1)
    t_end.record(stream)
    t_end.synchronize()
    torch.cuda.synchronize()
    clock_info = clocks.stop()
    ms = max_over_ranks(t_start.elapsed_time(t_end), dist)
    if dist:
        dist.barrier()
    value = world * args.steps / (ms / 1000.0)
    # recompose + one kernel per cascade + the shared walk of the narrow levels
    launches_per_step = 1 + params.num_cascades + 1

    # ---- e2e: public API, host buffers, H2D of the frame's spheres, D2H of every frame's
    # fluence into pinned host memory (the read-back of frame f overlaps the solve of f+1)
    nflu = 3 * int(np.prod(eng.probes0))
    host_out = [torch.empty(nflu, dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    for f in range(2):
        eng.set_spheres(sph)
        eng.solve()
        eng.fluence_async(host_out[f & 1])
        R.advance_spheres(sph, 256, 1)
    eng.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for f in range(args.steps):
        eng.set_spheres(sph)
        eng.solve()
        eng.fluence_async(host_out[f & 1])
        R.advance_spheres(sph, 256, 1)
    eng.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e_value = world * args.steps / e2e_s

    # ---- roofline of the level kernels (CUDA events around every launch)
    # per level with events between the kernels, then the level set as a solve runs it
    # (each level kernel may start while the previous one finishes): the roofline's time
    prof = eng.profile_levels(iters=10, whole=True)
    per_level_ms, level_ms = prof[:-1], float(prof[-1])
    elem = 2 if args.precision == "fp16" else 4
    B, per_launch = algorithmic_bytes(levels, 256, elem)
    achieved = B / (level_ms / 1000.0) / 1e9
    peak, peak_kind = measured_peak_gbs()
    traffic = profile_traffic_per_launch()

    line = {
        "metric": "frames/s at 256^3 (radiance cascades, fluence + per-probe radiance)",
        "value": round(value, 3), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f16" if args.precision == "fp16" else "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD_DESC, "precision": args.precision, "frames_per_rank": args.steps,
                   "parallelism": "replicas" if world > 1 else "single-gpu",
                   "l2": "inputs larger than L2 (~1.3 GB of scene + radiance per frame)"},
        "e2e": {"value": round(e2e_value, 3), "unit": "frames/s",
                "h2d_bytes_per_step": int(sph.nbytes), "d2h_bytes_per_step": int(nflu * 4)},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                     "traffic": traffic,
                     "frac_measured": (round(traffic / (level_ms / 1000.0) / 1e9 / peak, 4)
                                       if traffic else None),
                     "frac_basis": "frac: algorithmic bytes B (8 B/voxel scene read per cascade, radiance "
                                   "written and read once, fluence) / the frame's level time (its kernels "
                                   "launched as a solve launches them) / measured HBM peak; "
                                   "frac_measured: DRAM bytes of the level kernels measured by ncu "
                                   "(profiles/frame_c256_launch_list.md) / the same time / the same peak",
                     "kernel": "cascade levels: k_level0_tma + k_level_bits_up (wide) + k_walk_queue / k_level_merge (narrow)",
                     "algorithmic_bytes_per_frame": B,
                     "level_ms_per_frame": round(level_ms, 4),
                     "level_ms_serialised": round(float(per_level_ms[1:].sum()), 4),
                     "per_level_ms": [round(float(x), 4) for x in per_level_ms[1:]],
                     "compose_ms": round(float(per_level_ms[0]), 4)},
    }
    if clock_info:
        line["clocks"] = clock_info

    if rank == 0 and world == 1 and not args.no_accuracy:
        from oracle import oracle as O
        fb, fs = R.workload_scene(WORKLOAD)
        eng.set_spheres(fs)
        eng.solve()
        g = eng.fluence().astype(np.float64)
        ref, _ = O.solve(O.params(256, 6), O.voxelise(256, fb, fs), jump=True)
        line["accuracy"] = {"frame": 0, "fluence_rel_l2_vs_fp64":
                            float(np.linalg.norm(g - ref) / np.linalg.norm(ref)),
                            "fluence_max_abs_vs_fp64": float(np.abs(g - ref).max())}
    if rank == 0 and world == 1 and not args.no_learned:
        line["learned"] = learned_form(args, R, local, boxes, spheres, value)
    if rank == 0 and world == 1 and not args.no_accuracy:
        line["fp16"] = fp16_report(R, local)
    if rank == 0 and world == 1 and not args.no_batch:
        m = batch_measure(args, R, local, None, 1, min(args.steps, 50))
        line["batch"] = {"workload": BATCH_DESC, "scenes": len(m["items"]), "scenes_per_s": round(m["value"], 3),
                         "ms_per_batch": round(m["ms_per_step"], 4), "e2e": m["e2e"],
                         "per_scene_contexts_ms_per_batch": round(m["seq_ms"], 4), "tile": m["tile"],
                         "form": m["form"],
                         "persistent_kernel_ms_per_batch": (round(m["persistent_ms"], 4)
                                                            if m["persistent_ms"] else None),
                         "roofline": m["roofline"]}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, _ = cpu_port_frames_per_s(args.cpu_frames, threads)
        line["cpu_baseline"] = {"value": round(v, 4), "unit": "frames/s", "cores": threads, "kind": "port",
                                "sample": "%d frames of the same workload (voxelise + 6 cascades + fluence, "
                                          "FP32, OpenMP)" % args.cpu_frames}
    eng.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
