"""Runs the engine on small scenes with the checked library (RC_LIBRARY
points at librc_checked.so) and prints one JSON line per case: the fluence
error against the FP64 oracle and the checked build's failure count.  Driven
by tests/test_gpu_checked.py in a process of its own."""
import ctypes as C
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import radiancecascade_gb300 as R  # noqa: E402
from oracle import oracle as O  # noqa: E402
from radiancecascade_gb300 import _ffi as F  # noqa: E402


def rel(a, b):
    a = np.asarray(a, np.float64).reshape(-1)
    b = np.asarray(b, np.float64).reshape(-1)
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / n) if n > 0 else float(np.linalg.norm(a - b))


def status():
    first, count = C.c_uint64(), C.c_uint32()
    st = F.lib().rc_check_status(0, C.byref(first), C.byref(count))
    return st, int(count.value), F.last_error() if st else ""


def scene(grid, seed):
    n = max(grid)
    spec = R.scene_spec(grid, max(3, n // 4), (1, max(2, n // 6)), max(1, n // 16), (1.0, max(1.5, n / 10)),
                        (1.0, 20.0))
    return R.generate_scene(spec, seed)


def emit(name, err, extra=None):
    st, count, msg = status()
    line = {"case": name, "rel_l2": err, "status": st, "failures": count, "message": msg}
    line.update(extra or {})
    print(json.dumps(line), flush=True)


def main():
    assert "checked" in (os.environ.get("RC_LIBRARY") or ""), "run with RC_LIBRARY=.../librc_checked.so"
    st, _, msg = status()
    assert st == F.RC_OK, msg  # the checked library answers, and no failure is pending
    cases = [((8, 8, 8), 2), ((16, 16, 16), 3), ((48, 48, 48), 4), ((16, 32, 48), 3), ((64, 64, 64), 5)]
    for k, (grid, N) in enumerate(cases):
        boxes, spheres = scene(grid, 100 + k)
        ref, _ = O.solve(O.params(grid, N), O.voxelise(grid, boxes, spheres), jump=True)
        for prec in ("fp32", "fp16"):
            with R.Engine(R.make_params(grid, N, precision=prec)) as e:
                e.set_boxes(boxes)
                e.set_spheres(spheres)
                e.solve()
                sph = spheres.copy()
                R.advance_spheres(sph, grid, 3)
                e.set_spheres(sph)  # an incremental emitter update
                e.set_spheres(spheres)
                e.solve()
                emit("%s %s" % ("x".join(map(str, grid)), prec), rel(e.fluence(), ref))
    # the batched persistent solve over the same scenes
    with R.Batch([R.make_params(g, N) for g, N in cases[:4]]) as b:
        for k, (grid, N) in enumerate(cases[:4]):
            b.set_scene(k, *scene(grid, 100 + k))
        b.solve()
        errs = []
        for k, (grid, N) in enumerate(cases[:4]):
            boxes, spheres = scene(grid, 100 + k)
            ref, _ = O.solve(O.params(grid, N), O.voxelise(grid, boxes, spheres), jump=True)
            errs.append(rel(b.fluence(k), ref))
        emit("batch", max(errs))
    # the learned form (every cache kernel) on a small scene
    grid, N = (32, 32, 32), 4
    boxes, spheres = scene(grid, 7)
    ref, _ = O.solve(O.params(grid, N), O.voxelise(grid, boxes, spheres), jump=True)
    with R.Engine(R.make_params(grid, N)) as e:
        e.set_boxes(boxes)
        e.set_spheres(spheres)
        e.nrc_enable(first_level=2, hash_log2_entries=14, plain_level_fraction=1.0)
        for _ in range(20):
            e.solve()
        q = e.nrc_query(2, np.arange(8, dtype=np.int32), np.arange(8, dtype=np.int32))
        emit("learned", rel(e.fluence(), ref), {"finite_query": bool(np.isfinite(q).all())})


if __name__ == "__main__":
    main()
