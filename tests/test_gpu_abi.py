"""GPU tests of the C ABI's contract: error statuses, state checks, injected
faults (host-side, no GPU fault), device-memory and external-stream paths."""
import ctypes as C

import numpy as np
import pytest

import radiancecascade_gb300 as R
from radiancecascade_gb300 import _ffi as F
from oracle import oracle as O
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def test_state_and_argument_errors():
    p = R.make_params(32, 4)
    with R.Engine(p) as e:
        L = F.lib()
        assert L.rc_solve(e.handle, None) == F.RC_ERR_STATE
        assert "scene" in F.last_error()
        assert L.rc_scene_set_spheres(e.handle, None, 0) == F.RC_ERR_STATE
        v = np.zeros(10, R.VOXEL_DT)
        assert L.rc_scene_upload(e.handle, F.ptr(v), 10, F.RC_MEM_HOST) == F.RC_ERR_INVALID_ARG
        e.set_boxes(np.zeros(0, R.BOX_DT))
        e.solve()
        out = np.zeros(5, np.float32)
        assert L.rc_get_fluence(e.handle, F.ptr(out), 5, F.RC_MEM_HOST) == F.RC_ERR_INVALID_ARG
        assert L.rc_get_radiance(e.handle, 9, F.ptr(out), 20, F.RC_MEM_HOST) == F.RC_ERR_INVALID_ARG
        assert L.rc_get_fluence(e.handle, F.ptr(out), 5, 7) == F.RC_ERR_INVALID_ARG
        # the context is still usable after the errors
        e.solve()
        assert not e.fluence().any()
    h = C.c_void_p()
    assert F.lib().rc_create(C.byref(p), 99, C.byref(h)) == F.RC_ERR_INVALID_ARG


def test_injected_allocation_and_upload_faults(monkeypatch):
    p = R.make_params(32, 4)
    monkeypatch.setenv("RC_FAULT", "alloc")
    with pytest.raises(R.RCError) as ex:
        R.Engine(p)
    assert ex.value.status == F.RC_ERR_OOM
    monkeypatch.setenv("RC_FAULT", "upload")
    monkeypatch.delenv("RC_FAULT")
    e = R.Engine(p)
    monkeypatch.setenv("RC_FAULT", "upload")
    with pytest.raises(R.RCError) as ex:
        e.upload(np.zeros(32 ** 3, R.VOXEL_DT))
    assert ex.value.status == F.RC_ERR_CUDA
    monkeypatch.delenv("RC_FAULT")
    e.upload(np.zeros(32 ** 3, R.VOXEL_DT))
    e.solve()
    assert not e.fluence().any()
    e.close()


def test_device_upload_external_stream_and_device_outputs():
    torch = pytest.importorskip("torch")
    boxes, spheres = R.workload_scene("c64")
    vox = R.voxelise_host(64, boxes, spheres)
    dev = torch.from_numpy(vox.view(np.uint16).reshape(-1, 4).copy()).cuda()
    p = R.make_params(64, 5)
    with R.Engine(p) as e:
        e.upload_device(dev.data_ptr(), vox.size)
        s = torch.cuda.Stream()
        e.solve(stream=s.cuda_stream)
        s.synchronize()
        host = e.fluence()
        n = host.size
        out = torch.empty(n, dtype=torch.float32, device="cuda")
        assert F.lib().rc_get_fluence(e.handle, C.c_void_p(out.data_ptr()), n, F.RC_MEM_DEVICE) == F.RC_OK
        assert np.array_equal(out.cpu().numpy().reshape(-1, 3), host)
        assert e.fluence_device_ptr() != 0 and e.radiance_device_ptr(2) != 0
    oflu, _ = O.solve(O.params(64, 5), vox)
    assert rel_l2(host, oflu) <= 1e-4


def test_gi_stage_render_stage_cycle():
    """update -> render -> read, then resize to another shape (RenderStage call order)."""
    boxes, spheres = R.workload_scene("c64")
    stage = R.GiStage(R.make_params(64, 5), boxes=boxes)
    got = []
    for f in R.frames(stage, spheres, 64, 3):
        got.append(stage.fluence().copy())
    assert len(got) == 3 and not np.array_equal(got[0], got[2])
    stage.resize(R.make_params(64, 4))
    stage.update(R.GiState(spheres=spheres))
    stage.render()
    assert stage.fluence().shape == (32 ** 3, 3)
    stage.close()


def test_async_fluence_readback_matches_sync_per_frame():
    """Each frame's fluence, read back asynchronously into alternating host
    buffers while the next frame solves, equals the synchronous read-back."""
    boxes, spheres = R.workload_scene("c64")
    with R.Engine(R.make_params(64, 5)) as e, R.Engine(R.make_params(64, 5)) as ref:
        e.set_boxes(boxes)
        ref.set_boxes(boxes)
        outs = [np.zeros(3 * 32 ** 3, np.float32) for _ in range(4)]
        want = []
        sph = spheres.copy()
        for f in range(4):
            e.set_spheres(sph)
            e.solve()
            e.fluence_async(outs[f])
            ref.set_spheres(sph)
            ref.solve()
            want.append(ref.fluence().reshape(-1).copy())
            R.advance_spheres(sph, 64, 3)
        e.synchronize()
        for f in range(4):
            assert np.array_equal(outs[f], want[f]), f
        with pytest.raises(ValueError):
            e.fluence_async(np.zeros(10, np.float32))



def test_cpp_driver_solve_matches_python_binding(tmp_path):
    """The same solve through the C++ driver and through ctypes is bit-identical."""
    import subprocess
    from tests.helpers import build_abi_driver
    exe = build_abi_driver(tmp_path)
    out = str(tmp_path / "flu.bin")
    r = subprocess.run([exe, "gpu", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, np.float32)
    spec = R.scene_spec(32, 6, (3, 10), 3, (1.5, 4.0), (1.0, 20.0))
    boxes, spheres = R.generate_scene(spec, 77)
    with R.Engine(R.make_params(32, 4)) as e:
        e.set_boxes(boxes)
        e.set_spheres(spheres)
        e.solve()
        want = e.fluence().reshape(-1)
    assert np.array_equal(got, want)


def test_contexts_of_different_sizes_coexist():
    """A context created after a larger one must not break the larger one's
    kernels (per-kernel launch limits are shared by all contexts)."""
    spec = R.scene_spec(96, 10, (3, 12), 3, (1.5, 4.0), (1.0, 20.0))
    boxes, spheres = R.generate_scene(spec, 3)
    big = R.Engine(R.make_params(96, 5))
    small = R.Engine(R.make_params(32, 3))
    try:
        big.set_boxes(boxes)
        big.set_spheres(spheres)
        small.upload(O.voxelise(32, np.zeros(0, R.BOX_DT), np.zeros(0, R.SPHERE_DT)))
        small.solve()
        big.solve()
        got = big.fluence().astype(np.float64)
        want, _ = O.solve(O.params(96, 5), O.voxelise(96, boxes, spheres), jump=True)
        assert rel_l2(got, want) <= 1e-4
    finally:
        small.close()
        big.close()


def test_stage_timing_and_frame_log(tmp_path):
    """Stage timing records events inside every solve: the cascades' times are
    non-negative and add up to the whole solve; the JSONL frame log writes one
    line per frame with them, the algorithmic GB/s and the cache's figures."""
    import json
    params = R.make_params(64, 5)
    boxes, spheres = R.workload_scene("c64")
    with R.Engine(params) as e:
        e.set_boxes(boxes)
        e.set_spheres(spheres)
        with pytest.raises(R.RCError):
            e.stage_ms()  # timing is off
        log = R.FrameLog(str(tmp_path / "frames.jsonl"), e, algorithmic_bytes=29e6)
        for f in range(3):
            e.solve()
            log.write(f, note="plain")
        e.nrc_enable(first_level=3)
        e.solve()
        log.write(3)
        log.close()
        ms = None
        with pytest.raises(R.RCError):
            ms = e.stage_ms()
    lines = [json.loads(x) for x in open(tmp_path / "frames.jsonl")]
    assert [x["frame"] for x in lines] == [0, 1, 2, 3] and ms is None
    for x in lines:
        assert x["solve_ms"] > 0 and len(x["cascade_ms"]) == 5
        assert min(x["cascade_ms"]) >= 0 and abs(sum(x["cascade_ms"]) - x["solve_ms"]) <= 1e-3 + 1e-3 * x["solve_ms"]
        assert x["algorithmic_gb_per_s"] > 0
    assert lines[0]["note"] == "plain" and "nrc_loss" not in lines[0]
    assert 0.0 <= lines[3]["nrc_fallback_fraction"] <= 1.0


def test_overlapped_level_launches_match_serialised_ones():
    """The level kernels start while the previous level's kernel finishes
    (programmatic launches; each waits on the device for what it reads).  With
    stage timing on, events between the kernels serialise them: both orders
    must give the same bits, frame after frame, at 128^3 (every level kind:
    walk queue, merges, TMA-staged wide levels, cascade 0)."""
    params = R.make_params(128, 5)
    boxes, spheres = R.generate_scene(R.scene_spec(128, 96, (4, 24), 12, (2.0, 6.0), (1.0, 30.0)), 21)
    out = []
    for timing in (False, True):
        with R.Engine(params) as e:
            e.set_boxes(boxes)
            e.set_stage_timing(timing)
            s2 = spheres.copy()
            frames = []
            for _ in range(3):
                e.set_spheres(s2)
                e.solve()
                R.advance_spheres(s2, 128, 2)
                frames.append((e.fluence().copy(), [e.radiance(i).copy() for i in range(5)]))
            out.append(frames)
    for (fa, la), (fb, lb) in zip(*out):
        assert np.array_equal(fa, fb)
        for x, y in zip(la, lb):
            assert np.array_equal(x, y)


def test_profile_levels_per_launch_and_whole_frame():
    """rc_profile_levels: the per-launch means, and with one more float the
    frame's level set timed as a solve launches it (no events between the
    kernels), which cannot take much longer than the per-launch sum."""
    params = R.make_params(128, 5)
    boxes, spheres = R.generate_scene(R.scene_spec(128, 96, (4, 24), 12, (2.0, 6.0), (1.0, 30.0)), 21)
    with R.Engine(params) as e:
        e.set_boxes(boxes)
        e.set_spheres(spheres)
        e.solve()
        per = e.profile_levels(3)
        both = e.profile_levels(3, whole=True)
        assert per.shape == (6,) and both.shape == (7,)
        assert (per > 0).all() and (both > 0).all()
        assert both[-1] <= 1.25 * float(both[1:-1].sum()) + 0.05
        bad = np.zeros(8, np.float32)
        assert F.lib().rc_profile_levels(e.handle, 1, F.ptr(bad), 8) == F.RC_ERR_INVALID_ARG
