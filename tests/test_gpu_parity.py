"""GPU parity: the CUDA path through the C ABI against the FP64 oracle.

Tolerances (fluence and every level's merged radiance, against FP64):
  FP32 path: relative L2 <= 1e-4 (the bar), and since every voxel decision is
             exact integer arithmetic, max relative error per value <= 1e-5;
  FP16 path: relative L2 <= 1e-2.
"""
import math
import os

import numpy as np
import pytest

import radiancecascade_gb300 as R
from oracle import oracle as O
from tests.helpers import mirror_x, rel_l2, volume

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FP32_REL_L2 = 1e-4
FP32_MAX_REL = 1e-5
FP16_REL_L2 = 1e-2


def _solve_gpu(params, vox=None, boxes=None, spheres=None):
    with R.Engine(params) as e:
        if vox is not None:
            e.upload(vox)
        else:
            e.set_boxes(boxes)
            e.set_spheres(spheres)
        e.solve()
        e.synchronize()
        return e.fluence().astype(np.float64), [e.radiance(i).astype(np.float64)
                                                for i in range(params.num_cascades)]


def _check(gflu, gL, oflu, oL, rel=FP32_REL_L2, max_rel=FP32_MAX_REL):
    assert rel_l2(gflu, oflu) <= rel, rel_l2(gflu, oflu)
    for g, o in zip(gL, oL):
        assert g.shape == o.shape
        assert rel_l2(g, o) <= rel
        if max_rel is not None:
            assert np.abs(g - o).max() <= max_rel * max(1.0, np.abs(o).max())


@pytest.fixture(params=["default", "no_tma", "scalar"])
def walk(request, monkeypatch):
    """Runs a test with the default kernels (bit-parallel walks, TMA-staged
    cascade 0), without the TMA cascade-0 kernel, and with the scalar walk."""
    monkeypatch.delenv("RC_WALK", raising=False)
    monkeypatch.delenv("RC_TMA", raising=False)
    if request.param == "scalar":
        monkeypatch.setenv("RC_WALK", "scalar")
    elif request.param == "no_tma":
        monkeypatch.setenv("RC_TMA", "0")
    return request.param


@pytest.mark.parametrize("frame", [0, 37])
def test_c64_fp32_matches_fp64_oracle(frame, walk):
    boxes, spheres = R.workload_scene("c64", frame=frame)
    vox = O.voxelise(64, boxes, spheres)
    oflu, oL = O.solve(O.params(64, 5), vox)
    gflu, gL = _solve_gpu(R.make_params(64, 5), boxes=boxes, spheres=spheres)
    _check(gflu, gL, oflu, oL)


def test_c64_fp16_storage_within_one_percent(walk):
    boxes, spheres = R.workload_scene("c64")
    vox = O.voxelise(64, boxes, spheres)
    oflu, oL = O.solve(O.params(64, 5), vox)
    gflu, gL = _solve_gpu(R.make_params(64, 5, precision="fp16"), boxes=boxes, spheres=spheres)
    err = rel_l2(gflu, oflu)
    assert err <= FP16_REL_L2
    _check(gflu, gL, oflu, oL, rel=FP16_REL_L2, max_rel=None)


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz")))
def test_golden_fixtures(name, walk):
    z = np.load(os.path.join(GOLDEN, name))
    grid = tuple(int(x) for x in z["grid"])
    N = int(z["num_cascades"])
    gflu, gL = _solve_gpu(R.make_params(grid, N), vox=z["voxels"].view(R.VOXEL_DT).reshape(-1))
    _check(gflu, gL, z["fluence"], [z["radiance_%d" % i] for i in range(N)])


@pytest.mark.parametrize("grid,N,kw", [
    ((32, 16, 48), 3, {}),
    ((32, 32, 32), 2, dict(spacing0=4, dir_res0=2, interval0=2, ratio=3)),
    ((48, 48, 48), 4, {}),
    # elongated grids: 1024 voxels (the largest edge) along one axis, few along the others
    ((1024, 32, 64), 5, {}),
    ((32, 512, 32), 4, dict(dir_res0=6)),
    # cascade 0 through the staged kernel at the compiled row widths 32 and 128
    # (64 is the 256^3 workload's), and at a width of 48 that none fixes
    ((128, 24, 40), 3, {}),
    ((512, 48, 32), 4, {}),
    ((192, 32, 24), 3, {}),
    # 100 directions at cascade 0: more than the walk-free kernel keeps in lanes
    ((64, 64, 64), 3, dict(dir_res0=10)),
])
def test_other_shapes_match_oracle(grid, N, kw, walk):
    spec = R.scene_spec(grid, 12, (3, 12), 3, (1.5, 4.0), (1.0, 20.0))
    boxes, spheres = R.generate_scene(spec, 77)
    vox = O.voxelise(grid, boxes, spheres)
    oflu, oL = O.solve(O.params(grid, N, **kw), vox)
    gflu, gL = _solve_gpu(R.make_params(grid, N, **kw), vox=vox)
    _check(gflu, gL, oflu, oL)


@pytest.mark.parametrize("precision", ["fp32", "fp16"])
def test_c128_staged_merge_matches_oracle(precision):
    """128^3: cascade 1 (32^3 probes) is a wide bit-parallel level whose merge
    reads cascade 2 through TMA-staged shared-memory tiles."""
    spec = R.scene_spec(128, 100, (4, 24), 12, (2.0, 6.0), (1.0, 20.0))
    boxes, spheres = R.generate_scene(spec, 31)
    vox = O.voxelise(128, boxes, spheres)
    oflu, oL = O.solve(O.params(128, 5), vox, jump=True)
    gflu, gL = _solve_gpu(R.make_params(128, 5, precision=precision), vox=vox)
    if precision == "fp32":
        _check(gflu, gL, oflu, oL)
    else:
        _check(gflu, gL, oflu, oL, rel=FP16_REL_L2, max_rel=None)


@pytest.mark.parametrize("grid,N", [(64, 5), (128, 5), ((96, 64, 160), 5)])
def test_walk_step_tables_match_the_walk_dda_bit_for_bit(grid, N, monkeypatch):
    """The narrow levels' walks replay per-direction step tables built on the
    host; with RC_WALK_TABLES=0 they run their own DDA.  Both visit the same
    voxels, so every level's radiance is identical bit for bit."""
    g3 = (grid,) * 3 if isinstance(grid, int) else grid
    spec = R.scene_spec(g3, 60, (3, 20), 8, (1.5, 5.0), (1.0, 20.0))
    boxes, spheres = R.generate_scene(spec, 9)
    monkeypatch.delenv("RC_WALK_TABLES", raising=False)
    f1, L1 = _solve_gpu(R.make_params(g3, N), boxes=boxes, spheres=spheres)
    monkeypatch.setenv("RC_WALK_TABLES", "0")
    f2, L2 = _solve_gpu(R.make_params(g3, N), boxes=boxes, spheres=spheres)
    assert np.array_equal(f1, f2)
    for a, b in zip(L1, L2):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("grid,N", [(64, 5), ((96, 64, 160), 5), (256, 6)])
def test_cooperative_walk_groups_match_one_lane_per_item_bit_for_bit(grid, N, monkeypatch):
    """The step-table walk runs G lanes per item (RC_WALK_GROUP = 4, 8, 16,
    32: lane j takes every G-th step, first hits by an OR-scan over the
    group) or one lane per item (1).  All give the same records, so every
    level's radiance and the fluence are identical bit for bit."""
    g3 = (grid,) * 3 if isinstance(grid, int) else grid
    if grid == 256:
        boxes, spheres = R.workload_scene("c256", frame=5)
    else:
        boxes, spheres = R.generate_scene(R.scene_spec(g3, 60, (3, 20), 8, (1.5, 5.0), (1.0, 20.0)), 9)
    out = {}
    for g in ("1", "2", "4", "8", "16", "32"):
        monkeypatch.setenv("RC_WALK_GROUP", g)
        out[g] = _solve_gpu(R.make_params(g3, N), boxes=boxes, spheres=spheres)
    f1, L1 = out["1"]
    for g in ("2", "4", "8", "16", "32"):
        f, L = out[g]
        assert np.array_equal(f, f1), g
        for a, b in zip(L, L1):
            assert np.array_equal(a, b), g


def test_moving_emitters_incremental_update_matches_fresh_solve():
    boxes, spheres = R.workload_scene("c64")
    p = R.make_params(64, 5)
    checks = {0, 1, 9, 40}
    with R.Engine(p) as e:
        e.set_boxes(boxes)
        sph = spheres.copy()
        for f in range(41):
            e.set_spheres(sph)
            if f in checks:
                e.solve()
                gflu = e.fluence().astype(np.float64)
                ob, os_ = O.config_scene("c64", frame=f)
                oflu, _ = O.solve(O.params(64, 5), O.voxelise(64, ob, os_))
                assert rel_l2(gflu, oflu) <= FP32_REL_L2
                assert np.abs(gflu - oflu).max() <= FP32_MAX_REL * oflu.max()
            R.advance_spheres(sph, 64, 1)


def test_incremental_updates_keep_the_volume_exact():
    """Per-frame emitter updates recompose only the regions the spheres left
    and entered.  Small steps (one region per sphere) and long jumps (old and
    new regions apart), a sphere leaving the grid and one growing: after every
    update the composed volume equals a fresh voxelisation bit for bit."""
    boxes, spheres = R.workload_scene("c64")
    rng = np.random.default_rng(5)
    with R.Engine(R.make_params(64, 5)) as e:
        e.set_boxes(boxes)
        sph = spheres.copy()
        for f in range(10):
            e.set_spheres(sph)
            want = O.voxelise(64, boxes, sph)
            assert np.array_equal(e.volume().view(np.uint64), want.view(np.uint64)), f
            k = len(sph)
            sph["centre"][: k // 2] += rng.uniform(-0.75, 0.75, (k // 2, 3))
            sph["centre"][k // 2:] = rng.uniform(-4.0, 68.0, (k - k // 2, 3))
            sph["radius"][0] = 2.0 + f
        e.set_spheres(sph)
        e.solve()
        oflu, _ = O.solve(O.params(64, 5), O.voxelise(64, boxes, sph))
        assert rel_l2(e.fluence().astype(np.float64), oflu) <= FP32_REL_L2


def test_large_and_small_updates_keep_the_volume_exact():
    """An update whose spheres, regions and sphere lists fit 4 KB travels in
    the compose launch's parameters; a larger one (here 120 moving spheres,
    5.8 KB of spheres alone) goes through the pinned staging copy.  Through
    moves of each kind (the sphere count fixed, so only the regions the
    spheres left and entered are recomposed) the composed volume equals a
    fresh voxelisation bit for bit, and the solve matches the oracle."""
    boxes, _ = R.workload_scene("c64")
    rng = np.random.default_rng(11)
    many = np.zeros(120, R.SPHERE_DT)
    many["centre"] = rng.uniform(0.0, 64.0, (120, 3))
    many["radius"] = rng.uniform(1.0, 3.0, 120)
    many["value"]["emission"] = np.float16(2.0).view(np.uint16)
    many["value"]["albedo_occ"] = 0x8000
    with R.Engine(R.make_params(64, 5)) as e:
        e.set_boxes(boxes)
        for sph in (many, many[:6].copy()):
            for f in range(4):  # the first set recomposes the whole grid, then moves
                if f:
                    sph["centre"] += rng.uniform(-0.6, 0.6, (len(sph), 3))
                e.set_spheres(sph)
                want = O.voxelise(64, boxes, sph)
                assert np.array_equal(e.volume().view(np.uint64), want.view(np.uint64)), (len(sph), f)
            e.solve()
            oflu, _ = O.solve(O.params(64, 5), O.voxelise(64, boxes, sph))
            assert rel_l2(e.fluence().astype(np.float64), oflu) <= FP32_REL_L2


def test_empty_scene_is_dark():
    gflu, gL = _solve_gpu(R.make_params(32, 4), vox=volume(np.zeros((32, 32, 32), bool), 0))
    assert not gflu.any() and all(not x.any() for x in gL)


def test_furnace_all_emitting():
    gflu, _ = _solve_gpu(R.make_params(32, 4), vox=volume(np.ones((32, 32, 32), bool), O.float_to_half(3.0)))
    assert np.abs(gflu - 4 * math.pi * 3.0).max() <= 1e-5 * 4 * math.pi * 3.0


def test_furnace_cavity_and_slab_single_cascade():
    occ = np.ones((32, 32, 32), bool)
    occ[8:24, 8:24, 8:24] = False
    gflu, _ = _solve_gpu(R.make_params(32, 1, interval0=64), vox=volume(occ, O.float_to_half(5.0)))
    assert np.abs(gflu - 4 * math.pi * 5.0).max() <= 1e-5 * 4 * math.pi * 5.0

    occ = np.zeros((32, 32, 32), bool)
    occ[:, :, 0:3] = True
    em = np.where(occ, O.float_to_half(3.0), 0).astype(np.uint16)
    occ[:, :, 10:12] = True
    gflu, _ = _solve_gpu(R.make_params(32, 1, interval0=64), vox=volume(occ, em))
    f = gflu.reshape(16, 16, 16, 3)
    assert f[:, :, 6:, :].max() == 0.0 and f[:, :, 2:5, :].min() > 0.0


def test_mirror_symmetry_on_gpu():
    spec = R.scene_spec(32, 10, (3, 10), 3, (1.5, 3.5), (1.0, 20.0))
    boxes, spheres = R.generate_scene(spec, 5)
    vox = R.voxelise_host(32, boxes, spheres)
    p = R.make_params(32, 4)
    f, _ = _solve_gpu(p, vox=vox)
    mf, _ = _solve_gpu(p, vox=mirror_x(vox, 32))
    mf = mf.reshape(16, 16, 16, 3)[:, :, ::-1].reshape(-1, 3)
    assert np.abs(f - mf).max() <= 1e-5 * f.max()


def test_c256_frame0_matches_fp64_oracle(walk):
    boxes, spheres = R.workload_scene("c256")
    vox = O.voxelise(256, boxes, spheres)
    gflu, gL = _solve_gpu(R.make_params(256, 6), boxes=boxes, spheres=spheres)
    oflu, oL = O.solve(O.params(256, 6), vox, jump=True)
    _check(gflu, gL, oflu, oL)


@pytest.mark.parametrize("frame", [1, 239])
def test_c256_later_frames_match_fp64_oracle(frame):
    """Frames 1 and 239 of the moving-emitter workload, reached by incremental
    emitter updates frame after frame, against the oracle's fresh solve."""
    boxes, spheres = R.workload_scene("c256")
    with R.Engine(R.make_params(256, 6)) as e:
        e.set_boxes(boxes)
        sph = spheres.copy()
        for _ in range(frame):
            e.set_spheres(sph)
            R.advance_spheres(sph, 256, 1)
        e.set_spheres(sph)
        e.solve()
        gflu = e.fluence().astype(np.float64)
    ob, os_ = O.config_scene("c256", frame=frame)
    oflu, _ = O.solve(O.params(256, 6), O.voxelise(256, ob, os_), jump=True)
    assert rel_l2(gflu, oflu) <= FP32_REL_L2
    assert np.abs(gflu - oflu).max() <= FP32_MAX_REL * oflu.max()


def test_c256_size_independent_properties():
    """Full size: energy bounds, furnace and FP16 error."""
    boxes, spheres = R.workload_scene("c256", frame=120)
    p = R.make_params(256, 6)
    gflu, _ = _solve_gpu(p, boxes=boxes, spheres=spheres)
    emax = float(np.max(spheres["value"]["emission"].view(np.float16).astype(np.float64)))
    assert gflu.min() >= 0.0 and gflu.max() <= 4 * math.pi * emax * (1 + 1e-6)
    h, _ = _solve_gpu(R.make_params(256, 6, precision="fp16"), boxes=boxes, spheres=spheres)
    assert rel_l2(h, gflu) <= FP16_REL_L2
    full = np.zeros(1, R.BOX_DT)
    full[0]["lo"], full[0]["hi"] = (0, 0, 0), (256, 256, 256)
    full[0]["value"]["albedo_occ"] = 0x8000
    full[0]["value"]["emission"] = [O.float_to_half(2.0)] * 3
    ff, _ = _solve_gpu(p, boxes=full, spheres=np.zeros(0, R.SPHERE_DT))
    assert np.abs(ff - 4 * math.pi * 2.0).max() <= 1e-5 * 8 * math.pi
