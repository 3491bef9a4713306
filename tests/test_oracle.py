"""Pins the CPU oracle (test infrastructure) before anything is checked against it.

The reference has no radiance-cascade implementation, tests or golden vectors
(its only GPU programs are src/shader.wgsl and src/light.wgsl), so the oracle
is pinned by (1) an independent Python restatement of the same method, (2)
known-answer tests that hold exactly by construction, and (3) the committed
golden fixtures in tests/golden/.
"""
import math
import os

import numpy as np
import pytest

from oracle import oracle as O
from oracle import oracle_np as T
from tests.helpers import mirror_x, mirror_y, rel_l2, volume

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _twin_spec(grid, nb, edge, ns, rad, em):
    return dict(grid=list(grid), num_boxes=nb, box_edge_min=edge[0], box_edge_max=edge[1], num_spheres=ns,
                radius_min=rad[0], radius_max=rad[1], emission_min=em[0], emission_max=em[1],
                albedo_min=0.2, albedo_max=0.9, speed=0.5)


@pytest.mark.parametrize("grid,N,seed,kw", [
    ((16, 16, 16), 3, 7, {}),
    ((16, 8, 24), 2, 11, {}),
    ((16, 16, 16), 2, 3, dict(spacing0=4, dir_res0=2, interval0=2, ratio=3)),
])
def test_oracle_matches_independent_python_restatement(grid, N, seed, kw):
    spec = O.scene_spec(grid, 5, 2, 6, 2, 1.0, 2.5, 1.0, 20.0)
    boxes, spheres = O.generate(spec, seed)
    O.advance(spheres, grid, 3)
    vox = O.voxelise(grid, boxes, spheres)

    tb, ts = T.generate(_twin_spec(grid, 5, (2, 6), 2, (1.0, 2.5), (1.0, 20.0)), seed)
    T.advance(ts, list(grid), 3)
    occ, em, ao = T.voxelise(list(grid), tb, ts)
    assert np.array_equal(vox["albedo_occ"].reshape(occ.shape), ao)
    assert occ.any()

    p = O.params(grid, N, **kw)
    flu, L = O.solve(p, vox)
    tflu, tL = T.solve(list(grid), occ, em, N, spacing0=kw.get("spacing0", 2), dir_res0=kw.get("dir_res0", 4),
                       b1=kw.get("interval0", 1), ratio=kw.get("ratio", 4))
    assert flu.max() > 0
    assert rel_l2(flu, tflu) <= 1e-12
    for a, b in zip(L, tL):
        assert a.shape == b.shape
        assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max())


def test_generator_and_motion_match_python_restatement():
    g = (64, 64, 64)
    spec = O.scene_spec(g, 24, 4, 20, 4, 2.0, 5.0, 1.0, 20.0)
    boxes, spheres = O.generate(spec, 1001)
    tb, ts = T.generate(_twin_spec(g, 24, (4, 20), 4, (2.0, 5.0), (1.0, 20.0)), 1001)
    for b, t in zip(boxes, tb):
        assert list(b["lo"]) == t["lo"] and list(b["hi"]) == t["hi"] and b["value"]["albedo_occ"] == t["albedo_occ"]
    O.advance(spheres, g, 239)
    T.advance(ts, list(g), 239)
    for s, t in zip(spheres, ts):
        assert list(s["centre"]) == t["centre"] and s["radius"] == t["radius"]
        assert tuple(s["value"]["emission"]) == t["emission"]
        # the sphere stays inside the grid
        assert all(t["radius"] <= c <= 64 - t["radius"] for c in t["centre"])


def test_jump_walk_equals_walk_from_probe_centre():
    boxes, spheres = O.config_scene("c64", frame=5)
    vox = O.voxelise(64, boxes, spheres)
    p = O.params(64, 5)
    f0, L0 = O.solve(p, vox, jump=False)
    f1, L1 = O.solve(p, vox, jump=True)
    assert np.array_equal(f0, f1)
    for a, b in zip(L0, L1):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("n", [2, 4, 8, 16, 64])
def test_solid_angles_cover_the_sphere(n):
    om = O.solid_angles(n)
    assert om.min() > 0
    assert abs(om.sum() - 4 * math.pi) < 1e-12
    assert np.abs(om - T.solid_angles(n)).max() < 1e-13


def test_crossing_counts_are_exact():
    for D in [(1, 2, 2), (3, 4, 0), (5, -3, 8), (-7, 1, -8)]:
        S = sum(c * c for c in D)
        for b in [0, 1, 5, 21, 85, 341, 1365]:
            for a in D:
                k = O.crossings_before(b, a, S)
                # k*sqrt(S) < b*|a| <= (k+1)*sqrt(S)
                assert k * k * S < b * b * a * a or k == 0
                assert (k + 1) ** 2 * S >= b * b * a * a


def test_empty_scene_is_dark():
    G = 32
    vox = volume(np.zeros((G, G, G), bool), 0)
    flu, L = O.solve(O.params(G, 4), vox)
    assert not flu.any()
    assert all(not x.any() for x in L)


def test_furnace_all_emitting():
    """Every voxel opaque with radiance E: every level-0 ray hits its first voxel -> 4*pi*E."""
    G = 32
    E = O.float_to_half(3.0)
    flu, L = O.solve(O.params(G, 4), volume(np.ones((G, G, G), bool), E))
    assert np.abs(flu - 4 * math.pi * 3.0).max() < 1e-12


def test_furnace_enclosed_cavity_single_cascade():
    """Empty cavity inside emissive walls; one cascade whose interval reaches every wall."""
    G = 32
    occ = np.ones((G, G, G), bool)
    occ[8:24, 8:24, 8:24] = False
    E = O.float_to_half(5.0)
    flu, _ = O.solve(O.params(G, 1, interval0=64), volume(occ, E))
    assert np.abs(flu - 4 * math.pi * 5.0).max() < 1e-12


def test_opaque_slab_blocks_all_light_single_cascade():
    G = 32
    occ = np.zeros((G, G, G), bool)
    occ[:, :, 0:3] = True
    em = np.where(occ, O.float_to_half(3.0), 0).astype(np.uint16)
    occ[:, :, 10:12] = True  # non-emissive slab across the whole grid
    flu, _ = O.solve(O.params(G, 1, interval0=64), volume(occ, em))
    f = flu.reshape(16, 16, 16, 3)
    assert f[:, :, 6:, :].max() == 0.0  # probes at x >= 13: behind the slab
    assert f[:, :, 2:5, :].min() > 0.0  # probes between emitter and slab


@pytest.mark.parametrize("mirror", ["x", "y"])
def test_mirror_symmetry(mirror):
    G = 32
    spec = O.scene_spec(G, 10, 3, 10, 3, 1.5, 3.5, 1.0, 20.0)
    boxes, spheres = O.generate(spec, 5)
    vox = O.voxelise(G, boxes, spheres)
    p = O.params(G, 4)
    flu, _ = O.solve(p, vox)
    mv = mirror_x(vox, G) if mirror == "x" else mirror_y(vox, G)
    mflu, _ = O.solve(p, mv)
    M = G // 2
    f = flu.reshape(M, M, M, 3)
    mf = mflu.reshape(M, M, M, 3)
    mf = mf[:, :, ::-1] if mirror == "x" else mf[:, ::-1, :]
    assert flu.max() > 0
    assert np.abs(f - mf).max() <= 1e-12 * flu.max()


def test_fp32_port_tracks_fp64_oracle():
    boxes, spheres = O.config_scene("c64")
    vox = O.voxelise(64, boxes, spheres)
    p = O.params(64, 5)
    f64, _ = O.solve(p, vox)
    f32, _ = O.solve(p, vox, dtype=np.float32, jump=True)
    assert rel_l2(f32, f64) < 1e-6


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz")))
def test_oracle_reproduces_golden_fixture(name):
    z = np.load(os.path.join(GOLDEN, name))
    p = O.params(tuple(int(x) for x in z["grid"]), int(z["num_cascades"]), precision=0)
    flu, L = O.solve(p, z["voxels"].view(O.VOXEL_DT))
    assert rel_l2(flu, z["fluence"]) <= 1e-12
    for i, x in enumerate(L):
        assert np.abs(x - z["radiance_%d" % i]).max() <= 1e-12 * max(1.0, np.abs(x).max())
