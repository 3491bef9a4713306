"""Mesh voxelisation on the GPU: bit-exact against the oracle, and the solve
of a voxelised mesh scene against the FP64 oracle (FP32: rel-L2 <= 1e-4)."""
import numpy as np
import pytest

import radiancecascade_gb300 as R
from oracle import oracle as O
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def test_random_triangles_bit_exact():
    rng = np.random.default_rng(4)
    g = 32
    n = 300
    pos = rng.uniform(-3, g + 3, (3 * n, 3)).astype(np.float32)
    small = rng.random(n) < 0.7  # most triangles small, some spanning the grid
    for t in np.nonzero(small)[0]:
        c = rng.uniform(0, g, 3)
        pos[3 * t:3 * t + 3] = (c + rng.uniform(-1.5, 1.5, (3, 3))).astype(np.float32)
    pos[:30] = np.round(pos[:30])  # vertices on voxel corners
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    mats = np.zeros(5, R.VOXEL_DT)
    mats["albedo_occ"] = 0x8000 | np.arange(1, 6)
    mats["emission"][:, 0] = np.arange(5) * 1000
    tm = rng.integers(0, 5, n).astype(np.uint16)
    want = O.voxelise_mesh(g, pos, idx, tm, mats)
    with R.Engine(R.make_params(g, 3)) as e:
        e.set_mesh(pos, idx, mats, tm)
        got = e.volume()
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_room_mesh_scene_matches_fp64_oracle():
    g = 64
    pos, idx, tm, mats = R.room_mesh(g)
    spec = R.scene_spec(g, 0, (4, 8), 3, (2.0, 4.0), (1.0, 20.0))
    _, spheres = R.generate_scene(spec, 9)
    vox = O.voxelise_mesh(g, pos, idx, tm, mats)
    # spheres composed on top, as the context does
    sv = O.voxelise(g, np.zeros(0, R.BOX_DT), spheres)
    occ = sv["albedo_occ"] != 0
    vox[occ] = sv[occ]
    oflu, _ = O.solve(O.params(g, 5), vox)
    with R.Engine(R.make_params(g, 5)) as e:
        e.set_mesh(pos, idx, mats, tm)
        e.set_spheres(spheres)
        assert np.array_equal(e.volume().view(np.uint64), vox.view(np.uint64))
        e.solve()
        gflu = e.fluence().astype(np.float64)
    assert rel_l2(gflu, oflu) <= 1e-4
    assert oflu.max() > 0
