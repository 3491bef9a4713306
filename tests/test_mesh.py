"""Triangle-mesh voxelisation: the oracle's exact separating-axis test pinned
by known answers and by a third restatement (Python integers), and the OBJ
loader against the reference's own assets when they are present."""
import os

import numpy as np
import pytest

import radiancecascade_gb300 as R
from oracle import oracle as O

# Directory of the reference renderer's OBJ assets (its resources/ folder);
# the asset test is skipped when RC_REFERENCE_ASSETS is unset.
REF = os.environ.get("RC_REFERENCE_ASSETS", "")


def _mats(n):
    m = np.zeros(n, R.VOXEL_DT)
    m["albedo_occ"] = 0x8000 | np.arange(1, n + 1)
    return m


def _grid(vox, g):
    return (vox["albedo_occ"] != 0).reshape(g, g, g)  # [z][y][x]


def test_triangle_inside_one_voxel():
    pos = np.array([[1.2, 1.2, 1.2], [1.8, 1.2, 1.2], [1.2, 1.8, 1.7]], np.float32)
    v = _grid(O.voxelise_mesh(4, pos, [[0, 1, 2]], None, _mats(1)), 4)
    assert v.sum() == 1 and v[1, 1, 1]


def test_quad_on_a_voxel_face_marks_both_sides():
    pos = np.array([[0.5, 0.5, 2.0], [3.5, 0.5, 2.0], [3.5, 3.5, 2.0], [0.5, 3.5, 2.0]], np.float32)
    v = _grid(O.voxelise_mesh(4, pos, [[0, 1, 2], [0, 2, 3]], None, _mats(1)), 4)
    assert v[1].all() and v[2].all() and not v[0].any() and not v[3].any()


def test_later_triangle_wins():
    pos = np.array([[0.2, 0.2, 0.5], [3.8, 0.2, 0.5], [0.2, 3.8, 0.5]], np.float32)
    out = O.voxelise_mesh(4, pos, [[0, 1, 2], [2, 1, 0]], [0, 1], _mats(2))
    occ = out["albedo_occ"] != 0
    assert occ.sum() > 0 and np.all(out["albedo_occ"][occ] == (0x8000 | 2))


def _sat_python(tri, x, y, z):
    c = (256 * x + 128, 256 * y + 128, 256 * z + 128)
    q = [[tri[k][a] - c[a] for a in range(3)] for k in range(3)]
    e = [[q[(i + 1) % 3][a] - q[i][a] for a in range(3)] for i in range(3)]
    axes = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
    n = (e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
         e[0][0] * e[1][1] - e[0][1] * e[1][0])
    axes.append(n)
    for ei in e:
        for u in ((1, 0, 0), (0, 1, 0), (0, 0, 1)):
            axes.append((ei[1] * u[2] - ei[2] * u[1], ei[2] * u[0] - ei[0] * u[2], ei[0] * u[1] - ei[1] * u[0]))
    for a in axes:
        p = [a[0] * v[0] + a[1] * v[1] + a[2] * v[2] for v in q]
        r = 128 * (abs(a[0]) + abs(a[1]) + abs(a[2]))
        if min(p) > r or max(p) < -r:
            return False
    return True


def test_oracle_matches_a_python_integer_restatement():
    rng = np.random.default_rng(11)
    g = 6
    for trial in range(40):
        pos = rng.uniform(-1, g + 1, (3, 3)).astype(np.float32)
        if trial % 4 == 0:  # snap to voxel faces to exercise touching
            pos = np.round(pos).astype(np.float32)
        got = _grid(O.voxelise_mesh(g, pos, [[0, 1, 2]], None, _mats(1)), g)
        tri = [[int(round(float(v) * 256.0)) for v in p] for p in pos]
        want = np.zeros((g, g, g), bool)
        for z in range(g):
            for y in range(g):
                for x in range(g):
                    want[z, y, x] = _sat_python(tri, x, y, z)
        assert np.array_equal(got, want), trial


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="RC_REFERENCE_ASSETS not set to the assets folder")
def test_obj_loader_on_reference_assets():
    for rel in ("test_room/test_room.obj", "cube/cube.obj"):
        path = os.path.join(REF, rel)
        m = R.load_obj(path)
        faces = []
        with open(path) as f:
            for line in f:
                t = line.split()
                if t and t[0] == "f":
                    faces.append([int(v.split("/")[0]) - 1 for v in t[1:]])
        assert len(m["indices"]) == sum(len(fc) - 2 for fc in faces)
        # fan triangulation with the winding reversed (src/primitives.rs:369-376)
        assert list(m["indices"][0]) == [faces[0][2], faces[0][1], faces[0][0]]
        g = R.mesh_to_grid(m["positions"], 32)
        assert g.min() >= 1.0 - 1e-4 and g.max() <= 31.0 + 1e-4
        vox = O.voxelise_mesh(32, g, m["indices"], m["tri_material"], R.mesh_materials(m["materials"]))
        assert (vox["albedo_occ"] != 0).sum() > 0
    assert R.load_obj(os.path.join(REF, "test_room/test_room.obj"))["light"] is None
