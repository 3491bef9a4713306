"""The emitter update's host logic (csrc/rc_host.cpp: update_regions,
sphere_lists) against brute force on small grids: every voxel that a moving
sphere covers before or after the move lies in a recomposed region, and every
sphere that covers a voxel of a region is in that region's sphere list (the
kernel tests only the listed spheres).  Voxel (x, y, z) is inside a sphere
when its centre ((2x+1)·128, ...) in 1/256 voxel is within the radius."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "radiancecascade_gb300", "csrc")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("regions") / "emitter_regions_driver")
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", os.path.join(ROOT, "tests", "emitter_regions_driver.cpp"),
                    os.path.join(CSRC, "rc_host.cpp"), "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def _covered(grid, sph):
    """[z][y][x] mask of the voxels inside sphere (cx, cy, cz, r)."""
    gx, gy, gz = grid
    z, y, x = np.meshgrid(np.arange(gz), np.arange(gy), np.arange(gx), indexing="ij")
    cx, cy, cz, r = sph
    d = ((2 * x + 1) * 128 - cx) ** 2 + ((2 * y + 1) * 128 - cy) ** 2 + ((2 * z + 1) * 128 - cz) ** 2
    return d <= r * r


def _run(exe, grid, old, new):
    lines = ["%d %d %d %d" % (*grid, len(old))] + ["%d %d %d %d" % tuple(s) for s in list(old) + list(new)]
    out = subprocess.run([exe], input="\n".join(lines), check=True, capture_output=True, text=True).stdout.split()
    v = list(map(int, out))
    nreg, listed = v[0], v[1]
    regs = [v[2 + 8 * r: 10 + 8 * r] for r in range(nreg)]
    lst = v[2 + 8 * nreg: 2 + 8 * nreg + listed]
    return regs, lst


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_regions_cover_every_changed_voxel_and_lists_every_covering_sphere(driver, seed):
    rng = np.random.default_rng(seed)
    grid = (48, 40, 64)
    n = 24
    old = np.stack([rng.integers(-8 * 256, (g + 8) * 256, n) for g in grid] + [rng.integers(256, 7 * 256, n)], 1)
    new = old.copy()
    step = rng.integers(-200, 201, (n, 3))
    new[:, :3] += step
    jump = rng.random(n) < 0.3  # some spheres jump far, some grow
    new[jump, :3] = np.stack([rng.integers(0, g * 256, jump.sum()) for g in grid], 1)
    new[rng.random(n) < 0.2, 3] += 512
    regs, lst = _run(driver, grid, old, new)
    gx, gy, gz = grid
    inreg = np.zeros((gz, gy, gx), bool)
    cover_new = [_covered(grid, s) for s in new]
    for w0, w1, y0, y1, z0, z1, s0, sn in regs:
        box = np.zeros_like(inreg)
        box[z0:z1, y0:y1, 32 * w0:min(32 * w1, gx)] = True
        inreg |= box
        listed = set(range(n)) if sn < 0 else set(lst[s0:s0 + sn])
        if sn >= 0:
            assert lst[s0:s0 + sn] == sorted(lst[s0:s0 + sn])
        for i in range(n):
            if (cover_new[i] & box).any():
                assert i in listed, (i, (w0, w1, y0, y1, z0, z1))
    for i in range(n):
        changed = _covered(grid, old[i]) | cover_new[i]
        assert not (changed & ~inreg).any(), i
