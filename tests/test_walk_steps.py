"""The walk step tables the narrow levels' GPU walk replays (rcx::walk_steps,
host code in csrc/rc_host.cpp) against an independent restatement of the
walk: exact rational crossing times (as oracle/oracle_np.py's _march), ties
x before y before z, a voxel belongs to the interval when it is entered at a
distance in [b_lo, b_hi), the start voxel first at cascade 0.  Each table
entry's (phase, coarse cell) must decode to that walk's next voxel offset,
and the table must end where every probe of the level has left the grid on
some axis.  CPU only: the driver is built from the host sources with g++."""
import math
import os
import subprocess
from fractions import Fraction

import pytest

from oracle import oracle_np as ON

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "radiancecascade_gb300", "csrc")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("walk") / "walk_steps_driver")
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", os.path.join(ROOT, "tests", "walk_steps_driver.cpp"),
                    os.path.join(CSRC, "rc_host.cpp"), "-I", CSRC, "-I", os.path.join(ROOT, "include"), "-o", exe],
                   check=True, capture_output=True, text=True)
    return exe


def _tables(exe, grid, num, level):
    out = subprocess.run([exe, *map(str, grid), str(num), str(level)], check=True, capture_output=True,
                         text=True).stdout.split()
    vals, k, tabs = list(map(int, out)), 0, []
    while k < len(vals):
        d, n = vals[k], vals[k + 1]
        k += 2
        tabs.append([(vals[k + 2 * j], vals[k + 2 * j + 1]) for j in range(n)])
        k += 2 * n
        assert d == len(tabs) - 1
    return tabs


def _walk(D, s, M, grid, blo, bhi, test_start):
    """Voxel offsets from the probe's cell origin, in walk order."""
    h = s // 2
    S = sum(c * c for c in D)
    reach = math.ceil(math.sqrt(sum(g * g for g in grid))) + 1
    blo, bhi = min(blo, reach), min(bhi, reach)
    V = [h - (1 if D[a] < 0 else 0) for a in range(3)]
    out = []

    def gone():  # every probe of the level outside the grid on some axis
        return any(V[a] >= grid[a] or V[a] + (M[a] - 1) * s < 0 for a in range(3))

    if test_start and blo == 0:
        if gone():
            return out
        out.append(tuple(V))
    k = [0, 0, 0]
    while True:
        times = [Fraction(k[a] + 1, abs(D[a])) if D[a] != 0 else None for a in range(3)]
        best = min((a for a in range(3) if times[a] is not None), key=lambda a: (times[a], a))
        t = times[best]
        k[best] += 1
        V[best] += 1 if D[best] > 0 else -1
        d2 = t * t * S
        if d2 >= bhi * bhi:
            return out
        if d2 >= blo * blo:
            if gone():
                return out
            out.append(tuple(V))


def _decode(entry, l2s):
    phase, cell = entry
    s = 1 << l2s
    p = (phase & (s - 1), (phase >> l2s) & (s - 1), phase >> (2 * l2s))
    c = [((cell >> (8 * a)) & 0xFF) - (256 if (cell >> (8 * a)) & 0x80 else 0) for a in range(3)]
    return tuple(c[a] * s + p[a] for a in range(3))


@pytest.mark.parametrize("grid,num,level", [
    ((64, 64, 64), 5, 0), ((64, 64, 64), 5, 2), ((64, 64, 64), 5, 3), ((64, 64, 64), 5, 4),
    ((48, 32, 80), 4, 2), ((48, 32, 80), 4, 3),
])
def test_step_tables_replay_the_exact_walk(driver, grid, num, level):
    tabs = _tables(driver, grid, num, level)
    s = 2 << level
    l2s = s.bit_length() - 1
    M = [g // s for g in grid]
    n = 4 << level
    b = ON.intervals(num, 1, 4)
    dirs = ON.directions(n)
    assert len(tabs) == n * n
    stride = max(1, len(dirs) // 256)  # every direction up to 256 per level, else a spread sample
    for d in range(0, len(dirs), stride):
        want = _walk(dirs[d], s, M, grid, b[level], b[level + 1], level == 0)
        got = [_decode(e, l2s) for e in tabs[d]]
        assert got == want, (grid, level, d)
