"""Second, independent restatement of the radiance-cascade method in Python.

TEST INFRASTRUCTURE ONLY: used by tests/ to pin the C++ oracle
(oracle/rc_oracle.cpp) on tiny grids.  It shares no code with the C++ oracle
or with the product and deliberately computes some steps another way:

  * the DDA compares crossing times as Python fractions.Fraction values;
  * the merge gathers all 32 taps (8 parent probes x 4 child directions)
    directly instead of averaging the child directions first;
  * texel solid angles use Girard's theorem (spherical excess) instead of
    Van Oosterom & Strackee.

The reference repository has no radiance-cascade code to cite; the method is
Sannikov's radiance cascades (2023) with Amanatides & Woo voxel traversal and
the Engelhardt & Dachsbacher octahedral map.
"""
from __future__ import annotations

import math
from fractions import Fraction

import numpy as np

M64 = (1 << 64) - 1
OPAQUE = 0x8000


# ---------------------------------------------------------------- generator
def _mix64(z: int) -> int:
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


class _Rng:
    def __init__(self, seed: int, stream: int):
        self.s = _mix64(seed ^ _mix64(stream ^ 0xD1B54A32D192ED03))

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & M64
        return _mix64(self.s)

    def uniform(self) -> float:
        return (self.next() >> 11) * 2.0 ** -53


def half_bits(x: float) -> int:
    """float32 value -> binary16 bits, round to nearest even (via numpy)."""
    return int(np.array([x], dtype=np.float32).astype(np.float16).view(np.uint16)[0])


def half_value(h: int) -> float:
    return float(np.array([h], dtype=np.uint16).view(np.float16)[0])


def generate(spec: dict, seed: int):
    """Return (boxes, spheres) as lists of dicts, same draw order as the spec."""
    G = spec["grid"]
    boxes, spheres = [], []
    for b in range(spec["num_boxes"]):
        r = _Rng(seed, b)
        e = []
        for a in range(3):
            span = spec["box_edge_max"] - spec["box_edge_min"] + 1
            v = spec["box_edge_min"] + math.floor(r.uniform() * span)
            e.append(min(v, spec["box_edge_max"], G[a]))
        lo = []
        for a in range(3):
            lo.append(min(math.floor(r.uniform() * (G[a] - e[a] + 1)), G[a] - e[a]))
        alb = []
        for _ in range(3):
            x = spec["albedo_min"] + r.uniform() * (spec["albedo_max"] - spec["albedo_min"])
            alb.append(min(max(math.floor(x * 31.0 + 0.5), 0), 31))
        boxes.append(dict(lo=lo, hi=[lo[a] + e[a] for a in range(3)], emission=(0, 0, 0),
                          albedo_occ=OPAQUE | (alb[0] << 10) | (alb[1] << 5) | alb[2]))
    for s in range(spec["num_spheres"]):
        r = _Rng(seed, (1 << 32) + s)
        rad = spec["radius_min"] + r.uniform() * (spec["radius_max"] - spec["radius_min"])
        c = []
        for a in range(3):
            u = r.uniform()
            c.append(rad + u * (G[a] - 2.0 * rad) if G[a] >= 2.0 * rad else 0.5 * G[a])
        em = []
        for _ in range(3):
            x = spec["emission_min"] + r.uniform() * (spec["emission_max"] - spec["emission_min"])
            em.append(half_bits(float(np.float32(x))))
        while True:
            v = [2.0 * r.uniform() - 1.0 for _ in range(3)]
            q = v[0] * v[0] + v[1] * v[1] + v[2] * v[2]
            if 1e-6 < q <= 1.0:
                break
        inv = spec["speed"] / math.sqrt(q)
        spheres.append(dict(centre=c, radius=rad, velocity=[x * inv for x in v],
                            emission=tuple(em), albedo_occ=OPAQUE))
    return boxes, spheres


def advance(spheres, grid, frames):
    for _ in range(frames):
        for s in spheres:
            for a in range(3):
                lo, hi = s["radius"], grid[a] - s["radius"]
                if hi < lo:
                    s["centre"][a] = 0.5 * grid[a]
                    continue
                c = s["centre"][a] + s["velocity"][a]
                if c < lo:
                    c = 2.0 * lo - c
                    s["velocity"][a] = -s["velocity"][a]
                elif c > hi:
                    c = 2.0 * hi - c
                    s["velocity"][a] = -s["velocity"][a]
                s["centre"][a] = c


def voxelise(grid, boxes, spheres):
    """-> (occ[z,y,x] bool, emission[z,y,x,3] float64, albedo_occ[z,y,x] uint16)."""
    Gx, Gy, Gz = grid
    ao = np.zeros((Gz, Gy, Gx), np.uint16)
    em = np.zeros((Gz, Gy, Gx, 3), np.uint16)
    for b in boxes:
        lo = [max(b["lo"][a], 0) for a in range(3)]
        hi = [min(b["hi"][a], grid[a]) for a in range(3)]
        ao[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = b["albedo_occ"]
        em[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = b["emission"]
    zz, yy, xx = np.meshgrid(np.arange(Gz), np.arange(Gy), np.arange(Gx), indexing="ij")
    for s in spheres:
        cq = [int(round_half_away(s["centre"][a] * 256.0)) for a in range(3)]
        rq = int(round_half_away(s["radius"] * 256.0))
        d2 = ((2 * xx + 1) * 128 - cq[0]) ** 2 + ((2 * yy + 1) * 128 - cq[1]) ** 2 \
            + ((2 * zz + 1) * 128 - cq[2]) ** 2
        inside = d2 <= rq * rq
        ao[inside] = s["albedo_occ"]
        em[inside] = s["emission"]
    emf = em.view(np.float16).astype(np.float64)
    return (ao & OPAQUE) != 0, emf, ao


def round_half_away(x: float) -> int:
    return int(math.floor(abs(x) + 0.5)) * (1 if x >= 0 else -1)


# ---------------------------------------------------------------- geometry
def directions(n: int):
    out = []
    for k in range(n):
        for j in range(n):
            u = Fraction(2 * j + 1, n) - 1
            v = Fraction(2 * k + 1, n) - 1
            z = 1 - abs(u) - abs(v)
            if z >= 0:
                d = (u, v, z)
            else:
                d = ((1 - abs(v)) * (1 if u > 0 else -1), (1 - abs(u)) * (1 if v > 0 else -1), z)
            out.append(tuple(int(c * n) for c in d))
    return out


def intervals(num, b1, ratio):
    b = [0, b1]
    while len(b) < num + 1:
        b.append(b[-1] * ratio + b1)
    return b


def _march(occ, O, D, blo, bhi):
    """First opaque voxel entered at a distance in [blo, bhi), or None.

    Crossing j on axis a happens at ray parameter t = j / |D_a| (ray O + t D);
    its distance is t * |D|.  Exact comparisons with Fractions."""
    Gz, Gy, Gx = occ.shape
    S = sum(c * c for c in D)
    V = [O[a] - (1 if D[a] < 0 else 0) for a in range(3)]
    if blo == 0 and occ[V[2], V[1], V[0]]:
        return tuple(V)
    k = [0, 0, 0]
    while True:
        times = [Fraction(k[a] + 1, abs(D[a])) if D[a] != 0 else None for a in range(3)]
        best = min((a for a in range(3) if times[a] is not None), key=lambda a: (times[a], a))
        t = times[best]
        k[best] += 1
        V[best] += 1 if D[best] > 0 else -1
        # distance^2 = t^2 * S compared with b^2
        d2 = t * t * S
        if d2 >= bhi * bhi:
            return None
        if not (0 <= V[0] < Gx and 0 <= V[1] < Gy and 0 <= V[2] < Gz):
            return None
        if d2 >= blo * blo and occ[V[2], V[1], V[0]]:
            return tuple(V)


def solid_angles(n: int):
    """Girard's theorem on the radial projection of each texel polygon."""
    def sph_poly_area(P):
        P = [np.array(p, float) / np.linalg.norm(p) for p in P]
        m = len(P)
        tot = 0.0
        for i in range(m):
            A, B, C = P[i - 1], P[i], P[(i + 1) % m]
            t1 = A - np.dot(A, B) * B
            t2 = C - np.dot(C, B) * B
            tot += math.atan2(np.linalg.norm(np.cross(t1, t2)), np.dot(t1, t2))
        return tot - (m - 2) * math.pi

    def clip(poly, below):
        out = []
        f = (lambda q: 1.0 - q[0] - q[1]) if below else (lambda q: q[0] + q[1] - 1.0)
        for i in range(len(poly)):
            A, B = poly[i], poly[(i + 1) % len(poly)]
            fa, fb = f(A), f(B)
            if fa >= 0:
                out.append(A)
            if fa * fb < 0:
                t = fa / (fa - fb)
                out.append((A[0] + t * (B[0] - A[0]), A[1] + t * (B[1] - A[1])))
        return out

    res = np.zeros(n * n)
    for k in range(n):
        for j in range(n):
            us = sorted(abs(2.0 * x / n - 1.0) for x in (j, j + 1))
            vs = sorted(abs(2.0 * x / n - 1.0) for x in (k, k + 1))
            sq = [(us[0], vs[0]), (us[1], vs[0]), (us[1], vs[1]), (us[0], vs[1])]
            tot = 0.0
            for lower in (False, True):
                poly = clip(sq, below=not lower)
                # drop repeated vertices created by clipping through a corner
                dedup = []
                for q in poly:
                    if not dedup or abs(q[0] - dedup[-1][0]) + abs(q[1] - dedup[-1][1]) > 1e-15:
                        dedup.append(q)
                if len(dedup) > 1 and abs(dedup[0][0] - dedup[-1][0]) + abs(dedup[0][1] - dedup[-1][1]) <= 1e-15:
                    dedup.pop()
                if len(dedup) < 3:
                    continue
                if lower:
                    P3 = [(1 - c, 1 - a, 1 - a - c) for a, c in dedup]
                else:
                    P3 = [(a, c, 1 - a - c) for a, c in dedup]
                tot += sph_poly_area(P3)
            res[k * n + j] = tot
    return res


# ---------------------------------------------------------------- solver
def solve(grid, occ, emission, num_cascades, spacing0=2, dir_res0=4, b1=1, ratio=4):
    """Returns (fluence[P0,3], [L_i planar [3][dirs][Mz][My][Mx]] for each level)."""
    N = num_cascades
    b = intervals(N, b1, ratio)
    levels = []
    for i in range(N):
        s = spacing0 << i
        levels.append(dict(s=s, M=[grid[a] // s for a in range(3)], n=dir_res0 << i,
                           blo=b[i], bhi=b[i + 1]))
    L = [None] * N
    for i in range(N - 1, -1, -1):
        lv = levels[i]
        dirs = directions(lv["n"])
        Mx, My, Mz = lv["M"]
        Li = np.zeros((3, len(dirs), Mz, My, Mx))
        for di, D in enumerate(dirs):
            for mz in range(Mz):
                for my in range(My):
                    for mx in range(Mx):
                        O = [(2 * m + 1) * lv["s"] // 2 for m in (mx, my, mz)]
                        h = _march(occ, O, D, lv["blo"], lv["bhi"])
                        if h is not None:
                            Li[:, di, mz, my, mx] = emission[h[2], h[1], h[0]]
                        elif i < N - 1:
                            Li[:, di, mz, my, mx] = _merge(L[i + 1], levels[i + 1], lv, di, (mx, my, mz))
        L[i] = Li
    l0 = levels[0]
    om = solid_angles(l0["n"])
    P0 = l0["M"][0] * l0["M"][1] * l0["M"][2]
    flu = np.einsum("d,cdzyx->zyxc", om, L[0]).reshape(P0, 3)
    return flu, L


def _merge(Lup, up, lv, d, m):
    n = lv["n"]
    j, k = d % n, d // n
    nu = up["n"]
    kids = [(2 * k + bb) * nu + (2 * j + aa) for bb in (0, 1) for aa in (0, 1)]
    taps = []
    for a in range(3):
        f = Fraction(m[a], 2) - Fraction(1, 4)
        q0 = math.floor(f)
        w1 = f - q0
        hi = up["M"][a] - 1
        taps.append([(min(max(q0, 0), hi), 1 - w1), (min(max(q0 + 1, 0), hi), w1)])
    acc = np.zeros(3)
    for qz, wz in taps[2]:
        for qy, wy in taps[1]:
            for qx, wx in taps[0]:
                w = float(wx * wy * wz)
                for c in kids:
                    acc += 0.25 * w * Lup[:, c, qz, qy, qx]
    return acc
