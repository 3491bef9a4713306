"""Generates the golden fixtures in this directory.

Each fixture is a small seeded scene solved by the FP64 C++ oracle and
confirmed, at generation time, against the independent Python restatement
(oracle/oracle_np.py) to 1e-12.  The reference repository has no
radiance-cascade code or vectors of its own, so these fixtures pin the
oracle and the GPU path to one another across machines.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from oracle import oracle_np as T  # noqa: E402

CASES = [
    # name, grid, cascades, boxes, edges, spheres, radius, emission, seed, frames advanced
    ("scene16_n3", (16, 16, 16), 3, 6, (2, 6), 2, (1.0, 2.5), (1.0, 20.0), 21, 0),
    ("scene16x8x24_n2", (16, 8, 24), 2, 5, (2, 6), 2, (1.0, 2.5), (1.0, 20.0), 22, 4),
]


def main():
    for name, grid, N, nb, edge, ns, rad, em, seed, frames in CASES:
        spec = O.scene_spec(grid, nb, edge[0], edge[1], ns, rad[0], rad[1], em[0], em[1])
        boxes, spheres = O.generate(spec, seed)
        O.advance(spheres, grid, frames)
        vox = O.voxelise(grid, boxes, spheres)
        p = O.params(grid, N)
        flu, L = O.solve(p, vox)
        occ = (vox["albedo_occ"] & 0x8000).astype(bool).reshape(grid[2], grid[1], grid[0])
        emf = vox["emission"].view(np.float16).astype(np.float64).reshape(grid[2], grid[1], grid[0], 3)
        tflu, tL = T.solve(list(grid), occ, emf, N)
        assert np.linalg.norm(flu - tflu) <= 1e-12 * np.linalg.norm(tflu)
        for a, b in zip(L, tL):
            assert np.abs(a - b).max() <= 1e-12 * max(1.0, np.abs(b).max())
        out = dict(grid=np.array(grid, np.int32), num_cascades=np.int32(N),
                   voxels=vox.view(np.uint16).reshape(-1, 4), fluence=flu)
        for i, x in enumerate(L):
            out["radiance_%d" % i] = x
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "fluence max %.4f" % flu.max(), os.path.getsize(os.path.join(HERE, name + ".npz")), "bytes")


if __name__ == "__main__":
    main()
