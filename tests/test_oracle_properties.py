"""Size-independent properties of the method, checked on the FP64 oracle
(the checker the GPU path is compared with): the solve is linear in the
emission.  Doubling every emission doubles every radiance and the fluence
bit for bit (scaling by 2 is exact in binary16 and in every FP64 step); two
emitter sets over the same opaque voxels add up to the solve of their sum."""
import numpy as np

from oracle import oracle as O
from tests.helpers import rel_l2, volume


def _scene(seed, g=32):
    rng = np.random.default_rng(seed)
    occ = np.zeros((g, g, g), bool)
    for _ in range(12):
        lo = rng.integers(0, g - 4, 3)
        hi = lo + rng.integers(2, 9, 3)
        occ[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] = True
    em_a = np.where(occ & (rng.random(occ.shape) < 0.05), rng.uniform(1, 20, occ.shape), 0.0)
    em_b = np.where(occ & (em_a == 0) & (rng.random(occ.shape) < 0.05), rng.uniform(1, 20, occ.shape), 0.0)
    return occ, em_a, em_b


def _bits(em):
    return np.vectorize(O.float_to_half, otypes=[np.uint16])(em)


def test_doubling_the_emission_doubles_every_value_exactly():
    occ, em_a, _ = _scene(3)
    bits = _bits(em_a)
    flu, L = O.solve(O.params(32, 4), volume(occ, bits))
    flu2, L2 = O.solve(O.params(32, 4), volume(occ, _bits(2.0 * em_a)))
    assert flu.any()
    assert np.array_equal(flu2, 2.0 * flu)
    for a, b in zip(L, L2):
        assert np.array_equal(b, 2.0 * a)


def test_two_emitter_sets_superpose():
    occ, em_a, em_b = _scene(5)
    # the same opaque voxels in all three solves; emission only where each set has it
    fa, La = O.solve(O.params(32, 4), volume(occ, _bits(em_a)))
    fb, Lb = O.solve(O.params(32, 4), volume(occ, _bits(em_b)))
    fab, Lab = O.solve(O.params(32, 4), volume(occ, _bits(em_a + em_b)))
    assert fa.any() and fb.any()
    assert rel_l2(fa + fb, fab) <= 1e-12
    for a, b, ab in zip(La, Lb, Lab):
        assert rel_l2(a + b, ab) <= 1e-12
