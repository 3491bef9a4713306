"""Batched persistent solve: many scenes of uneven size in one graph launch.

Every scene of a batch must match the FP64 oracle with the single-context
tolerances (FP32: relative L2 <= 1e-4, max relative <= 1e-5), whatever the
queue's tile shape, and a wait that runs out must come back as
RC_ERR_TIMEOUT with the batch still usable.
"""
import numpy as np
import pytest

import radiancecascade_gb300 as R
from radiancecascade_gb300 import _ffi as F
from oracle import oracle as O
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu
FP32_REL_L2 = 1e-4
FP32_MAX_REL = 1e-5

# (grid, cascades, scene seed): uneven sizes and depths in one queue
SCENES = [
    ((32, 32, 32), 3, 11),
    ((80, 48, 64), 4, 12),
    ((64, 64, 64), 5, 13),
    ((128, 64, 32), 5, 14),
    ((96, 96, 96), 5, 15),
]


def _scene(grid, seed):
    n = max(grid)
    spec = R.scene_spec(grid, max(6, n // 4), (3, max(6, n // 6)), max(2, n // 16), (1.5, 4.0), (1.0, 20.0))
    return R.generate_scene(spec, seed)


@pytest.fixture(scope="module")
def oracle_results():
    out = []
    for grid, N, seed in SCENES:
        boxes, spheres = _scene(grid, seed)
        vox = O.voxelise(grid, boxes, spheres)
        out.append(O.solve(O.params(grid, N), vox, jump=True))
    return out


def _batch(precision="fp32"):
    b = R.Batch([R.make_params(g, N, precision=precision) for g, N, _ in SCENES])
    for k, (grid, _, seed) in enumerate(SCENES):
        b.set_scene(k, *_scene(grid, seed))
    return b


def _check_all(b, oracle_results, rel=FP32_REL_L2, max_rel=FP32_MAX_REL):
    for k, (oflu, oL) in enumerate(oracle_results):
        gflu = b.fluence(k).astype(np.float64)
        assert rel_l2(gflu, oflu) <= rel, (k, rel_l2(gflu, oflu))
        for i, o in enumerate(oL):
            g = b.radiance(k, i).astype(np.float64)
            assert g.shape == o.shape
            assert rel_l2(g, o) <= rel, (k, i)
            if max_rel is not None:
                assert np.abs(g - o).max() <= max_rel * max(1.0, np.abs(o).max()), (k, i)


def test_batch_matches_oracle(oracle_results):
    with _batch() as b:
        b.solve()
        b.synchronize()
        _check_all(b, oracle_results)
        b.solve()  # the graph replays: same results
        _check_all(b, oracle_results)


@pytest.mark.parametrize("ppi,qpi", [(1, 1), (32, 3), (128, 2), (1000, 64)])
def test_batch_tile_shapes_give_the_same_results(ppi, qpi, oracle_results):
    with _batch() as b:
        b.set_tiles(ppi, qpi)
        b.solve()
        _check_all(b, oracle_results)


def test_batch_matches_single_contexts():
    with _batch() as b:
        b.solve()
        for k, (grid, N, seed) in enumerate(SCENES):
            with R.Engine(R.make_params(grid, N)) as e:
                boxes, spheres = _scene(grid, seed)
                e.set_boxes(boxes)
                e.set_spheres(spheres)
                e.solve()
                ref = e.fluence()
            got = b.fluence(k)
            assert np.abs(got - ref).max() <= 1e-6 * max(1.0, float(np.abs(ref).max()))


def test_batch_autotuner_keeps_a_candidate(oracle_results):
    with _batch() as b:
        ppi, qpi, ms = b.tune(iters=1)
        assert ppi in (128, 256, 512, 1024) and qpi in (1, 2, 4, 8) and ms > 0
        b.solve()
        _check_all(b, oracle_results)


def test_batch_fp16(oracle_results):
    with _batch("fp16") as b:
        b.solve()
        _check_all(b, oracle_results, rel=1e-2, max_rel=None)


def test_batch_state_and_argument_errors():
    with pytest.raises(R.RCError) as ei:
        R.Batch([R.make_params(32, 3), R.make_params(32, 3, precision="fp16")])
    assert ei.value.status == F.RC_ERR_INVALID_ARG
    with R.Batch([R.make_params(32, 3)] * 2) as b:
        with pytest.raises(R.RCError) as ei:
            b.solve()
        assert ei.value.status == F.RC_ERR_STATE
        out = np.zeros(3 * 16 ** 3, np.float32)
        assert F.lib().rc_batch_get_fluence(b.handle, 2, F.ptr(out), out.size, F.RC_MEM_HOST) == F.RC_ERR_INVALID_ARG
        with pytest.raises(R.RCError):
            b.set_tiles(0, 1)


def test_batch_timeout_is_reported_and_batch_stays_usable(monkeypatch, oracle_results):
    """Fault injection on the host: the level table claims one more top-level
    tile than the queue holds, so the next level's bounded wait runs out."""
    monkeypatch.setenv("RC_FAULT", "timeout")
    b = _batch()
    try:
        b.solve()
        with pytest.raises(R.RCError) as ei:
            b.synchronize()
        assert ei.value.status == F.RC_ERR_TIMEOUT
        monkeypatch.delenv("RC_FAULT")
        b.set_tiles(256, 2)  # rebuilds the level table without the fault
        b.solve()
        b.synchronize()
        _check_all(b, oracle_results)
    finally:
        b.close()
