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


def test_batch_matches_oracle(oracle_results, walk):
    with _batch() as b:
        b.solve()
        b.synchronize()
        _check_all(b, oracle_results)
        b.solve()  # the graph replays: same results
        _check_all(b, oracle_results)


@pytest.fixture(params=["default", "scalar"])
def walk(request, monkeypatch):
    """Batch scenes with the bit-parallel wide levels and walk-free cascade 0
    (default), or with every level on the scalar walk."""
    monkeypatch.delenv("RC_WALK", raising=False)
    if request.param == "scalar":
        monkeypatch.setenv("RC_WALK", "scalar")
    return request.param


@pytest.mark.parametrize("ppi,qpi,upi,wpi", [(1, 1, 1, 1), (32, 3, 2, 77), (128, 2, 3, 1024),
                                             (1000, 64, 64, 65536)])
def test_batch_tile_shapes_give_the_same_results(ppi, qpi, upi, wpi, oracle_results, walk):
    with _batch() as b:
        b.set_tiles(ppi, qpi, upi, wpi)
        assert b.tiles() == dict(probes_per_item=ppi, dirs_per_item=qpi, blocks_per_item=upi, walks_per_item=wpi)
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
    """The tuner times the persistent kernel's tile shapes and the scenes' own
    launches, keeps the faster form (persistent until tuned), and either gives
    the oracle's results."""
    with _batch() as b:
        assert b.form() == "persistent"
        tiles, ms = b.tune(iters=1)
        assert tiles == b.tiles() and ms > 0 and b.form() in ("persistent", "scenes")
        b.solve()
        _check_all(b, oracle_results)


def test_batch_fp16(oracle_results, walk):
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
            b.set_tiles(0, 1, 1, 1)


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
        b.set_tiles(256, 2, 1, 1024)  # rebuilds the level table without the fault
        b.solve()
        b.synchronize()
        _check_all(b, oracle_results)
    finally:
        b.close()


def test_batch64_workload_parity_and_properties():
    """The 64-scene batched workload at full size: one scene of each edge
    against the FP64 oracle, every scene within the energy bound."""
    items = R.batch_workload()
    with R.Batch([R.make_params(e, N) for e, N, _, _ in items]) as b:
        for k, (_, _, boxes, spheres) in enumerate(items):
            b.set_scene(k, boxes, spheres)
        b.tune(iters=1)
        b.solve()
        seen = set()
        for k, (edge, N, boxes, spheres) in enumerate(items):
            g = b.fluence(k).astype(np.float64)
            emax = float(np.max(spheres["value"]["emission"].view(np.float16).astype(np.float64)))
            assert g.min() >= 0.0 and g.max() <= 4 * np.pi * emax * (1 + 1e-6)
            if edge in seen:
                continue
            seen.add(edge)
            ref, _ = O.solve(O.params(edge, N), O.voxelise(edge, boxes, spheres), jump=True)
            assert rel_l2(g, ref) <= FP32_REL_L2, (k, edge)
            assert np.abs(g - ref).max() <= FP32_MAX_REL * max(1.0, ref.max()), (k, edge)
        assert seen == set(R.BATCH_EDGES)


def test_moving_emitters_between_solves_and_one_fluence_read():
    """rc_batch_set_spheres updates each scene's emitters on the batch stream
    with no host wait, in order with the solves: after three solves with the
    spheres advanced one frame before each, every scene matches the oracle on
    the third frame's spheres, and rc_batch_get_fluence_all returns the same
    floats as the per-scene reads, scene after scene."""
    b = _batch()
    try:
        sph = [_scene(grid, seed)[1].copy() for grid, _, seed in SCENES]
        for frame in range(1, 4):
            for k, (grid, _, _) in enumerate(SCENES):
                R.advance_spheres(sph[k], grid, 1)
                b.set_spheres(k, sph[k])
            b.solve()
        flat = b.fluence_all()
        off = 0
        for k, (grid, N, seed) in enumerate(SCENES):
            one = b.fluence(k).reshape(-1)
            assert np.array_equal(flat[off:off + one.size], one), k
            off += one.size
            boxes, _ = _scene(grid, seed)
            oflu, _ = O.solve(O.params(grid, N), O.voxelise(grid, boxes, sph[k]), jump=True)
            assert rel_l2(one.reshape(-1, 3), oflu) <= FP32_REL_L2, k
        assert off == flat.size
        with pytest.raises(R.RCError):
            F.check(F.lib().rc_batch_get_fluence_all(b.handle, F.ptr(flat), flat.size - 1, F.RC_MEM_HOST))
    finally:
        b.close()


def test_batch_as_parallel_scene_launches_matches_oracle(monkeypatch, oracle_results):
    """The other form of the batched solve (RC_BATCH_MODE=scenes): every
    scene's own level launches as parallel branches of one graph.  Every
    scene matches the oracle, a second launch of the graph gives the same
    results, and moving emitters between solves are seen in order."""
    monkeypatch.setenv("RC_BATCH_MODE", "scenes")
    with _batch() as b:
        assert b.form() == "scenes"
        b.solve()
        _check_all(b, oracle_results)
        b.solve()
        _check_all(b, oracle_results)
        tiles, ms = b.tune(iters=1)  # the form is fixed: only timed
        assert ms > 0 and b.form() == "scenes"
        sph = [_scene(grid, seed)[1].copy() for grid, _, seed in SCENES]
        for k, (grid, _, _) in enumerate(SCENES):
            R.advance_spheres(sph[k], grid, 2)
            b.set_spheres(k, sph[k])
        b.solve()
        for k, (grid, N, seed) in enumerate(SCENES):
            boxes, _ = _scene(grid, seed)
            oflu, _ = O.solve(O.params(grid, N), O.voxelise(grid, boxes, sph[k]), jump=True)
            assert rel_l2(b.fluence(k).reshape(-1, 3).astype(np.float64), oflu) <= FP32_REL_L2, k


def test_batch_as_parallel_scene_launches_fp16(monkeypatch, oracle_results):
    """The scene-launch form with FP16 radiance storage: every scene within
    1% of the FP64 oracle."""
    monkeypatch.setenv("RC_BATCH_MODE", "scenes")
    with _batch("fp16") as b:
        assert b.form() == "scenes"
        b.solve()
        _check_all(b, oracle_results, rel=1e-2, max_rel=None)


def test_async_fluence_read_matches_the_synchronous_one():
    """rc_batch_get_fluence_all_async starts the read on the batch stream and
    returns; after synchronize it holds the same floats as the synchronous
    read, and an emitter update plus solve enqueued right after it do not
    disturb it (they run after the copies)."""
    b = _batch()
    try:
        b.solve()
        want = b.fluence_all()
        got = np.full(want.size, np.nan, np.float32)
        b.fluence_all_async(got)
        sph = _scene(SCENES[0][0], SCENES[0][2])[1].copy()
        R.advance_spheres(sph, SCENES[0][0], 3)
        b.set_spheres(0, sph)
        b.solve()
        b.synchronize()
        assert np.array_equal(got, want)
        with pytest.raises(R.RCError):
            F.check(F.lib().rc_batch_get_fluence_all_async(b.handle, F.ptr(got), got.size - 1))
    finally:
        b.close()


def test_async_reads_in_flight_over_moving_frames():
    """Four moving-emitter frames, each read asynchronously into one of two
    pinned buffers with no wait in between (the copy to the host runs beside
    the next solve, from the device staging buffer): after the final
    synchronize the two buffers hold the last two frames, equal to a second
    batch stepped the same way and read synchronously."""
    torch = pytest.importorskip("torch")
    a, b = _batch(), _batch()
    try:
        n = a.fluence_elems()
        bufs = [torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
        for x in bufs:
            x[:] = np.nan
        sph_a = [_scene(g, seed)[1].copy() for g, _, seed in SCENES]
        sph_b = [x.copy() for x in sph_a]
        want = []
        for f in range(4):
            for k, (grid, _, _) in enumerate(SCENES):
                R.advance_spheres(sph_a[k], grid, 1)
                a.set_spheres(k, sph_a[k])
                R.advance_spheres(sph_b[k], grid, 1)
                b.set_spheres(k, sph_b[k])
            a.solve()
            a.fluence_all_async(bufs[f & 1])
            b.solve()
            want.append(b.fluence_all())
        a.synchronize()
        assert not np.array_equal(want[2], want[3])  # the emitters moved
        assert np.array_equal(bufs[0], want[2])
        assert np.array_equal(bufs[1], want[3])
    finally:
        a.close()
        b.close()
