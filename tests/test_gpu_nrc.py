"""Neural radiance cache: the tcgen05 network against its NumPy restatement,
training, the learned solve against the FP64 oracle, save / load.

Tolerances: served (R, G, B, T) within 2e-3 absolute (radiance units after
1/scale) of the BF16-emulating NumPy forward, away from the T threshold; the tile gradient within 3e-2
relative L2 (BF16 rounding of the backward operands); the learned solve,
with the network serving at least one far cascade, within 1% relative L2 of
the FP64 oracle with the per-tile fallback and within 2% with no fallback.
"""
import numpy as np
import pytest

import radiancecascade_gb300 as R
from radiancecascade_gb300 import _ffi as F
from oracle import oracle as O
from tests import nrc_ref as N
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def _engine(grid=64, cascades=5, workload="c64", **kw):
    e = R.Engine(R.make_params(grid, cascades))
    boxes, spheres = R.workload_scene(workload)
    e.set_boxes(boxes)
    e.set_spheres(spheres)
    e.nrc_enable(**kw)
    return e, boxes, spheres


def _model(e, prm):
    mlp, table = N.unpack_save(e.nrc_save(), prm.hash_log2_entries)
    W, b = N.layers(mlp)
    return W, b, table.astype(np.float16)


def _inputs(e, prm, table16, level, probes, dirs):
    info = e.levels[level]
    px, py, pz = info.probes
    xyz = np.stack([probes % px, (probes // px) % py, probes // (px * py)], 1)
    res = N.resolutions(prm.base_resolution, prm.max_resolution)
    pos = N.encode(table16, res, N.dir_resolutions(), prm.hash_log2_entries, xyz, info.spacing,
                   max(e.params.grid), dirs.astype(np.int64), info.dir_res, level)
    x = np.zeros((len(probes), 64), np.float32)
    x[:, :32] = pos
    x[:, 32:48] = N.dir_features(info.dir_res, dirs, level - prm.first_level)
    return x


def test_forward_matches_numpy():
    e, _, _ = _engine()
    prm = R.Engine.nrc_params()
    try:
        W, b, t16 = _model(e, prm)
        rng = np.random.default_rng(3)
        for level in (2, 3, 4):
            info = e.levels[level]
            P = int(np.prod(info.probes))
            probes = rng.integers(0, P, 300).astype(np.int32)
            dirs = rng.integers(0, info.num_dirs, 300).astype(np.int32)
            got = e.nrc_query(level, probes, dirs)
            o, _ = N.forward(W, b, _inputs(e, prm, t16, level, probes, dirs))
            want = N.served(o, prm.radiance_scale)
            clear = np.abs(o[:, 3] - 0.5) > 1e-2  # away from the T threshold
            assert clear.mean() > 0.9
            err = np.abs(got - want)[clear].max()
            assert err <= 2e-3, (level, err)
    finally:
        e.close()


def test_tile_gradient_matches_numpy():
    e, _, _ = _engine()
    prm = R.Engine.nrc_params()
    try:
        W, b, t16 = _model(e, prm)
        rng = np.random.default_rng(5)
        for level, probe, d0, n in [(2, 17, 128, 128), (3, 40, 0, 77), (4, 3, 1024, 128)]:
            y = np.zeros((n, 4), np.float32)
            y[:, :3] = rng.uniform(0, 20, (n, 3)) * (rng.random((n, 1)) < 0.3)
            y[:, 3] = rng.random(n) < 0.5
            pg, eg = e.nrc_tile_gradient(level, probe, d0, y)
            dirs = np.arange(d0, d0 + n, dtype=np.int32)
            x = _inputs(e, prm, t16, level, np.full(n, probe, np.int32), dirs)
            rg, reg = N.backward(W, b, x, y.astype(np.float64), prm.radiance_scale)
            assert rel_l2(pg, rg) <= 3e-2, (level, rel_l2(pg, rg))
            assert rel_l2(eg, reg) <= 3e-2, (level, rel_l2(eg, reg))
    finally:
        e.close()


def test_training_lowers_loss():
    e, boxes, spheres = _engine()
    try:
        losses = []
        for f in range(48):
            e.solve()
            if f % 8 == 7:
                losses.append(e.nrc_stats()["last_loss"])
        st = e.nrc_stats()
        assert st["solves"] == 48 and st["steps"] == 48
        assert losses[-1] < losses[0]
    finally:
        e.close()


def _served(st, level):
    return (st["served_levels"] >> level) & 1


@pytest.mark.parametrize("first,plain_fraction", [(3, 0.5), (2, 1.0)])
def test_learned_solve_serves_from_the_network_within_one_percent(first, plain_fraction):
    """64^3: after 48 solves the network serves at least one far cascade (in
    whole, or per tile next to walked fallback tiles) and the fluence stays
    within 1% relative L2 of the FP64 oracle."""
    e, boxes, spheres = _engine(first_level=first, plain_level_fraction=plain_fraction)
    try:
        for _ in range(48):
            e.solve()
        st = e.nrc_stats()
        g = e.fluence().astype(np.float64)
    finally:
        e.close()
    assert st["served_levels"] != 0, st
    assert st["fallback_tiles"] < st["tiles"], st
    ref, _ = O.solve(O.params(64, 5), O.voxelise(64, boxes, spheres))
    err, max_abs = rel_l2(g, ref), float(np.abs(g - ref).max())
    print("64^3 learned (first %d): served %s, fallback %d/%d tiles, rel-L2 %.3e, max-abs %.3e"
          % (first, bin(st["served_levels"]), st["fallback_tiles"], st["tiles"], err, max_abs))
    assert err <= 1e-2, err
    assert np.isfinite(max_abs)


def _scene_256(frame):
    boxes, sph = R.workload_scene("c256")
    sph = sph.copy()
    R.advance_spheres(sph, 256, frame)
    return boxes, sph


@pytest.mark.parametrize("threshold,bound", [(0.01, 1e-2), (1e9, 2e-2)])
def test_learned_256_frames_0_1_239(threshold, bound):
    """256^3 FP16, the cache on cascades 4 and 5: it learns for 48 solves on
    frame 0, then solves frame 1, then jumps to frame 239 (8 solves).  With
    the 1% per-tile fallback the cache serves cascade 5 and the fluence is
    within 1% of the FP64 oracle on every frame; with no fallback at all (the
    network serves every tile of both cascades) within 2%."""
    e = R.Engine(R.make_params(256, 6, precision="fp16"))
    boxes, _ = _scene_256(0)
    e.set_boxes(boxes)
    e.nrc_enable(first_level=4, fallback_threshold=threshold)
    try:
        for frame, solves in ((0, 48), (1, 1), (239, 8)):
            _, sph = _scene_256(frame)
            e.set_spheres(sph)
            for _ in range(solves):
                e.solve()
            st = e.nrc_stats()
            g = e.fluence().astype(np.float64)
            ref, _ = O.solve(O.params(256, 6), O.voxelise(256, boxes, sph), jump=True)
            err, max_abs = rel_l2(g, ref), float(np.abs(g - ref).max())
            print("256^3 frame %d: served %s, fallback %d/%d, rel-L2 %.3e, max-abs %.3e"
                  % (frame, bin(st["served_levels"]), st["fallback_tiles"], st["tiles"], err, max_abs))
            assert _served(st, 5), st
            assert st["fallback_tiles"] < st["tiles"], st
            if threshold > 1.0:
                assert st["fallback_tiles"] == 0 and _served(st, 4), st
            assert err <= bound, (frame, err)
    finally:
        e.close()


def test_save_load_round_trip_and_disable():
    e, boxes, spheres = _engine()
    try:
        for _ in range(5):
            e.solve()
        blob = e.nrc_save()
        q = e.nrc_query(3, np.arange(50, dtype=np.int32), np.arange(50, dtype=np.int32) * 7)
        e2, _, _ = _engine()
        try:
            e2.nrc_load(blob)
            q2 = e2.nrc_query(3, np.arange(50, dtype=np.int32), np.arange(50, dtype=np.int32) * 7)
            assert np.array_equal(q, q2)
            with pytest.raises(R.RCError):
                e2.nrc_load(blob[:-4])
        finally:
            e2.close()
        e.nrc_disable()
        e.solve()
        g = e.fluence().astype(np.float64)
        ref, _ = O.solve(O.params(64, 5), O.voxelise(64, boxes, spheres))
        assert rel_l2(g, ref) <= 1e-4
        with pytest.raises(R.RCError) as ei:
            e.nrc_stats()
        assert ei.value.status == F.RC_ERR_STATE
    finally:
        e.close()
