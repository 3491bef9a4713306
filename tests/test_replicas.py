"""The N>1 path of bench.py on CPU: two gloo ranks rendezvous on 127.0.0.1,
agree on the slowest rank's time, take disjoint frame ranges, and the
reference arm runs on rank 0 only (the other rank exits 0 silently)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist = bench.init_replicas(world, rank)
    try:
        slowest = bench.max_over_ranks(1.5 + rank, dist)
        first = bench.replica_first_frame(rank, 60, 5)
        ranges = [None] * world
        dist.all_gather_object(ranges, (first, first + 65))
        q.put((rank, slowest, ranges))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_disjoint_frames():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, ranges in out:
        assert slowest == 1.5 + (world - 1)
        (a0, a1), (b0, b1) = ranges
        assert a1 <= b0  # rank 0's frames end before rank 1's begin


def test_reference_arm_runs_on_rank_zero_only(capsys):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench

    class Args:
        steps, warmup = 1, 0

    assert bench.run_reference(Args(), rank=1, world=2) == 0
    assert capsys.readouterr().out == ""
