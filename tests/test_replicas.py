"""The multi-GPU form of the path is replicas only (rays are independent;
no data-path collective): bench.py's ranks each render their own frames and
report the whole job's rays over the slowest rank's time.  These tests run
that aggregation on two gloo ranks on the CPU, and the reference arm's rule
that ranks other than 0 do no work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, q):
    import torch.distributed as td
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        total = bench.max_over_ranks(times[rank], td, "cpu")
        value = bench.whole_job_mrays(1_000_000, 10, world, total)
        q.put((rank, total, value))
    finally:
        td.destroy_process_group()


def test_replicas_report_the_slowest_rank_and_all_rays():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [250.0, 400.0]
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, total, value in got:
        assert total == 400.0  # the slowest replica's timed region
        # 2 ranks x 10 frames x 1 M rays over 0.4 s
        assert value == pytest.approx(2 * 10 * 1.0 / 0.4)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(123.0) == 123.0
    assert bench.whole_job_mrays(2_000_000, 5, 1, 1000.0) == pytest.approx(10.0)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup = 1, 0
    assert bench.run_reference(Args(), 1, 2) is None
    assert capsys.readouterr().out == ""


def test_bench_tile_order_is_a_permutation():
    """The roofline launch queues the frame's primary rays in the render's
    8 x 4 tile order: a permutation of the pixels, tile by tile."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import bench
    for w, h in ((1920, 1080), (33, 17), (8, 4), (5, 3)):
        t = bench.tile_order(w, h)
        assert np.array_equal(np.sort(t), np.arange(w * h))
    t = bench.tile_order(16, 8)
    assert list(t[:8]) == list(range(8)) and list(t[8:16]) == list(range(16, 24))
    assert list(t[32:40]) == list(range(8, 16))
