"""The N>1 host path of bench.py on CPU: two gloo ranks (world size 2) run the
rank setup, the barrier, the max-over-ranks step time and the whole-job rate,
and the reference arm's non-zero ranks exit without work."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, world, port):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)


def _rank_timing(rank, world, port, q):
    _env(rank, world, port)
    import bench
    w, r, local, pg = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank) and pg is not None
    bench.barrier(pg)
    # each rank reports its own step time; the job's time is the slowest rank's
    ms = bench.max_over_ranks(pg, 10.0 * (rank + 1))
    rate = bench.job_rate(1000.0, w, ms)
    bench.barrier(pg)
    q.put((rank, ms, rate))
    pg.destroy_process_group()


def _rank_reference(rank, world, port, q):
    _env(rank, world, port)
    import argparse
    import bench
    if rank == 0:
        # rank 0 would run the timed CPU sample; here it only joins the group
        w, r, local, pg = bench.dist_setup()
        q.put((rank, None))
        pg.destroy_process_group()
        return
    out = bench.run_reference(argparse.Namespace(steps=1, warmup=0, gpus=world, impl="reference"))
    q.put((rank, out))


def _run(fn, world=2):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=fn, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    codes = [p.exitcode for p in procs]
    for p in procs:
        if p.is_alive():
            p.kill()
    assert codes == [0] * world, codes
    return sorted(q.get(timeout=5) for _ in range(world))


def test_two_rank_max_over_ranks_and_job_rate():
    out = _run(_rank_timing)
    for rank, ms, rate in out:
        assert ms == 20.0
        assert rate == pytest.approx(1000.0 * 2 / 0.020)


def test_reference_arm_runs_on_rank_zero_only():
    out = _run(_rank_reference)
    assert out == [(0, None), (1, None)]


def test_single_rank_helpers_are_no_ops():
    sys.path.insert(0, ROOT)
    import bench
    bench.barrier(None)
    assert bench.max_over_ranks(None, 3.5) == 3.5
    assert bench.job_rate(10.0, 1, 1000.0) == 10.0
