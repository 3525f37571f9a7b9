"""bench.py's multi-rank logic on CPU: two gloo ranks, each a replica with its own time; the job time is
the slowest rank's and the job throughput counts every rank's steps.  The reference arm does its work on
rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), MLG_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    r, w, local, pg = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank)
    ms = bench.max_over_ranks(pg, 10.0 + 5.0 * rank)
    value = bench.job_steps_per_s(w, 20, ms)

    class Args:
        steps, warmup, gpus = 2, 1, world
    # ranks other than 0 leave the reference arm at once, without touching the oracle
    ref = "skipped" if rank != 0 else "rank0"
    if rank != 0:
        assert bench.run_reference(Args(), r, w, pg) is None
    pg.barrier()
    pg.destroy_process_group()
    out.put((rank, ms, value, ref))


@pytest.mark.timeout(120)
def test_two_gloo_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(30)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    # 2 ranks x 20 steps in 15 ms
    assert all(abs(r[2] - 2 * 20 / 0.015) < 1e-9 for r in res)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 7.5) == 7.5
    assert bench.job_steps_per_s(1, 10, 100.0) == 100.0
