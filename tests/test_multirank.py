"""The N-GPU bench path is replicas (one independent box per rank, no data
exchange): check its host-side rank logic with two gloo ranks on CPU - the
max-over-ranks timing and the whole-job aggregation the bench reports."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms_local = 100.0 + 25.0 * rank  # rank 1 is the slow one
    ms = bench.max_over_ranks(ms_local, dist, "cpu")
    value = bench.whole_job_rate(world, 256 ** 3, 10, ms)
    dist.barrier()
    q.put((rank, ms, value))
    dist.destroy_process_group()


def test_replicas_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench

    for rank, ms, value in res:
        assert ms == 125.0  # every rank reports the slowest rank's time
        assert value == pytest.approx(bench.whole_job_rate(2, 256 ** 3, 10, 125.0))
        assert value == pytest.approx(2 * 256 ** 3 * 10 / 0.125 / 1e6)


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.max_over_ranks(3.5, None) == 3.5
    assert bench.whole_job_rate(1, 1000, 4, 2.0) == pytest.approx(1000 * 4 / 2e-3 / 1e6)
