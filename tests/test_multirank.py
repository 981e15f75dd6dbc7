"""The replica (N > 1) host logic of bench.py on CPU: two gloo ranks on 127.0.0.1 take the
barrier, agree on the slowest rank's time and report the whole-job throughput."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.rank_barrier(world)
        ms = bench.max_over_ranks(10.0 * (rank + 1), world, "cpu")  # rank r took 10 (r + 1) ms
        out[rank] = (ms, bench.job_throughput(ms, world))
        bench.rank_barrier(world)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    mp_ctx = mp.get_context("spawn")
    with mp_ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [mp_ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        res = dict(out)
    for r in range(2):
        ms, thr = res[r]
        assert ms == 20.0
        assert thr == pytest.approx(2 / 0.020)


def test_single_rank_is_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    bench.rank_barrier(1)
    assert bench.max_over_ranks(7.5, 1, "cpu") == 7.5
    assert bench.job_throughput(8.0, 1) == pytest.approx(125.0)
