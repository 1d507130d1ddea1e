"""The bench's multi-rank timing on CPU: two gloo ranks, each with its own
timed-region length; both report the slowest rank's, and the whole-job rate
counts the units of every rank over that time."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, ms, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group('gloo', init_method='tcp://127.0.0.1:%d' % port, rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(ms[rank], dist, 'cpu')
        out.put((rank, got, bench.whole_job_rate(got, 4, 1000, world)))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context('spawn')
    out = ctx.Queue()
    ms = [3.0, 5.0]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, ms, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = [out.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, (ms_step, rate) in res:
        assert got == 5.0
        assert ms_step == 1.25
        assert abs(rate - 2 * 1000 / 1.25e-3) < 1e-6


def test_single_process_keeps_its_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.5) == 7.5
    ms_step, rate = bench.whole_job_rate(7.5, 3, 600, 1)
    assert ms_step == 2.5 and abs(rate - 600 / 2.5e-3) < 1e-6
