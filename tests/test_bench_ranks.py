"""Replica ranks of bench.py on the CPU: two gloo processes (world size 2).

bench.py under torchrun runs one full replica of the workload per GPU; the only
cross-rank steps are the barriers around the timed region and the maximum of
the per-rank times.  This checks bench.Ranks (barrier, max over ranks) with
real process groups, and that one rank needs no process group at all.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    r = bench.Ranks(world, "gloo")
    r.barrier()
    got = r.max(10.0 + 3.5 * rank)  # rank 1 is the slowest
    r.barrier()
    out.put((rank, got))
    r.dist.destroy_process_group()


def test_ranks_barrier_and_max_two_gloo_processes():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    out = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 13.5, 1: 13.5}


def test_ranks_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    r = bench.Ranks(1, "gloo")
    assert r.dist is None
    r.barrier()
    assert r.max(7.25) == 7.25
