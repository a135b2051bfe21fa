"""The benchmark's multi-GPU path is replicas only (independent solves, no
data-path collective): its one collective is the max of the timed region over
ranks.  Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from hemocell_gb300 import hemocell
    hemocell.set_default_device(rank)  # as bench.py does with LOCAL_RANK: each replica on its own GPU
    ms = 10.0 + 5.0 * rank            # rank 1 is the slower replica
    m = bench.max_over_ranks(ms)
    q.put((rank, m, bench.replicas_mlups(world, 1_000_000, 100, m), hemocell.default_device()))
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [15.0, 15.0]
    # 2 replicas x 1e6 nodes x 100 steps in 15 ms
    assert got[0][2] == pytest.approx(2 * 1e6 * 100 / 15e3)
    assert [g[3] for g in got] == [0, 1]


def test_single_process_is_identity():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
