"""The multi-process plumbing of bench.py on CPU: two gloo ranks, barrier and
the max over ranks that makes the timed region the slowest rank's."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    ws, r, local = bench.dist_env()
    dist = bench.init_dist(ws)
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 1.5 + r)
    bench.barrier(dist)
    q.put((r, local, ws, t))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    assert [o[0] for o in out] == [0, 1]
    assert all(o[2] == 2 for o in out)
    assert all(o[3] == pytest.approx(2.5) for o in out)


def test_single_process_needs_no_process_group():
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    ws, r, local = bench.dist_env()
    assert (ws, r, local) == (1, 0, 0)
    assert bench.init_dist(ws) is None
    assert bench.max_over_ranks(None, 3.0) == 3.0
