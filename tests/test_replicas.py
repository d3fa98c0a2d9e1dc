"""The replica bookkeeping of bench.py (tealeaf_ref_gb300/replicas.py) on two CPU processes
with the gloo backend: barrier, maximum over ranks, whole-job rate."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from tealeaf_ref_gb300 import replicas

    g = replicas.init("gloo")
    g.barrier()
    t = g.max(1.5 + rank)  # each rank's "time"; the job takes the slowest
    rate = replicas.whole_job_rate(g.world, 100, 10, t)
    g.barrier()
    g.close()
    q.put((rank, g.world, t, rate))


def test_two_replicas_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, world, t, rate in got:
        assert world == 2
        assert t == 2.5
        assert rate == 2 * 100 * 10 / 2.5


def test_single_process_group():
    from tealeaf_ref_gb300 import replicas

    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        g = replicas.init()
        assert (g.world, g.rank, g.dist) == (1, 0, None)
        assert g.max(3.0) == 3.0
        g.barrier()
        g.close()
    finally:
        os.environ.update(env)
