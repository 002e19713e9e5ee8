"""The multi-GPU path runs replicas (one independent domain per rank): the
host logic around the timed region - barrier, max of the per-rank times,
whole-job throughput - on two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from apc_524_project_gb300 import replicas

    w, r, barrier, dmax, close = replicas.comm("gloo")
    barrier()
    t = 1.0 + 0.5 * r  # this rank's timed region
    tmax = dmax(t)
    barrier()
    close()
    out.put((r, w, tmax, replicas.job_throughput(1000, 20, w, tmax)))


def test_two_gloo_ranks_take_the_slowest_time():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1]
    for r, w, tmax, value in res:
        assert w == 2
        assert tmax == 1.5
        assert value == pytest.approx(1000 * 20 * 2 / 1.5)


def test_single_process_is_a_no_op():
    from apc_524_project_gb300 import replicas

    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK") if k in os.environ}
    try:
        w, r, barrier, dmax, close = replicas.comm("gloo")
        assert (w, r) == (1, 0)
        barrier()
        assert dmax(3.0) == 3.0
        close()
    finally:
        os.environ.update(env)
