"""The N > 1 path of bench.py on CPU: replicas time their steps independently
and the job reports the slowest rank (gloo, world size 2, 127.0.0.1)."""
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_max_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    from helpers import multirank_worker
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=multirank_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(ws):
        rank, ms, env = q.get(timeout=180)
        out[rank] = (ms, env)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 11.0
    assert out[0][1] == (2, 0, 0) and out[1][1] == (2, 1, 0)


def test_max_over_ranks_without_a_group():
    import bench
    assert bench.max_over_ranks(7.5, torch.device("cpu")) == 7.5
