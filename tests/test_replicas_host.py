"""The replicated (N > 1) bench path on CPU: two gloo ranks agree on the slowest rank's time and
report the whole-job edges/s (multi-GPU here is replicas only, with no data-path collective)."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=ws)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, "cpu")
    out.put((rank, ms, bench.replica_value(1000, ms, ws)))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert res[0][2] == pytest.approx(2 * 1000 / 0.015)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.0, "cpu") == 3.0
    assert bench.replica_value(500, 2.0, 1) == pytest.approx(250000.0)
