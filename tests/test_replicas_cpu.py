"""The multi-rank bench path on the CPU: one independent simulation per rank
(replicas; the time loop is not sharded), the timed region taken as the
maximum over ranks and the whole-job throughput summed over replicas.  Two
``gloo`` ranks on 127.0.0.1, started with ``spawn``."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, got_local = bench.dist_env()
        ms = 10.0 + 5.0 * rank  # the ranks' own timed regions differ
        dist.barrier()
        ms_max = bench.max_over_ranks(ms, device="cpu")
        out.put((rank, got_ws, got_rank, got_local, ms_max, bench.replica_throughput(1000, 20, ms_max, ws)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, out)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(out.get(timeout=10) for _ in range(ws))
    for rank, got_ws, got_rank, got_local, ms_max, value in res:
        assert (got_ws, got_rank, got_local) == (ws, rank, rank)
        assert ms_max == 15.0  # every rank reports the slowest rank's time
        assert value == pytest.approx(ws * 1000 * 20 / 0.015 / 1e6)


def test_single_process_is_its_own_maximum():
    import bench

    assert bench.max_over_ranks(3.5, device="cpu") == 3.5
    assert bench.replica_throughput(10, 4, 2.0, 1) == pytest.approx(10 * 4 / 0.002 / 1e6)
