"""The N > 1 host logic of bench.py (replicas: one process per GPU, a
barrier, the slowest rank's step time, whole-job frames/s) with two gloo
ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench._dist() == (ws, rank, rank)
        bench._barrier(ws)
        ms_local = [2.0, 5.0][rank]  # rank 1 is the slow replica
        ms, fps = bench._whole_job(ms_local, ws)
        q.put((rank, ms, fps))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(ws))
    # every rank sees the max over ranks; whole-job frames/s = ws frames per slowest step
    assert got == [(0, 5.0, 400.0), (1, 5.0, 400.0)]


def test_single_process_is_unchanged():
    import bench
    assert bench._whole_job(4.0, 1) == (4.0, 250.0)
