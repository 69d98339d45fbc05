"""CPU: the multi-GPU form is replicas (one independent solve stream per
rank, no collective on the data path). Two ``gloo`` ranks check the host
logic of ``bench.py``: every rank sees the slowest rank's time, and the job's
rate counts all ranks' solves; each rank draws its own seeded model."""
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


def _rank(rank, world, port, out):
    import bench
    from extreme_gb300.model import random_model
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = [1000.0, 1500.0][rank]
        e2e = [1100.0, 1400.0][rank]
        ms_max, e2e_max, value = bench.job_rate(ms, e2e, 4, world, "cpu")
        m = random_model(8, 8, 4, seed=1 + rank)
        out[rank] = (ms_max, e2e_max, value, float(m.sigma.sum()))
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        r0, r1 = out[0], out[1]
    assert r0[:3] == r1[:3] == (1500.0, 1400.0, pytest.approx(8 / 1.5))
    assert r0[3] != r1[3]   # each rank solves its own model


def test_one_rank_needs_no_group():
    import bench
    assert bench.job_rate(500.0, 600.0, 3, 1) == (500.0, 600.0, pytest.approx(6.0))
