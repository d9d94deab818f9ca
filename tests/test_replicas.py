"""Replicas on several ranks (gloo on CPU, world size 2): distinct
frequencies per rank, the job time is the slowest rank's, and the job rate
counts every rank's units."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from wtomo3d_gb300 import replicas

FREQS = [0.5, 1.0, 1.5, 2.0]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        freqs = [replicas.rank_frequency(i, rank, FREQS) for i in range(3, 7)]
        t = replicas.max_over_ranks(1.0 + rank, world)     # rank 1 is the slow one
        rate = replicas.job_rate(world, 32 * 4, t)
        out.put((rank, freqs, t, rate))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    world, port = 2, _free_port()
    ps = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get() for _ in range(world))
    f0, f1 = res[0][1], res[1][1]
    assert all(a != b for a, b in zip(f0, f1))          # the ranks factor different frequencies
    assert sorted(f0) == sorted(FREQS) and sorted(f1) == sorted(FREQS)
    assert res[0][2] == res[1][2] == 2.0                 # max over ranks
    assert res[0][3] == pytest.approx(2 * 128 / 2.0)


def test_single_rank_is_identity():
    assert replicas.max_over_ranks(3.5, 1) == 3.5
    assert replicas.rank_frequency(5, 0, FREQS) == FREQS[1]
