"""Host logic of `bench.py --gpus N` (independent replicas, no collective on the data path),
with two gloo ranks on the CPU: disjoint frame pools, barrier, max-over-ranks timing."""
from __future__ import annotations

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        frames = bench.frames_for_rank(5, rank, world)
        bench.barrier(world)
        slowest = bench.max_over_ranks(10.0 + rank, world, torch.device("cpu"))
        out.put((rank, frames, slowest))
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = [out.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    by_rank = {r: (f, s) for r, f, s in results}
    assert set(by_rank) == {0, 1}
    assert not set(by_rank[0][0]) & set(by_rank[1][0])        # disjoint frames
    assert by_rank[0][1] == by_rank[1][1] == pytest.approx(11.0)  # both ranks see the max


def test_single_process_helpers():
    assert bench.frames_for_rank(3, 0, 1) == [0, 1, 2]
    assert bench.max_over_ranks(4.5, 1, None) == 4.5
