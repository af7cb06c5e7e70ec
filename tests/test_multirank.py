"""The N>1 path of bench.py on CPU: two gloo ranks shard the configuration's p
slices with no overlap and no gap, and the timing and count reductions give
the max and the sum over ranks (the only process-group traffic the path has)."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, ws: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        total = 47
        mine = bench.shard_slices(total, ws, rank)
        # a rank's "elapsed" and "primes" stand-ins: rank-dependent numbers
        elapsed = 1.0 + rank
        primes = 1000.0 * (rank + 1) * len(mine)
        q.put((rank, mine, bench.reduce_over_ranks(elapsed, "max", ws, "cpu"),
               bench.reduce_over_ranks(primes, "sum", ws, "cpu")))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_and_reduce():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    slices = [s for _, mine, _, _ in got for s in mine]
    assert sorted(slices) == list(range(47)) and len(set(slices)) == 47
    assert all(mx == 2.0 for _, _, mx, _ in got)  # max over ranks of 1.0, 2.0
    want = 1000.0 * (1 * len(got[0][1]) + 2 * len(got[1][1]))
    assert all(sm == want for _, _, _, sm in got)


def test_single_rank_is_identity():
    import bench

    assert bench.shard_slices(5, 1, 0) == [0, 1, 2, 3, 4]
    assert bench.reduce_over_ranks(3.5, "max", 1, "cpu") == 3.5
