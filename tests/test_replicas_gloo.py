"""The multi-GPU path on CPU: two ranks over gloo.

Fields (and branches) are independent, so a multi-GPU run is N replicas
with no data exchange; the only collective reduces the timer (max over
ranks) and the point counts (sum).  These tests run that reduction, the
sharding of fields and requests, and the replica seeds in two processes.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, ws: int, port: int, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        t = bench.reduce_over_ranks(1.5 + rank, "max", ws, device="cpu")
        p = bench.reduce_over_ranks(100.0 * (rank + 1), "sum", ws, device="cpu")
        fields = bench.batch_fields()
        mine = [f["random_seed"] for f in bench.shard(fields, rank, ws)]
        reqs = [p_["random_seed"] for _, p_ in bench.shard(bench.serving_requests(10), rank, ws)]
        seed = bench.replica_seed(1235, rank)
        q.put((rank, t, p, mine, reqs, seed))
    finally:
        dist.destroy_process_group()


def test_two_ranks_reduce_shard_and_seed():
    ws = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    # the timer is the slowest rank's, the points are everyone's
    assert all(o[1] == 2.5 for o in out)
    assert all(o[2] == 300.0 for o in out)
    # every field and request goes to exactly one rank
    fields = sorted(out[0][3] + out[1][3])
    assert fields == sorted(f["random_seed"] for f in bench.batch_fields())
    assert not set(out[0][3]) & set(out[1][3])
    reqs = sorted(out[0][4] + out[1][4])
    assert reqs == sorted(p["random_seed"] for _, p in bench.serving_requests(10))
    # the single-field replicas draw different star fields
    assert out[0][5] != out[1][5]


def test_one_rank_is_the_identity():
    assert bench.reduce_over_ranks(3.25, "max", 1) == 3.25
    assert bench.shard([1, 2, 3], 0, 1) == [1, 2, 3]
    assert bench.replica_seed(7, 0) == 7
