"""The multi-rank path on CPU (gloo, world size 2): round-robin sharding of independent instances
and the whole-job aggregation of a sharded batch (max wall time over ranks, summed instances,
gathered latencies)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from seemps2_gb300.distributed import combine_batch_reports, shard_indices  # noqa: E402


def test_shard_indices_cover_once():
    n, world = 17, 3
    parts = [shard_indices(n, r, world) for r in range(world)]
    assert sorted(i for p in parts for i in p) == list(range(n))
    assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
    with pytest.raises(ValueError):
        shard_indices(5, 3, 3)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        idx = shard_indices(10, rank, world)
        wall = 2.0 if rank == 0 else 3.0
        lat = [0.1 * (i + 1) for i in idx]
        rep = combine_batch_reports(wall, len(idx), lat)
        out.put((rank, rep))
    finally:
        dist.destroy_process_group()


def test_combine_batch_reports_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    reps = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        rep = reps[rank]
        assert rep["ranks"] == 2 and rep["instances"] == 10
        assert rep["wall_s"] == 3.0  # the slowest rank
        assert abs(rep["instances_per_s"] - 10 / 3.0) < 1e-12
        assert abs(rep["p50_s"] - 0.6) < 1e-12 or abs(rep["p50_s"] - 0.5) < 1e-12
        assert abs(rep["p99_s"] - 1.0) < 1e-12
