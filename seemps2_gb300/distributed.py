"""Multi-GPU use of the library: independent instances spread over ranks.

A simplify sweep does not shard (each two-site step needs the environment the previous one
produced), so the library's multi-GPU story is replicas and, for batches of independent MPS,
sharding: every rank (one process per GPU) takes a round-robin share of the instances, runs them with
seemps2_gb300.batch, and the ranks combine their timings with one collective at the end (the data path
itself has no exchange).  The helpers take a torch.distributed process group (NCCL on GPUs; the tests
use gloo on the CPU).
"""

from __future__ import annotations


def shard_indices(n: int, rank: int, world: int) -> list:
    """Round-robin share of `n` instances for `rank` of `world` (balances uneven sizes that come
    in sorted order)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("need 0 <= rank < world")
    return list(range(rank, n, world))


def combine_batch_reports(wall_s: float, instances: int, latencies_s: list, group=None,
                          device=None) -> dict:
    """Whole-job figures of a sharded batch: wall time = the slowest rank's (max over ranks),
    instances summed, per-instance latencies gathered from every rank; MPS/s over the whole job."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    dev = device if device is not None else torch.device("cpu")
    t = torch.tensor([wall_s, float(instances)], dtype=torch.float64, device=dev)
    w = t[:1].clone()
    dist.all_reduce(w, op=dist.ReduceOp.MAX, group=group)
    c = t[1:].clone()
    dist.all_reduce(c, op=dist.ReduceOp.SUM, group=group)
    lat = [None] * world
    dist.all_gather_object(lat, list(latencies_s), group=group)
    flat = sorted(x for part in lat for x in part)

    def pct(q):
        if not flat:
            return 0.0
        return flat[min(len(flat) - 1, max(0, int(round(q / 100.0 * (len(flat) - 1)))))]

    wall = float(w.item())
    count = int(round(float(c.item())))
    return {"ranks": world, "instances": count, "wall_s": wall,
            "instances_per_s": count / wall if wall > 0 else 0.0,
            "p50_s": pct(50), "p99_s": pct(99)}
