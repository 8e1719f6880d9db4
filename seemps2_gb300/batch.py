"""Batched ``MPO.apply`` + ``simplify`` over many independent MPS.

Each instance is an independent sweep (``MPO.apply``, operators/mpo.py:229-281, then ``simplify``,
state/simplification.py:32-144), and each of its splits ends in a truncation decision that the sweep
driver reads back before it sizes the next contraction, so a single small instance (bond 8..128)
leaves most of a GB300 idle.  A batch keeps S instances in flight: S worker threads, each with its
own library context (scratch memory, pinned words) and its own CUDA stream; the C calls release the
GIL (ctypes), so the kernels of different instances run concurrently on the GPU.  S is picked by
``tune_streams``, which times the candidates on a sample of the batch itself.  Worker contexts are
marked concurrent (``sm_ctx_set_concurrent``): the FP64 SVD's grid-barrier kernels then run as one
CTA, because a multi-CTA grid barrier can wait on CTAs that the other streams' kernels keep off the
SMs; the mixed forms' cluster kernel is co-scheduled by the hardware and needs no such care.

Instances keep their own dtype (complex64 storage is promoted to complex128 on the device, as the
reference's SVD and GEMM wrappers do, cython/svd.pxi:74-77, gemm.pxi:29-58); truncation decisions are
the FP64 ones of the selected precision mode.  Results are identical whatever S is (every kernel reduces
in a fixed order).
"""

from __future__ import annotations

import statistics
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

from . import _lib
from .core import Strategy

DEFAULT_STREAM_CANDIDATES = (1, 2, 4, 8, 12, 16, 24, 32)


@dataclass
class BatchReport:
    """Timing of one batch: wall time, per-instance latencies (seconds) and the stream count."""

    streams: int
    wall_s: float
    latencies_s: list = field(default_factory=list)

    @property
    def instances_per_s(self) -> float:
        return len(self.latencies_s) / self.wall_s if self.wall_s > 0 else 0.0

    def percentile(self, q: float) -> float:
        xs = sorted(self.latencies_s)
        if not xs:
            return 0.0
        k = min(len(xs) - 1, max(0, int(round(q / 100.0 * (len(xs) - 1)))))
        return xs[k]

    def summary(self) -> dict:
        return {"streams": self.streams, "instances": len(self.latencies_s),
                "wall_s": self.wall_s, "instances_per_s": self.instances_per_s,
                "p50_s": self.percentile(50), "p99_s": self.percentile(99),
                "mean_s": statistics.mean(self.latencies_s) if self.latencies_s else 0.0}


_worker = threading.local()
_pool_lock = threading.Lock()
_pool: ThreadPoolExecutor | None = None
_POOL_THREADS = max(DEFAULT_STREAM_CANDIDATES)


def _executor() -> ThreadPoolExecutor:
    """One persistent pool: its threads keep their library contexts and streams across batches
    (a context per short-lived thread would leave its device scratch behind)."""
    global _pool
    with _pool_lock:
        if _pool is None:
            _pool = ThreadPoolExecutor(max_workers=_POOL_THREADS, thread_name_prefix="sm-batch")
        return _pool


def _worker_stream(device: int, precision: str | None, contractions: str):
    import torch

    st = getattr(_worker, "stream", None)
    if st is None:
        torch.cuda.set_device(device)
        st = _worker.stream = torch.cuda.Stream(device=device)
        _worker.mode = None
        # this context shares the device with the other workers' streams
        _lib.check(_lib.load().sm_ctx_set_concurrent(_lib.context(device), 1))
    mode = (precision, contractions)
    if precision is not None and _worker.mode != mode:
        from ._lib import set_precision

        with torch.cuda.stream(st):
            set_precision(precision, device=device, contractions=contractions)
        _worker.mode = mode
    return st


def apply_batch(mpos, states, strategy: Strategy | None = None, streams: int = 8, device: int = 0,
                precision: str | None = None, contractions: str = "fp64"):
    """``[mpo.apply(state, strategy) for mpo, state in zip(mpos, states)]`` with ``streams``
    instances in flight.  ``precision`` (None keeps each worker context's mode) is one of
    ``seemps2_gb300.set_precision``'s modes.  Returns (results in input order, BatchReport)."""
    import torch

    if len(mpos) != len(states):
        raise ValueError("apply_batch needs one MPO per state")
    n = len(states)
    out = [None] * n
    lat = [0.0] * n
    streams = max(1, min(int(streams), _POOL_THREADS))
    gate = threading.Semaphore(streams)  # at most `streams` instances in flight

    def run(i):
        with gate:
            st = _worker_stream(device, precision, contractions)
            _lib.context(device)
            t0 = time.perf_counter()
            with torch.cuda.stream(st):
                mpo = mpos[i]
                res = mpo.apply(states[i], strategy=strategy or mpo.strategy)
                st.synchronize()
            lat[i] = time.perf_counter() - t0
            out[i] = res

    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    futures = [_executor().submit(run, i) for i in range(n)]
    for f in futures:
        f.result()  # re-raises an instance's exception
    torch.cuda.synchronize(device)
    wall = time.perf_counter() - t0
    return out, BatchReport(streams=streams, wall_s=wall, latencies_s=lat)


def tune_streams(mpos, states, strategy: Strategy | None = None, candidates=DEFAULT_STREAM_CANDIDATES,
                 sample: int = 64, device: int = 0, precision: str | None = None,
                 contractions: str = "fp64"):
    """The stream count with the highest instances/s on ``sample`` instances of the batch (the
    first ``sample`` of them, each candidate timed after one warm-up pass of the sample).
    Returns (best count, {count: instances/s})."""
    k = min(sample, len(states))
    mp, sts = mpos[:k], states[:k]
    apply_batch(mp, sts, strategy, streams=max(candidates), device=device, precision=precision,
                contractions=contractions)  # grows every worker's scratch once
    table = {}
    for s in candidates:
        _, rep = apply_batch(mp, sts, strategy, streams=s, device=device, precision=precision,
                             contractions=contractions)
        table[s] = rep.instances_per_s
    best = max(table, key=table.get)
    return best, table
