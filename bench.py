#!/usr/bin/env python
"""Benchmark of the MPO·MPS + simplify path: sweeps/s at n=30, chi=256.

Workload (one "step"): MPO.apply of the second-difference (Laplacian) MPO of
bond 3, tridiagonal [1,-2,1]/h^2 with h = 2^-30, on a random n=30 float64 MPS
of bond 256 (i.i.d. normal cores, QR-orthonormalised, normalised), followed by
variational simplify with tolerance 1e-12, max bond 256 and exactly 2 sweeps
(simplification_tolerance = 0 so the sweep count is fixed).  A step includes
the site products, the canonical-form guess and both sweeps.

Reported (one JSON line on rank 0):
  value        sweeps/s with inputs resident in GPU memory (CUDA events)
  e2e          same through the public API from pinned host arrays, host<->device
               copies inside the timed region
  phases       the step split into the MPO x MPS product, the canonical form
               of the product and the state norm + sweeps (by difference), with
               the sweep loop's own rate
  roofline     the dominant kernel: in the mixed forms the FP32 cluster
               factorisation (latency bound; the algorithmic SVD flops
               4mn^2 + 8n^3 of its splits against the FP32 SIMT peak of the
               whole GPU, the FP32 work as run beside it), else the dominant
               FP64 kernel (FP64 GEMM or Jacobi SVD) against the FP64 peak
               measured in this run (the library's FP64 GEMM; GB300 has no FP64
               tensor path); plus the FP64-accurate and 3xTF32 tensor-core
               products
  cpu_baseline the CPU oracle (NumPy/SciPy LAPACK, all host threads) on the
               same workload
`--impl reference` times that CPU implementation alone, same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

SEED = 20241203
METRIC = "MPO·MPS+simplify sweeps/s, n=30 χ=256: mixed+learned vs plain FP64, err≤1e-10"


def make_workload(n: int, chi: int, seed: int = SEED):
    """Seeded host arrays: (mps tensors, mpo tensors)."""
    from oracle import seemps_oracle as so

    rng = np.random.default_rng(seed)
    raw = so.random_mps(2, n, chi, rng)
    # QR-orthonormalise the cores left to right, normalise the last one
    mps = []
    carry = np.eye(1)
    for i, A in enumerate(raw):
        A = np.tensordot(carry, A, axes=1)
        a, d, b = A.shape
        if i < n - 1:
            Q, R = np.linalg.qr(A.reshape(a * d, b))
            mps.append(np.ascontiguousarray(Q.reshape(a, d, Q.shape[1])))
            carry = R
        else:
            mps.append(A / np.linalg.norm(A))
    h = 2.0 ** (-n)
    mpo = so.tridiagonal_mpo(n, -2.0 / h**2, 1.0 / h**2, 1.0 / h**2)
    return mps, [np.ascontiguousarray(O) for O in mpo]


def strategy_kwargs(chi: int, sweeps: int = 2):
    return dict(tolerance=1e-12, max_bond_dimension=chi, max_sweeps=sweeps,
                simplification_tolerance=0.0)


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_bf16_tflops() -> float:
    """Dense BF16 TFLOP/s measured on the GB300s (MEASURED_PEAKS.json, burst
    figure); 1900 (an earlier GB300 measurement) when the file is absent."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"])
    except (OSError, KeyError, ValueError):
        return 1900.0


def fp64_peak(torch, lib_mod) -> float:
    """Measured FP64 FLOP/s of this GPU: best of the library's FP64 GEMM (2048^3)."""
    import ctypes as C

    lib = lib_mod.load()
    ctx = lib_mod.context()
    n = 2048
    A = torch.randn(n, n, dtype=torch.float64, device="cuda")
    B = torch.randn(n, n, dtype=torch.float64, device="cuda")
    Cm = torch.empty(n, n, dtype=torch.float64, device="cuda")
    st = lib_mod.stream_handle()
    best = 0.0
    for _ in range(2):
        lib.sm_gemm(ctx, 0, 0, 0, n, n, n, lib_mod.ptr(A), n, lib_mod.ptr(B), n, lib_mod.ptr(Cm), n, st)
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            lib.sm_gemm(ctx, 0, 0, 0, n, n, n, lib_mod.ptr(A), n, lib_mod.ptr(B), n, lib_mod.ptr(Cm),
                        n, st)
        e1.record()
        e1.synchronize()
        best = max(best, 3 * 2.0 * n**3 / (e0.elapsed_time(e1) / 1e3))
    del C
    return best


def cpu_run(mps, mpo, chi, sweeps=2, want_result=False):
    """One oracle call (all host BLAS threads); returns (seconds, sweeps run[, result])."""
    from oracle import seemps_oracle as so

    st = so.DEFAULT_STRATEGY.replace(**strategy_kwargs(chi, sweeps))
    t = time.perf_counter()
    res = so.mpo_apply(mpo, mps, st)
    dt = time.perf_counter() - t
    return (dt, res.sweeps, res) if want_result else (dt, res.sweeps)


def phase_split(torch, sg, O, psi, st, step, flush, reps: int, sweeps: int) -> dict:
    """Where one MPO.apply + simplify step spends its time, each phase timed on its own
    with CUDA events (mean of `reps` runs, L2 flushed before each): the MPO x MPS
    product, the canonical form of the product that starts the sweeps (centre 0, with
    truncation, as the step runs it), and the rest of the step by difference: the state
    norm from the factors and the sweeps.  `sweep_loop` is the sweep rate of that rest."""

    def timed(fn):
        ts, r = [], None
        for _ in range(reps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            r = fn()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return sum(ts) / len(ts), r

    product_ms, prod = timed(lambda: O.apply(psi, strategy=st, simplify=False))
    canon_ms, _ = timed(lambda: sg.CanonicalMPS(prod, center=0, normalize=False, strategy=st))
    del prod
    step_ms, _ = timed(step)
    rest = step_ms - product_ms - canon_ms
    return {"product_ms": product_ms, "canonical_form_ms": canon_ms,
            "norm_and_sweeps_ms": rest, "step_ms": step_ms,
            "sweep_loop": {"value": sweeps / (rest / 1e3) if rest > 0 else None,
                           "unit": "sweeps/s", "sweeps": sweeps},
            "method": "product and canonical form timed as separate calls; the state norm "
                      "and the sweeps are the step minus both"}


def run_reference(args):
    """CPU implementation of the path (the oracle port) on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    mps, mpo = make_workload(args.n, args.chi)
    for _ in range(args.warmup):
        cpu_run(mps, mpo, args.chi)
    times, sw = [], 0
    for _ in range(args.steps):
        t, s = cpu_run(mps, mpo, args.chi)
        times.append(t)
        sw += s
    tot = sum(times)
    value = sw / tot
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "sweeps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": "sweeps/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full MPO.apply+simplify calls (2 sweeps each); "
                                   "NumPy/SciPy LAPACK gesdd restatement of the reference path"},
        "e2e": {"value": value, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args):
    return {"workload": f"MPO.apply(Laplacian bond-3 MPO, n={args.n} float64 MPS chi={args.chi}) "
                        f"+ variational simplify, tol 1e-12, max bond {args.chi}, 2 sweeps",
            "n": args.n, "chi": args.chi, "mpo_bond": 3, "tolerance": 1e-12,
            "max_bond_dimension": args.chi, "sweeps_per_step": 2, "form": args.form,
            "rank_cap": [getattr(args, "cap_margin", 1.15), getattr(args, "cap_extra", 10)],
            "learned_use": "range finder (rank + 10, %d power iterations)" % getattr(args, "rf_power", 0)
            if getattr(args, "range_finder", False) else "QR cap",
            "contractions": getattr(args, "contractions", "fp32"),
            "l2": "flushed between timed steps (256 MB write); the product MPS is >256 MB",
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


def run_split_case(args):
    """Single two-site splits (left-orthogonal, as in a left-to-right sweep) of an
    M x N matrix whose spectrum has the shape of the n=30, chi=256 workload's
    splits (256 values from 1 to 3e-3, two more at 2.5e-3 and 2.4e-3, then
    zeros), timed with CUDA events for both precision modes."""
    import torch

    import __graft_entry__

    __graft_entry__.build()
    import seemps2_gb300 as sg
    from seemps2_gb300 import _lib, core

    m, n = args.split_case
    rng = np.random.default_rng(SEED)
    k = min(m, n)
    s = np.concatenate([np.geomspace(1.0, 3e-3, 256), [2.5e-3, 2.4e-3]])[:k]
    Qa, _ = np.linalg.qr(rng.normal(size=(m, len(s))))
    Qb, _ = np.linalg.qr(rng.normal(size=(n, len(s))))
    A = (Qa * s) @ Qb.T
    AA = torch.from_numpy(np.ascontiguousarray(A.reshape(m // 2, 2, 2, n // 2))).cuda()
    st = sg.Strategy(tolerance=1e-12, max_bond_dimension=256)
    out = {"split_case": [m, n], "steps": args.steps}
    for form in ("plain", "mixed", "range_finder"):
        if form == "range_finder":  # the learned form's range finder at rank 256 + 10
            sg.set_precision("mixed+learned", range_finder=True, rank_hint=256,
                             power_iters=args.rf_power)
        else:
            sg.set_precision("fp64" if form == "plain" else "mixed")
        for _ in range(max(1, args.warmup)):
            core._left_orth_2site(AA, st)
        torch.cuda.synchronize()
        _lib.stats_reset()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            U, SV, err = core._left_orth_2site(AA, st)
        e1.record()
        e1.synchronize()
        stt = _lib.stats_read()
        out[form] = {"ms_per_split": e0.elapsed_time(e1) / args.steps, "D": int(U.shape[-1]),
                     "err": float(err), "launches_per_split": stt["launches"] / args.steps,
                     "mixed_fallbacks": stt["mixed_fallbacks"],
                     "fallback_reasons": {k: stt[k] for k in (
                         "mixed_fallback_cut", "mixed_fallback_fp32", "mixed_fallback_over",
                         "mixed_fallback_unconverged", "mixed_cap_redone", "rf_splits")},
                     "cluster_qr_ms": stt["cluster_qr_ms"] / args.steps,
                     "cluster_jacobi_ms": stt["cluster_jacobi_ms"] / args.steps,
                     "jacobi_sweeps_per_split": stt["jacobi_sweeps"] / args.steps}
    sg.set_precision("fp64")
    print(json.dumps(out), flush=True)


def make_batch_workload(count: int, seed: int = SEED + 4):
    """The batching configuration: `count` independent random MPS, complex64 storage, lengths
    n ~ U[10, 40], d = 2, uniform bond chi from {8, 16, 32, 64, 128} (i.i.d. complex normal,
    normalised), each with its own random complex MPO of bond D in {2, 4} (entries / sqrt(D d))."""
    from oracle import seemps_oracle as so

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(10, 41))
        chi = int(rng.choice([8, 16, 32, 64, 128]))
        D = int(rng.choice([2, 4]))
        mps = so.random_mps(2, n, chi, rng, complex_=True)
        nrm = np.sqrt(abs(so.scprod(mps, mps)))
        mps[0] = mps[0] / nrm
        mpo = so.random_mpo(2, n, D, rng, complex_=True)
        out.append(([t.astype(np.complex64) for t in mps], [t.astype(np.complex64) for t in mpo], chi))
    return out


def run_batch(args):
    """Batched compression: `--batch-count` instances (see make_batch_workload), each MPO.apply +
    simplify to tolerance 1e-8 with max bond = the instance's own chi (the product, bond chi D, is
    compressed back to chi), 2 sweeps, FP64 truncation decisions.  The stream autotuner picks the
    number of instances in flight on a 64-instance sample; the whole batch is then timed with it and
    with one instance at a time.  Reports MPS/s and p50 / p99 per-instance latency."""
    import torch

    import __graft_entry__

    __graft_entry__.build()
    import seemps2_gb300 as sg
    from seemps2_gb300 import batch
    from seemps2_gb300.distributed import combine_batch_reports, shard_indices

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:  # independent instances: a round-robin share per rank, no data exchange
        import torch.distributed as dist

        dist.init_process_group("nccl")
    inst_all = make_batch_workload(args.batch_count)
    mine = shard_indices(len(inst_all), rank, world)
    inst = [inst_all[i] for i in mine]
    mpos = [sg.MPO(mpo, sg.DEFAULT_STRATEGY.replace(tolerance=1e-8, max_bond_dimension=chi,
                                                    max_sweeps=2, simplification_tolerance=0.0))
            for mps, mpo, chi in inst]
    states = [sg.MPS(mps) for mps, mpo, chi in inst]
    precision = {"plain": "fp64", "mixed": "mixed", "mixed+learned": "mixed"}[args.form]
    best, table = batch.tune_streams(mpos, states, sample=64, device=local, precision=precision)
    if dist:
        dist.barrier()
    res, rep = batch.apply_batch(mpos, states, streams=best, device=local, precision=precision)
    job = None
    if dist:
        job = combine_batch_reports(rep.wall_s, len(rep.latencies_s), rep.latencies_s,
                                    device=torch.device("cuda", local))
    if world > 1 and rank != 0:
        dist.destroy_process_group()
        return
    _, rep1 = batch.apply_batch(mpos, states, streams=1, device=local, precision=precision)
    check = None
    if not args.no_cpu:
        from oracle import seemps_oracle as so

        worst = 0.0
        for (mps, mpo, chi), out in list(zip(inst, res))[:8]:
            ref = so.mpo_apply([t.astype(np.complex128) for t in mpo],
                               [t.astype(np.complex128) for t in mps],
                               so.DEFAULT_STRATEGY.replace(tolerance=1e-8, max_bond_dimension=chi,
                                                           max_sweeps=2,
                                                           simplification_tolerance=0.0))
            fe = so.fidelity_error([x.detach().cpu().numpy() for x in out._data], ref.tensors)
            worst = max(worst, float(fe))
        check = {"instances_checked": 8, "max_fidelity_error_vs_oracle": worst}
    sizes = [(len(m), chi) for m, _, chi in inst_all]
    value = job["instances_per_s"] if job else rep.instances_per_s
    print(json.dumps({
        "metric": "batched MPO.apply+simplify, MPS/s", "value": value, "unit": "MPS/s",
        "higher_is_better": True, "n_gpus": world, "form": args.form,
        "scaling": "strong (the batch is split over the ranks)",
        "whole_job": job,
        "config": {"workload": f"{len(inst_all)} MPS, n~U[10,40], chi in {{8..128}}, D in {{2,4}}, "
                               "complex64 storage, tol 1e-8, max bond = chi, 2 sweeps",
                   "sites_total": sum(n for n, _ in sizes)},
        "streams": best, "autotune_instances_per_s": table,
        "p50_s": rep.percentile(50), "p99_s": rep.percentile(99), "wall_s": rep.wall_s,
        "one_in_flight": rep1.summary(), "speedup_vs_one_in_flight":
            rep.instances_per_s / rep1.instances_per_s if rep1.instances_per_s else None,
        "oracle_check": check}), flush=True)
    if dist:
        dist.destroy_process_group()


def run_dmrg_matvec(args):
    """The DMRG configuration's hot operation: the two-site effective-Hamiltonian matvec at
    chi = 256 of a Heisenberg chain (MPO bond 5, d = 2), environments with i.i.d. normal entries
    (the cost does not depend on their values), the two-site MPO of the chain's bulk.  Each
    precision is timed over 50 matvecs with CUDA events and compared with the FP64 result; the
    oracle's NumPy matvec is timed on the host cores; a 30-vector Lanczos run (FP64
    re-orthogonalisation) is timed at FP64 and BF16."""
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from oracle import dmrg_oracle as do
    from seemps2_gb300 import dmrg

    chi, D, d = 256, 5, 2
    rng = np.random.default_rng(SEED + 7)
    W = do.heisenberg_mpo(8)
    H = do.two_site_hamiltonian(W[3], W[4])
    L = rng.normal(size=(chi, D, chi))
    R = rng.normal(size=(chi, D, chi))
    L = 0.5 * (L + L.transpose(2, 1, 0))
    R = 0.5 * (R + R.transpose(2, 1, 0))
    v = rng.normal(size=(chi, d, d, chi))
    Ld, Hd, Rd, vd = (torch.from_numpy(x).cuda() for x in (L, H, R, v))
    flops = 2.0 * chi * D * chi * d * d * chi * 2 + 2.0 * chi * chi * (D * d * d) ** 2
    out = {"workload": f"two-site matvec, chi={chi}, MPO bond {D} (Heisenberg), d={d}",
           "flops_per_matvec": flops}
    ref = None
    for prec in ("fp64", "fp64tc", "tf32x3", "bf16"):
        o = torch.empty((chi, d, d, chi), dtype=torch.float64, device="cuda")
        for _ in range(3):
            dmrg.two_site_matvec(Ld, Hd, Rd, vd, prec, out=o)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(50):
            dmrg.two_site_matvec(Ld, Hd, Rd, vd, prec, out=o)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / 50
        res = o.cpu().numpy()
        if ref is None:
            ref = res
        out[prec] = {"ms_per_matvec": ms, "matvecs_per_s": 1e3 / ms,
                     "tflops": flops / (ms / 1e3) / 1e12,
                     "rel_err_vs_fp64": float(np.linalg.norm(res - ref) / np.linalg.norm(ref))}
    for prec in ("tf32x3", "bf16"):  # prepared operator: environments converted once
        op = dmrg.TwoSiteOperator(Ld, Hd, Rd, prec)
        o = torch.empty((chi, d, d, chi), dtype=torch.float64, device="cuda")
        for _ in range(3):
            op.matvec(vd, out=o)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(50):
            op.matvec(vd, out=o)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / 50
        res = o.cpu().numpy()
        out[f"{prec}_prepared"] = {"ms_per_matvec": ms, "matvecs_per_s": 1e3 / ms,
                                   "tflops": flops / (ms / 1e3) / 1e12,
                                   "rel_err_vs_fp64": float(np.linalg.norm(res - ref) /
                                                            np.linalg.norm(ref))}
    out["bf16"]["frac_of_bf16_peak"] = out["bf16"]["tflops"] / measured_bf16_tflops()
    out["bf16_prepared"]["frac_of_bf16_peak"] = (out["bf16_prepared"]["tflops"] /
                                                 measured_bf16_tflops())
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        do.two_site_matvec(L, H, R, v)
    cpu_ms = (time.perf_counter() - t0) / reps * 1e3
    out["cpu_oracle"] = {"ms_per_matvec": cpu_ms, "cores": os.cpu_count(),
                         "kind": "port (NumPy, the reference's own reshape/GEMM sequence)"}
    for prec in ("fp64", "bf16"):
        dmrg.lanczos_ground_state(Ld, Hd, Rd, vd, krylov=4, precision=prec)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ev, _, steps = dmrg.lanczos_ground_state(Ld, Hd, Rd, vd, krylov=30, precision=prec)
        torch.cuda.synchronize()
        out[f"lanczos_{prec}"] = {"s": time.perf_counter() - t0, "steps": steps, "eigenvalue": ev}
    out["lanczos_bf16"]["rel_diff_vs_fp64"] = abs(out["lanczos_bf16"]["eigenvalue"] -
                                                  out["lanczos_fp64"]["eigenvalue"]) / abs(
        out["lanczos_fp64"]["eigenvalue"])
    print(json.dumps(out), flush=True)


def make_dmrg_workload(L: int, chi: int, seed: int = SEED + 11):
    """The DMRG configuration's inputs: the spin-1/2 Heisenberg chain's MPO (J = 1, open
    boundaries, bond 5) as the reference's HeisenbergHamiltonian(L).to_mpo() builds it
    (recorded from the reference in tests/golden/heisenberg_mpo_L100.npz; its bulk tensor
    repeats, so shorter chains take the first and last tensors around L - 2 bulk ones),
    and a random float64 guess of bond chi (i.i.d. normal cores, each scaled to unit
    Frobenius norm so that the chain's norm stays in range; the driver normalises it)."""
    from oracle import seemps_oracle as so

    z = np.load(os.path.join(ROOT, "tests", "golden", "heisenberg_mpo_L100.npz"))
    W100 = [z[f"W{i}"] for i in range(100)]
    W = [W100[0]] + [W100[1]] * (L - 2) + [W100[99]] if L != 100 else W100
    rng = np.random.default_rng(seed)
    guess = [A / np.linalg.norm(A) for A in so.random_mps(2, L, chi, rng)]
    return W, guess


def run_dmrg(args):
    """The DMRG configuration end to end: two two-site DMRG sweeps of the L-site Heisenberg
    chain from a random bond-chi guess, truncation tolerance 1e-10, max bond chi.  Forms:
    "fp64" (FP64 matvecs and FP64 splits, the reference's arithmetic) and "bf16" (the
    precision pattern: BF16 tensor-core matvecs with FP32 accumulation for the Krylov
    basis, re-orthogonalised in FP64, each eigenpair polished with FP64-accurate
    tensor-core matvecs; mixed-precision splits with FP64 truncation decisions).  Reports
    sweeps/s, ms per two-site step and the energies.  The eigensolver tolerance is the
    reference's default (tol_eigs = tol = 1e-10).  The CPU oracle (scipy eigsh, NumPy, all
    host cores) is timed on the first steps of the first sweep."""
    import torch

    import __graft_entry__

    __graft_entry__.build()
    import seemps2_gb300 as sg
    from oracle import dmrg_oracle as do
    from oracle import seemps_oracle as so
    from seemps2_gb300 import _lib, dmrg

    L, chi = args.dmrg_sites, args.dmrg_chi
    W, guess = make_dmrg_workload(L, chi)
    st = sg.DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=chi)
    H = sg.MPO(W)
    out = {"workload": f"two-site DMRG, Heisenberg chain L={L} (MPO bond 5, the reference's "
                       f"to_mpo), random guess of bond {chi}, tolerance 1e-10, max bond {chi}, "
                       "2 sweeps", "sweeps": 2}
    for form, prec, split in (("fp64", "fp64", "fp64"), ("bf16", "bf16", "mixed")):
        sg.set_precision(split)
        # warm-up on a short chain (kernels loaded, buffers sized)
        Ws, gs = make_dmrg_workload(6, 8)
        dmrg.dmrg(sg.MPO(Ws), guess=sg.MPS(gs), maxiter=1, strategy=st, precision=prec)
        torch.cuda.synchronize()
        _lib.stats_reset()
        t0 = time.perf_counter()
        res = dmrg.dmrg(H, guess=sg.MPS(guess), maxiter=2, strategy=st, precision=prec)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        stt = _lib.stats_read()
        nsw = len(res.trajectory) - 1
        out[form] = {"s": dt, "sweeps_per_s": nsw / dt, "ms_per_step": 1e3 * dt / (nsw * (L - 1)),
                     "trajectory": res.trajectory, "variances": res.variances,
                     "bonds_max": max(res.state.bond_dimensions()),
                     "launches": stt["launches"], "mixed_splits": stt["mixed_splits"],
                     "mixed_fallbacks": stt["mixed_fallbacks"]}
    sg.set_precision("fp64")
    out["bf16"]["energy_diff_vs_fp64"] = out["bf16"]["trajectory"][-1] - out["fp64"]["trajectory"][-1]
    if not args.no_cpu:
        nsteps = args.dmrg_cpu_steps
        t0 = time.perf_counter()
        do.dmrg(W, guess, maxiter=1,
                strategy=so.DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=chi),
                max_steps=nsteps)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {
            "kind": "port", "cores": os.cpu_count(),
            "sample": f"the oracle's canonical form, environments and first {nsteps} two-site "
                      f"steps of sweep 1 ({dt:.1f} s), scaled to a sweep of {L - 1} steps",
            "s_per_step": dt / nsteps, "sweeps_per_s": nsteps / (dt * (L - 1))}
    print(json.dumps(out), flush=True)


def run_gemm_case(args):
    """One real M x N x K product (op N, N) timed with CUDA events: the FP64 SIMT
    GEMM, the tensor-core 3xTF32 GEMM (FP32 accuracy) and the FP64-accurate
    tensor-core GEMM (BF16 slices), each with its operand preparation and
    split-K reduction."""
    import ctypes as C

    import torch

    import __graft_entry__

    __graft_entry__.build()
    from seemps2_gb300 import _lib

    M, N, K = args.gemm_case
    rng = np.random.default_rng(SEED)
    A = torch.from_numpy(rng.normal(size=(M, K))).cuda()
    B = torch.from_numpy(rng.normal(size=(K, N))).cuda()
    out = {"gemm_case": [M, N, K], "steps": args.steps}
    ref = None
    for name, fn in (("fp64", "sm_gemm"), ("tf32x3", "sm_gemm_f32"),
                     ("fp64_tensor_cores", "sm_gemm_f64tc")):
        Cm = torch.empty((M, N), dtype=torch.float64, device="cuda")
        f = getattr(_lib.load(), fn)
        call = lambda: _lib.check(f(_lib.context(), 0, 0, 0, M, N, K, C.c_void_p(A.data_ptr()), K,
                                    C.c_void_p(B.data_ptr()), N, C.c_void_p(Cm.data_ptr()), N,
                                    _lib.stream_handle()))
        for _ in range(max(1, args.warmup)):
            call()
        torch.cuda.synchronize()
        _lib.stats_reset()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            call()
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        res = Cm.cpu().numpy()
        if ref is None:
            ref = res
        out[name] = {"ms": ms, "tflops": 2.0 * M * N * K / (ms / 1e3) / 1e12,
                     "tc_launches": _lib.stats_read()["gemm_tc_launches"] / args.steps,
                     "oz_launches": _lib.stats_read()["gemm_oz_launches"] / args.steps,
                     "rel_err_vs_fp64": float(np.linalg.norm(res - ref) / np.linalg.norm(ref))}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=30)
    ap.add_argument("--chi", type=int, default=256)
    ap.add_argument("--form", default="mixed+learned", choices=["plain", "mixed", "mixed+learned"],
                    help="plain = FP64 splits (reference ranks); mixed = FP32 cluster "
                         "factorisation + FP64 refinement; mixed+learned = mixed with the rank "
                         "predictor capping the FP32 QR (the metric's headline form)")
    ap.add_argument("--contractions", default="fp32", choices=["fp64", "fp32"],
                    help="accuracy of the sweep contractions in the mixed forms: fp32 = 3xTF32 "
                         "on the tensor cores (FP32 SIMT for small or complex shapes); the "
                         "state norm, the refinement and the final estimate stay FP64")
    ap.add_argument("--rank-model", default=None,
                    help="trained rank predictor (.npz); default: the packaged model "
                         "(seemps2_gb300/data/rank_model.npz), else trained here")
    ap.add_argument("--train-count", type=int, default=90,
                    help="training workloads recorded when the predictor is trained here")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--cap-margin", type=float, default=1.15,
                    help="learned cap of the FP32 QR: ceil(margin * predicted rank) + extra rows")
    ap.add_argument("--cap-extra", type=int, default=10)
    ap.add_argument("--range-finder", action="store_true",
                    help="mixed+learned: the predicted rank sizes a randomized range finder (rank + "
                         "10 columns) instead of capping the FP32 QR")
    ap.add_argument("--rf-power", type=int, default=0,
                    help="subspace (power) iterations of the range finder")
    ap.add_argument("--split-case", type=int, nargs=2, metavar=("M", "N"),
                    help="time single M x N two-site splits in both precision modes and exit")
    ap.add_argument("--gemm-case", type=int, nargs=3, metavar=("M", "N", "K"),
                    help="time one real M x N x K product on the tensor cores (3xTF32) and as "
                         "the FP64 GEMM, and exit")
    ap.add_argument("--dmrg", action="store_true",
                    help="two DMRG sweeps of the Heisenberg chain (FP64 and the BF16 pattern), "
                         "sweeps/s and energies, and exit")
    ap.add_argument("--dmrg-sites", type=int, default=100)
    ap.add_argument("--dmrg-chi", type=int, default=256)
    ap.add_argument("--dmrg-cpu-steps", type=int, default=8)
    ap.add_argument("--dmrg-matvec", action="store_true",
                    help="time the DMRG two-site matvec (chi 256, MPO bond 5) per precision and exit")
    ap.add_argument("--batch", action="store_true",
                    help="batched compression of many independent MPS (MPS/s, p50/p99) and exit")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--profile-step", action="store_true",
                    help="after the warm-up, run one step of --form between cudaProfilerStart "
                         "and cudaProfilerStop (for ncu --profile-from-start off) and exit")
    args = ap.parse_args()
    if args.split_case:
        return run_split_case(args)
    if args.gemm_case:
        return run_gemm_case(args)
    if args.batch:
        return run_batch(args)
    if args.dmrg_matvec:
        return run_dmrg_matvec(args)
    if args.dmrg:
        return run_dmrg(args)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    import __graft_entry__

    __graft_entry__.build()
    import seemps2_gb300 as sg
    from seemps2_gb300 import _lib

    mps_h, mpo_h = make_workload(args.n, args.chi)
    st = sg.DEFAULT_STRATEGY.replace(**strategy_kwargs(args.chi))
    psi = sg.MPS(mps_h)
    O = sg.MPO(mpo_h, st)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def step():
        return O.apply(psi, strategy=st)

    # ---- rank predictor (outside every timed region) ---------------------------
    learned_info = None
    if args.form == "mixed+learned":
        from seemps2_gb300 import learned

        t0 = time.perf_counter()
        path = args.rank_model or learned.PACKAGED_MODEL
        if path and os.path.exists(path):
            model = learned.RankModel.load(path)
            meta = np.load(path)
            learned_info = {"model": os.path.relpath(path, ROOT),
                            **{k: meta[k].item() for k in ("truncations", "workloads", "record_s",
                                                           "train_s", "loss_last") if k in meta}}
        else:
            model, rep = learned.train_default(count=args.train_count, epochs=40, seed=1)
            learned_info = {"model": "trained in this run on the GPU (library kernels)", **rep}
        model.install()
        learned_info["setup_s"] = time.perf_counter() - t0

    # ---- plain FP64 form on the same workload (the metric's comparison) -------
    plain = None
    if args.profile_step:
        sg.set_precision({"plain": "fp64", "mixed": "mixed", "mixed+learned": "mixed+learned"}[
            args.form], contractions=args.contractions)
        for _ in range(max(3, args.warmup)):
            step()
        torch.cuda.synchronize()
        _lib.stats_reset(timing=False)
        torch.cuda.profiler.start()
        step()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        stt = _lib.stats_read()
        print(json.dumps({"profile_step": args.form, "contractions": args.contractions,
                          "launches": stt["launches"]}), flush=True)
        return
    def time_form(precision, **kw):
        sg.set_precision(precision, **kw)
        step()
        torch.cuda.synchronize()
        pt = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            step()
            e1.record()
            e1.synchronize()
            pt.append(e0.elapsed_time(e1))
        psw = sg.state.last_report["sweeps"]
        return {"value": psw * len(pt) / (sum(pt) / 1e3), "unit": "sweeps/s",
                "ms_per_step": sum(pt) / len(pt)}

    no_predictor = rf_form = None
    if args.form != "plain":
        plain = time_form("fp64")
    if args.form == "mixed+learned":
        # the same mixed form without the rank predictor: what the learned part gains
        no_predictor = time_form("mixed", contractions=args.contractions)
        # the other use of the predicted rank: sizing a randomized range finder
        _lib.stats_reset(timing=False)
        rf_form = time_form("mixed+learned", contractions=args.contractions,
                            range_finder=not args.range_finder, power_iters=args.rf_power)
        s_rf = _lib.stats_read()
        kk = max(1, args.steps + 1)
        rf_form.update({"range_finder": not args.range_finder,
                        "rf_splits_per_step": s_rf["rf_splits"] / kk,
                        "redone_per_step": s_rf["mixed_cap_redone"] / kk,
                        "fallbacks_per_step": s_rf["mixed_fallbacks"] / kk})
    sg.set_precision({"plain": "fp64", "mixed": "mixed", "mixed+learned": "mixed+learned"}[args.form],
                     contractions=args.contractions,
                     range_finder=args.range_finder and args.form == "mixed+learned",
                     power_iters=args.rf_power)
    _lib.check(_lib.load().sm_ctx_set_rank_cap(_lib.context(), args.cap_margin, args.cap_extra))

    for _ in range(max(3, args.warmup)):
        out = step()
    torch.cuda.synchronize()
    sweeps_per_step = sg.state.last_report["sweeps"]

    # ---- device-resident timing ---------------------------------------------
    _lib.stats_reset(timing=False)
    times = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            out = step()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    timed_stats = _lib.stats_read()
    launches = timed_stats["launches"]
    total_ms = sum(times)
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.barrier()
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * sweeps_per_step * args.steps / (total_ms / 1e3)

    # ---- end to end through the public API with host buffers -----------------
    mps_pin = [torch.from_numpy(a).pin_memory() for a in mps_h]
    mpo_pin = [torch.from_numpy(a).pin_memory() for a in mpo_h]
    h2d = sum(a.nbytes for a in mps_h) + sum(a.nbytes for a in mpo_h)
    e2e_times, d2h = [], 0
    for k in range(args.steps + 1):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = sg.MPO(mpo_pin, st).apply(sg.MPS(mps_pin), strategy=st)
        host = [t.cpu() for t in res._data]
        torch.cuda.synchronize()
        if k:  # first call warms the pinned path
            e2e_times.append(time.perf_counter() - t0)
        d2h = sum(t.numel() * t.element_size() for t in host)
    e2e_value = world * sweeps_per_step / statistics.mean(e2e_times)

    # ---- phase split of the step ----------------------------------------------
    try:
        phases = phase_split(torch, sg, O, psi, st, step, flush, max(1, args.steps),
                             sweeps_per_step)
    except Exception as exc:  # a reporting extra must not hide the line
        phases = {"failed": f"{type(exc).__name__}: {exc}"}

    # ---- roofline of the dominant kernel (one instrumented step) -----------
    _lib.stats_reset(timing=True)
    torch.cuda.synchronize()
    ei0 = torch.cuda.Event(enable_timing=True)
    ei1 = torch.cuda.Event(enable_timing=True)
    ei0.record()
    step()
    ei1.record()
    ei1.synchronize()
    inst_ms = ei0.elapsed_time(ei1)
    stt = _lib.stats_read()
    _lib.stats_reset(timing=False)
    peak = fp64_peak(torch, _lib)
    # the dominant FP64 kernel of the step (event-timed per launch in this step)
    cands = {"k_jacobi (one-sided Jacobi SVD, FP64)": ("jacobi", stt["jacobi_flops"],
                                                      stt["jacobi_ms"], stt["jacobi_launches"]),
             "k_gemm (SIMT FP64 GEMM, split-K)": ("gemm", stt["gemm_flops"], stt["gemm_ms"],
                                                  stt["gemm_launches"])}
    kname, (tag, kfl, kms, kl) = max(cands.items(), key=lambda kv: kv[1][2])
    achieved = kfl / (kms / 1e3) if kms else 0.0
    fp64_roof = {
        "bound": "fp64", "kernel": kname,
        "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
        "frac": achieved / peak if peak else None, "traffic": None,
        "peak_source": "measured in this run: the library's FP64 GEMM at 2048^3 (GB300 FP64 has "
                       "no tensor-core path; MEASURED_PEAKS.json lists HBM and bf16 only)",
        "flops_per_launch": kfl / max(1, kl), "launches_per_step": kl,
        "avg_launch_ms": kms / max(1, kl), "share_of_step": kms / inst_ms if inst_ms else None,
    }
    roofline = dict(fp64_roof)
    if stt["cluster_ms"] > kms and stt["mixed_splits"]:
        # the mixed forms' dominant kernel: the FP32 cluster factorisation, one launch per mixed
        # split on the 16 SMs of one thread-block cluster; bound by latency (barriers and each
        # pair step's dependent chain), so its FP32 rate is reported against the SIMT peak of
        # those 16 SMs and of the whole GPU at the sampled SM clock
        nl = stt["mixed_splits"]
        sec = stt["cluster_ms"] / 1e3
        alg = stt["cluster_alg_flops"] / sec  # algorithmic SVD flops (4mn^2 + 8n^3 per split)
        run = stt["cluster_flops"] / sec      # FP32 flops as run (QR reflectors, Jacobi pairs)
        mhz = clk.summary().get("sm_mhz") or 2070.0
        fp32_sm = 128 * 2 * mhz * 1e6  # FP32 FMA lanes per SM x 2 flops x clock
        n_sm = torch.cuda.get_device_properties(0).multi_processor_count
        roofline = {
            "bound": "latency", "kernel": "k_split_cluster (FP32 blocked QR + block-cyclic "
                                          "one-sided Jacobi, 16-CTA cluster)",
            "achieved": alg / 1e12, "peak": n_sm * fp32_sm / 1e12, "unit": "TFLOP/s",
            "frac": alg / (n_sm * fp32_sm),
            "work_convention": "algorithmic SVD flops 4mn^2 + 8n^3 per m x n split (m >= n), "
                               "summed over the step's cluster launches at their real shapes",
            "peak_source": f"nominal FP32 SIMT rate of the whole GPU ({n_sm} SMs x 128 FMA lanes "
                           "x 2 at the sampled SM clock); MEASURED_PEAKS.json has no FP32 SIMT "
                           "figure",
            "flops_per_launch": stt["cluster_alg_flops"] / nl, "launches_per_step": nl,
            "avg_launch_ms": stt["cluster_ms"] / nl,
            "share_of_step": stt["cluster_ms"] / inst_ms if inst_ms else None,
            "traffic": stt["cluster_bytes"] / nl,
            "traffic_source": "derived per launch: the split matrix read once and the converged "
                              "rows written (FP64); an ncu capture of a 512 x 512 launch read "
                              "1.1x the matrix bytes, everything else stays on chip",
            "as_run": {"achieved": run / 1e12, "unit": "TFLOP/s (FP32 work as run)",
                       "frac_of_16_sms": run / (16 * fp32_sm),
                       "frac_of_gpu": run / (n_sm * fp32_sm)},
            "fp64_simt": fp64_roof,
        }
    if stt["gemm_oz_launches"]:
        oz_ach = stt["gemm_oz_flops"] / (stt["gemm_oz_ms"] / 1e3) if stt["gemm_oz_ms"] else 0.0
        roofline["fp64_tensor_core_gemm"] = {
            "kernel": "k_gemm_oz (FP64-accurate: 8 BF16 slices, 36 tcgen05 products; slicing "
                      "and split-K reduce included)",
            "launches_per_step": stt["gemm_oz_launches"],
            "flops_per_launch": stt["gemm_oz_flops"] / stt["gemm_oz_launches"],
            "achieved": oz_ach / 1e12, "unit": "TFLOP/s (FP64-equivalent 2MNK / time)",
            "vs_fp64_peak": oz_ach / peak if peak else None,
            "share_of_step": stt["gemm_oz_ms"] / inst_ms if inst_ms else None,
        }
    if stt["gemm_tc_launches"]:
        tc_ach = stt["gemm_tc_flops"] / (stt["gemm_tc_ms"] / 1e3) if stt["gemm_tc_ms"] else 0.0
        tf32_peak = measured_bf16_tflops() / 2.0
        roofline["tensor_core_gemm"] = {
            "kernel": "k_gemm_tc (3xTF32, tcgen05 + TMA; split and split-K reduce included)",
            "launches_per_step": stt["gemm_tc_launches"],
            "flops_per_launch": stt["gemm_tc_flops"] / stt["gemm_tc_launches"],
            "achieved": tc_ach / 1e12, "unit": "TFLOP/s (2MNK / time)",
            "peak": tf32_peak, "frac": tc_ach / 1e12 / tf32_peak if tf32_peak else None,
            "peak_source": "half the measured bf16 dense rate (MEASURED_PEAKS.json): GB300 runs "
                           "TF32 at half the BF16 rate; each product issues 3 TF32 MMAs",
            "share_of_step": stt["gemm_tc_ms"] / inst_ms if inst_ms else None,
        }

    # ---- CPU baseline (oracle, bounded sample) -------------------------------
    cpu = None
    oracle_check = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import seemps_oracle as so

        try:
            t, s, res = cpu_run(mps_h, mpo_h, args.chi, want_result=True)
            import numpy as _np

            out_np = [x.detach().cpu().numpy() for x in out._data]
            oracle_check = {"fidelity_error_vs_oracle": float(so.fidelity_error(out_np, res.tensors)),
                            "error_bound": float(out.error()), "oracle_error_bound": float(res.error),
                            "bonds_equal": out.bond_dimensions()[:-1] == [x.shape[0] for x in res.tensors]}
            del _np
            cpu = {"value": s / t, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": "one full MPO.apply+simplify call of this workload (2 sweeps), "
                             f"{t:.1f} s; NumPy/SciPy BLAS+LAPACK restatement of the reference "
                             f"path (gesdd; gesvd retries: {so.GESDD_RETRIES[0]})"}
        except Exception as exc:  # a CPU-side LAPACK failure must not hide the GPU line
            cpu = {"value": None, "unit": "sweeps/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {type(exc).__name__}: {exc}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.form == "plain" else "f32+f64",
            "data": "synthetic", "config": workload_config(args),
            "e2e": {"value": e2e_value, "unit": "sweeps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk.summary(),
            "gpu_launches": launches, "bonds_out": out.bond_dimensions()[: args.n // 2 + 1],
            "error": out.error(), "oracle_check": oracle_check, "phases": phases,
        }
        if plain:
            line["plain_fp64"] = plain
            line["speedup_vs_plain_fp64"] = value / plain["value"] if plain["value"] else None
        if args.form != "plain":
            k = max(1, args.steps)
            line["mixed"] = {
                "splits_per_step": timed_stats["mixed_splits"] / k,
                "fallbacks_per_step": timed_stats["mixed_fallbacks"] / k,
                "rows_per_split": timed_stats["mixed_rows"] / max(1, timed_stats["mixed_splits"]),
                "cluster_ms_per_step": stt["cluster_ms"],
                "cluster_qr_ms_per_step": timed_stats["cluster_qr_ms"] / k,
                "cluster_jacobi_ms_per_step": timed_stats["cluster_jacobi_ms"] / k,
                "fallbacks_coupling_per_step": timed_stats["mixed_fallback_cut"] / k,
                "fallbacks_fp32_per_step": timed_stats["mixed_fallback_fp32"] / k,
                "fallbacks_over_tolerance_per_step": timed_stats["mixed_fallback_over"] / k,
                "fallbacks_unconverged_per_step": timed_stats["mixed_fallback_unconverged"] / k,
                "capped_per_step": timed_stats["mixed_capped"] / k,
                "cap_redone_per_step": timed_stats["mixed_cap_redone"] / k,
                "mean_predicted_rank": timed_stats["rank_predicted_sum"]
                / max(1, timed_stats["rank_predictions"]),
            }
            if learned_info:
                line["learned"] = learned_info
            if no_predictor:
                line["mixed_without_predictor"] = no_predictor
                line["predictor_gain"] = value / no_predictor["value"] if no_predictor["value"] else None
            if rf_form:
                line["learned_other_use"] = rf_form
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
