"""Generate golden fixtures by running the reference SeeMPS itself.

The reference is built out of tree by ``oracle/build_reference.sh REF_DIR OUT_DIR``
(this script reads OUT_DIR, ``/tmp/seemps_ref`` unless given).  This script runs
each case twice in child processes:

* with the reference's compiled Cython backend (its production path) to record
  the final outputs of ``MPO.apply`` / ``simplify`` and of the truncation rule,
  and every SVD split of the run: the splits happen inside compiled kernels, so
  the run's Python-level call sites are wrapped (``CanonicalMPS``'s
  ``_canonicalize`` restated as the loop of the compiled
  ``_update_in_canonical_form_*`` kernels it runs, and the two-site
  ``_left/_right_orth_2site``); each wrapper takes the singular values of the
  matrix about to be split with LAPACK gesdd, as the compiled kernel does, and the
  kept rank and discarded weight from the compiled kernel's own result;
* with its pure-NumPy backend (``SEEMPS_BACKEND=python``), whose module-level
  ``_truncate`` can be wrapped, to record every split of the small cases a second
  way (its unoptimised environment einsums make it impractical at bond 128+);
  both records must agree.

Inputs are generated from fixed seeds by ``oracle.seemps_oracle.random_mps`` /
``random_mpo`` / ``tridiagonal_mpo``; each fixture stores the seed and a SHA-256
of the generated input bytes so a consumer can verify it regenerated the same
arrays.  Outputs go to ``tests/golden/*.npz`` and ``truncation_cases.json``.

The DMRG fixtures (``dmrg_*.npz``, ``heisenberg_mpo_L100.npz``) come from the
reference's ``HeisenbergHamiltonian(L).to_mpo()``, ``QuadraticForm.two_site_operator``
and ``dmrg`` run with the Cython backend (see ``_dmrg_child``).

Usage:  oracle/build_reference.sh REF_DIR OUT_DIR && python tests/golden/make_golden.py [OUT_DIR]
"""

from __future__ import annotations

import hashlib
import json
import os
import pickle
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import seemps_oracle as so  # noqa: E402

# name -> (kind, params)
CASES = {
    # configuration 1 of the workload list at reduced size (dense-checkable)
    "c1_small": dict(kind="mpo_apply", n=10, d=2, chi=16, D=4, complex=True,
                     tol=1e-10, maxchi=24, sweeps=2, seed=101),
    # configuration 1 at full size: n=20, chi=32, complex128, D=4, tol 1e-10, maxchi 64
    "c1": dict(kind="mpo_apply", n=20, d=2, chi=32, D=4, complex=True,
               tol=1e-10, maxchi=64, sweeps=2, seed=102),
    # real Laplacian (tridiagonal [1,-2,1]/h^2) on a random real MPS
    # These results are exact up to rounding, so the sweep estimate `err` sits at
    # ~1e-15, next to the default simplification tolerance (eps): whether the
    # loop stops after sweep 1 is decided by rounding noise (the reference's own
    # two backends disagree).  stol=0 makes the sweep count deterministic.
    "lap_small": dict(kind="laplacian", n=12, d=2, chi=16, tol=1e-12, maxchi=32,
                      sweeps=2, seed=103, stol=0.0),
    "lap_n30_chi32": dict(kind="laplacian", n=30, d=2, chi=32, tol=1e-12, maxchi=64,
                          sweeps=2, seed=104, stol=0.0),
    # Euler step x + dt * L x simplified as an MPSSum
    "euler_small": dict(kind="euler", n=10, d=2, chi=16, tol=1e-12, maxchi=32,
                        sweeps=2, seed=105, dt=1e-3, stol=0.0),
    # plain simplify of a random real MPS with a bond cap
    "simplify_real": dict(kind="simplify", n=12, d=2, chi=64, complex=False,
                          tol=1e-8, maxchi=12, sweeps=3, seed=106),
    # configuration 2 proper: n=30 float64 MPS of bond 128 with QR-orthonormalised
    # random cores, explicit Euler step x + 1e-3 L x (Laplacian, h = 2^-30) as an
    # MPSSum, simplified to tolerance 1e-12 with max bond 256.  Singular values are
    # stored up to the kept rank + 16 (s_keep) to keep the fixture small.
    "c2": dict(kind="euler", n=30, d=2, chi=128, ortho=True, tol=1e-12, maxchi=256,
               sweeps=2, seed=107, dt=1e-3, stol=0.0, s_keep=16, large=True),
    # the benchmark's own workload (same seed and input construction): n=30, bond 256,
    # QR-orthonormalised cores, Laplacian MPO, tolerance 1e-12, max bond 256, 2 sweeps
    "northstar": dict(kind="laplacian", n=30, d=2, chi=256, ortho=True, tol=1e-12,
                      maxchi=256, sweeps=2, seed=20241203, stol=0.0, s_keep=16, large=True),
}

# DMRG fixtures: Heisenberg chain (J = 1, open boundaries) from the reference's own
# HeisenbergHamiltonian(L).to_mpo()
DMRG_CASES = {
    # one effective two-site matvec at the middle of an L=10 chain, bond-8 state
    "dmrg_matvec_L10": dict(L=10, chi=8, site=4, seed=201),
    # two DMRG sweeps from a seeded random guess, tolerance 1e-10, max bond 32
    "dmrg_run_L10": dict(L=10, chi=4, seed=202, tol=1e-10, maxchi=32, maxiter=2),
}


def _norm(mps) -> float:
    """|psi| by a plain NumPy left-environment contraction (fixed, oracle-independent)."""
    rho = np.eye(1)
    for A in mps:
        a, d, b = A.shape
        t = (rho @ A.reshape(a, d * b)).reshape(a * d, b)
        rho = A.reshape(a * d, b).conj().T @ t
    return float(np.sqrt(abs(rho[0, 0].real)))


def _orthonormalise(raw):
    """QR-orthonormalise the cores left to right (numpy QR), normalise the last one."""
    out = []
    carry = np.eye(1)
    for i, A in enumerate(raw):
        A = np.tensordot(carry, A, axes=1)
        a, d, b = A.shape
        if i < len(raw) - 1:
            Q, R = np.linalg.qr(A.reshape(a * d, b))
            out.append(np.ascontiguousarray(Q.reshape(a, d, Q.shape[1])))
            carry = R
        else:
            out.append(A / np.linalg.norm(A))
    return out


def make_inputs(p: dict):
    rng = np.random.default_rng(p["seed"])
    n, d = p["n"], p["d"]
    if p.get("ortho"):
        mps = _orthonormalise(so.random_mps(d, n, p["chi"], rng, complex_=False))
        h = 2.0 ** (-n)
        mpo = so.tridiagonal_mpo(n, -2.0 / h**2, 1.0 / h**2, 1.0 / h**2)
        return mps, mpo
    if p["kind"] == "mpo_apply":
        mps = so.random_mps(d, n, p["chi"], rng, complex_=p["complex"])
        nrm = _norm(mps)
        mps = so.scale(mps, 1.0 / nrm)
        mpo = so.random_mpo(d, n, p["D"], rng, complex_=p["complex"])
        return mps, mpo
    if p["kind"] in ("laplacian", "euler"):
        mps = so.random_mps(d, n, p["chi"], rng, complex_=False)
        nrm = _norm(mps)
        mps = so.scale(mps, 1.0 / nrm)
        h = 2.0 ** (-n)
        mpo = so.tridiagonal_mpo(n, -2.0 / h**2, 1.0 / h**2, 1.0 / h**2)
        return mps, mpo
    if p["kind"] == "simplify":
        mps = so.random_mps(d, n, p["chi"], rng, complex_=p["complex"])
        nrm = _norm(mps)
        mps = so.scale(mps, 1.0 / nrm)
        return mps, None
    raise ValueError(p["kind"])


def input_hash(mps, mpo) -> str:
    h = hashlib.sha256()
    for A in mps:
        h.update(np.ascontiguousarray(A).tobytes())
    for O in mpo or []:
        h.update(np.ascontiguousarray(O).tobytes())
    return h.hexdigest()


# ---------------------------------------------------------------------------
# Child side: runs inside a process that imported the reference
# ---------------------------------------------------------------------------


def _child(backend: str, payload_path: str, out_path: str):
    import seemps  # noqa: F401
    from seemps.state import MPS, MPSSum, simplify, scprod
    from seemps.operators import MPO
    from seemps.cython import (
        DEFAULT_STRATEGY,
        Strategy,
        Truncation,
        destructively_truncate_vector,
    )

    records = []
    if backend == "python":
        from seemps.cython import _python_core as pc

        orig = pc._truncate

        def recording_truncate(s, strategy):
            D, err = orig(s, strategy)
            records.append((np.array(s, dtype=np.float64), int(D), float(err)))
            return D, err

        pc._truncate = recording_truncate
    else:
        import scipy.linalg as sla
        from seemps.cython import _update_in_canonical_form_left as upd_left
        from seemps.cython import _update_in_canonical_form_right as upd_right
        from seemps.state import canonical_mps as cm

        def svals(M):
            return sla.svd(np.array(M), compute_uv=False, lapack_driver="gesdd")

        def canonicalize(state, center, truncation):
            # cython/schmidt.pxi:109-120, one compiled update per site
            err = 0.0
            L = len(state)
            for i in range(0, center):
                A = state[i]
                s = svals(A.reshape(A.shape[0] * A.shape[1], A.shape[2]))
                _, e = upd_right(state, A, i, truncation)
                records.append((s, int(state[i].shape[2]), float(e) ** 2))
                err += e
            for i in range(L - 1, center, -1):
                A = state[i]
                s = svals(A.reshape(A.shape[0], A.shape[1] * A.shape[2]))
                _, e = upd_left(state, A, i, truncation)
                records.append((s, int(state[i].shape[0]), float(e) ** 2))
                err += e
            return err

        def wrap_split(fn):
            def split(AA, strategy):
                a, d1, d2, b = AA.shape
                s = svals(AA.reshape(a * d1, d2 * b))
                U, V, err = fn(AA, strategy)
                records.append((s, int(U.shape[-1]), float(err) ** 2))
                return U, V, err
            return split

        cm._canonicalize = canonicalize
        cm._left_orth_2site = wrap_split(cm._left_orth_2site)
        cm._right_orth_2site = wrap_split(cm._right_orth_2site)

    with open(payload_path, "rb") as f:
        payload = pickle.load(f)
    results = {}
    for name, (p, mps, mpo) in payload["cases"].items():
        records.clear()
        if backend == "python" and p.get("large"):
            continue
        strategy = DEFAULT_STRATEGY.replace(
            tolerance=p["tol"], max_bond_dimension=p["maxchi"], max_sweeps=p["sweeps"]
        )
        if p.get("stol") is not None:
            strategy = strategy.replace(simplification_tolerance=p["stol"])
        psi = MPS([np.array(A) for A in mps])
        if p["kind"] in ("mpo_apply", "laplacian"):
            O = MPO([np.array(A) for A in mpo], strategy)
            out = O.apply(psi, strategy=strategy)
            product = O.apply(psi, simplify=False)
            target = product
        elif p["kind"] == "euler":
            O = MPO([np.array(A) for A in mpo], strategy)
            Lx = O.apply(psi, simplify=False)
            target = MPSSum([1.0, p["dt"]], [psi, Lx])
            out = simplify(target, strategy=strategy)
        else:
            out = simplify(psi, strategy=strategy)
            target = psi
        r = dict(
            bonds=np.array(out.bond_dimensions()),
            error=float(out.error()),
            center=int(out.center),
            norm2=float(out.norm_squared()),
            overlap=complex(scprod(out, target) if not isinstance(target, MPSSum)
                            else sum(w * scprod(out, s) for w, s in
                                     zip(target.weights, target.states))),
            splits=[(s, D, e) for (s, D, e) in records],
        )
        if p["n"] <= 12:
            r["vector"] = out.to_vector()
        results[name] = r

    # truncation known-answer cases
    tr = []
    for (s, method, tol, maxb) in payload["truncation"]:
        st = Strategy(method=method, tolerance=tol, max_bond_dimension=maxb)
        v = np.array(s, dtype=np.float64)
        err = destructively_truncate_vector(v, st)
        tr.append(dict(s=list(map(float, s)), method=method, tol=tol, maxb=maxb,
                       size=int(len(v)), err=float(err),
                       effective_method=int(st.get_method())))
    results["__truncation__"] = tr
    with open(out_path, "wb") as f:
        pickle.dump(results, f)


def truncation_inputs():
    """Known-answer inputs: the reference test vectors plus seeded random ones."""
    base = [
        [1.0, 0.1, 0.01, 0.001, 0.0001],  # tests/test_truncate/test_truncation.py:46
        [1.0, 0.2, 0.01, 0.005, 0.0005],  # :9
        [0.0, 0.0, 0.0, 0.0],  # :16
        [1e-16, 1e-12, 1e-10, 1e-8, 1e-6, 1e-4, 1e-2, 1.0],  # :33 (not sorted)
        [1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7],  # tests/test_strategy.py:14
    ]
    rng = np.random.default_rng(7)
    for n in (1, 2, 3, 17, 64, 300):
        base.append(sorted(np.exp(rng.normal(scale=4.0, size=n)).tolist(), reverse=True))
    out = []
    for s in base:
        for method in (0, 1, 2, 3):
            for tol in (0.0, 1e-12, 1e-9, 1e-5, 1e-3, 0.05, 0.5):
                for maxb in (0x7FFFFFFF, 1, 2, 4):
                    out.append((s, method, tol, maxb))
    return out


def make_dmrg_inputs(p: dict):
    """Seeded random guess state (float64, normalised) for a DMRG fixture."""
    rng = np.random.default_rng(p["seed"])
    mps = so.random_mps(2, p["L"], p["chi"], rng, complex_=False)
    return so.scale(mps, 1.0 / _norm(mps))


def _dmrg_child(payload_path: str, out_path: str):
    """Runs inside a process that imported the reference (Cython backend)."""
    from seemps.state import MPS, CanonicalMPS, DEFAULT_STRATEGY
    from seemps.hamiltonians import HeisenbergHamiltonian
    from seemps.operators.quadratic import QuadraticForm
    from seemps.optimization import dmrg

    with open(payload_path, "rb") as f:
        payload = pickle.load(f)
    results = {}
    H100 = HeisenbergHamiltonian(100).to_mpo()
    results["heisenberg_mpo_L100"] = [np.array(W) for W in H100]
    for name, (p, guess) in payload["dmrg"].items():
        H = HeisenbergHamiltonian(p["L"]).to_mpo()
        W = [np.array(x) for x in H]
        if name.startswith("dmrg_matvec"):
            i = p["site"]
            state = CanonicalMPS([np.array(A) for A in guess], center=i, normalize=True)
            QF = QuadraticForm(H, state, start=i)
            L, H12, R = QF.two_site_block(i)
            Op = QF.two_site_operator(i)
            rng = np.random.default_rng(p["seed"] + 1)
            b, k, l, f = L.shape[2], H12.shape[2], H12.shape[4], R.shape[2]
            v = rng.normal(size=(b, k, l, f))
            out = Op.matvec(v.reshape(-1)).reshape(L.shape[0], H12.shape[1], H12.shape[3],
                                                    R.shape[0])
            results[name] = dict(mpo=W, state=[np.array(A) for A in state], L=np.array(L),
                                 H12=np.array(H12), R=np.array(R), v=v, out=out)
        else:
            st = DEFAULT_STRATEGY.replace(tolerance=p["tol"], max_bond_dimension=p["maxchi"])
            res = dmrg(H, guess=MPS([np.array(A) for A in guess]), maxiter=p["maxiter"],
                       tol=1e-14, strategy=st)
            results[name] = dict(mpo=W, energy=float(res.energy),
                                 trajectory=np.array(res.trajectory, dtype=np.float64),
                                 bonds=np.array(res.state.bond_dimensions()),
                                 vector=res.state.to_vector())
    with open(out_path, "wb") as f:
        pickle.dump(results, f)


def make_dmrg(ref: str):
    env_path = f"{ref}/shim:{ref}/src"
    payload = {"dmrg": {name: (p, make_dmrg_inputs(p)) for name, p in DMRG_CASES.items()}}
    tmp = "/tmp/_golden_dmrg_payload.pkl"
    with open(tmp, "wb") as f:
        pickle.dump(payload, f)
    out = "/tmp/_golden_dmrg.pkl"
    env = dict(os.environ, PYTHONPATH=env_path, SEEMPS_BACKEND="cython", OPENBLAS_NUM_THREADS="1")
    subprocess.run([sys.executable, __file__, "--dmrg-child", tmp, out], check=True, env=env)
    with open(out, "rb") as f:
        res = pickle.load(f)
    W100 = res.pop("heisenberg_mpo_L100")
    np.savez_compressed(os.path.join(HERE, "heisenberg_mpo_L100.npz"),
                        **{f"W{i}": W for i, W in enumerate(W100)})
    for name, p in DMRG_CASES.items():
        r = res[name]
        arrs = {f"W{i}": W for i, W in enumerate(r.pop("mpo"))}
        if "state" in r:
            arrs.update({f"A{i}": A for i, A in enumerate(r.pop("state"))})
        arrs.update(r)
        arrs["meta"] = np.frombuffer(json.dumps(dict(params=p)).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)
        print(name, {k: (v.shape if hasattr(v, "shape") else v) for k, v in r.items()})


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/tmp/seemps_ref"
    if "--dmrg-only" in sys.argv:
        return make_dmrg(ref)
    env_path = f"{ref}/shim:{ref}/src"
    cases = {}
    meta = {}
    for name, p in CASES.items():
        mps, mpo = make_inputs(p)
        cases[name] = (p, mps, mpo)
        meta[name] = dict(params=p, input_sha256=input_hash(mps, mpo))
    payload = dict(cases=cases, truncation=truncation_inputs())
    tmp = "/tmp/_golden_payload.pkl"
    with open(tmp, "wb") as f:
        pickle.dump(payload, f)
    outs = {}
    for backend in ("cython", "python"):
        env = dict(os.environ, PYTHONPATH=env_path, SEEMPS_BACKEND=backend,
                   OPENBLAS_NUM_THREADS="1")
        out = f"/tmp/_golden_{backend}.pkl"
        subprocess.run([sys.executable, __file__, "--child", backend, tmp, out],
                       check=True, env=env)
        with open(out, "rb") as f:
            outs[backend] = pickle.load(f)
    cy, py = outs["cython"], outs["python"]
    # the two reference backends must agree before anything is written
    for name in CASES:
        if name not in py:
            continue
        # the two ways of recording the splits agree
        assert [D for (_, D, _) in cy[name]["splits"]] == [D for (_, D, _) in py[name]["splits"]]
        for (s1, _, e1), (s2, _, e2) in zip(cy[name]["splits"], py[name]["splits"]):
            assert len(s1) == len(s2) and np.max(np.abs(s1 - s2)) <= 1e-12 * max(s2[0], 1e-300)
            # discarded weights made of rounding noise (~(1e-16 s_max)^2 each) differ
            # between two SVDs of the same matrix
            assert abs(e1 - e2) <= 1e-8 * e2 + 1e-24 * s2[0] ** 2
        assert np.array_equal(cy[name]["bonds"], py[name]["bonds"]), name
        assert cy[name]["center"] == py[name]["center"], name
        # error() is sqrt(err estimate); at noise level only its square is stable
        e1, e2 = cy[name]["error"] ** 2, py[name]["error"] ** 2
        assert abs(e1 - e2) <= 1e-13 + 1e-9 * e1, name
    assert [t["size"] for t in cy["__truncation__"]] == [t["size"] for t in py["__truncation__"]]
    for name, p in CASES.items():
        c, q = cy[name], cy[name]
        keep = p.get("s_keep")
        # singular values as stored: all of them, or the kept rank + s_keep
        kept_s = [s if keep is None else s[: min(len(s), D + keep)] for (s, D, _) in q["splits"]]
        arrs = dict(
            bonds=c["bonds"], error=np.float64(c["error"]), center=np.int64(c["center"]),
            norm2=np.float64(c["norm2"]), overlap=np.complex128(c["overlap"]),
            split_rank=np.array([D for (_, D, _) in q["splits"]], dtype=np.int64),
            split_err2=np.array([e for (_, _, e) in q["splits"]], dtype=np.float64),
            split_len=np.array([len(s) for s in kept_s], dtype=np.int64),
            split_full_len=np.array([len(s) for (s, _, _) in q["splits"]], dtype=np.int64),
            split_s=np.concatenate(kept_s) if kept_s else np.zeros(0),
            meta=np.frombuffer(json.dumps(meta[name]).encode(), dtype=np.uint8),
        )
        if "vector" in c:
            arrs["vector"] = c["vector"]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)
        print(name, "bonds", c["bonds"].tolist(), "err", c["error"],
              "splits", len(q["splits"]))
    vectors, cases_out, index = [], [], {}
    for t in cy["__truncation__"]:
        key = tuple(t["s"])
        if key not in index:
            index[key] = len(vectors)
            vectors.append(t["s"])
        cases_out.append(dict(v=index[key], **{k: t[k] for k in
                                               ("method", "tol", "maxb", "size", "err",
                                                "effective_method")}))
    with open(os.path.join(HERE, "truncation_cases.json"), "w") as f:
        json.dump(dict(vectors=vectors, cases=cases_out), f)
    print("truncation cases:", len(cy["__truncation__"]))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--child":
        _child(sys.argv[2], sys.argv[3], sys.argv[4])
    elif len(sys.argv) > 1 and sys.argv[1] == "--dmrg-child":
        _dmrg_child(sys.argv[2], sys.argv[3])
    else:
        main()
