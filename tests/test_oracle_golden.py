"""Pins the CPU oracle to the reference's own outputs (no GPU needed)."""

import numpy as np
import pytest

from oracle import seemps_oracle as so
from tests.golden_cases import CASE_NAMES, load_case, run_oracle, truncation_cases


@pytest.mark.parametrize("chunk", range(4))
def test_truncation_known_answers(chunk):
    """Every reference truncation case: same kept size, bit-identical error."""
    cases = truncation_cases()
    for s, c in cases[chunk::4]:
        st = so.Strategy(method=c["method"], tolerance=c["tol"], max_bond_dimension=c["maxb"])
        assert st.method == c["effective_method"]
        size, err = so.truncate(s, st)
        assert size == c["size"], (c, size)
        if st.method == so.Truncation.RELATIVE_NORM_SQUARED_ERROR:
            # prefix sums are stored one by one: the order is fixed, bit-exact
            assert err == c["err"], (c, err)
        else:
            # the reference core is built with -ffast-math, which may reassociate
            # the plain sum of dropped s^2 of the singular-value rules
            assert abs(err - c["err"]) <= 8 * np.finfo(float).eps * abs(c["err"]), (c, err)


def test_reference_inline_vectors():
    """tests/test_truncate/test_truncation.py:83-147 of the reference, restated."""
    s = np.array([1.0, 0.1, 0.01, 0.001, 0.0001])
    expected = [1.01010100e-02, 1.01010000e-04, 1.01000000e-06, 9.99999994e-09, 0.0]
    for k, tol in enumerate([0.1, 1e-3, 1e-5, 1e-7, 1e-9]):
        st = so.Strategy(method=so.Truncation.RELATIVE_NORM_SQUARED_ERROR, tolerance=tol)
        size, err = so.truncate(s, st)
        assert size == k + 1
        assert abs(err - expected[k]) < 1e-7


def test_strategy_validation():
    with pytest.raises(AssertionError):
        so.Strategy(tolerance=-1.0)
    with pytest.raises(AssertionError):
        so.Strategy(tolerance=1.0)
    with pytest.raises(AssertionError):
        so.Strategy(max_bond_dimension=0)
    with pytest.raises(AssertionError):
        so.Strategy(max_sweeps=-1)
    assert so.Strategy(tolerance=0.0).method == so.Truncation.ABSOLUTE_SINGULAR_VALUE


@pytest.mark.parametrize("name", CASE_NAMES)
def test_oracle_matches_reference_run(name):
    p, mps, mpo, g, same = load_case(name)
    if not same:
        pytest.skip("this numpy regenerates different seeded inputs than the fixture's")
    rec = so.Recorder()
    res, target = run_oracle(p, mps, mpo, rec)
    bonds = [A.shape[0] for A in res.tensors] + [res.tensors[-1].shape[-1]]
    assert bonds == g["bonds"].tolist()
    assert res.center == int(g["center"])
    # every split: identical kept rank, singular values within 1e-10 of s_max
    assert [sp.rank for sp in rec.splits] == g["split_rank"].tolist()
    # (large fixtures store each split's values up to the kept rank + 16)
    for sp, s_ref, n_full in zip(rec.splits, g["splits_s"], g["split_full_len"]):
        assert len(sp.s) == n_full
        smax = max(float(s_ref[0]), 1e-300)
        assert np.max(np.abs(sp.s[: len(s_ref)] - s_ref)) <= 1e-10 * smax
    # error bound: its square is the stable quantity (see make_golden.py)
    e1, e2 = res.error ** 2, float(g["error"]) ** 2
    assert abs(e1 - e2) <= 1e-13 + 1e-8 * e2
    n2 = so.norm_squared(res.tensors)
    assert abs(n2 - float(g["norm2"])) <= 1e-10 * float(g["norm2"])
    if "vector" in g:
        v = so.to_vector(res.tensors)
        ref = g["vector"]
        assert np.linalg.norm(v - ref) <= 1e-9 * np.linalg.norm(ref)


def _dmrg_fixture(name):
    import json
    import os

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))
    W = [z[f"W{i}"] for i in range(sum(1 for k in z.files if k.startswith("W")))]
    return z, W, json.loads(bytes(z["meta"]).decode())["params"]


def test_dmrg_matvec_oracle_matches_reference():
    """The oracle's environments and two-site matvec against the reference's QuadraticForm
    on HeisenbergHamiltonian(10).to_mpo() (fixture made by tests/golden/make_golden.py)."""
    from oracle import dmrg_oracle as do

    z, W, p = _dmrg_fixture("dmrg_matvec_L10")
    i = p["site"]
    state = [z[f"A{k}"] for k in range(p["L"])]
    L = do.begin_mpo_environment()
    for k in range(i):
        L = do.update_left_mpo_environment(L, state[k], W[k], state[k])
    R = do.begin_mpo_environment()
    for k in range(p["L"] - 1, i + 1, -1):
        R = do.update_right_mpo_environment(R, state[k], W[k], state[k])
    assert np.allclose(L, z["L"], atol=1e-13)
    assert np.allclose(R, z["R"], atol=1e-13)
    assert np.allclose(do.two_site_hamiltonian(W[i], W[i + 1]), z["H12"], atol=1e-15)
    out = do.two_site_matvec(z["L"], z["H12"], z["R"], z["v"])
    assert np.allclose(out, z["out"], atol=1e-13 * np.abs(z["out"]).max())


def test_dmrg_oracle_matches_reference_run():
    """The oracle's DMRG driver (scipy eigsh, as the reference) reproduces the reference's
    two-sweep run: energies per sweep, bonds and the final state."""
    import importlib.util
    import os

    from oracle import dmrg_oracle as do

    z, W, p = _dmrg_fixture("dmrg_run_L10")
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    guess = mg.make_dmrg_inputs(p)
    st = so.DEFAULT_STRATEGY.replace(tolerance=p["tol"], max_bond_dimension=p["maxchi"])
    energy, state, traj, _, _, _ = do.dmrg(W, guess, maxiter=p["maxiter"], tol=1e-14, strategy=st)
    assert np.max(np.abs(np.array(traj) - z["trajectory"])) <= 1e-9 * max(1.0, abs(energy))
    assert abs(energy - float(z["energy"])) <= 1e-9
    assert [A.shape[0] for A in state] + [1] == z["bonds"].tolist()
    v = so.to_vector(state)
    ref = z["vector"].reshape(-1)
    assert 1.0 - abs(np.vdot(ref, v)) / (np.linalg.norm(ref) * np.linalg.norm(v)) <= 1e-8


def _mpo_dense(W):
    """Dense operator of an MPO O[a, i, j, b] (small chains only)."""
    M = W[0][0]  # (i, j, b)
    for O in W[1:]:
        M = np.einsum("ijb,bklc->ikjlc", M, O)
        n = M.shape[0] * M.shape[1]
        M = M.reshape(n, n, -1)
    return M[:, :, 0]


def test_heisenberg_oracle_matches_reference_mpo():
    """The oracle's Heisenberg MPO is the operator of the reference's
    HeisenbergHamiltonian(100).to_mpo() (fixture heisenberg_mpo_L100.npz): the same
    energy <psi|H|psi> for seeded random states on all 100 sites, and the same dense
    operator on 6 sites built from the fixture's edge and bulk tensors."""
    import os

    from oracle import dmrg_oracle as do

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "heisenberg_mpo_L100.npz"))
    ref = [z[f"W{i}"] for i in range(100)]
    ours = do.heisenberg_mpo(100)
    rng = np.random.default_rng(7)
    for _ in range(3):
        psi = [A / np.linalg.norm(A) for A in so.random_mps(2, 100, 3, rng)]
        e = []
        for W in (ref, ours):
            L = do.begin_mpo_environment()
            for A, O in zip(psi, W):
                L = do.update_left_mpo_environment(L, A, O, A)
            e.append(float(L.reshape(-1)[0]))
        assert abs(e[0] - e[1]) <= 1e-12 * max(1.0, abs(e[0]))
    small = [ref[0]] + [ref[1]] * 4 + [ref[99]]
    assert np.allclose(_mpo_dense(small), _mpo_dense(do.heisenberg_mpo(6)), atol=1e-14)
