"""CPU oracle of the DMRG two-site effective-Hamiltonian matvec (test and benchmark
infrastructure only: the tests and bench.py compare the GPU kernels with it).

Restates, in NumPy:
  * QuadraticForm.two_site_operator._matvec (operators/quadratic.py:187-237):
    out[a,ko,lo,g] = sum L[a,c,b] v[b,k,l,f] H[c,ko,k,lo,l,d] R[g,d,f];
  * the two-site MPO H = _contract_last_and_first(O[i], O[i+1])
    (operators/quadratic.py:102-104, cython/contractions.pxi:6-38);
  * update_left_mpo_environment / update_right_mpo_environment
    (state/environments.py:19-42) and begin_mpo_environment (:15-16);
  * the effective operator as a dense matrix, for eigenvalue checks.
The spin-1/2 Heisenberg MPO (bond 5, J (S+S- + S-S+)/2 + J SzSz) is the textbook
finite-state-machine construction written here for the benchmark's inputs; only
its shape (bond 5) and sparsity matter to the kernels.
"""

from __future__ import annotations

import numpy as np


def contract_last_and_first(A, B):
    """Last index of A against the first of B (cython/_python_core.py:220-227)."""
    return np.tensordot(A, B, axes=(-1, 0))


def two_site_hamiltonian(O1, O2):
    """H[c, ko, k, lo, l, d] of two neighbouring MPO sites O[c, i, j, e]
    (the H12 of QuadraticForm.two_site_block, operators/quadratic.py:102-104)."""
    return contract_last_and_first(O1, O2)


def two_site_matvec(L, H, R, v):
    """operators/quadratic.py:198-219 (the reshape / transpose sequence of _matvec)."""
    a, c, b = L.shape
    _, ko, k, lo, l, d = H.shape
    g, _, f = R.shape
    Lm = L.reshape(a * c, b)
    Hm = np.ascontiguousarray(H.transpose(0, 2, 4, 1, 3, 5)).reshape(c * k * l, ko * lo * d)
    Rm = np.ascontiguousarray(R.transpose(2, 1, 0)).reshape(f * d, g)
    x = (Lm @ v.reshape(b, k * l * f)).reshape(a, c, k, l, f)
    x = x.transpose(0, 4, 1, 2, 3).reshape(a * f, c * k * l)
    x = (x @ Hm).reshape(a, f, ko, lo, d)
    x = x.transpose(0, 2, 3, 1, 4).reshape(a * ko * lo, f * d)
    return (x @ Rm).reshape(a, ko, lo, g)


def dense_operator(L, H, R):
    """The matvec as a dense (a ko lo g) x (b k l f) matrix (small sizes only)."""
    b = L.shape[2]
    k, l = H.shape[2], H.shape[4]
    f = R.shape[2]
    n = b * k * l * f
    cols = []
    for j in range(n):
        e = np.zeros(n, dtype=np.result_type(L, H, R))
        e[j] = 1.0
        cols.append(two_site_matvec(L, H, R, e.reshape(b, k, l, f)).reshape(-1))
    return np.stack(cols, axis=1)


def begin_mpo_environment():
    """The trivial 1 x 1 x 1 edge environment (state/environments.py:15-16)."""
    return np.ones((1, 1, 1))


def update_left_mpo_environment(rho, A, O, B):
    """state/environments.py:19-29: "acb,ajd,cjie,bif->def"."""
    aux = np.tensordot(B, rho, (0, 2))
    aux = np.tensordot(aux, O, ([0, 3], [2, 0]))
    return np.tensordot(aux, np.conj(A), ((1, 2), (0, 1))).transpose(2, 1, 0)


def update_right_mpo_environment(rho, A, O, B):
    """state/environments.py:32-42: "def,ajd,cjie,bif->acb"."""
    aux = np.tensordot(np.conj(A), rho, (2, 0))
    aux = np.tensordot(aux, O, ((1, 2), (1, 3)))
    return np.tensordot(aux, B, ((1, 3), (2, 1)))


def heisenberg_mpo(n: int, J: float = 1.0):
    """Open-chain spin-1/2 Heisenberg MPO, bond 5 (edges 1): the operator of
    HeisenbergHamiltonian(n).to_mpo() (hamiltonians/nearest_neighbor.py:318, :105-150),
    checked against the reference-made heisenberg_mpo_L100.npz fixture."""
    Sp = np.array([[0.0, 1.0], [0.0, 0.0]])
    Sm = Sp.T
    Sz = np.diag([0.5, -0.5])
    I2 = np.eye(2)
    W = np.zeros((5, 2, 2, 5))
    W[0, :, :, 0] = I2
    W[0, :, :, 1] = Sp
    W[0, :, :, 2] = Sm
    W[0, :, :, 3] = Sz
    W[1, :, :, 4] = 0.5 * J * Sm
    W[2, :, :, 4] = 0.5 * J * Sp
    W[3, :, :, 4] = J * Sz
    W[4, :, :, 4] = I2
    return [W[:1]] + [W] * (n - 2) + [W[:, :, :, 4:]]


# ---------------------------------------------------------------------------
# The two-site DMRG driver (optimization/dmrg.py:15-199) with scipy's eigsh, as the
# reference runs it; uses the MPS oracle's canonical forms and two-site splits.
# ---------------------------------------------------------------------------


def mpo_expectation(W, state, center):
    """<state|W|state> (operators/mpo.py:378-416) for a state in canonical form about center."""
    left = right = begin_mpo_environment()
    for i in range(0, center):
        left = update_left_mpo_environment(left, state[i], W[i], state[i])
    for i in range(len(W) - 1, center - 1, -1):
        right = update_right_mpo_environment(right, state[i], W[i], state[i])
    return np.dot(left.reshape(-1), right.reshape(-1))


def _energy_and_variance(W, state, center):
    """optimization/dmrg.py:56-60: <H> and |<H psi|H psi> - <H>^2|."""
    from oracle import seemps_oracle as so

    energy = mpo_expectation(W, state, center).real
    hpsi = [so.mpo_multiply_tensor(O, A) for O, A in zip(W, state)]
    return energy, abs(so.norm_squared(hpsi) - energy * energy)


def dmrg(W, guess, maxiter=20, tol=1e-10, tol_up=None, tol_eigs=None, strategy=None,
         max_steps=None):
    """optimization/dmrg.py:76-199 on lists of tensors: guess canonicalised at site 0 and
    normalised, sweeps of eigsh(which="SA") on the two-site operators from the current
    two-site tensor, left/right splits with the strategy (normalize=True), energy and
    variance after each sweep, the same stop rule.  Returns (best energy, best state,
    trajectory, variances, converged, sweeps).  ``max_steps`` (timing samples only) stops
    after that many two-site steps."""
    import scipy.sparse.linalg as sla

    from oracle import seemps_oracle as so

    tol_up = tol if tol_up is None else tol_up
    tol_eigs = tol if tol_eigs is None else tol_eigs
    strat = (so.DEFAULT_STRATEGY if strategy is None else strategy).replace(normalize=True)
    size = len(W)
    state, center, _ = so.canonical_mps([np.array(A) for A in guess], 0, strat)
    state[center] = state[center] / np.linalg.norm(state[center])
    # environments: right ones for the first sweep (quadratic.py:40-76)
    left = [begin_mpo_environment()] * size
    right = [begin_mpo_environment()] * size
    env = right[-1]
    for i in range(size - 1, 0, -1):
        right[i - 1] = env = update_right_mpo_environment(env, state[i], W[i], state[i])
    energy, variance = _energy_and_variance(W, state, center)
    best = (energy, [A.copy() for A in state])
    trajectory, variances = [energy], [variance]
    direction, last_energy, converged, sweeps = +1, energy, False, 0
    steps = 0
    for sweep in range(1, maxiter + 1):
        sweeps = sweep
        sites = range(size - 1) if direction > 0 else range(size - 2, -1, -1)
        for i in sites:
            if max_steps is not None and steps >= max_steps:
                return best[0], state, trajectory, variances, False, sweeps
            steps += 1
            L, R = left[i], right[i + 1]
            H = two_site_hamiltonian(W[i], W[i + 1])
            v = np.tensordot(state[i], state[i + 1], axes=1)
            n = v.size
            op = sla.LinearOperator((n, n), matvec=lambda x, L=L, H=H, R=R, s=v.shape:
                                    two_site_matvec(L, H, R, x.reshape(s)).reshape(-1),
                                    dtype=np.float64)
            _, evec = sla.eigsh(op, 1, which="SA", v0=v.reshape(-1), tol=tol_eigs)
            AB = evec.reshape(v.shape)
            if direction > 0:
                state[i], state[i + 1], _ = so.left_orth_2site(AB, strat)
                center = i + 1
                if i < size - 2:
                    left[i + 1] = update_left_mpo_environment(left[i], state[i], W[i], state[i])
            else:
                state[i], state[i + 1], _ = so.right_orth_2site(AB, strat)
                center = i
                if i > 0:
                    right[i] = update_right_mpo_environment(right[i + 1], state[i + 1],
                                                            W[i + 1], state[i + 1])
        direction = -direction
        energy, variance = _energy_and_variance(W, state, center)
        trajectory.append(energy)
        variances.append(variance)
        if energy < best[0]:
            best = (energy, [A.copy() for A in state])
        change = energy - last_energy
        scale = max(1.0, abs(energy))
        if change > tol_up * scale or -tol * scale <= change <= 0:
            converged = True
            break
        last_energy = energy
    return best[0], best[1], trajectory, variances, converged, sweeps
