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
    return np.tensordot(A, B, axes=(-1, 0))


def two_site_hamiltonian(O1, O2):
    """H[c, ko, k, lo, l, d] of two neighbouring MPO sites O[c, i, j, e]."""
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
    """Open-chain spin-1/2 Heisenberg MPO, bond 5 (edges 1)."""
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
