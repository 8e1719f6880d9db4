"""Regression input for the mixed split: a strongly graded two-site matrix.

MPO.apply of the Laplacian (bond-3, 1/h^2 = 2^60 entries) to the seeded
n=30, chi=256 MPS of the benchmark, with tol 1e-12 and max bond 256, first
brings the product state (bond 768) to canonical form with truncation; near
the right end of that sweep it meets matrices whose rows span 1e-14 of the
largest and a third of whose entries are exact zeros.  The first SVD of shape
192 x 250 of that run (oracle, FP64) is saved here; its FP32 QR leaves rows of
R far below FP32 resolution that are nearly parallel, which once broke the
mixed split's refinement.

    python tests/golden/make_graded_split.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import seemps_oracle as so  # noqa: E402

SHAPE = (192, 250)
SEED = 20241203  # the benchmark's workload seed


class _Found(Exception):
    pass


def workload(n=30, chi=256, seed=SEED):
    """The benchmark's seeded inputs (left-orthonormal MPS, Laplacian MPO)."""
    rng = np.random.default_rng(seed)
    raw = so.random_mps(2, n, chi, rng)
    mps, carry = [], np.eye(1)
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
    return mps, mpo


def main():
    mps, mpo = workload()
    st = so.DEFAULT_STRATEGY.replace(tolerance=1e-12, max_bond_dimension=256, max_sweeps=2,
                                     simplification_tolerance=0.0)
    orig = so.svd

    def hook(A):
        if A.shape == SHAPE:
            raise _Found(np.array(A))
        return orig(A)

    so.svd = hook
    try:
        so.mpo_apply(mpo, mps, st)
    except _Found as f:
        A = f.args[0]
        np.savez_compressed(os.path.join(HERE, "graded_split_192x250.npz"), A=A)
        print("saved", A.shape)
        return
    finally:
        so.svd = orig
    raise SystemExit("no split of shape %s met" % (SHAPE,))


if __name__ == "__main__":
    main()
