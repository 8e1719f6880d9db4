"""CPU oracle for the MPO·MPS + ``simplify`` path (test infrastructure only).

This module is the checker that the CUDA path of ``seemps2_gb300`` is compared
against.  It is a NumPy/SciPy restatement of the reference algorithm of SeeMPS
(``juanjosegarciaripoll/seemps2``), written from its published behaviour; every
function cites the reference file:line it follows.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline leg and its
``--impl reference`` arm) may import it.  The product package never does.

Parity of this oracle is pinned two ways (see ``tests/test_oracle_golden.py``):
  * against the exact known-answer vectors of the reference's own truncation
    tests (``tests/test_truncate/test_truncation.py:7-147``,
    ``tests/test_strategy.py:16-114``), restated in ``tests/golden/``;
  * against fixtures produced by running the reference itself (SeeMPS 3.2,
    Cython backend) on seeded inputs, made by ``tests/golden/make_golden.py``.

Conventions (reference ``state/mps.py:23-38``, ``operators/mpo.py:51-54``): MPS
site tensors are ``A[a, i, b]``, MPO site tensors ``O[a, i, j, b]``, C order,
float64 or complex128.  The economy SVD uses LAPACK ``gesdd`` like the
reference (``cython/svd.pxi:23``).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from math import sqrt

import numpy as np
import scipy.linalg
import scipy.linalg.blas
import scipy.linalg.lapack

# --------------------------------------------------------------------------
# Strategy (reference cython/truncation.pxi:1-220, mirror _python_core.py:60-183)
# --------------------------------------------------------------------------

MAX_BOND_DIMENSION = 0x7FFFFFFF
DEFAULT_TOLERANCE = float(np.finfo(np.float64).eps)


class Truncation:
    """Truncation method codes (cython/truncation.pxi:23-42)."""

    DO_NOT_TRUNCATE = 0
    RELATIVE_SINGULAR_VALUE = 1
    RELATIVE_NORM_SQUARED_ERROR = 2
    ABSOLUTE_SINGULAR_VALUE = 3


class Simplification:
    """Simplification method codes (cython/truncation.pxi:44-61)."""

    DO_NOT_SIMPLIFY = 0
    CANONICAL_FORM = 1
    VARIATIONAL = 2
    VARIATIONAL_EXACT_GUESS = 3


class Strategy:
    """Truncation / simplification settings (reference truncation.pxi:66-130)."""

    def __init__(
        self,
        method: int = Truncation.RELATIVE_NORM_SQUARED_ERROR,
        tolerance: float = DEFAULT_TOLERANCE,
        simplification_tolerance: float = DEFAULT_TOLERANCE,
        max_bond_dimension: int = MAX_BOND_DIMENSION,
        normalize: bool = False,
        simplify: int = Simplification.VARIATIONAL,
        max_sweeps: int = 16,
    ):
        if tolerance < 0 or tolerance >= 1.0:
            raise AssertionError("Invalid tolerance argument passed to Strategy")
        if tolerance == 0 and method != Truncation.DO_NOT_TRUNCATE:
            method = Truncation.ABSOLUTE_SINGULAR_VALUE  # truncation.pxi:105-106
        if max_bond_dimension <= 0 or max_bond_dimension > MAX_BOND_DIMENSION:
            raise AssertionError("Invalid bond dimension in Strategy")
        if simplify < 0 or simplify > 3:
            raise AssertionError("Invalid simplify argument passed to Strategy")
        if max_sweeps < 0:
            raise AssertionError("Negative or zero number of sweeps in Strategy")
        if method not in (0, 1, 2, 3):
            raise AssertionError("Invalid method argument passed to Strategy")
        self.method = int(method)
        self.tolerance = float(tolerance)
        self.simplification_tolerance = float(simplification_tolerance)
        self.max_bond_dimension = int(max_bond_dimension)
        self.normalize = bool(normalize)
        self.simplify = int(simplify)
        self.max_sweeps = int(max_sweeps)

    def replace(self, **kw) -> "Strategy":
        args = dict(
            method=self.method,
            tolerance=self.tolerance,
            simplification_tolerance=self.simplification_tolerance,
            max_bond_dimension=self.max_bond_dimension,
            normalize=self.normalize,
            simplify=self.simplify,
            max_sweeps=self.max_sweeps,
        )
        args.update({k: v for k, v in kw.items() if v is not None})
        return Strategy(**args)


DEFAULT_STRATEGY = Strategy()
NO_TRUNCATION = DEFAULT_STRATEGY.replace(
    method=Truncation.DO_NOT_TRUNCATE, simplify=Simplification.DO_NOT_SIMPLIFY
)
# reference state/simplification.py:22-29
SIMPLIFICATION_STRATEGY = Strategy(normalize=True, max_sweeps=4)


# --------------------------------------------------------------------------
# Truncation rule (reference truncation.pxi:222-334)
# --------------------------------------------------------------------------


def truncate(s: np.ndarray, strategy: Strategy) -> tuple[int, float]:
    """Kept size and squared discarded weight for descending singular values.

    Follows ``_truncate_relative_norm_squared_error`` (truncation.pxi:251-287),
    ``_truncate_relative_singular_value`` (:289-307) and
    ``_truncate_absolute_singular_value`` (:309-327) literally, including the
    summation order (smallest value first) and the strict ``>`` test, so that
    ties resolve the same way.
    """
    s = np.asarray(s, dtype=np.float64)
    N = s.shape[0]
    method = strategy.method
    if method == Truncation.DO_NOT_TRUNCATE:
        return N, 0.0
    if method == Truncation.RELATIVE_NORM_SQUARED_ERROR:
        errors = np.empty(N + 1)
        total = 0.0
        for i in range(N):  # cumulative sum from the smallest value upwards
            errors[i] = total
            v = float(s[N - 1 - i])
            total += v * v
        errors[N] = total
        max_error = total * strategy.tolerance
        i = N - 1
        for j in range(N):
            if errors[j] > max_error:
                i = j - 1
                break
        final_size = min(N - i, strategy.max_bond_dimension)
        return final_size, float(errors[N - final_size])
    if method == Truncation.RELATIVE_SINGULAR_VALUE:
        max_error = strategy.tolerance * float(s[0])
    else:  # ABSOLUTE_SINGULAR_VALUE
        max_error = strategy.tolerance
    final_size = min(N, strategy.max_bond_dimension)
    for i in range(1, final_size):
        if s[i] <= max_error:
            final_size = i
            break
    err = 0.0
    for i in range(final_size, N):
        err += float(s[i]) * float(s[i])
    return final_size, err


# --------------------------------------------------------------------------
# Kernels (reference svd.pxi, contractions.pxi, environments.pxi, mpo.py)
# --------------------------------------------------------------------------


GESDD_RETRIES = [0]


def svd(A: np.ndarray):
    """Economy SVD through LAPACK ?gesdd called directly, as the reference's
    Cython core does (svd.pxi:35-83, gesdd being its default driver :23)."""
    if A.dtype == np.complex64:
        A = A.astype(np.complex128)
    elif A.dtype not in (np.float64, np.complex128):
        A = A.astype(np.float64)
    f = scipy.linalg.lapack.zgesdd if np.iscomplexobj(A) else scipy.linalg.lapack.dgesdd
    U, s, Vh, info = f(A, compute_uv=1, full_matrices=0)
    if info > 0:
        # Some LAPACK builds (seen with OpenBLAS on aarch64) report that the
        # divide-and-conquer stage did not converge on matrices that gesvd
        # handles; the reference offers gesvd as its other driver
        # (svd.pxi:25-32).  The retry is counted so callers can report it.
        GESDD_RETRIES[0] += 1
        g = scipy.linalg.lapack.zgesvd if np.iscomplexobj(A) else scipy.linalg.lapack.dgesvd
        U, s, Vh, info = g(A, compute_uv=1, full_matrices=0)
    if info > 0:
        raise np.linalg.LinAlgError("SVD did not converge")
    if info < 0:
        raise RuntimeError(f"Wrong argument {-info} to LAPACK SVD.")
    return U, s, Vh


def gemm(A: np.ndarray, B: np.ndarray, opA: str = "N", opB: str = "N") -> np.ndarray:
    """op(A) @ op(B) through SciPy's BLAS ?gemm, the library the reference's
    _gemm calls (gemm.pxi:21-122).  Using one BLAS for GEMM and LAPACK keeps a
    single OpenBLAS thread pool busy, as in the reference's process."""
    cplx = np.iscomplexobj(A) or np.iscomplexobj(B)
    dt = np.complex128 if cplx else np.float64
    A = np.asarray(A, dtype=dt)
    B = np.asarray(B, dtype=dt)
    f = scipy.linalg.blas.zgemm if cplx else scipy.linalg.blas.dgemm
    code = {"N": 0, "T": 1, "C": 2}
    # row-major C = op(A) op(B)  <=>  column-major C^T = op(B)^T op(A)^T
    Ct = f(1.0, B.T if B.flags.c_contiguous else np.asfortranarray(B.T),
           A.T if A.flags.c_contiguous else np.asfortranarray(A.T),
           trans_a=code[opB], trans_b=code[opA])
    return Ct.T


def contract_last_and_first(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Contract the last index of A with the first of B (contractions.pxi:6-38)."""
    Am = np.ascontiguousarray(A.reshape(-1, A.shape[-1]))
    Bm = np.ascontiguousarray(B.reshape(B.shape[0], -1))
    return gemm(Am, Bm).reshape(A.shape[:-1] + B.shape[1:])


def mpo_multiply_tensor(O: np.ndarray, B: np.ndarray) -> np.ndarray:
    """C[c*a, i, d*b] = sum_j B[c,j,d] O[a,i,j,b] (operators/mpo.py:26-45)."""
    a, i, j, b = O.shape
    c, j2, d = B.shape
    assert j == j2
    C = np.einsum("cjd,aijb->caidb", B, O)
    return C.reshape(c * a, i, d * b)


def update_left_environment(B: np.ndarray, A: np.ndarray, rho: np.ndarray):
    """rho'[n,k] = sum conj(B[l,j,n]) rho[l,i] A[i,j,k] (environments.pxi:10-37)."""
    l, j, n = B.shape
    i, j2, k = A.shape
    tmp = np.ascontiguousarray(gemm(np.ascontiguousarray(rho), np.ascontiguousarray(A).reshape(i, j * k)))
    return np.ascontiguousarray(gemm(np.ascontiguousarray(B).reshape(l * j, n), tmp.reshape(l * j, k), "C", "N"))


def update_right_environment(B: np.ndarray, A: np.ndarray, rho: np.ndarray):
    """rho'[i,l] = sum A[i,j,k] rho[k,n] conj(B[l,j,n]) (environments.pxi:39-67)."""
    i, j, k = A.shape
    l, j2, n = B.shape
    tmp = np.ascontiguousarray(gemm(np.ascontiguousarray(A).reshape(i * j, k), np.ascontiguousarray(rho)))
    return np.ascontiguousarray(gemm(tmp.reshape(i, j * n), np.ascontiguousarray(B).reshape(l, j * n), "N", "C"))


def scprod(bra: list, ket: list):
    """<bra|ket> through left environments (environments.pxi:87-118)."""
    rho = np.eye(1)
    for B, A in zip(bra, ket):
        rho = update_left_environment(B, A, rho)
    return rho.flat[0]


def norm_squared(state: list) -> float:
    """|scprod(state, state).real| (state/mps.py:240-242)."""
    return abs(scprod(state, state).real)


# --------------------------------------------------------------------------
# Truncation recorder: every SVD split is logged for rank-parity checks
# --------------------------------------------------------------------------


@dataclass
class Split:
    kind: str  # "canon_right", "canon_left", "2site_right", "2site_left"
    site: int
    shape: tuple
    s: np.ndarray  # all singular values, descending
    rank: int
    err2: float


@dataclass
class Recorder:
    splits: list = field(default_factory=list)

    def add(self, kind, site, shape, s, rank, err2):
        self.splits.append(Split(kind, site, tuple(shape), np.array(s), rank, err2))


_NULL = None


def _record(rec, *args):
    if rec is not None:
        rec.add(*args)


# --------------------------------------------------------------------------
# Canonical form (reference cython/schmidt.pxi:18-174)
# --------------------------------------------------------------------------


def update_canonical_right(state, A, site, strategy, rec=None) -> float:
    """SVD of A as (a*i, b); keep U at `site`, absorb s*V into `site+1`.

    reference schmidt.pxi:18-42.  Returns sqrt(err^2).
    """
    a, i, b = A.shape
    U, s, V = svd(np.array(A, copy=True).reshape(a * i, b))
    D, err2 = truncate(s, strategy)
    _record(rec, "canon_right", site, (a * i, b), s, D, err2)
    state[site] = U[:, :D].reshape(a, i, D)
    state[site + 1] = contract_last_and_first(s[:D, None] * V[:D, :], state[site + 1])
    return sqrt(err2)


def update_canonical_left(state, A, site, strategy, rec=None) -> float:
    """SVD of A as (a, i*b); keep V at `site`, absorb U*s into `site-1`.

    reference schmidt.pxi:59-82.  Returns sqrt(err^2).
    """
    a, i, b = A.shape
    U, s, V = svd(np.array(A, copy=True).reshape(a, i * b))
    D, err2 = truncate(s, strategy)
    _record(rec, "canon_left", site, (a, i * b), s, D, err2)
    state[site] = V[:D, :].reshape(D, i, b)
    state[site - 1] = contract_last_and_first(state[site - 1], U[:, :D] * s[:D])
    return sqrt(err2)


def canonicalize(state: list, center: int, strategy: Strategy, rec=None) -> float:
    """reference schmidt.pxi:109-120."""
    L = len(state)
    err = 0.0
    for i in range(0, center):
        err += update_canonical_right(state, state[i], i, strategy, rec)
    for i in range(L - 1, center, -1):
        err += update_canonical_left(state, state[i], i, strategy, rec)
    return err


def recanonicalize(state, oldcenter, newcenter, strategy, rec=None) -> float:
    """reference schmidt.pxi:96-106."""
    err = 0.0
    while oldcenter > newcenter:
        err += update_canonical_left(state, state[oldcenter], oldcenter, strategy, rec)
        oldcenter -= 1
    while oldcenter < newcenter:
        err += update_canonical_right(state, state[oldcenter], oldcenter, strategy, rec)
        oldcenter += 1
    return err


def left_orth_2site(AA, strategy, rec=None, site=-1):
    """(U, s*V, sqrt(err^2)) of AA as (a*d1, d2*b) (schmidt.pxi:123-147)."""
    a, d1, d2, b = AA.shape
    U, s, V = svd(AA.reshape(a * d1, d2 * b))
    D, err2 = truncate(s, strategy)
    _record(rec, "2site_right", site, (a * d1, d2 * b), s, D, err2)
    return (
        U[:, :D].reshape(a, d1, D),
        (s[:D, None] * V[:D, :]).reshape(D, d2, b),
        sqrt(err2),
    )


def right_orth_2site(AA, strategy, rec=None, site=-1):
    """(U*s, V, sqrt(err^2)) of AA as (a*d1, d2*b) (schmidt.pxi:150-174)."""
    a, d1, d2, b = AA.shape
    U, s, V = svd(AA.reshape(a * d1, d2 * b))
    D, err2 = truncate(s, strategy)
    _record(rec, "2site_left", site, (a * d1, d2 * b), s, D, err2)
    return (
        (U[:, :D] * s[:D]).reshape(a, d1, D),
        V[:D, :].reshape(D, d2, b),
        sqrt(err2),
    )


# --------------------------------------------------------------------------
# Antilinear form (reference state/antilinear.py:13-146)
# --------------------------------------------------------------------------


class AntilinearForm:
    """<bra|ket> with cached left/right environments (state/antilinear.py:13-146)."""

    def __init__(self, bra: list, ket: list, center: int = 0):
        size = len(bra)
        rho = np.eye(1)
        R = [rho] * size
        for i in range(size - 1, center, -1):
            R[i - 1] = rho = update_right_environment(bra[i], ket[i], rho)
        rho = np.eye(1)
        L = [rho] * size
        for i in range(0, center):
            L[i + 1] = rho = update_left_environment(bra[i], ket[i], rho)
        self.bra, self.ket, self.size = bra, ket, size
        self.L, self.R, self.center = L, R, center

    def tensor1site(self):
        c = self.center
        return contract_last_and_first(
            self.L[c], contract_last_and_first(self.ket[c], self.R[c])
        )

    def tensor2site(self, direction: int):
        if direction > 0:
            i = self.center
            j = i + 1
        else:
            j = self.center
            i = j - 1
        LA = contract_last_and_first(self.L[i], self.ket[i])
        BR = contract_last_and_first(self.ket[j], self.R[j])
        return contract_last_and_first(LA, BR)

    def update_right(self):
        prev = self.center
        self.L[prev + 1] = update_left_environment(
            self.bra[prev], self.ket[prev], self.L[prev]
        )
        self.center = prev + 1

    def update_left(self):
        prev = self.center
        self.R[prev - 1] = update_right_environment(
            self.bra[prev], self.ket[prev], self.R[prev]
        )
        self.center = prev - 1


# --------------------------------------------------------------------------
# simplify (reference state/simplification.py:32-280)
# --------------------------------------------------------------------------


@dataclass
class SimplifyResult:
    tensors: list
    center: int
    error: float
    sweeps: int = 0
    errs: list = field(default_factory=list)  # per-sweep err estimates
    norm_state_sqr: float = 0.0


def canonical_mps(tensors, center, strategy, normalize=None, rec=None):
    """CanonicalMPS(data, center, normalize, strategy) (canonical_mps.py:76-108)."""
    data = list(tensors)
    L = len(data)
    c = center if center >= 0 else center + L
    err = canonicalize(data, c, strategy, rec)
    if normalize is True or (normalize is None and strategy.normalize):
        N = np.linalg.norm(data[c].reshape(-1))
        if N:
            data[c] = data[c] / N
    return data, c, err


def simplify(
    tensors: list,
    strategy: Strategy = SIMPLIFICATION_STRATEGY,
    direction: int = +1,
    error: float = 0.0,
    rec: Recorder | None = None,
    guess: list | None = None,
) -> SimplifyResult:
    """Variational simplification of one MPS (simplification.py:32-144)."""
    size = len(tensors)
    start = 0 if direction > 0 else -1
    method = strategy.simplify
    if method == Simplification.CANONICAL_FORM:
        data, c, err = canonical_mps(tensors, start, strategy, rec=rec)
        newc = (-1 - start) % size
        err += recanonicalize(data, c, newc, strategy, rec)
        return SimplifyResult(data, newc, error + err)
    if method == Simplification.DO_NOT_SIMPLIFY:
        data, c, err = canonical_mps(tensors, -1 - start, strategy, rec=rec)
        return SimplifyResult(data, c, error + err)

    mps, center, _ = canonical_mps(
        tensors if guess is None else guess, start, strategy, normalize=False, rec=rec
    )
    norm_state_sqr = norm_squared(tensors)
    if not norm_state_sqr:
        zero = [np.zeros((1, A.shape[1], 1)) for A in tensors]
        return SimplifyResult(zero, 0, 0.0)
    form = AntilinearForm(mps, tensors, center=center)
    err = 2.0
    norm_mps_sqr = 0.0
    errs = []
    sweeps = 0
    last = None
    for _sweep in range(max(1, strategy.max_sweeps)):
        sweeps += 1
        if direction > 0:
            for n in range(0, size - 1):
                mps[n], mps[n + 1], _e = left_orth_2site(
                    form.tensor2site(direction), strategy, rec, n
                )
                form.update_right()
            center = size - 1
        else:
            for n in reversed(range(0, size - 1)):
                mps[n], mps[n + 1], _e = right_orth_2site(
                    form.tensor2site(direction), strategy, rec, n
                )
                form.update_left()
            center = 0
        last = mps[center]
        norm_mps_sqr = np.vdot(last, last).real
        mps_state_scprod = np.vdot(last, form.tensor1site())
        old_err = err
        err = 2 * abs(1.0 - mps_state_scprod.real / sqrt(norm_mps_sqr * norm_state_sqr))
        errs.append(err)
        if err < strategy.simplification_tolerance or err > old_err:
            break
        direction = -direction
    total_error_bound = error + sqrt(err)
    if strategy.normalize and norm_mps_sqr:
        factor = sqrt(norm_mps_sqr)
        mps[center] = last / factor
        total_error_bound /= factor
    return SimplifyResult(mps, center, total_error_bound, sweeps, errs, norm_state_sqr)


def mpssum_join(weights: list, states: list) -> list:
    """Block-diagonal join of a weighted sum (state/mpssum.py:130-167)."""
    L = len(states[0])
    out = []
    for i in range(L):
        As = [s[i] for s in states]
        if i == 0:
            out.append(np.concatenate([w * A for w, A in zip(weights, As)], axis=2))
        elif i == L - 1:
            out.append(np.concatenate(As, axis=0))
        else:
            DL = sum(A.shape[0] for A in As)
            DR = sum(A.shape[2] for A in As)
            d = As[0].shape[1]
            dt = np.result_type(*As)
            B = np.zeros((DL, d, DR), dtype=dt)
            l = r = 0
            for A in As:
                a, _, b = A.shape
                B[l : l + a, :, r : r + b] = A
                l += a
                r += b
            out.append(B)
    return out


def mpssum_norm_squared(weights, states) -> float:
    """delete_zero_components' norm (state/mpssum.py:204-228), zero terms kept out."""
    c = 0.0
    fw, fs = [], []
    for wi, si in zip(weights, states):
        wic = np.conj(wi)
        ni = (wic * wi).real * norm_squared(si)
        if ni:
            for wj, sj in zip(fw, fs):
                c += 2 * (wic * wj * scprod(si, sj)).real
            fs.append(si)
            fw.append(wi)
            c += ni
    return abs(c), fw, fs


def simplify_mps_sum(
    weights: list,
    states: list,
    strategy: Strategy = SIMPLIFICATION_STRATEGY,
    direction: int = +1,
    errors: list | None = None,
    rec: Recorder | None = None,
    guess: list | None = None,
) -> SimplifyResult:
    """Variational simplification of sum_i w_i psi_i (simplification.py:150-280); a guess
    replaces the joined sum as the starting state (:214-219)."""
    norm_state_sqr, weights, states = mpssum_norm_squared(weights, states)
    if errors is None:
        errors = [0.0] * len(states)
    if not norm_state_sqr:
        zero = [np.zeros((1, A.shape[1], 1)) for A in states[0]]
        return SimplifyResult(zero, 0, 0.0)
    start = 0 if direction > 0 else -1
    mps, center, _ = canonical_mps(
        mpssum_join(weights, states) if guess is None else guess, start, strategy,
        normalize=False, rec=rec
    )
    size = len(mps)
    forms = [AntilinearForm(mps, si, center=center) for si in states]
    err = 2.0
    norm_mps_sqr = 0.0
    errs = []
    sweeps = 0
    last = None
    for _sweep in range(max(1, strategy.max_sweeps)):
        sweeps += 1
        if direction > 0:
            for n in range(0, size - 1):
                AA = sum(w * f.tensor2site(direction) for w, f in zip(weights, forms))
                mps[n], mps[n + 1], _e = left_orth_2site(AA, strategy, rec, n)
                for f in forms:
                    f.update_right()
            center = size - 1
        else:
            for n in reversed(range(0, size - 1)):
                AA = sum(w * f.tensor2site(direction) for w, f in zip(weights, forms))
                mps[n], mps[n + 1], _e = right_orth_2site(AA, strategy, rec, n)
                for f in forms:
                    f.update_left()
            center = 0
        last = mps[center]
        norm_mps_sqr = np.vdot(last, last).real
        sc = np.vdot(last, sum(w * f.tensor1site() for w, f in zip(weights, forms)))
        old_err = err
        err = 2 * abs(1.0 - sc.real / sqrt(norm_mps_sqr * norm_state_sqr))
        errs.append(err)
        if err < strategy.simplification_tolerance or err > old_err:
            break
        direction = -direction
    total_error_bound = sum(abs(w) * e for w, e in zip(weights, errors)) + sqrt(err)
    if strategy.normalize and norm_mps_sqr:
        factor = sqrt(norm_mps_sqr)
        mps[center] = last / factor
        total_error_bound /= factor
    return SimplifyResult(mps, center, total_error_bound, sweeps, errs, norm_state_sqr)


def contract_nrjl_ijk_klm(U, A, B):
    """np.einsum('ijk,klm,nrjl -> inrm', A, B, U) (cython/contractions.pxi:102-127)."""
    a, d, b = A.shape
    _, e, c = B.shape
    AB = (A.reshape(a * d, b) @ B.reshape(b, e * c)).reshape(a, d * e, c)
    return np.matmul(U, AB).reshape(a, d, e, c)


def mpo_join(mpos: list) -> list:
    """MPOList.join (operators/mpo.py:679-711): per site, the tensors joined from the last
    MPO backwards, aijb,cjkd->acikbd with the later MPO's tensor first."""
    out = []
    for s in range(len(mpos[0])):
        ts = [m[s] for m in mpos]

        def join(A, *args):
            if not args:
                return A
            B = join(*args)
            a, d, _, b = A.shape
            c, _, _, e = B.shape
            aux = np.tensordot(B, A, ((2,), (1,)))
            return np.ascontiguousarray(aux.transpose(0, 3, 1, 4, 2, 5).reshape(a * c, d, d, b * e))

        out.append(join(*ts))
    return out


def simplify_mpo(mpo: list, strategy: Strategy, direction: int = +1, guess: list | None = None):
    """simplify_mpo (operators/simplify_mpo.py:50-89) on a list of MPO tensors: as an MPS of
    physical dimension i*j, simplified, and back."""
    as_mps = [O.reshape(O.shape[0], O.shape[1] * O.shape[2], O.shape[3]) for O in mpo]
    g = None if guess is None else [O.reshape(O.shape[0], -1, O.shape[3]) for O in guess]
    res = simplify(as_mps, strategy, direction, guess=g)
    s = int(round(np.sqrt(mpo[0].shape[1] * mpo[0].shape[2])))
    return [A.reshape(A.shape[0], s, s, A.shape[2]) for A in res.tensors], res


def mpo_apply(
    mpo: list,
    state: list,
    strategy: Strategy = DEFAULT_STRATEGY,
    simplify_flag: bool | None = None,
    error: float = 0.0,
    rec: Recorder | None = None,
):
    """MPO.apply on an MPS (operators/mpo.py:229-281)."""
    if simplify_flag is None:
        simplify_flag = strategy.simplify != Simplification.DO_NOT_SIMPLIFY
    prod = [mpo_multiply_tensor(O, B) for O, B in zip(mpo, state)]
    if simplify_flag:
        return simplify(prod, strategy, +1, error, rec)
    return SimplifyResult(prod, -1, error)


# --------------------------------------------------------------------------
# Helpers shared by tests and the benchmark: seeded inputs and comparisons
# --------------------------------------------------------------------------


def random_mps(d: int, n: int, D: int, rng, complex_: bool = False, truncate_=True):
    """Random MPS with the reference factory's bond rule (state/factories.py:180-215)."""
    out = []
    DR = 1
    for i in range(n):
        DL = DR
        if not truncate_ and i != n - 1:
            DR = D
        else:
            DR = min(DR * d, D, d ** (n - i - 1))
        T = rng.normal(size=(DL, d, DR))
        if complex_:
            T = T + 1j * rng.normal(size=T.shape)
        out.append(T)
    return out


def random_mpo(d: int, n: int, D: int, rng, complex_: bool = False):
    """Random MPO with bond D (edges 1), entries N(0,1)/sqrt(D*d)."""
    out = []
    for i in range(n):
        Dl = 1 if i == 0 else D
        Dr = 1 if i == n - 1 else D
        T = rng.normal(size=(Dl, d, d, Dr))
        if complex_:
            T = T + 1j * rng.normal(size=T.shape)
        out.append(T / sqrt(D * d))
    return out


def tridiagonal_mpo(n: int, a: float, b: float, c: float, closed: bool = True):
    """Second-difference style MPO of bond 3 (analysis/derivatives/finite_differences.py:9-38)."""
    A = np.zeros((3, 2, 2, 3))
    A[0, 0, 0, 0] = 1.0
    A[0, 1, 1, 0] = 1.0
    A[0, 1, 0, 1] = 1.0
    A[1, 0, 1, 1] = 1.0
    A[2, 1, 0, 2] = 1.0
    A[0, 0, 1, 2] = 1.0
    R = a * A[:, :, :, [0]] + b * A[:, :, :, [1]] + c * A[:, :, :, [2]]
    if closed:
        Lt = A[[0], :, :, :] + A[[1], :, :, :] + A[[2], :, :, :]
    else:
        Lt = A[[0], :, :, :]
    return [Lt] + [A] * (n - 2) + [R]


def scale(tensors: list, factor) -> list:
    out = list(tensors)
    out[0] = out[0] * factor
    return out


def to_vector(tensors: list) -> np.ndarray:
    """Dense state vector (state/mps.py:457-472); small sizes only."""
    psi = np.ones(1)
    for A in reversed(tensors):
        a, d, b = A.shape
        psi = (A.reshape(a * d, b) @ psi).reshape(a, -1)
    return psi.reshape(-1)


def fidelity_error(a: list, b: list) -> float:
    """1 - |<a|b>|^2 / (<a|a><b|b>) computed through environments."""
    ab = scprod(a, b)
    aa = scprod(a, a).real
    bb = scprod(b, b).real
    return float(1.0 - (abs(ab) ** 2) / (aa * bb))
