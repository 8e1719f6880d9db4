"""Two-site DMRG on the GPU (the reference's optimization/dmrg.py:26-199 with
QuadraticForm, operators/quadratic.py:31-348, and the MPO environments of
state/environments.py:15-48).

The effective-Hamiltonian matvec (QuadraticForm.two_site_operator, operators/quadratic.py:
187-237) is diagonalised by a Lanczos solver here where the reference calls scipy's eigsh
(optimization/dmrg.py:15-23).

``two_site_matvec`` is one call of ``sm_two_site_matvec``: GEMM, two-site MPO
contraction, GEMM, in FP64 or at the reduced precisions of the DMRG pattern
("fp64tc": FP64-accurate on the BF16 tensor cores; "tf32x3": FP32-accurate;
"bf16": one BF16 product with FP32 accumulation).  ``TwoSiteOperator`` is the
prepared form for the reduced precisions (environments converted once).  ``lanczos_ground_state`` runs a
Krylov iteration with those matvecs and re-orthogonalises the basis in FP64 with
the library's FP64 GEMM; the small tridiagonal problem is solved on the host,
as ARPACK does for the reference.
"""

from __future__ import annotations

import ctypes as C
import dataclasses

import numpy as np

from . import _lib
from .core import DEFAULT_STRATEGY, Strategy, _contract_last_and_first, as_device, dtype_code

PRECISIONS = {"fp64": 0, "fp64tc": 1, "tf32x3": 2, "bf16": 3}


def two_site_matvec(L, H, R, v, precision: str = "fp64", out=None):
    """out[a,ko,lo,g] = sum L[a,c,b] v[b,k,l,f] H[c,ko,k,lo,l,d] R[g,d,f] (device tensors or
    arrays; returns a device tensor)."""
    import torch

    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
    cplx = any((t.is_complex() if hasattr(t, "is_complex") else np.iscomplexobj(t))
               for t in (L, H, R, v))
    L, H, R, v = (as_device(t, cplx) for t in (L, H, R, v))
    a, c, b = L.shape
    c2, p1, k1, p2, k2, e = H.shape
    g, e2, f = R.shape
    if (c2, k1, p1, k2, p2, e2) != (c, p1, k1, p2, k2, e) or tuple(v.shape) != (b, p1, p2, f):
        raise ValueError("two_site_matvec: inconsistent shapes")
    if out is None:
        out = torch.empty((a, p1, p2, g), dtype=v.dtype, device=v.device)
    dims = _lib.int_array([a, c, b, p1, p2, e, g, f])
    _lib.check(_lib.load().sm_two_site_matvec(
        _lib.context(), _lib.SM_COMPLEX128 if cplx else _lib.SM_FLOAT64, dims, _lib.ptr(L),
        _lib.ptr(H), _lib.ptr(R), _lib.ptr(v), _lib.ptr(out), PRECISIONS[precision],
        _lib.stream_handle()))
    return out


def _ctx_key(ctx):
    return getattr(ctx, "value", ctx)


class TwoSiteOperator:
    """The two-site operator of fixed environments for a Lanczos run (real operands, "tf32x3" or
    "bf16"): ``sm_two_site_prepare`` turns L and R into tensor-core operand planes once, and each
    ``matvec`` (``sm_two_site_matvec_prepared``) converts only v.  The planes live in the library
    context, one prepared operator at a time: a matvec after another operator was prepared prepares
    this one again.  The operator keeps its device tensors alive."""

    _current = {}  # context handle -> id of the prepared operator

    def __init__(self, L, H, R, precision: str = "bf16"):
        if precision not in ("tf32x3", "bf16"):
            raise ValueError("TwoSiteOperator: precision must be 'tf32x3' or 'bf16'")
        self.L, self.H, self.R = (as_device(t, False) for t in (L, H, R))
        a, c, b = self.L.shape
        c2, p1, k1, p2, k2, e = self.H.shape
        g, e2, f = self.R.shape
        if (c2, k1, k2, e2) != (c, p1, p2, e):
            raise ValueError("TwoSiteOperator: inconsistent shapes")
        self.shape = (b, p1, p2, f)
        self.out_shape = (a, p1, p2, g)
        self.precision = precision
        self._dims = _lib.int_array([a, c, b, p1, p2, e, g, f])
        self._prepare()

    def _prepare(self):
        ctx = _lib.context()
        _lib.check(_lib.load().sm_two_site_prepare(
            ctx, self._dims, _lib.ptr(self.L), _lib.ptr(self.R), PRECISIONS[self.precision],
            _lib.stream_handle()))
        TwoSiteOperator._current[_ctx_key(ctx)] = id(self)

    def matvec(self, v, out=None):
        import torch

        v = as_device(v, False)
        if tuple(v.shape) != self.shape:
            raise ValueError("TwoSiteOperator.matvec: v has the wrong shape")
        if out is None:
            out = torch.empty(self.out_shape, dtype=torch.float64, device=v.device)
        if TwoSiteOperator._current.get(_ctx_key(_lib.context())) != id(self):
            self._prepare()
        _lib.check(_lib.load().sm_two_site_matvec_prepared(
            _lib.context(), _lib.ptr(self.H), _lib.ptr(v), _lib.ptr(out), _lib.stream_handle()))
        return out


def _gemm(opA, opB, M, N, K, A, lda, B, ldb, Cm, ldc, alpha=1.0, beta=0.0):
    """C = alpha op(A) op(B) + beta C with the library's FP64 GEMM (real)."""
    _lib.check(_lib.load().sm_gemm_ex(
        _lib.context(), _lib.SM_FLOAT64, opA, opB, M, N, K, _lib.dbl_array([alpha, 0.0]),
        _lib.ptr(A), lda, _lib.ptr(B), ldb, _lib.dbl_array([beta, 0.0]), _lib.ptr(Cm), ldc,
        _lib.stream_handle()))


def _lanczos_cycle(apply, x0, m: int):
    """One Lanczos run of at most m steps from x0 (real, FP64 basis): every new vector is
    re-orthogonalised against the basis twice (classical Gram-Schmidt with the library's
    FP64 GEMM); the tridiagonal problem is solved on the host.  Returns (lowest Ritz value,
    Ritz vector shaped like x0, residual norm estimate beta_m |y_m|, steps)."""
    import torch

    shape = tuple(x0.shape)
    n = x0.numel()
    m = max(1, min(m, n))
    dev = x0.device
    V = torch.empty((m, n), dtype=torch.float64, device=dev)
    coef = torch.empty((m, 1), dtype=torch.float64, device=dev)
    s = torch.empty((1, 1), dtype=torch.float64, device=dev)
    one = torch.ones((1, 1), dtype=torch.float64, device=dev)
    w = torch.empty(shape, dtype=torch.float64, device=dev)
    alpha, beta = [], []
    q = x0.reshape(-1)
    _gemm(0, 0, 1, 1, n, q, n, q, 1, s, 1)
    _gemm(0, 0, n, 1, 1, q, 1, one, 1, V[0], 1, alpha=1.0 / float(s.sqrt().item()))
    steps, b = 0, 0.0
    for j in range(m):
        apply(V[j].reshape(shape), w)
        wf = w.reshape(-1)
        _gemm(0, 0, j + 1, 1, n, V, n, wf, 1, coef, 1)
        alpha.append(float(coef[j].item()))
        for rep in range(2):
            if rep:
                _gemm(0, 0, j + 1, 1, n, V, n, wf, 1, coef, 1)
            _gemm(1, 0, n, 1, j + 1, V, n, coef, 1, wf, 1, alpha=-1.0, beta=1.0)
        _gemm(0, 0, 1, 1, n, wf, n, wf, 1, s, 1)
        b = float(s.sqrt().item())
        steps = j + 1
        # an invariant subspace (breakdown) ends the run: the Ritz pair is then exact
        if j + 1 == m or b <= 1e-14 * max(abs(a) for a in alpha):
            break
        beta.append(b)
        _gemm(0, 0, n, 1, 1, wf, 1, one, 1, V[j + 1], 1, alpha=1.0 / b)
    T = np.diag(alpha) + np.diag(beta[: steps - 1], 1) + np.diag(beta[: steps - 1], -1)
    evals, evecs = np.linalg.eigh(T)
    y = torch.from_numpy(np.ascontiguousarray(evecs[:, 0].reshape(1, steps))).to(dev)
    x = torch.empty((1, n), dtype=torch.float64, device=dev)
    _gemm(0, 0, 1, n, steps, y, steps, V, n, x, n)
    return float(evals[0]), x.reshape(shape), b * abs(float(evecs[steps - 1, 0])), steps


def lanczos_ground_state(L, H, R, v0, krylov: int = 30, precision: str = "fp64", tol: float = 0.0,
                         restarts: int = 0, polish: int = 0, polish_precision: str = "fp64tc"):
    """Lowest eigenpair of the (Hermitian, real) two-site operator from the start vector v0.

    Each cycle is ``krylov`` Lanczos steps (FP64 basis, full re-orthogonalisation) with the
    matvecs in ``precision``; up to ``restarts`` more cycles restart from the Ritz vector
    while the residual estimate is above ``tol`` |lambda| (scipy's eigsh, which the reference
    calls with this tol, stops on the same relative criterion; tol = 0 means rounding level).
    For a reduced precision, ``polish`` > 0 then runs cycles of ``polish`` steps with
    FP64-accurate matvecs (``polish_precision``: "fp64tc", the FP64-accurate tensor-core
    products, or "fp64") from the result until the same criterion holds (or ``restarts`` is
    used up), so the pair reaches FP64 accuracy with most matvecs at the reduced precision.  Returns (eigenvalue,
    eigenvector as a device tensor shaped like v0, matvecs run)."""
    L, H, R = (as_device(t, False) for t in (L, H, R))
    x = as_device(v0, False)
    thr = max(tol, 1e-14)
    op = TwoSiteOperator(L, H, R, precision) if precision in ("tf32x3", "bf16") else None

    def reduced(v, out):
        if op is not None:
            op.matvec(v, out=out)
        else:
            two_site_matvec(L, H, R, v, precision, out=out)

    def full(v, out):
        two_site_matvec(L, H, R, v, polish_precision, out=out)

    total = 0
    lam = 0.0
    # a reduced-precision operator cannot resolve the residual below its own rounding:
    # one cycle of it, then the FP64-accurate polish
    cycles = 1 if (op is not None and polish > 0) else 1 + max(0, restarts)
    for _ in range(cycles):
        lam, x, res, steps = _lanczos_cycle(reduced, x, krylov)
        total += steps
        if res <= thr * max(abs(lam), 1e-300) or steps < krylov:
            break
    if op is not None and polish > 0:
        for _ in range(1 + max(0, restarts)):
            lam, x, res, steps = _lanczos_cycle(full, x, polish)
            total += steps
            if res <= thr * max(abs(lam), 1e-300) or steps < polish:
                break
    return lam, x, total


# ---------------------------------------------------------------------------
# MPO environments (state/environments.py:15-48)
# ---------------------------------------------------------------------------


def begin_mpo_environment(dtype=None):
    """(1, 1, 1) ones (state/environments.py:15-16)."""
    import torch

    return torch.ones((1, 1, 1), dtype=torch.float64 if dtype is None else dtype, device="cuda")


def _mpo_env(fn, rho, A, O, B, out_shape):
    import torch

    cplx = any(t.is_complex() if hasattr(t, "is_complex") else np.iscomplexobj(t)
               for t in (rho, A, O, B))
    rho, A, O, B = (as_device(t, cplx) for t in (rho, A, O, B))
    a, j, d = A.shape
    c, j2, i, e = O.shape
    b, i2, f = B.shape
    if j2 != j or i2 != i:
        raise ValueError("MPO environment: physical dimensions differ")
    out = torch.empty(out_shape(a, c, b, d, e, f), dtype=A.dtype, device=A.device)
    _lib.check(fn(_lib.context(), dtype_code(A), _lib.ptr(rho), _lib.ptr(A), a, j, d, _lib.ptr(O),
                  c, i, e, _lib.ptr(B), b, f, _lib.ptr(out), _lib.stream_handle()))
    return out


def update_left_mpo_environment(rho, A, O, B):
    """out[d,e,f] = sum conj(A[a,j,d]) rho[a,c,b] O[c,j,i,e] B[b,i,f] (environments.py:19-30)."""
    if tuple(rho.shape) != (A.shape[0], O.shape[0], B.shape[0]):
        raise ValueError("update_left_mpo_environment: rho does not match the sites")
    return _mpo_env(_lib.load().sm_update_left_mpo_environment, rho, A, O, B,
                    lambda a, c, b, d, e, f: (d, e, f))


def update_right_mpo_environment(rho, A, O, B):
    """out[a,c,b] = sum conj(A[a,j,d]) rho[d,e,f] O[c,j,i,e] B[b,i,f] (environments.py:33-42)."""
    if tuple(rho.shape) != (A.shape[2], O.shape[3], B.shape[2]):
        raise ValueError("update_right_mpo_environment: rho does not match the sites")
    return _mpo_env(_lib.load().sm_update_right_mpo_environment, rho, A, O, B,
                    lambda a, c, b, d, e, f: (a, c, b))


def end_mpo_environment(rho):
    return rho.reshape(-1)[0].item()


def join_mpo_environments(left, right):
    return (left.reshape(-1) * right.reshape(-1)).sum().item()


def mpo_expectation(O, bra, ket=None):
    """<bra|O|ket> (operators/mpo.py:378-416): left environments up to the bra's centre
    (the last site for a plain MPS), right environments from the end down to it."""
    from .state import CanonicalMPS, MPS

    if isinstance(bra, CanonicalMPS):
        center = bra.center
    elif isinstance(bra, MPS):
        center = O.size - 1
    else:
        raise TypeError("MPS required")
    if ket is None:
        ket = bra
    elif not isinstance(ket, MPS):
        raise TypeError("MPS required")
    left = right = begin_mpo_environment()
    for i in range(0, center):
        left = update_left_mpo_environment(left, bra[i], O[i], ket[i])
    for i in range(O.size - 1, center - 1, -1):
        right = update_right_mpo_environment(right, bra[i], O[i], ket[i])
    return join_mpo_environments(left, right)


# ---------------------------------------------------------------------------
# QuadraticForm and the two-site DMRG driver
# ---------------------------------------------------------------------------


class QuadraticForm:
    """<state|O|ket> with MPO environments left and right of the active site
    (operators/quadratic.py:31-100, 348-370), device tensors throughout."""

    def __init__(self, O, state, start: int = 0, ket=None):
        from .state import CanonicalMPS

        if not isinstance(state, CanonicalMPS):
            raise TypeError("QuadraticForm: state must be a CanonicalMPS")
        if state.center not in (start, start + 1):
            raise ValueError(f"QuadraticForm: state must be centered at start={start} or {start + 1}")
        self.O, self.state = O, state
        self.ket = ket if ket is not None else state
        self.size = size = state.size
        if size != O.size:
            raise ValueError("QuadraticForm: MPO and MPS do not have the same size")
        if any(int(Op.shape[1]) != int(A.shape[1]) for Op, A in zip(O, state)):
            raise ValueError("QuadraticForm: MPO and MPS dimensions do not match")
        env = begin_mpo_environment(state[0].dtype)
        self.left_env = [env] * size
        self.right_env = [env] * size
        for i in range(size - 1, max(0, start - 1), -1):
            self.right_env[i - 1] = env = update_right_mpo_environment(env, state[i], O[i],
                                                                       self.ket[i])
        env = self.left_env[0]
        for i in range(0, start):
            self.left_env[i + 1] = env = update_left_mpo_environment(env, state[i], O[i],
                                                                     self.ket[i])
        self.site = start

    def two_site_block(self, i: int):
        """(L, H12, R) with H12 = O[i] O[i+1] (operators/quadratic.py:102-104)."""
        return self.left_env[i], _contract_last_and_first(self.O[i], self.O[i + 1]), \
            self.right_env[i + 1]

    def ket_2site(self, i: int):
        return _contract_last_and_first(self.ket[i], self.ket[i + 1])

    def diagonalize_two_site(self, i: int, tol_eigs: float, precision: str = "fp64",
                             krylov: int = 30, restarts: int = 20):
        """Lowest eigenpair of the effective two-site operator from the current two-site
        tensor (optimization/dmrg.py:15-23)."""
        L, H12, R = self.two_site_block(i)
        v = _contract_last_and_first(self.state[i], self.state[i + 1])
        lam, x, _ = lanczos_ground_state(L, H12, R, v, krylov=krylov, precision=precision,
                                         tol=tol_eigs, restarts=restarts,
                                         polish=12 if precision in ("tf32x3", "bf16") else 0)
        return lam, x

    def update_2site_right(self, AB, i: int, strategy: Strategy) -> None:
        self.state.update_2site_right(AB, i, strategy)
        if i < self.size - 2:
            self.site = j = i + 1
            self.left_env[j] = update_left_mpo_environment(self.left_env[i], self.state[i],
                                                           self.O[i], self.ket[i])

    def update_2site_left(self, AB, i: int, strategy: Strategy) -> None:
        self.state.update_2site_left(AB, i, strategy)
        if i > 0:
            j = i + 1
            self.right_env[i] = update_right_mpo_environment(self.right_env[j], self.state[j],
                                                             self.O[j], self.ket[j])
            self.site = i - 1


@dataclasses.dataclass
class OptimizeResults:
    """Result of a ground-state search (optimization/descent.py:22-49)."""

    state: object
    energy: float
    converged: bool
    message: str
    trajectory: list = dataclasses.field(default_factory=list)
    variances: list = dataclasses.field(default_factory=list)


def _energy_and_variance(H, state):
    """<H> and |<H^2> - <H>^2| (optimization/dmrg.py:56-60); |H psi|^2 is taken from the MPO
    and MPS factors (sm_mpo_scprod) instead of the bond-(chi D) product."""
    from .operators import mpo_scprod

    energy = float(np.real(mpo_expectation(H, state)))
    h2 = float(np.real(mpo_scprod(H, state, state)))
    return energy, abs(h2 - energy * energy)


def _state_deepcopy(state):
    from .state import CanonicalMPS, MPS

    data = [A.clone() for A in state]
    if isinstance(state, CanonicalMPS):
        return CanonicalMPS(data, center=state.center, normalize=False, strategy=state.strategy,
                            is_canonical=True, error=state.error())
    return MPS(data, error=state.error())


def dmrg(H, guess=None, maxiter: int = 20, tol: float = 1e-10, tol_up: float | None = None,
         tol_eigs: float | None = None, strategy: Strategy = DEFAULT_STRATEGY, callback=None,
         precision: str = "fp64", krylov: int = 30) -> OptimizeResults:
    """Ground state of an MPO Hamiltonian by two-site DMRG (optimization/dmrg.py:76-199),
    with the same sweep order, convergence rule and results record.  The two-site
    eigenproblems run the Lanczos solver of this module; ``precision`` sets its matvec
    precision ("fp64", or "bf16" / "tf32x3" with an FP64 polish of the eigenpair).
    H must be a (real) MPO: a nearest-neighbour Hamiltonian is converted by the caller
    (the reference's H.to_mpo())."""
    from .operators import MPO
    from .state import CanonicalMPS, random_mps

    if maxiter < 1:
        raise ValueError("maxiter must be positive")
    if not isinstance(H, MPO):
        raise TypeError("dmrg: H must be an MPO")
    if H.size < 2:
        raise ValueError("DMRG requires at least two sites")
    if guess is None:
        guess = random_mps(H.physical_dimensions(), D=2)
    if tol < 0:
        raise ValueError("tol must be non-negative")
    if tol_up is None:
        tol_up = tol
    elif tol_up < 0:
        raise ValueError("tol_up must be non-negative")
    if tol_eigs is None:
        tol_eigs = tol
    strat = strategy.replace(normalize=True)
    if not isinstance(guess, CanonicalMPS) or guess.center not in (0, H.size - 1):
        guess = CanonicalMPS(guess, center=0, strategy=strat)
    guess.normalize_inplace()
    if guess.center == 0:
        direction = +1
        QF = QuadraticForm(H, guess, start=0)
    else:
        direction = -1
        QF = QuadraticForm(H, guess, start=H.size - 2)
    energy, variance = _energy_and_variance(H, QF.state)
    results = OptimizeResults(state=_state_deepcopy(QF.state), energy=energy, converged=False,
                              message=f"Exceeded maximum number of steps {maxiter}",
                              trajectory=[energy], variances=[variance])
    if callback is not None:
        callback(QF.state, results)
    last_energy = energy
    for _sweep in range(1, maxiter + 1):
        sites = range(H.size - 1) if direction > 0 else range(H.size - 2, -1, -1)
        for i in sites:
            _, AB = QF.diagonalize_two_site(i, tol_eigs, precision, krylov)
            if direction > 0:
                QF.update_2site_right(AB, i, strat)
            else:
                QF.update_2site_left(AB, i, strat)
        direction = -direction
        energy, variance = _energy_and_variance(H, QF.state)
        results.trajectory.append(energy)
        results.variances.append(variance)
        if energy < results.energy:
            results.energy, results.state = energy, _state_deepcopy(QF.state)
        if callback is not None:
            callback(QF.state, results)
        energy_change = energy - last_energy
        energy_scale = max(1.0, abs(energy))
        if energy_change > tol_up * energy_scale:
            results.converged = True
            results.message = f"Energy fluctuation above tolerance {tol_up}"
            break
        if -tol * energy_scale <= energy_change <= 0:
            results.converged = True
            results.message = f"Energy decrease slower than tolerance {tol}"
            break
        last_energy = energy
    return results
