"""DMRG two-site effective-Hamiltonian matvec on the GPU and a Lanczos solver
around it (the reference's QuadraticForm.two_site_operator, operators/quadratic.py:
187-237, diagonalised by scipy's eigsh in optimization/dmrg.py:15-23).

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

import numpy as np

from . import _lib
from .core import as_device

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


def lanczos_ground_state(L, H, R, v0, krylov: int = 30, precision: str = "fp64", tol: float = 0.0):
    """Lowest eigenpair of the (Hermitian, real) two-site operator from the start vector v0:
    ``krylov`` Lanczos steps, each new vector fully re-orthogonalised against the basis in FP64
    (classical Gram-Schmidt applied twice, library GEMMs), the tridiagonal eigenproblem on the
    host.  Returns (eigenvalue, eigenvector as a device tensor shaped like v0, steps run)."""
    import torch

    L, H, R = (as_device(t, False) for t in (L, H, R))
    v0 = as_device(v0, False)
    shape = tuple(v0.shape)
    n = v0.numel()
    m = min(krylov, n)
    dev = v0.device
    V = torch.empty((m, n), dtype=torch.float64, device=dev)
    coef = torch.empty((m, 1), dtype=torch.float64, device=dev)
    s = torch.empty((1, 1), dtype=torch.float64, device=dev)
    one = torch.ones((1, 1), dtype=torch.float64, device=dev)
    w = torch.empty(shape, dtype=torch.float64, device=dev)
    alpha, beta = [], []
    op = TwoSiteOperator(L, H, R, precision) if precision in ("tf32x3", "bf16") else None
    q = v0.reshape(-1)
    _gemm(0, 0, 1, 1, n, q, n, q, 1, s, 1)
    _gemm(0, 0, n, 1, 1, q, 1, one, 1, V[0], 1, alpha=1.0 / float(s.sqrt().item()))
    steps = 0
    for j in range(m):
        if op is not None:
            op.matvec(V[j].reshape(shape), out=w)
        else:
            two_site_matvec(L, H, R, V[j].reshape(shape), precision, out=w)
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
        if j + 1 == m or b <= tol:
            break
        beta.append(b)
        _gemm(0, 0, n, 1, 1, wf, 1, one, 1, V[j + 1], 1, alpha=1.0 / b)
    T = np.diag(alpha) + np.diag(beta[: steps - 1], 1) + np.diag(beta[: steps - 1], -1)
    evals, evecs = np.linalg.eigh(T)
    y = torch.from_numpy(np.ascontiguousarray(evecs[:, 0].reshape(1, steps))).to(dev)
    x = torch.empty((1, n), dtype=torch.float64, device=dev)
    _gemm(0, 0, 1, n, steps, y, steps, V, n, x, n)
    return float(evals[0]), x.reshape(shape), steps
