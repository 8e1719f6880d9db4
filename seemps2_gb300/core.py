"""Strategy / Truncation / Simplification and the GPU kernel table.

The configuration classes keep the reference's names, defaults, validation and
error types (cython/truncation.pxi:1-220); the kernel functions mirror the
reference's kernel table (cython/__init__.py:25-54) but take and return CUDA
tensors (torch, float64 or complex128) and run the sm_103a kernels of
libseemps_gb300.so through its C ABI.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

MAX_BOND_DIMENSION = 0x7FFFFFFF
DEFAULT_TOLERANCE = float(np.finfo(np.float64).eps)


class Truncation:
    """SVD truncation rules (cython/truncation.pxi:22-43)."""

    DO_NOT_TRUNCATE = 0
    RELATIVE_SINGULAR_VALUE = 1
    RELATIVE_NORM_SQUARED_ERROR = 2
    ABSOLUTE_SINGULAR_VALUE = 3


class Simplification:
    """Tensor-network simplification methods (cython/truncation.pxi:45-61)."""

    DO_NOT_SIMPLIFY = 0
    CANONICAL_FORM = 1
    VARIATIONAL = 2
    VARIATIONAL_EXACT_GUESS = 3


class GemmOrder:
    NORMAL = 0
    TRANSPOSE = 1
    ADJOINT = 2


class Strategy:
    """MPS and MPO simplification strategies (cython/truncation.pxi:66-220).

    Same parameters, defaults and AssertionError checks as the reference:
    a zero tolerance turns any truncating method into ABSOLUTE_SINGULAR_VALUE.
    """

    __slots__ = ("_method", "_tolerance", "_simplification_tolerance", "_max_bond_dimension",
                 "_normalize", "_simplify", "_max_sweeps")

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
            method = Truncation.ABSOLUTE_SINGULAR_VALUE
        if max_bond_dimension <= 0 or max_bond_dimension > MAX_BOND_DIMENSION:
            raise AssertionError("Invalid bond dimension in Strategy")
        if simplify < 0 or simplify > Simplification.VARIATIONAL_EXACT_GUESS:
            raise AssertionError("Invalid simplify argument passed to Strategy")
        if max_sweeps < 0:
            raise AssertionError("Negative or zero number of sweeps in Strategy")
        if method not in (0, 1, 2, 3):
            raise AssertionError("Invalid method argument passed to Strategy")
        self._method = int(method)
        self._tolerance = float(tolerance)
        self._simplification_tolerance = float(simplification_tolerance)
        self._max_bond_dimension = int(max_bond_dimension)
        self._normalize = bool(normalize)
        self._simplify = int(simplify)
        self._max_sweeps = int(max_sweeps)

    def replace(self, method=None, tolerance=None, simplification_tolerance=None,
                max_bond_dimension=None, normalize=None, simplify=None, max_sweeps=None):
        return Strategy(
            method=self._method if method is None else method,
            tolerance=self._tolerance if tolerance is None else tolerance,
            simplification_tolerance=(self._simplification_tolerance
                                      if simplification_tolerance is None
                                      else simplification_tolerance),
            max_bond_dimension=(self._max_bond_dimension if max_bond_dimension is None
                                else max_bond_dimension),
            normalize=self._normalize if normalize is None else normalize,
            simplify=self._simplify if simplify is None else simplify,
            max_sweeps=self._max_sweeps if max_sweeps is None else max_sweeps,
        )

    def set_normalization(self, normalize: bool) -> "Strategy":
        return self.replace(normalize=normalize)

    def get_method(self) -> int:
        return self._method

    def get_simplification_method(self) -> int:
        return self._simplify

    def get_tolerance(self) -> float:
        return self._tolerance

    def get_simplification_tolerance(self) -> float:
        return self._simplification_tolerance

    def get_max_bond_dimension(self) -> int:
        return self._max_bond_dimension

    def get_normalize_flag(self) -> bool:
        return self._normalize

    def get_max_sweeps(self) -> int:
        return self._max_sweeps

    def get_simplify_flag(self) -> bool:
        return self._simplify != Simplification.DO_NOT_SIMPLIFY

    def to_c(self) -> _lib.sm_strategy:
        return _lib.sm_strategy(self._method, self._max_bond_dimension, self._tolerance,
                                self._simplification_tolerance, int(self._normalize),
                                self._simplify, self._max_sweeps, 0)

    def __str__(self) -> str:
        m = {0: "None", 1: "RelativeSVD", 2: "RelativeNorm", 3: "AbsoluteSVD"}
        s = {0: "None", 1: "CanonicalForm", 2: "Variational", 3: "Variational (exact guess)"}
        return (f"Strategy(method={m[self._method]}, tolerance={self._tolerance:5g}, "
                f"max_bond_dimension={self._max_bond_dimension}, normalize={self._normalize}, "
                f"simplify={s[self._simplify]}, "
                f"simplification_tolerance={self._simplification_tolerance:5g}, "
                f"max_sweeps={self._max_sweeps})")

    __repr__ = __str__


DEFAULT_STRATEGY = Strategy(method=Truncation.RELATIVE_NORM_SQUARED_ERROR,
                            simplify=Simplification.VARIATIONAL,
                            tolerance=DEFAULT_TOLERANCE,
                            simplification_tolerance=DEFAULT_TOLERANCE,
                            max_bond_dimension=MAX_BOND_DIMENSION, normalize=False)
NO_TRUNCATION = DEFAULT_STRATEGY.replace(method=Truncation.DO_NOT_TRUNCATE,
                                         simplify=Simplification.DO_NOT_SIMPLIFY)

# ---------------------------------------------------------------------------
# Tensor plumbing: device tensors in the library's two dtypes
# ---------------------------------------------------------------------------


def _torch():
    import torch

    return torch


def dtype_code(t) -> int:
    torch = _torch()
    return _lib.SM_COMPLEX128 if t.dtype == torch.complex128 else _lib.SM_FLOAT64


def as_device(x, complex_: bool | None = None, device=None):
    """CUDA, contiguous, float64 or complex128 copy/view of an array or tensor.

    float32/complex64 inputs are promoted like the reference's SVD/GEMM
    wrappers do (cython/svd.pxi:74-77, gemm.pxi:29-58).
    """
    torch = _torch()
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
    if not isinstance(x, torch.Tensor):
        x = torch.from_numpy(np.ascontiguousarray(x))
    is_c = x.is_complex() if complex_ is None else complex_
    dt = torch.complex128 if is_c else torch.float64
    if x.is_complex() and not is_c:
        raise TypeError("cannot store a complex tensor as float64")
    return x.to(device=dev, dtype=dt).contiguous()


def _common_complex(tensors) -> bool:
    return any(t.is_complex() if hasattr(t, "is_complex") else np.iscomplexobj(t) for t in tensors)


# ---------------------------------------------------------------------------
# Kernel table (reference seemps.cython)
# ---------------------------------------------------------------------------


def destructively_truncate_vector(s, strategy: Strategy):
    """Truncate descending singular values; returns (kept view, squared error).

    The reference resizes its numpy vector in place and returns the error
    (cython/truncation.pxi:329-334); a CUDA tensor cannot be resized in place,
    so the kept prefix is returned as a view together with the error.
    """
    torch = _torch()
    s = as_device(s, complex_=False)
    if s.ndim != 1:
        raise TypeError("destructively_truncate_vector requires a 1D float64 vector")
    rank = C.c_int()
    err = C.c_double()
    _lib.check(_lib.load().sm_truncate(_lib.context(), _lib.ptr(s), s.numel(),
                                       C.byref(strategy.to_c()), C.byref(rank), C.byref(err),
                                       _lib.stream_handle()))
    del torch
    return s[: rank.value], err.value


def _gemm(B, BT: int, A, AT: int):
    """op(B) @ op(A) (cython/gemm.pxi:21-122)."""
    torch = _torch()
    cplx = _common_complex([A, B])
    B = as_device(B, cplx)
    A = as_device(A, cplx)
    M, K = (B.shape if BT == 0 else (B.shape[1], B.shape[0]))
    K2, N = (A.shape if AT == 0 else (A.shape[1], A.shape[0]))
    if K != K2:
        raise ValueError("Invalid GEMM dimensions")
    out = torch.empty((M, N), dtype=A.dtype, device=A.device)
    _lib.check(_lib.load().sm_gemm(_lib.context(), dtype_code(A), BT, AT, M, N, K, _lib.ptr(B),
                                   B.shape[1], _lib.ptr(A), A.shape[1], _lib.ptr(out), N,
                                   _lib.stream_handle()))
    return out


def _contract_last_and_first(A, B):
    """Contract the last index of A with the first of B (cython/contractions.pxi:6-38)."""
    cplx = _common_complex([A, B])
    A = as_device(A, cplx)
    B = as_device(B, cplx)
    out = _gemm(A.reshape(-1, A.shape[-1]), 0, B.reshape(B.shape[0], -1), 0)
    return out.reshape(tuple(A.shape[:-1]) + tuple(B.shape[1:]))


def _destructive_svd(A):
    """Economy SVD (U, s, Vh) of a matrix (cython/svd.pxi:17-21)."""
    torch = _torch()
    A = as_device(A)
    if A.ndim != 2:
        raise ValueError("Invalid argument to SVD")
    m, n = A.shape
    r = min(m, n)
    U = torch.empty((m, r), dtype=A.dtype, device=A.device)
    V = torch.empty((r, n), dtype=A.dtype, device=A.device)
    s = torch.empty((r,), dtype=torch.float64, device=A.device)
    _lib.check(_lib.load().sm_svd(_lib.context(), dtype_code(A), _lib.ptr(A), m, n, _lib.ptr(U),
                                  _lib.ptr(s), _lib.ptr(V), _lib.stream_handle()))
    return U, s, V


def _split_2site(fn, AA, strategy: Strategy):
    torch = _torch()
    AA = as_device(AA)
    if AA.ndim != 4:
        raise ValueError("two-site split needs a 4-index tensor")
    a, d1, d2, b = AA.shape
    r = min(a * d1, d2 * b)
    L = torch.empty(a * d1 * r, dtype=AA.dtype, device=AA.device)
    R = torch.empty(r * d2 * b, dtype=AA.dtype, device=AA.device)
    D = C.c_int()
    err = C.c_double()
    _lib.check(fn(_lib.context(), dtype_code(AA), _lib.ptr(AA), a, d1, d2, b,
                  C.byref(strategy.to_c()), _lib.ptr(L), _lib.ptr(R), C.byref(D), C.byref(err),
                  _lib.stream_handle()))
    D = D.value
    return (L[: a * d1 * D].view(a, d1, D), R[: D * d2 * b].view(D, d2, b), err.value)


def _left_orth_2site(AA, strategy: Strategy):
    """(U[a,d1,D], (sV)[D,d2,b], sqrt(err)) (cython/schmidt.pxi:123-147)."""
    return _split_2site(_lib.load().sm_left_orth_2site, AA, strategy)


def _right_orth_2site(AA, strategy: Strategy):
    """((Us)[a,d1,D], V[D,d2,b], sqrt(err)) (cython/schmidt.pxi:150-174)."""
    return _split_2site(_lib.load().sm_right_orth_2site, AA, strategy)


def _begin_environment(D: int = 1):
    torch = _torch()
    return torch.eye(D, dtype=torch.float64, device="cuda")


def _env(fn, B, A, rho, out_shape):
    torch = _torch()
    cplx = _common_complex([A, B, rho])
    A, B, rho = as_device(A, cplx), as_device(B, cplx), as_device(rho, cplx)
    if A.ndim != 3 or B.ndim != 3 or rho.ndim != 2:
        raise ValueError("Invalid arguments to environment update")
    i, j, k = A.shape
    l, j2, n = B.shape
    if j != j2:
        raise ValueError("Invalid arguments to environment update")
    out = torch.empty(out_shape(i, j, k, l, n), dtype=A.dtype, device=A.device)
    _lib.check(fn(_lib.context(), dtype_code(A), _lib.ptr(B), l, j, n, _lib.ptr(A), i, k,
                  _lib.ptr(rho), _lib.ptr(out), _lib.stream_handle()))
    return out


def _update_left_environment(B, A, rho):
    """rho'[n,k] = sum conj(B[l,j,n]) rho[l,i] A[i,j,k] (cython/environments.pxi:10-37)."""
    return _env(_lib.load().sm_update_left_environment, B, A, rho,
                lambda i, j, k, l, n: (n, k))


def _update_right_environment(B, A, rho):
    """rho'[i,l] = sum A[i,j,k] rho[k,n] conj(B[l,j,n]) (cython/environments.pxi:39-67)."""
    return _env(_lib.load().sm_update_right_environment, B, A, rho,
                lambda i, j, k, l, n: (i, l))


def _end_environment(rho):
    return rho.reshape(-1)[0].item()


def _join_environments(rhoL, rhoR):
    if rhoL.shape[0] == 1:
        return _end_environment(rhoL) * _end_environment(rhoR)
    return (rhoL.reshape(-1) * rhoR.transpose(0, 1).reshape(-1)).sum().item()


def _canonical_buffers(state: list, cplx: bool):
    """Private device copies of a list of site tensors, flat, with their bonds."""
    bufs = [as_device(t, cplx).clone().reshape(-1) for t in state]
    phys = [int(t.shape[1]) for t in state]
    bonds = [int(state[0].shape[0])] + [int(t.shape[2]) for t in state]
    return bufs, phys, bonds


def _write_back(state: list, bufs, phys, bonds):
    for i in range(len(state)):
        n = bonds[i] * phys[i] * bonds[i + 1]
        state[i] = bufs[i][:n].view(bonds[i], phys[i], bonds[i + 1])


def _canonicalize(state: list, center: int, truncation: Strategy) -> float:
    """Bring a list of site tensors to canonical form about `center`, in place
    (cython/schmidt.pxi:109-120): right updates below the centre, left updates above it,
    each a truncated SVD.  The list's entries are replaced by device tensors; returns the
    summed sqrt(discarded weight)."""
    if not isinstance(state, list):
        raise TypeError("_canonicalize needs a list of tensors")
    L = len(state)
    if not 0 <= center < L:
        raise IndexError("center out of range")
    bufs, phys, bonds = _canonical_buffers(state, _common_complex(state))
    cb = _lib.int_array(bonds)
    err = C.c_double()
    _lib.check(_lib.load().sm_canonicalize(
        _lib.context(), dtype_code(bufs[0]), L, _lib.int_array(phys), cb, _lib.ptr_array(bufs),
        _lib.i64_array([b.numel() for b in bufs]), center, C.byref(truncation.to_c()),
        C.byref(err), _lib.stream_handle()))
    _write_back(state, bufs, phys, list(cb))
    return err.value


def _recanonicalize(state: list, oldcenter: int, newcenter: int, truncation: Strategy) -> float:
    """Move the orthogonality centre of a canonical list of site tensors from `oldcenter`
    to `newcenter` one site at a time, in place (cython/schmidt.pxi:96-106)."""
    if not isinstance(state, list):
        raise TypeError("_recanonicalize needs a list of tensors")
    L = len(state)
    if not (0 <= oldcenter < L and 0 <= newcenter < L):
        raise IndexError("center out of range")
    bufs, phys, bonds = _canonical_buffers(state, _common_complex(state))
    cb = _lib.int_array(bonds)
    err = C.c_double()
    _lib.check(_lib.load().sm_recanonicalize(
        _lib.context(), dtype_code(bufs[0]), L, _lib.int_array(phys), cb, _lib.ptr_array(bufs),
        _lib.i64_array([b.numel() for b in bufs]), oldcenter, newcenter,
        C.byref(truncation.to_c()), C.byref(err), _lib.stream_handle()))
    _write_back(state, bufs, phys, list(cb))
    return err.value


def _update_in_canonical_form_right(state: list, A, site: int, truncation: Strategy):
    """Insert A at `site` and move the centre one site right (cython/schmidt.pxi:18-56):
    A = U s V truncated, state[site] = U, state[site+1] = (s V) state[site+1].  Returns
    (new centre, sqrt(discarded weight)); at the last site A is stored as is."""
    torch = _torch()
    if site + 1 == len(state):
        state[site] = A
        return site, 0.0
    cplx = _common_complex([A, state[site + 1]])
    A = as_device(A, cplx)
    nxt = as_device(state[site + 1], cplx)
    a, i, b = A.shape
    b2, j, c = nxt.shape
    if b2 != b:
        raise ValueError("Invalid arguments to _update_in_canonical_form_right")
    r = min(a * i, b)
    U = torch.empty(a * i * r, dtype=A.dtype, device=A.device)
    out = torch.empty(r * j * c, dtype=A.dtype, device=A.device)
    D = C.c_int()
    err = C.c_double()
    _lib.check(_lib.load().sm_update_in_canonical_form_right(
        _lib.context(), dtype_code(A), _lib.ptr(A), a, i, b, _lib.ptr(nxt), j, c,
        C.byref(truncation.to_c()), _lib.ptr(U), _lib.ptr(out), C.byref(D), C.byref(err),
        _lib.stream_handle()))
    D = D.value
    state[site] = U[: a * i * D].view(a, i, D)
    state[site + 1] = out[: D * j * c].view(D, j, c)
    return site + 1, err.value


def _update_in_canonical_form_left(state: list, A, site: int, truncation: Strategy):
    """Insert A at `site` and move the centre one site left (cython/schmidt.pxi:59-93):
    A = U s V truncated, state[site] = V, state[site-1] = state[site-1] (U s).  Returns
    (new centre, sqrt(discarded weight)); at site 0 A is stored as is."""
    torch = _torch()
    if site == 0:
        state[0] = A
        return 0, 0.0
    cplx = _common_complex([A, state[site - 1]])
    A = as_device(A, cplx)
    prv = as_device(state[site - 1], cplx)
    a, i, b = A.shape
    p, j, a2 = prv.shape
    if a2 != a:
        raise ValueError("Invalid arguments to _update_in_canonical_form_left")
    r = min(a, i * b)
    V = torch.empty(r * i * b, dtype=A.dtype, device=A.device)
    out = torch.empty(p * j * r, dtype=A.dtype, device=A.device)
    D = C.c_int()
    err = C.c_double()
    _lib.check(_lib.load().sm_update_in_canonical_form_left(
        _lib.context(), dtype_code(A), _lib.ptr(A), a, i, b, _lib.ptr(prv), p, j,
        C.byref(truncation.to_c()), _lib.ptr(V), _lib.ptr(out), C.byref(D), C.byref(err),
        _lib.stream_handle()))
    D = D.value
    state[site] = V[: D * i * b].view(D, i, b)
    state[site - 1] = out[: p * j * D].view(p, j, D)
    return site - 1, err.value


def _contract_nrjl_ijk_klm(U, A, B):
    """np.einsum('ijk,klm,nrjl -> inrm', A, B, U) with U (n*r x j*l)
    (cython/contractions.pxi:102-127); the result has A's and B's physical shapes."""
    torch = _torch()
    cplx = _common_complex([U, A, B])
    U, A, B = as_device(U, cplx), as_device(A, cplx), as_device(B, cplx)
    if A.ndim != 3 or B.ndim != 3 or U.ndim != 2:
        raise ValueError("Invalid arguments to _contract_nrjl_ijk_klm")
    a, d, b = A.shape
    b2, e, c = B.shape
    if b2 != b or U.shape != (d * e, d * e):
        raise ValueError("Invalid arguments to _contract_nrjl_ijk_klm")
    out = torch.empty((a, d, e, c), dtype=A.dtype, device=A.device)
    _lib.check(_lib.load().sm_contract_nrjl_ijk_klm(
        _lib.context(), dtype_code(A), _lib.ptr(U), d * e, _lib.ptr(A), a, d, b, _lib.ptr(B), e, c,
        _lib.ptr(out), _lib.stream_handle()))
    return out


def _select_svd_driver(name: str) -> None:
    """Select the reference's LAPACK SVD driver by name (cython/svd.pxi:25-32): "gesdd" or
    "gesvd", else ValueError.  The device SVD is one algorithm whose kept ranks and singular
    values agree with either driver's, so the choice is recorded and changes no result."""
    if _lib.load().sm_select_svd_driver(str(name).encode()) != _lib.SM_OK:
        raise ValueError(f"Invalid LAPACK SVD driver name: {name}")


def _tensor2site(L, A, B, R):
    """LA = L A, BR = B R, AA = LA BR: the two-site tensor [l, d1, d2, r] of an
    AntilinearForm (state/antilinear.py:68-98), one library call."""
    torch = _torch()
    cplx = _common_complex([L, A, B, R])
    L, A, B, R = (as_device(x, cplx) for x in (L, A, B, R))
    l, i = L.shape
    i2, d1, k = A.shape
    k2, d2, n = B.shape
    n2, r = R.shape
    if i2 != i or k2 != k or n2 != n:
        raise ValueError("Invalid arguments to tensor2site")
    out = torch.empty((l, d1, d2, r), dtype=A.dtype, device=A.device)
    _lib.check(_lib.load().sm_tensor2site(
        _lib.context(), dtype_code(A), _lib.ptr(L), l, i, _lib.ptr(A), d1, k, _lib.ptr(B), d2, n,
        _lib.ptr(R), r, _lib.ptr(out), _lib.stream_handle()))
    return out


def _mpo_multiply_tensor(O, B):
    """C[c*a, i, d*b] = sum_j B[c,j,d] O[a,i,j,b] (operators/mpo.py:26-45)."""
    torch = _torch()
    cplx = _common_complex([O, B])
    O, B = as_device(O, cplx), as_device(B, cplx)
    a, i, j, b = O.shape
    c, j2, d = B.shape
    if j != j2:
        raise ValueError("MPO and MPS physical dimensions differ")
    out = torch.empty((c * a, i, d * b), dtype=O.dtype, device=O.device)
    _lib.check(_lib.load().sm_mpo_multiply_tensor(_lib.context(), dtype_code(O), _lib.ptr(O), a, i,
                                                  j, b, _lib.ptr(B), c, d, _lib.ptr(out),
                                                  _lib.stream_handle()))
    return out
