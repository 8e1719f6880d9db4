"""MPO and MPOList with ``apply`` / ``@`` on the GPU (operators/mpo.py:48-753)."""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .core import (DEFAULT_STRATEGY, NO_TRUNCATION, Simplification, Strategy,
                   _mpo_multiply_tensor, as_device, dtype_code)
from .state import SIMPLIFICATION_STRATEGY, MPS, MPSSum, TensorArray, _simplify_terms, simplify


class MPO(TensorArray):
    """Matrix product operator ``O[a, i, j, b]`` (operators/mpo.py:48-75)."""

    __array_priority__ = 10000

    def __init__(self, data, strategy: Strategy = DEFAULT_STRATEGY):
        data = list(data)
        cplx = any((t.is_complex() if hasattr(t, "is_complex") else np.iscomplexobj(t)) for t in data)
        super().__init__([as_device(t, cplx) for t in data])
        self.strategy = strategy

    def copy(self) -> "MPO":
        return MPO(self._data, self.strategy)

    def physical_dimensions(self) -> list[int]:
        return [int(A.shape[2]) for A in self._data]

    def bond_dimensions(self) -> list[int]:
        return [int(A.shape[-1]) for A in self._data][:-1]

    def max_bond_dimension(self) -> int:
        return max(int(A.shape[0]) for A in self._data)

    @property
    def T(self) -> "MPO":
        return MPO([A.permute(0, 2, 1, 3).contiguous() for A in self._data], self.strategy)

    def conj(self) -> "MPO":
        return MPO([A.conj().resolve_conj() for A in self._data], self.strategy)

    def set_strategy(self, strategy: Strategy) -> "MPO":
        return MPO(self._data, strategy)

    def __mul__(self, n):
        if isinstance(n, (int, float, complex)):
            absn = abs(n)
            if absn:
                phase = n / absn
                factor = np.exp(np.log(absn) / self.size)
            else:
                phase, factor = 0.0, 0.0
            return MPO([(factor if i > 0 else factor * phase) * A for i, A in enumerate(self._data)],
                       self.strategy)
        raise TypeError(f"Cannot multiply MPO by {type(n)}")

    __rmul__ = __mul__

    def to_matrix(self):
        """Dense matrix (small systems only)."""
        import torch

        out = torch.ones((1, 1, 1), dtype=self._data[0].dtype, device=self._data[0].device)
        Di = Dj = 1
        for A in self._data:
            _, i, j, b = A.shape
            Di *= i
            Dj *= j
            out = torch.tensordot(out, A, dims=1).permute(0, 2, 1, 3, 4).reshape(Di, Dj, b)
        return out[:, :, 0]

    def apply(self, state, strategy: Strategy | None = None, simplify: bool | None = None):
        """``self @ state`` followed by ``simplify`` when the strategy asks for it
        (operators/mpo.py:229-281)."""
        if strategy is None:
            strategy = self.strategy
        if strategy is None:
            raise RuntimeError("MPO has no truncation strategy")
        if simplify is None:
            simplify = strategy.get_simplify_flag()
        if isinstance(state, MPSSum):
            if self.size != state.size:
                raise ValueError("MPO and state must have the same size")
            out = None
            factors = list(zip(state.weights, state.states))
            for i, (w, mps) in enumerate(factors):
                Ostate = w * MPS([_mpo_multiply_tensor(A, B) for A, B in zip(self._data, mps._data)],
                                 error=mps.error())
                out = Ostate if i == 0 else out + Ostate
            state = out
        elif isinstance(state, MPS):
            if self.size != state.size:
                raise ValueError("MPO and state must have the same size")
            factors = [(1.0, state)]
            state = MPS([_mpo_multiply_tensor(A, B) for A, B in zip(self._data, state._data)],
                        error=state.error())
        else:
            raise TypeError(f"Cannot multiply MPO with {state}")
        if simplify:
            # the products' norms and overlaps come from the factors
            # (sm_mpo_scprod) instead of the bond-(chi D) product states
            terms = state.states if isinstance(state, MPSSum) else [state]
            weights = state.weights if isinstance(state, MPSSum) else [1.0]
            gram = _product_gram(self._data, factors) if len(terms) == len(factors) else None
            state = _simplify_terms(weights, terms, strategy, +1, gram=gram)
        return state

    def __matmul__(self, b):
        if isinstance(b, (MPS, MPSSum)):
            return self.apply(b)
        if isinstance(b, MPO):
            return MPOList([b, self])
        if isinstance(b, MPOList):
            return MPOList(b.mpos + [self], b.strategy)
        raise TypeError(f"Cannot multiply MPO with {b}")

    def __rmatmul__(self, b):
        if isinstance(b, (MPS, MPSSum)):
            return self.T.apply(b)
        raise TypeError(f"Cannot multiply {b} with MPO")


_simplify = simplify


def mpo_scprod(mpo: MPO, bra: MPS, ket: MPS):
    """<O bra|O ket> from the factors, without forming the products
    (the scprod of cython/environments.pxi:87-118 applied to O|bra>, O|ket>)."""
    return _mpo_scprod(mpo._data, bra, ket)


def _mpo_scprod(data, bra: MPS, ket: MPS):
    if not (len(data) == bra.size == ket.size):
        raise ValueError("Invalid arguments to mpo_scprod")
    cplx = (bra.is_complex() or ket.is_complex() or
            any((t.is_complex() if hasattr(t, "is_complex") else np.iscomplexobj(t)) for t in data))
    O = [as_device(t, cplx) for t in data]
    A = [as_device(t, cplx) for t in bra._data]
    B = [as_device(t, cplx) for t in ket._data]
    out = (C.c_double * 2)()
    _lib.check(_lib.load().sm_mpo_scprod(
        _lib.context(), _lib.SM_COMPLEX128 if cplx else _lib.SM_FLOAT64, len(O),
        _lib.int_array([t.shape[1] for t in O]), _lib.int_array([t.shape[2] for t in O]),
        _lib.int_array([O[0].shape[0]] + [t.shape[3] for t in O]), _lib.ptr_array(O),
        _lib.int_array(bra.bond_dimensions()), _lib.ptr_array(A),
        _lib.int_array(ket.bond_dimensions()), _lib.ptr_array(B), out, _lib.stream_handle()))
    return complex(out[0], out[1]) if cplx else out[0]


def _product_gram(data, factors):
    """<w_i O s_i|w_j O s_j> for the terms (w_i, s_i) of an MPO apply, as the
    nterms x nterms complex array sm_simplify_gram takes."""
    n = len(factors)
    G = np.zeros((n, n), dtype=complex)
    for i in range(n):
        for j in range(i, n):
            wi, si = factors[i]
            wj, sj = factors[j]
            v = np.conj(complex(wi)) * complex(wj)
            if v != 0:
                v *= complex(_mpo_scprod(data, si, sj))
            G[i, j] = v
            G[j, i] = np.conj(v)
    return G


class MPOList:
    """Sequence of MPOs applied right-to-left order of the list (operators/mpo.py:430-621)."""

    def __init__(self, mpos, strategy: Strategy = DEFAULT_STRATEGY):
        self.mpos = list(mpos)
        self.size = self.mpos[0].size
        self.strategy = strategy

    def copy(self) -> "MPOList":
        return MPOList(self.mpos, self.strategy)

    def apply(self, state, strategy: Strategy | None = None, simplify: bool | None = None):
        """Each MPO applied with its own strategy, then one final simplify (:585-621)."""
        if strategy is None:
            strategy = self.strategy
        if simplify is None:
            simplify = strategy.get_simplify_flag()
        for mpo in self.mpos:
            state = mpo.apply(state)
        if simplify:
            state = _simplify(state, strategy=strategy)
        return state

    def __matmul__(self, b):
        if isinstance(b, (MPS, MPSSum)):
            return self.apply(b)
        if isinstance(b, MPO):
            return MPOList([b] + self.mpos, self.strategy)
        if isinstance(b, MPOList):
            return MPOList(b.mpos + self.mpos, self.strategy)
        raise TypeError(f"Cannot multiply MPOList with {b}")

    def join(self, strategy: Strategy | None = None) -> MPO:
        """One MPO for the product of the list (operators/mpo.py:679-711): at each site the
        tensors are joined pairwise from the last MPO backwards, C[(a c), i, k, (b d)] =
        sum_j B[a, i, j, b] A[c, j, k, d] with A applied before B (sm_mpo_join)."""
        import torch

        cplx = any(m[0].is_complex() for m in self.mpos)

        def join2(A, B):  # A applied first, then B
            A = as_device(A, cplx)
            B = as_device(B, cplx)
            a, i, j, b = B.shape
            c, j2, k, d = A.shape
            if j2 != j:
                raise ValueError("MPOList.join: physical dimensions differ")
            out = torch.empty((a * c, i, k, b * d), dtype=A.dtype, device=A.device)
            _lib.check(_lib.load().sm_mpo_join(_lib.context(), dtype_code(A), _lib.ptr(B), a, i, j,
                                               b, _lib.ptr(A), c, k, d, _lib.ptr(out),
                                               _lib.stream_handle()))
            return out

        tensors = []
        for s in range(self.size):
            ts = [m[s] for m in self.mpos]
            acc = ts[-1]
            for A in reversed(ts[:-1]):
                acc = join2(A, acc)
            tensors.append(acc)
        return MPO(tensors, self.strategy if strategy is None else strategy)


#: MPO simplification does not normalise by default (operators/simplify_mpo.py:18-19)
MPO_SIMPLIFICATION_STRATEGY = SIMPLIFICATION_STRATEGY.replace(normalize=False)
#: canonical forms without truncation (operators/simplify_mpo.py:15-16)
CANONICALIZE_MPO = NO_TRUNCATION.replace(simplify=Simplification.DO_NOT_SIMPLIFY)


def mpo_as_mps(mpo: MPO) -> MPS:
    """The MPO's sites O[a, i, j, b] as MPS sites [a, (i j), b] (operators/simplify_mpo.py:22-29)."""
    return MPS([A.reshape(A.shape[0], A.shape[1] * A.shape[2], A.shape[3]) for A in mpo._data])


def mps_as_mpo(mps: MPS, mpo_strategy: Strategy = DEFAULT_STRATEGY) -> MPO:
    """MPS sites [a, p, b] with p a perfect square as MPO sites [a, s, s, b]
    (operators/simplify_mpo.py:32-47)."""
    from math import isqrt

    data = []
    for A in mps._data:
        bl, p, br = A.shape
        s = isqrt(p)
        if s * s != p:
            raise ValueError("The physical dimensions of the MPS must be a perfect square")
        data.append(A.reshape(bl, s, s, br))
    return MPO(data, strategy=mpo_strategy)


def simplify_mpo(operator, strategy: Strategy = MPO_SIMPLIFICATION_STRATEGY, direction: int = +1,
                 guess: MPO | None = None, mpo_strategy: Strategy | None = None) -> MPO:
    """Approximate an MPO (or the product of an MPOList) by one of smaller bond dimension
    (operators/simplify_mpo.py:50-89): the operator is recast as an MPS of physical
    dimension i*j, simplified variationally on the device (with the guess, if any, as the
    starting state) and recast as an MPO."""
    if isinstance(operator, MPOList):
        operator = operator.join()
    if not isinstance(operator, MPO):
        raise TypeError(f"Cannot simplify {type(operator)} as an MPO")
    if mpo_strategy is None:
        mpo_strategy = operator.strategy
    mps = mpo_as_mps(operator)
    guess_mps = None if guess is None else mpo_as_mps(guess)
    out = simplify(mps, strategy, direction, guess_mps)
    return mps_as_mpo(out, mpo_strategy=mpo_strategy)
