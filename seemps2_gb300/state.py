"""MPS, CanonicalMPS, MPSSum and simplify on device-resident tensors.

Same classes, methods and semantics as the reference (state/mps.py,
state/canonical_mps.py, state/mpssum.py, state/simplification.py), with site
tensors held as CUDA tensors (torch.float64 / torch.complex128, C order
``A[a, i, b]``).  All numerical work runs in libseemps_gb300.so: the whole
variational sweep of ``simplify`` is one C call (sm_simplify).
"""

from __future__ import annotations

import ctypes as C
import math
import warnings
from collections.abc import Iterable, Sequence

import numpy as np

from . import _lib
from .core import (
    DEFAULT_STRATEGY,
    DEFAULT_TOLERANCE,
    MAX_BOND_DIMENSION,
    Simplification,
    Strategy,
    Truncation,
    _update_left_environment,
    _update_right_environment,
    as_device,
    dtype_code,
)


def _torch():
    import torch

    return torch


class InvalidOperation(TypeError):
    def __init__(self, op, *args):
        super().__init__(f"Invalid operation {op} between arguments of types {[type(x) for x in args]}")


def _promote(tensors: list) -> list:
    cplx = any((t.is_complex() if hasattr(t, "is_complex") else np.iscomplexobj(t)) for t in tensors)
    return [as_device(t, cplx) for t in tensors]


class TensorArray(Sequence):
    """A list of site tensors that is copied (not its tensors) on clone (state/array.py:9-31)."""

    def __init__(self, data: Iterable):
        self._data = list(data)
        self.size = len(self._data)

    def __getitem__(self, k):
        return self._data[k]

    def __setitem__(self, k, value):
        if isinstance(k, slice):
            self._data[k] = list(value)
        else:
            self._data[k] = value
        return value

    def __iter__(self):
        return iter(self._data)

    def __reversed__(self):
        return reversed(self._data)

    def __len__(self):
        return self.size


class MPS(TensorArray):
    """Matrix product state with open boundaries (state/mps.py:23-60)."""

    __array_priority__ = 10000

    def __init__(self, data: Iterable, error: float = 0.0):
        super().__init__(_promote(list(data)))
        self._error = float(error)

    # --- structure ---------------------------------------------------------
    def copy(self) -> "MPS":
        return MPS(self._data, self._error)

    def as_mps(self) -> "MPS":
        return self

    @property
    def dtype(self):
        return self._data[0].dtype

    def is_complex(self) -> bool:
        return self._data[0].is_complex()

    def dimension(self) -> int:
        return math.prod(self.physical_dimensions())

    def physical_dimensions(self) -> list[int]:
        return [int(a.shape[1]) for a in self._data]

    def bond_dimensions(self) -> list[int]:
        return [int(a.shape[0]) for a in self._data] + [int(self._data[-1].shape[-1])]

    def max_bond_dimension(self) -> int:
        return max(int(a.shape[-1]) for a in self._data)

    def error(self) -> float:
        return self._error

    def update_error(self, delta: float) -> None:
        self._error += delta

    def to_numpy(self) -> list:
        return [a.detach().cpu().numpy() for a in self._data]

    def to_vector(self):
        """Dense wavefunction (small systems only; state/mps.py:457-472)."""
        torch = _torch()
        psi = torch.ones(1, dtype=self.dtype, device=self._data[0].device)
        for A in reversed(self._data):
            a, d, b = A.shape
            psi = (A.reshape(a * d, b) @ psi.reshape(b, -1)).reshape(a, -1)
        return psi.reshape(-1)

    def zero_state(self) -> "MPS":
        torch = _torch()
        return MPS([torch.zeros((1, int(A.shape[1]), 1), dtype=self.dtype, device=A.device)
                    for A in self._data])

    def conj(self) -> "MPS":
        return MPS([A.conj().resolve_conj() for A in self._data], self._error)

    def reverse(self) -> "MPS":
        """Sites in reverse order, each A[a, i, b] read as A[b, i, a] (state/mps.py:471-485;
        like the reference, the result carries no error bound)."""
        return MPS([A.permute(2, 1, 0).contiguous() for A in reversed(self._data)])

    def to_tensor(self):
        """The wavefunction as a tensor with one index per site (state/mps.py:103-106)."""
        return self.to_vector().reshape(self.physical_dimensions())

    def __copy__(self):
        return self.copy()

    # --- scalars -----------------------------------------------------------
    def norm2(self) -> float:
        """Deprecated alias of `norm_squared` (state/mps.py:233-238)."""
        warnings.warn("method norm2 is deprecated, use norm_squared", category=DeprecationWarning)
        return self.norm_squared()

    def norm_squared(self) -> float:
        return abs(scprod(self, self).real)

    def norm(self) -> float:
        return math.sqrt(abs(scprod(self, self)))

    # --- arithmetic (state/mps.py:150-230) -----------------------------------
    def __add__(self, state):
        if isinstance(state, MPS):
            return MPSSum([1.0, 1.0], [self, state], check_args=False)
        if isinstance(state, MPSSum):
            return MPSSum([1.0] + state.weights, [self] + state.states, check_args=False)
        raise InvalidOperation("+", self, state)

    def __sub__(self, state):
        if isinstance(state, MPS):
            return MPSSum([1, -1], [self, state], check_args=False)
        if isinstance(state, MPSSum):
            return MPSSum([1] + [-w for w in state.weights], [self] + state.states, check_args=False)
        raise InvalidOperation("-", self, state)

    def __mul__(self, n):
        if isinstance(n, (int, float, complex)):
            if n:
                out = self.copy()
                first = out._data[0]
                if isinstance(n, complex) and not first.is_complex():
                    out._data = [as_device(t, True) for t in out._data]
                    first = out._data[0]
                out._data[0] = n * first
                out._error *= abs(n)
                return out
            return self.zero_state()
        raise InvalidOperation("*", self, n)

    def __rmul__(self, n):
        if isinstance(n, (int, float, complex)):
            return self.__mul__(n)
        raise InvalidOperation("*", n, self)

    def __truediv__(self, n):
        if isinstance(n, (int, float, complex)):
            return self.__mul__(1.0 / n)
        raise InvalidOperation("/", self, n)

    def left_environment(self, site: int):
        torch = _torch()
        rho = torch.eye(1, dtype=self.dtype, device=self._data[0].device)
        for A in self._data[:site]:
            rho = _update_left_environment(A, A, rho)
        return rho

    def right_environment(self, site: int):
        torch = _torch()
        rho = torch.eye(1, dtype=self.dtype, device=self._data[0].device)
        for A in self._data[-1:site:-1]:
            rho = _update_right_environment(A, A, rho)
        return rho


def _site_arrays(states: Sequence[MPS]):
    L = states[0].size
    phys = states[0].physical_dimensions()
    bonds, ptrs = [], []
    for s in states:
        if s.size != L:
            raise ValueError("all states must have the same size")
        bonds.extend(s.bond_dimensions())
        ptrs.extend(s._data)
    return L, phys, bonds, ptrs


def scprod(bra: MPS, ket: MPS):
    """<bra|ket> (cython/environments.pxi:87-118), computed on the device."""
    if bra.size != ket.size:
        raise ValueError("Invalid arguments to scprod")
    cplx = bra.is_complex() or ket.is_complex()
    A = [as_device(t, cplx) for t in bra._data]
    B = [as_device(t, cplx) for t in ket._data]
    out = (C.c_double * 2)()
    _lib.check(_lib.load().sm_scprod(
        _lib.context(), _lib.SM_COMPLEX128 if cplx else _lib.SM_FLOAT64, bra.size,
        _lib.int_array(bra.physical_dimensions()), _lib.int_array(bra.bond_dimensions()),
        _lib.ptr_array(A), _lib.int_array(ket.bond_dimensions()), _lib.ptr_array(B), out,
        _lib.stream_handle()))
    return complex(out[0], out[1]) if cplx else out[0]


vdot = scprod


class AntilinearForm:
    """<bra|ket> with the environments kept left and right of `center`
    (state/antilinear.py:13-146): tensor1site / tensor2site give the tensors whose
    contraction with the bra's site(s) is the form; update_right / update_left move the
    centre after the bra changed.  Every contraction is a library call."""

    def __init__(self, bra: MPS, ket: MPS, center: int = 0):
        from .core import _begin_environment, _update_left_environment, _update_right_environment

        if bra.size != ket.size:
            raise ValueError("bra and ket must have the same size")
        size = bra.size
        rho = _begin_environment()
        R = [rho] * size
        for i in range(size - 1, center, -1):
            R[i - 1] = rho = _update_right_environment(bra[i], ket[i], rho)
        rho = _begin_environment()
        Lv = [rho] * size
        for i in range(0, center):
            Lv[i + 1] = rho = _update_left_environment(bra[i], ket[i], rho)
        self.bra, self.ket, self.size = bra, ket, size
        self.R, self.L, self.center = R, Lv, center

    def tensor1site(self):
        """L[c] ket[c] R[c] (antilinear.py:59-66)."""
        from .core import _contract_last_and_first

        c = self.center
        return _contract_last_and_first(self.L[c], _contract_last_and_first(self.ket[c], self.R[c]))

    def tensor2site(self, direction: int):
        """The two-site tensor on (center, center+1) if direction > 0, else on
        (center-1, center) (antilinear.py:68-98)."""
        from .core import _tensor2site

        if direction > 0:
            i = self.center
            j = i + 1
        else:
            j = self.center
            i = j - 1
        return _tensor2site(self.L[i], self.ket[i], self.ket[j], self.R[j])

    def update(self, direction: int) -> None:
        if direction > 0:
            self.update_right()
        else:
            self.update_left()

    def update_right(self) -> None:
        from .core import _update_left_environment

        prev = self.center
        nxt = prev + 1
        if nxt >= self.size:
            raise RuntimeError("Cannot move the center beyond the last site")
        self.L[nxt] = _update_left_environment(self.bra[prev], self.ket[prev], self.L[prev])
        self.center = nxt

    def update_left(self) -> None:
        from .core import _update_right_environment

        prev = self.center
        nxt = prev - 1
        if nxt < 0:
            raise RuntimeError("Cannot move the center before the first site")
        self.R[nxt] = _update_right_environment(self.bra[prev], self.ket[prev], self.R[prev])
        self.center = nxt


class CanonicalMPS(MPS):
    """MPS in canonical form with respect to `center` (state/canonical_mps.py:38-108)."""

    def __init__(self, data: Iterable, center: int | None = None, normalize: bool | None = None,
                 strategy: Strategy = DEFAULT_STRATEGY, is_canonical: bool = False,
                 error: float = 0.0):
        super().__init__(data, error)
        self.strategy = strategy
        if isinstance(data, CanonicalMPS):
            self._center = data.center
            self._error = data._error
            if center is not None:
                self.recenter(center)
            actual = self._center
        else:
            self._center = actual = self._interpret_center(0 if center is None else center)
            if not is_canonical:
                self._error += self._canonicalize(actual, strategy)
        if normalize is True or (normalize is None and strategy.get_normalize_flag()):
            self.normalize_inplace()

    @property
    def center(self) -> int:
        return self._center

    def _interpret_center(self, center: int) -> int:
        if 0 <= center < self.size:
            return center
        center += self.size
        if 0 <= center < self.size:
            return center
        raise IndexError()

    def _canonicalize(self, center: int, strategy: Strategy) -> float:
        # private copies (the caller's tensors are never modified), shrunk in place
        bufs = [t.clone().reshape(-1) for t in self._data]
        bonds = _lib.int_array(self.bond_dimensions())
        err = C.c_double()
        _lib.check(_lib.load().sm_canonicalize(
            _lib.context(), dtype_code(bufs[0]), self.size,
            _lib.int_array(self.physical_dimensions()), bonds, _lib.ptr_array(bufs),
            _lib.i64_array([b.numel() for b in bufs]), center, C.byref(strategy.to_c()),
            C.byref(err), _lib.stream_handle()))
        d = self.physical_dimensions()
        self._data = [bufs[i][: bonds[i] * d[i] * bonds[i + 1]].view(bonds[i], d[i], bonds[i + 1])
                      for i in range(self.size)]
        return err.value

    def norm_squared(self) -> float:
        A = self._data[self._center]
        return float((A.conj() * A).real.sum().item())

    def normalize_inplace(self) -> "CanonicalMPS":
        A = self._data[self._center]
        N = float(A.abs().pow(2).sum().sqrt().item())
        if N:
            self._data[self._center] = A / N
        return self

    def recenter(self, center: int, strategy: Strategy | None = None) -> "CanonicalMPS":
        """Move the orthogonality centre (cython/schmidt.pxi:96-106).

        The reference walks the centre one site at a time with SVD updates.
        On the segment between the old and the new centre that walk is exactly
        ``_canonicalize(segment, new centre)``: right updates from the old
        centre up to the new one, or left updates down to it.
        """
        newc = self._interpret_center(center)
        oldc = self._center
        if newc != oldc:
            st = self.strategy if strategy is None else strategy
            lo, hi = min(oldc, newc), max(oldc, newc)
            seg = CanonicalMPS.__new__(CanonicalMPS)
            MPS.__init__(seg, self._data[lo:hi + 1], 0.0)
            err = seg._canonicalize(newc - lo, st)
            self._data[lo:hi + 1] = seg._data
            self._error += err
            self._center = newc
        return self

    def update_2site_right(self, AA, site: int, strategy: Strategy) -> None:
        from .core import _left_orth_2site

        self._data[site], self._data[site + 1], err = _left_orth_2site(AA, strategy)
        self._center = site + 1
        self._error += err

    def update_2site_left(self, AA, site: int, strategy: Strategy) -> None:
        from .core import _right_orth_2site

        self._data[site], self._data[site + 1], err = _right_orth_2site(AA, strategy)
        self._center = site
        self._error += err

    def zero_state(self) -> "CanonicalMPS":
        return CanonicalMPS(MPS.zero_state(self)._data, center=0, is_canonical=True)

    def copy(self):
        return CanonicalMPS(self, center=self._center, strategy=self.strategy, error=self._error)

    __copy__ = copy


class MPSSum:
    """Weighted sum of MPS (state/mpssum.py:11-262)."""

    __array_priority__ = 10000

    def __init__(self, weights, states, check_args: bool = True):
        if check_args:
            self.weights, self.states = [], []
            for w, s in zip(weights, states):
                if isinstance(s, MPS):
                    self.weights.append(w)
                    self.states.append(s)
                elif isinstance(s, MPSSum):
                    self.weights.extend(w * wi for wi in s.weights)
                    self.states.extend(s.states)
                else:
                    raise ValueError(s)
        else:
            self.weights = list(weights)
            self.states = list(states)
        self.size = self.states[0].size

    def copy(self) -> "MPSSum":
        return MPSSum(self.weights.copy(), self.states.copy())

    def physical_dimensions(self):
        return self.states[0].physical_dimensions()

    def is_complex(self) -> bool:
        return any(isinstance(w, complex) for w in self.weights) or any(s.is_complex() for s in self.states)

    def __add__(self, state):
        if isinstance(state, MPS):
            return MPSSum(self.weights + [1.0], self.states + [state], check_args=False)
        if isinstance(state, MPSSum):
            return MPSSum(self.weights + state.weights, self.states + state.states, check_args=False)
        raise InvalidOperation("+", self, state)

    def __sub__(self, state):
        if isinstance(state, MPS):
            return MPSSum(self.weights + [-1], self.states + [state], check_args=False)
        if isinstance(state, MPSSum):
            return MPSSum(self.weights + [-w for w in state.weights], self.states + state.states,
                          check_args=False)
        raise InvalidOperation("-", self, state)

    def __mul__(self, n):
        if isinstance(n, (int, float, complex)):
            return MPSSum([n * w for w in self.weights], self.states, check_args=False)
        raise InvalidOperation("*", self, n)

    __rmul__ = __mul__

    def __truediv__(self, n):
        return self.__mul__(1.0 / n)

    def error(self) -> float:
        return sum(abs(w) * s._error for w, s in zip(self.weights, self.states))

    def norm_squared(self) -> float:
        w, s = self.weights, self.states
        L = len(w)
        total = 0.0
        for i in range(L):
            for j in range(i, L):
                v = np.conj(w[i]) * w[j] * scprod(s[i], s[j])
                total += (v.real if isinstance(v, complex) else v) * (1 if i == j else 2)
        return abs(total)

    def norm(self) -> float:
        return math.sqrt(self.norm_squared())

    def to_vector(self):
        return sum(w * s.to_vector() for w, s in zip(self.weights, self.states))

    def to_tensor(self):
        return self.to_vector().reshape(self.physical_dimensions())

    def __copy__(self):
        return self.copy()

    def conj(self) -> "MPSSum":
        """Complex conjugate: conjugated weights and states (state/mpssum.py:173-177)."""
        return MPSSum([w.conjugate() for w in self.weights], [s.conj() for s in self.states],
                      check_args=False)

    def reverse(self) -> "MPSSum":
        """Every state with its sites reversed (state/mpssum.py:247-252)."""
        return MPSSum(self.weights, [s.reverse() for s in self.states], check_args=False)

    def delete_zero_components(self) -> float:
        """Drop the terms whose weighted norm is zero and return the norm squared of
        the sum over the rest (state/mpssum.py:204-228): terms are taken in order, each
        kept term adds |w_i|^2 <s_i|s_i> and 2 Re(conj(w_i) w_j <s_i|s_j>) against the
        terms kept before it; with no term left the sum becomes 0 * zero_state.  The
        overlaps run on the device (the scprod kernel)."""
        c = 0.0
        weights: list = []
        states: list = []
        for wi, si in zip(self.weights, self.states):
            wic = wi.conjugate()
            ni = (wic * wi).real * si.norm_squared()
            if ni:
                for wj, sj in zip(weights, states):
                    c += 2 * (wic * wj * scprod(si, sj)).real
                weights.append(wi)
                states.append(si)
                c += ni
        if len(weights) < len(self.states):
            if not weights:
                self.weights = [0.0]
                self.states = [self.states[0].zero_state()]
                return 0.0
            self.weights, self.states = weights, states
        return abs(float(c))

    def join_canonical(self, *args, **kwargs) -> "CanonicalMPS":
        """`join` followed by the canonical form (state/mpssum.py:169-171)."""
        return CanonicalMPS(self.join(), *args, **kwargs)

    def join(self) -> MPS:
        """Block-diagonal join (state/mpssum.py:130-167)."""
        torch = _torch()
        cplx = self.is_complex()
        L = self.size
        out = []
        for i in range(L):
            As = [as_device(s[i], cplx) for s in self.states]
            if i == 0:
                out.append(torch.cat([w * A for w, A in zip(self.weights, As)], dim=2))
            elif i == L - 1:
                out.append(torch.cat(As, dim=0))
            else:
                DL = sum(A.shape[0] for A in As)
                DR = sum(A.shape[2] for A in As)
                B = torch.zeros((DL, As[0].shape[1], DR), dtype=As[0].dtype, device=As[0].device)
                l = r = 0
                for A in As:
                    a, _, b = A.shape
                    B[l:l + a, :, r:r + b] = A
                    l += a
                    r += b
                out.append(B)
        return MPS(out)

    def as_mps(self) -> MPS:
        return self.join()


# ---------------------------------------------------------------------------
# simplify (state/simplification.py:22-296)
# ---------------------------------------------------------------------------

SIMPLIFICATION_STRATEGY = Strategy(method=Truncation.RELATIVE_NORM_SQUARED_ERROR,
                                   tolerance=DEFAULT_TOLERANCE,
                                   max_bond_dimension=MAX_BOND_DIMENSION, normalize=True,
                                   max_sweeps=4, simplify=Simplification.VARIATIONAL)

# Report of the last simplify call on this thread (sweeps, err estimates, ...)
last_report: dict = {}


def _simplify_terms(weights, states, strategy: Strategy, direction: int,
                    gram=None, guess: MPS | None = None) -> CanonicalMPS:
    """simplify of sum_t w_t |s_t>; `gram` (optional, nterms x nterms complex,
    <s_i|s_j>) replaces the terms' scprods in the state norm; `guess` (optional) is the
    sweeps' starting state instead of the joined terms."""
    torch = _torch()
    cplx = any(isinstance(w, complex) and w.imag != 0 for w in weights) or any(s.is_complex() for s in states)
    if guess is not None:
        if guess.size != states[0].size or guess.physical_dimensions() != states[0].physical_dimensions():
            raise ValueError("simplify: the guess does not match the state's sites")
        cplx = cplx or guess.is_complex()
    states = [s if (s.is_complex() == cplx) else MPS(s._data, s._error) for s in states]
    kets = [[as_device(t, cplx) for t in s._data] for s in states]
    L, phys, bonds, _ = _site_arrays(states)
    nterms = len(states)
    st_c = strategy.to_c()
    caps = (C.c_int * (L + 1))()
    _lib.check(_lib.load().sm_simplify_bond_caps(L, _lib.int_array(phys), nterms,
                                                 _lib.int_array(bonds), C.byref(st_c), caps))
    dt = torch.complex128 if cplx else torch.float64
    dev = kets[0][0].device
    gsites = gbonds = None
    if guess is not None:
        gsites = [as_device(t, cplx) for t in guess._data]
        gbonds = guess.bond_dimensions()
        for i in range(L + 1):
            caps[i] = max(caps[i], gbonds[i])
    outs = [torch.empty(max(1, caps[i] * phys[i] * caps[i + 1]), dtype=dt, device=dev)
            for i in range(L)]
    wpairs = []
    for w in weights:
        w = complex(w)
        wpairs += [w.real, w.imag]
    out_bonds = (C.c_int * (L + 1))()
    rep = _lib.sm_simplify_report()
    flat = [t for k in kets for t in k]
    head = (_lib.context(), _lib.SM_COMPLEX128 if cplx else _lib.SM_FLOAT64, L,
            _lib.int_array(phys), nterms, _lib.dbl_array(wpairs), _lib.int_array(bonds),
            _lib.ptr_array(flat), _lib.dbl_array([s._error for s in states]))
    tail = (C.byref(st_c), int(direction), _lib.ptr_array(outs),
            _lib.i64_array([o.numel() for o in outs]), out_bonds, C.byref(rep), _lib.stream_handle())
    gram_arr = None
    if gram is not None:
        g = np.asarray(gram, dtype=complex).reshape(nterms, nterms)
        pairs = np.stack([g.real, g.imag], axis=-1).reshape(-1)
        gram_arr = _lib.dbl_array(pairs.tolist())
    if guess is not None:
        _lib.check(_lib.load().sm_simplify_guess(*head, gram_arr, _lib.int_array(gbonds),
                                                 _lib.ptr_array(gsites), *tail))
    elif gram is None:
        _lib.check(_lib.load().sm_simplify(*head, *tail))
    else:
        _lib.check(_lib.load().sm_simplify_gram(*head, gram_arr, *tail))
    data = [outs[i][: out_bonds[i] * phys[i] * out_bonds[i + 1]].view(out_bonds[i], phys[i],
                                                                         out_bonds[i + 1])
            for i in range(L)]
    last_report.clear()
    last_report.update(dict(error=rep.error, norm_state_sqr=rep.norm_state_sqr,
                            norm_mps_sqr=rep.norm_mps_sqr, last_err=rep.last_err,
                            sweeps=rep.sweeps, center=rep.center, splits=rep.splits,
                            zero_state=bool(rep.zero_state),
                            sweep_err=[rep.sweep_err[k] for k in range(min(64, rep.sweeps))]))
    out = CanonicalMPS.__new__(CanonicalMPS)
    MPS.__init__(out, data, rep.error)
    out.strategy = strategy
    out._center = rep.center
    return out


def simplify(state, strategy: Strategy = SIMPLIFICATION_STRATEGY, direction: int = +1,
             guess: MPS | None = None) -> CanonicalMPS:
    """Simplify an MPS or MPSSum (state/simplification.py:32-144, :150-280); a `guess`
    starts the variational sweeps instead of the state itself (:93-98, :214-219)."""
    if guess is not None and not isinstance(guess, MPS):
        raise TypeError("simplify: the guess must be an MPS")
    if isinstance(state, MPSSum):
        return _simplify_terms(state.weights, state.states, strategy, direction, guess=guess)
    if isinstance(state, MPS):
        return _simplify_terms([1.0], [state], strategy, direction, guess=guess)
    raise TypeError(f"Cannot simplify {type(state)}")


simplify_mps = simplify


def simplify_mps_sum(sum_state: MPSSum, strategy: Strategy = SIMPLIFICATION_STRATEGY,
                     direction: int = +1, guess: MPS | None = None) -> CanonicalMPS:
    return simplify(sum_state, strategy, direction, guess)


def random_uniform_mps(d: int, N: int, D: int = 1, truncate: bool = True, complex: bool = False,
                       rng: np.random.Generator | None = None) -> MPS:
    """Random MPS with the reference factory's bond rule (state/factories.py:141-215).

    Entries are drawn on the host with numpy's Generator (same stream as the
    reference for the same seed) and copied to the device.
    """
    return random_mps([d] * N, D, truncate, complex, rng)


def random_mps(dimensions, D: int = 1, truncate: bool = True, complex: bool = False,
               rng: np.random.Generator | None = None) -> MPS:
    rng = np.random.default_rng(0x874665212) if rng is None else rng
    N = len(dimensions)
    out = []
    DR = 1
    if N > 60:
        truncate = False
    for i, d in enumerate(dimensions):
        DL = DR
        if not truncate and i != N - 1:
            DR = D
        else:
            DR = min(DR * d, D, d ** (N - i - 1))
        T = rng.normal(size=(DL, d, DR))
        if complex:
            T = T + 1j * rng.normal(size=T.shape)
        out.append(T)
    return MPS(out)
