"""The allocation-free two-site split (sm_left_orth_2site_noalloc) against the
regular one (sm_left_orth_2site), both called through the C ABI.

The allocation-free entry point exists for callers that cannot allocate device
memory while they run (a host application that owns all device memory through
its own pool, a plugin that is only handed buffers): it keeps its work arrays
in a static device array instead of the context's scratch.  Its results must
match the regular entry point's within the tolerance of the other GPU tests,
on two calls in a row (the static array keeps the previous call's contents).
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from seemps2_gb300 import _lib  # noqa: E402
from seemps2_gb300.core import DEFAULT_STRATEGY  # noqa: E402


def _split(fn_name, AA, strategy, with_ctx):
    lib = _lib.load()
    a, d1, d2, b = AA.shape
    r = min(a * d1, d2 * b)
    U = torch.full((a * d1 * r,), float("nan"), dtype=AA.dtype, device=AA.device)
    SV = torch.full((r * d2 * b,), float("nan"), dtype=AA.dtype, device=AA.device)
    D = C.c_int()
    err = C.c_double()
    dtype = _lib.SM_COMPLEX128 if AA.is_complex() else _lib.SM_FLOAT64
    st = strategy.to_c()
    args = [dtype, _lib.ptr(AA), a, d1, d2, b, C.byref(st), _lib.ptr(U), _lib.ptr(SV),
            C.byref(D), C.byref(err), _lib.stream_handle()]
    if with_ctx:
        args = [_lib.context()] + args
    _lib.check(getattr(lib, fn_name)(*args))
    torch.cuda.synchronize()
    n = D.value
    return U[: a * d1 * n].reshape(a * d1, n), SV[: n * d2 * b].reshape(n, d2 * b), n, err.value


def _noalloc_call(AA, strategy, U, SV):
    """One call of the allocation-free entry point into preallocated outputs."""
    lib = _lib.load()
    a, d1, d2, b = AA.shape
    D = C.c_int()
    err = C.c_double()
    dtype = _lib.SM_COMPLEX128 if AA.is_complex() else _lib.SM_FLOAT64
    st = strategy.to_c()
    _lib.check(lib.sm_left_orth_2site_noalloc(dtype, _lib.ptr(AA), a, d1, d2, b, C.byref(st),
                                              _lib.ptr(U), _lib.ptr(SV), C.byref(D), C.byref(err),
                                              _lib.stream_handle()))
    torch.cuda.synchronize()
    return D.value, err.value


# square (64 x 64), tall (128 x 96, 14 x 10), strictly wide (10 x 18) and the
# largest accepted size (256 x 256)
SHAPES = [(32, 2, 2, 32), (64, 2, 2, 48), (7, 2, 2, 5), (5, 2, 2, 9), (128, 2, 2, 128)]


@pytest.mark.parametrize("cplx", [False, True])
def test_noalloc_split_matches_regular_split_twice(cplx):
    rng = np.random.default_rng(77)
    strategy = DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=40)
    for shape in SHAPES:
        x = rng.normal(size=shape)
        if cplx:
            x = x + 1j * rng.normal(size=shape)
        AA = torch.from_numpy(x).cuda()
        ref_U, ref_SV, ref_D, ref_err = _split("sm_left_orth_2site", AA, strategy, True)
        for _ in range(2):  # two calls in a row through the shared static array
            U, SV, D, err = _split("sm_left_orth_2site_noalloc", AA, strategy, False)
            # singular vectors are defined up to a phase per vector, so compare
            # what does not depend on it: kept rank, discarded weight, the
            # truncated product U @ SV, the isometry of U and the row norms of SV
            assert D == ref_D, shape
            assert abs(err - ref_err) <= 1e-12 * max(1.0, ref_err), shape
            rec = (U @ SV).cpu().numpy()
            ref = (ref_U @ ref_SV).cpu().numpy()
            assert np.allclose(rec, ref, rtol=0, atol=1e-12 * np.abs(ref).max()), shape
            eye = torch.eye(D, dtype=U.dtype, device=U.device)
            assert torch.allclose(U.conj().T @ U, eye, atol=1e-12), shape
            s = torch.linalg.vector_norm(SV, dim=1)
            s_ref = torch.linalg.vector_norm(ref_SV, dim=1)
            assert torch.allclose(s, s_ref, rtol=0, atol=1e-12 * float(s_ref.max())), shape


def test_noalloc_split_allocates_no_device_memory():
    """After a first call (which may load the kernels it uses), further calls leave the
    device's free memory unchanged: the entry point allocates nothing."""
    rng = np.random.default_rng(78)
    strategy = DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=64)
    for shape in [(64, 2, 2, 64), (5, 2, 2, 9)]:
        AA = torch.from_numpy(rng.normal(size=shape)).cuda()
        a, d1, d2, b = shape
        r = min(a * d1, d2 * b)
        U = torch.empty(a * d1 * r, dtype=AA.dtype, device="cuda")
        SV = torch.empty(r * d2 * b, dtype=AA.dtype, device="cuda")
        first = _noalloc_call(AA, strategy, U, SV)
        free_before, _ = torch.cuda.mem_get_info()
        for _ in range(3):
            assert _noalloc_call(AA, strategy, U, SV) == first
        free_after, _ = torch.cuda.mem_get_info()
        assert free_after == free_before, (shape, free_before - free_after)


def test_noalloc_split_rejects_sizes_beyond_its_limit():
    lib = _lib.load()
    AA = torch.zeros((200, 2, 2, 3), dtype=torch.float64, device="cuda")  # 400 rows > 256
    out = torch.zeros(400 * 12, dtype=torch.float64, device="cuda")
    D = C.c_int()
    err = C.c_double()
    st = DEFAULT_STRATEGY.to_c()
    status = lib.sm_left_orth_2site_noalloc(_lib.SM_FLOAT64, _lib.ptr(AA), 200, 2, 2, 3,
                                            C.byref(st), _lib.ptr(out), _lib.ptr(out), C.byref(D),
                                            C.byref(err), _lib.stream_handle())
    assert status == _lib.SM_ERR_VALUE
    assert b"exceeds" in lib.sm_last_error()
    # dimensions whose product overflows 32 bits are rejected by the same limit (the
    # check happens before any device access)
    status = lib.sm_left_orth_2site_noalloc(_lib.SM_FLOAT64, _lib.ptr(AA), 1 << 20, 1 << 12, 2, 3,
                                            C.byref(st), _lib.ptr(out), _lib.ptr(out), C.byref(D),
                                            C.byref(err), _lib.stream_handle())
    assert status == _lib.SM_ERR_VALUE
    assert b"exceeds" in lib.sm_last_error()
