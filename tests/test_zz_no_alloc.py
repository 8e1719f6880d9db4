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


@pytest.mark.parametrize("cplx", [False, True])
def test_noalloc_split_matches_regular_split_twice(cplx):
    rng = np.random.default_rng(77)
    strategy = DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=40)
    for shape in [(32, 2, 2, 32), (64, 2, 2, 48), (7, 2, 2, 5)]:
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
            assert D == ref_D
            assert abs(err - ref_err) <= 1e-12 * max(1.0, ref_err)
            rec = (U @ SV).cpu().numpy()
            ref = (ref_U @ ref_SV).cpu().numpy()
            assert np.allclose(rec, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
            eye = torch.eye(D, dtype=U.dtype, device=U.device)
            assert torch.allclose(U.conj().T @ U, eye, atol=1e-12)
            s = torch.linalg.vector_norm(SV, dim=1)
            s_ref = torch.linalg.vector_norm(ref_SV, dim=1)
            assert torch.allclose(s, s_ref, rtol=0, atol=1e-12 * float(s_ref.max()))


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
