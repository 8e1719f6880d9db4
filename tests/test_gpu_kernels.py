"""Kernel-level parity of the CUDA path against the CPU oracle (GPU required).

Mirrors the reference's kernel tests: test_states/test_svd.py:6-26 (sizes 1..5,
reconstruction), test_states/test_gemm.py:6-112 (all N/T/C flags),
test_contractions.py:7-29 (_mpo_multiply_tensor), test_truncate/*.
"""

import numpy as np
import pytest

from oracle import seemps_oracle as so
from tests.golden_cases import truncation_cases
from tests.gpu_util import sv_close, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import seemps2_gb300 as sg  # noqa: E402
from seemps2_gb300 import core  # noqa: E402

RNG = np.random.default_rng(0x1232388472)


def rand(shape, cplx):
    x = RNG.normal(size=shape)
    if cplx:
        x = x + 1j * RNG.normal(size=shape)
    return x


def test_truncation_rule_on_device_is_bit_exact():
    """Every golden truncation case: same size, same squared error (relative norm rule)."""
    for s, c in truncation_cases():
        st = sg.Strategy(method=c["method"], tolerance=c["tol"], max_bond_dimension=c["maxb"])
        kept, err = sg.destructively_truncate_vector(np.array(s), st)
        assert kept.numel() == c["size"], c
        o_size, o_err = so.truncate(np.array(s), so.Strategy(method=c["method"], tolerance=c["tol"],
                                                             max_bond_dimension=c["maxb"]))
        assert err == o_err, (c, err, o_err)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("opB", [0, 1, 2])
@pytest.mark.parametrize("opA", [0, 1, 2])
def test_gemm_flags(opA, opB, cplx):
    # the last three take the split-K path (fewer output tiles than SMs)
    for (M, N, K) in [(1, 1, 1), (5, 3, 4), (70, 65, 33), (130, 17, 200), (256, 256, 512),
                      (300, 258, 384), (64, 700, 1000)]:
        A = rand((M, K) if opA == 0 else (K, M), cplx)
        B = rand((K, N) if opB == 0 else (N, K), cplx)
        opn = {0: lambda x: x, 1: lambda x: x.T, 2: lambda x: x.conj().T}
        ref = opn[opA](A) @ opn[opB](B)
        out = to_np(core._gemm(A, opA, B, opB))
        assert np.allclose(out, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("cplx", [False, True])
def test_svd_small_sizes_reconstruct(cplx):
    for m in range(1, 6):
        for n in range(1, 6):
            A = rand((m, n), cplx)
            U, s, V = (to_np(x) for x in sg._destructive_svd(A))
            assert np.allclose((U * s) @ V, A, rtol=1e-10, atol=1e-12)
            sv_close(s, np.linalg.svd(A, compute_uv=False), 1e-12)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("shape", [(64, 64), (100, 37), (37, 100), (256, 512), (300, 300), (1, 50), (50, 1)])
def test_svd_against_lapack(shape, cplx):
    A = rand(shape, cplx)
    # graded spectrum like an MPS bond
    m, n = shape
    k = min(m, n)
    Q1, _ = np.linalg.qr(rand((m, k), cplx))
    Q2, _ = np.linalg.qr(rand((n, k), cplx))
    s0 = np.exp(-np.linspace(0, 30, k))
    A = (Q1 * s0) @ Q2.conj().T
    U, s, V = (to_np(x) for x in sg._destructive_svd(A))
    _, s_ref, _ = so.svd(A)
    sv_close(s, s_ref, 1e-12)
    assert np.allclose((U * s) @ V, A, atol=1e-12 * s_ref[0])
    assert np.allclose(U.conj().T @ U, np.eye(k), atol=1e-11)
    assert np.allclose(V @ V.conj().T, np.eye(k), atol=1e-11)


@pytest.mark.parametrize("cplx", [False, True])
def test_two_site_splits_match_oracle(cplx):
    st = sg.DEFAULT_STRATEGY.replace(tolerance=1e-8, max_bond_dimension=20)
    ost = so.DEFAULT_STRATEGY.replace(tolerance=1e-8, max_bond_dimension=20)
    for (a, b) in [(1, 1), (3, 5), (16, 16), (24, 9)]:
        AA = rand((a, 2, 2, b), cplx)
        for gpu_fn, ora_fn in [(sg._left_orth_2site, so.left_orth_2site),
                               (sg._right_orth_2site, so.right_orth_2site)]:
            L, R, e = gpu_fn(AA, st)
            Lo, Ro, eo = ora_fn(AA, ost)
            assert L.shape == Lo.shape and R.shape == Ro.shape
            D = L.shape[-1]
            rec = to_np(L).reshape(-1, D) @ to_np(R).reshape(D, -1)
            reco = Lo.reshape(-1, D) @ Ro.reshape(D, -1)
            assert np.allclose(rec, reco, atol=1e-11 * np.abs(AA).max())
            assert abs(e - eo) <= 1e-9 * max(1.0, eo)


@pytest.mark.parametrize("cplx", [False, True])
def test_environments_and_mpo_product(cplx):
    A = rand((5, 2, 7), cplx)
    B = rand((4, 2, 6), cplx)
    rhoL = rand((4, 5), cplx)
    rhoR = rand((7, 6), cplx)
    assert np.allclose(to_np(sg._update_left_environment(B, A, rhoL)),
                       so.update_left_environment(B, A, rhoL), atol=1e-12)
    assert np.allclose(to_np(sg._update_right_environment(B, A, rhoR)),
                       so.update_right_environment(B, A, rhoR), atol=1e-12)
    O = rand((3, 2, 2, 4), cplx)
    psi = rand((5, 2, 6), cplx)
    assert np.allclose(to_np(sg._mpo_multiply_tensor(O, psi)), so.mpo_multiply_tensor(O, psi),
                       atol=1e-12)


def test_invalid_arguments_raise_like_the_reference():
    with pytest.raises(ValueError):
        core._gemm(np.ones((2, 3)), 0, np.ones((4, 2)), 0)
    with pytest.raises(ValueError):
        sg._update_left_environment(np.ones((2, 2)), np.ones((2, 2, 2)), np.ones((2, 2)))
