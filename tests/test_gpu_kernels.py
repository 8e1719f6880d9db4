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


def _clustered_matrix(m, n, cplx, spectrum, rng):
    """Q1 diag(s) Q2^H with random orthonormal Q1, Q2 and the given leading singular
    values (the rest decays geometrically from the last one)."""
    k = min(m, n)
    s = np.array(spectrum[:k], dtype=np.float64)
    if s.size < k:
        s = np.concatenate([s, s[-1] * np.exp(-0.7 * np.arange(1, k - s.size + 1))])
    def q(r):
        x = rng.normal(size=(r, k))
        if cplx:
            x = x + 1j * rng.normal(size=(r, k))
        return np.linalg.qr(x)[0]
    return (q(m) * s) @ q(n).conj().T


def _spectra(rng):
    r5 = np.sqrt(5.0)
    return {
        # a threefold exact cluster, as the Laplacian's symmetry produces (sqrt 5)
        "threefold": [3.0, r5, r5, r5, 2.0, 1.0, 0.5],
        # several exactly repeated blocks
        "blocks": [1.0] * 8 + [0.5] * 8 + [0.25] * 4,
        # near-degenerate clusters: relative spread 1e-9 inside each
        "near": sorted((c * (1.0 + 1e-9 * rng.random()) for c in (1.0, 0.3, 0.01)
                        for _ in range(5)), reverse=True),
        # a cluster sitting at a truncation cut of tolerance 1e-12
        "at_cut": [1.0, 0.5, 0.5, 0.5] + [1e-7] * 6,
    }


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("shape", [(12, 12), (40, 24), (24, 40), (64, 64), (130, 100), (256, 128)])
def test_svd_converges_on_degenerate_spectra(shape, cplx):
    """The FP64 Jacobi converges inside exactly and nearly degenerate clusters (it formerly
    stalled there with an FP32 rotation angle), with singular values within 1e-12 s_max of
    LAPACK's and an orthonormal reconstruction."""
    rng = np.random.default_rng(hash((shape, cplx)) % (1 << 32))
    for name, spec in _spectra(rng).items():
        A = _clustered_matrix(*shape, cplx, spec, rng)
        U, s, V = (to_np(x) for x in sg._destructive_svd(A))
        _, s_ref, _ = so.svd(A)
        sv_close(s, s_ref, 1e-12)
        k = min(shape)
        assert np.allclose((U * s) @ V, A, atol=1e-12 * s_ref[0]), name
        assert np.allclose(U.conj().T @ U, np.eye(k), atol=1e-11), name
        assert np.allclose(V @ V.conj().T, np.eye(k), atol=1e-11), name


@pytest.mark.parametrize("cplx", [False, True])
def test_two_site_splits_on_degenerate_spectra_keep_reference_ranks(cplx):
    """Two-site splits (QR preconditioner + FP64 Jacobi) of clustered matrices: identical kept
    rank and discarded weight to the oracle's, under the relative-norm rule at 1e-12 and 1e-8."""
    rng = np.random.default_rng(4242 + cplx)
    for tol in (1e-12, 1e-8):
        st = sg.DEFAULT_STRATEGY.replace(tolerance=tol, max_bond_dimension=256)
        ost = so.DEFAULT_STRATEGY.replace(tolerance=tol, max_bond_dimension=256)
        for (a, b) in [(6, 6), (20, 12), (64, 64), (100, 64)]:
            for name, spec in _spectra(rng).items():
                AA = _clustered_matrix(2 * a, 2 * b, cplx, spec, rng).reshape(a, 2, 2, b)
                for gpu_fn, ora_fn in [(sg._left_orth_2site, so.left_orth_2site),
                                       (sg._right_orth_2site, so.right_orth_2site)]:
                    L, R, e = gpu_fn(AA, st)
                    Lo, Ro, eo = ora_fn(AA, ost)
                    assert L.shape == Lo.shape and R.shape == Ro.shape, (name, a, b, tol)
                    D = L.shape[-1]
                    rec = to_np(L).reshape(-1, D) @ to_np(R).reshape(D, -1)
                    reco = Lo.reshape(-1, D) @ Ro.reshape(D, -1)
                    assert np.allclose(rec, reco, atol=1e-11 * np.abs(AA).max()), (name, a, b)
                    assert abs(e - eo) <= 1e-9 * max(1e-2, eo), (name, a, b, e, eo)


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("e", [-480, -300, 0, 300, 505])
def test_fp64_splits_are_scale_invariant(e, cplx):
    """The FP64 splits give the same ranks and 2^e times the singular values for a matrix
    scaled by 2^e, far beyond where squared entries (or their squares) under- or overflow:
    the split runs on the matrix prescaled by a power of two, as LAPACK rescales."""
    rng = np.random.default_rng(abs(e) + cplx)
    s0 = np.concatenate([np.geomspace(1.0, 1e-9, 30), [1e-13] * 4])
    A = _clustered_matrix(64, 48, cplx, list(s0), rng)
    As = A * 2.0**e
    _, s_ref, _ = so.svd(A)
    U, s, V = (to_np(x) for x in sg._destructive_svd(As))
    sv_close(s * 2.0**-e, s_ref, 1e-12)
    assert np.allclose(U.conj().T @ U, np.eye(48), atol=1e-11)
    st = sg.DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=64)
    ost = so.DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=64)
    for gpu_fn, ora_fn in [(sg._left_orth_2site, so.left_orth_2site),
                           (sg._right_orth_2site, so.right_orth_2site)]:
        L, R, err = gpu_fn(As.reshape(32, 2, 2, 24), st)
        Lo, Ro, eo = ora_fn(A.reshape(32, 2, 2, 24), ost)
        assert L.shape == Lo.shape and R.shape == Ro.shape
        D = L.shape[-1]
        rec = (to_np(L).reshape(-1, D) @ to_np(R).reshape(D, -1)) * 2.0**-e
        reco = Lo.reshape(-1, D) @ Ro.reshape(D, -1)
        assert np.allclose(rec, reco, atol=1e-12 * np.abs(A).max())
        assert abs(err * 2.0**-e - eo) <= 1e-9 * max(1e-3, eo)


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
