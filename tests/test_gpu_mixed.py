"""The mixed-precision split (SM_PRECISION_MIXED) against the FP64 oracle.

The mixed form computes the kept subspace with an FP32 cluster factorisation
refined by FP64 GEMMs, so singular vectors are compared through gauge-free
quantities: the truncated product P = U (sV), the isometry of U, the exact
discarded weight and the fidelity of whole states.  Bars (stated per test):
fidelity error of the truncated product 1 - |<P, P_oracle>|^2 / (|P|^2
|P_oracle|^2) below 1e-10, discarded weights within 1e-10 |A|^2 of the
oracle's, isometries orthonormal to 1e-13, whole-state fidelity error below
1e-10.
"""

import numpy as np
import pytest

from oracle import seemps_oracle as so
from tests.gpu_util import mps_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import seemps2_gb300 as sg  # noqa: E402
from seemps2_gb300 import _lib  # noqa: E402
from seemps2_gb300 import core  # noqa: E402


@pytest.fixture
def mixed():
    sg.set_precision("mixed")
    _lib.stats_reset()
    try:
        yield
    finally:
        sg.set_precision("fp64")


def spectrum_matrix(rng, m, n, s, cplx):
    """m x n matrix with singular values s (len <= min(m, n))."""
    def haar(r, c):
        X = rng.normal(size=(r, c))
        if cplx:
            X = X + 1j * rng.normal(size=(r, c))
        Q, _ = np.linalg.qr(X)
        return Q
    r = len(s)
    return (haar(m, r) * np.asarray(s)) @ haar(n, r).conj().T


def product_fidelity_error(P, Q):
    """1 - |<P, Q>|^2 / (|P|^2 |Q|^2) of two matrices (Frobenius inner product)."""
    pq = np.vdot(P, Q)
    return 1.0 - abs(pq) ** 2 / (np.vdot(P, P).real * np.vdot(Q, Q).real)


def two_site(A, a, d1, d2, b):
    return np.ascontiguousarray(A.reshape(a, d1, d2, b))


def test_mixed_split_resolved_cut_stays_mixed(mixed):
    """A cut well above FP32 resolution (s_150 = 3e-2, s_151 = 1e-2): no
    fallback, product fidelity error below 1e-12, exact isometry."""
    rng = np.random.default_rng(12)
    s = np.concatenate([np.geomspace(1.0, 3e-2, 150), np.geomspace(1e-2, 1e-3, 60)])
    A = spectrum_matrix(rng, 384, 384, s, False)
    AA = two_site(A, 192, 2, 2, 192)
    st = sg.Strategy(tolerance=1e-12, max_bond_dimension=150)
    L, R, err = core._left_orth_2site(AA, st)
    oL, oR, oerr = so.left_orth_2site(AA, so.Strategy(tolerance=1e-12, max_bond_dimension=150))
    stats = _lib.stats_read()
    assert stats["mixed_splits"] == 1 and stats["mixed_fallbacks"] == 0
    L, R = L.cpu().numpy(), R.cpu().numpy()
    M = L.reshape(-1, 150)
    assert np.abs(M.T @ M - np.eye(150)).max() < 1e-13
    P = M @ R.reshape(150, -1)
    oP = oL.reshape(384, -1) @ oR.reshape(-1, 384)
    norm = np.linalg.norm(A)
    assert product_fidelity_error(P, oP) < 1e-12
    assert abs(err**2 - oerr**2) <= 1e-12 * norm**2


def spectra():
    # 258 significant values with a gap after 256 (the shape of the n=30, chi=256
    # workload), then rounding-level noise
    s1 = np.concatenate([np.geomspace(1.0, 3e-3, 256), [2.5e-3, 2.4e-3], 1e-17 * np.ones(20)])
    # a smooth tail that the tolerance cuts (no max-bond limit)
    s2 = np.geomspace(1.0, 1e-9, 120)
    return {"gap_at_max_bond": (s1, 256, 1e-12), "tolerance_cut": (s2, 10**6, 1e-12)}


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("case", ["gap_at_max_bond", "tolerance_cut"])
@pytest.mark.parametrize("side", ["left", "right"])
def test_mixed_split_against_oracle(mixed, cplx, case, side):
    rng = np.random.default_rng(11)
    s, maxb, tol = spectra()[case]
    a, d, b = (160, 2, 160) if case == "gap_at_max_bond" else (64, 2, 64)
    A = spectrum_matrix(rng, a * d, d * b, s, cplx)
    AA = two_site(A, a, d, d, b)
    st = sg.Strategy(tolerance=tol, max_bond_dimension=maxb)
    ost = so.Strategy(tolerance=tol, max_bond_dimension=maxb)
    fn, ofn = (core._left_orth_2site, so.left_orth_2site) if side == "left" else (
        core._right_orth_2site, so.right_orth_2site)
    L, R, err = fn(AA, st)
    oL, oR, oerr = ofn(AA, ost)
    L, R = L.cpu().numpy(), R.cpu().numpy()
    D = L.shape[-1]
    stats = _lib.stats_read()
    assert stats["mixed_splits"] >= 1
    # "tolerance_cut" cuts below 1e-4 s_max, beyond the FP32 stage's resolution of
    # individual values: the rank comes from the exact discarded weight instead
    # (never below the oracle's, a few above at most, weight within tolerance)
    norm2 = np.linalg.norm(A) ** 2
    # the kept rank: identical where the spectrum separates it
    if case == "gap_at_max_bond":
        assert D == oL.shape[-1] == 256
    else:
        assert oL.shape[-1] <= D <= oL.shape[-1] + 3
        assert err**2 <= 1e-12 * norm2 * (1 + 1e-9)
    # isometry of the orthogonal factor to FP64 rounding
    if side == "left":
        M = L.reshape(-1, D)
        assert np.abs(M.conj().T @ M - np.eye(D)).max() < 1e-13
    else:
        M = R.reshape(D, -1)
        assert np.abs(M @ M.conj().T - np.eye(D)).max() < 1e-13
    # truncated products: fidelity error below 1e-10
    P = L.reshape(a * d, D) @ R.reshape(D, d * b)
    oP = oL.reshape(a * d, -1) @ oR.reshape(-1, d * b)
    assert product_fidelity_error(P, oP) < 1e-10
    # discarded weight: reported value is the exact |A - P|^2, within 1e-10 |A|^2 of the oracle's
    assert abs(err**2 - np.linalg.norm(A - P) ** 2) <= 1e-13 * norm2
    assert abs(err**2 - oerr**2) <= 1e-10 * norm2


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("want_u", [0, 1])
@pytest.mark.parametrize("shape", [(96, 64), (64, 200), (320, 320), (512, 256)])
def test_cluster_rows_span_and_orthogonality(cplx, want_u, shape):
    """FP32 stage alone: rows mutually orthogonal to the stop rule's level, Y^H Y = W^H W
    (same row space and singular values) to FP32 accuracy."""
    import ctypes as C

    rng = np.random.default_rng(1)
    m, n = shape
    r = min(m, n) - 3
    s = np.geomspace(1.0, 1e-3, r)
    A = spectrum_matrix(rng, m, n, s, cplx)
    W = A.T if want_u else A
    kw, l = W.shape
    kcap = min(m, n) + 32
    dt = torch.complex128 if cplx else torch.float64
    Ad = torch.from_numpy(np.ascontiguousarray(A)).to("cuda")
    rows = torch.empty(kcap, l, dtype=dt, device="cuda")
    nrm = torch.empty(kcap, dtype=torch.float64, device="cuda")
    keff, sweeps = C.c_int(), C.c_int()
    _lib.check(_lib.load().sm_split_rows_f32(
        _lib.context(), 1 if cplx else 0, _lib.ptr(Ad), m, n, want_u, 1e-14, 0.0, _lib.ptr(rows),
        C.cast(nrm.data_ptr(), C.POINTER(C.c_double)), kcap, C.byref(keff), C.byref(sweeps),
        _lib.stream_handle()))
    torch.cuda.synchronize()
    Y = rows.cpu().numpy()
    nv = nrm.cpu().numpy()
    assert keff.value >= r and sweeps.value >= 1
    assert np.allclose(np.linalg.norm(Y, axis=1), nv, rtol=1e-12, atol=1e-300)
    # same Gram matrix as W (row space and singular values) to the backward
    # error of an FP32 QR + Jacobi: a few 1e-6 of |W|_F^2
    Gw = W.conj().T @ W
    Gy = Y.conj().T @ Y
    assert np.abs(Gy - Gw).max() <= 1e-5 * np.linalg.norm(W) ** 2
    # singular values = row norms (sorted), to FP32 backward error of |W|_F
    sv = np.sort(nv)[::-1][: len(s)]
    assert np.abs(sv - s).max() <= 2e-5 * np.linalg.norm(W)
    # mutual orthogonality of the significant rows: the Jacobi stops after a
    # sweep whose rotations all started below cosine 1e-2, so about 1e-4 is left
    # for the FP64 refinement
    big = nv > 1e-4
    Yb = Y[big] / nv[big, None]
    off = Yb.conj() @ Yb.T - np.eye(big.sum())
    assert np.abs(off).max() <= 1e-3


@pytest.mark.parametrize("cplx", [False, True])
def test_cluster_qr_pivots_heavy_columns_first(cplx):
    """Block column pivoting in the FP32 QR: W (256 x 256) whose first 192
    columns are zero and whose last 64 hold a rank-24 matrix.  Every panel takes
    the heaviest remaining columns, so the rank-revealing QR stops within a few
    blocks of the rank (keff <= 40; unpivoted it would first step through the
    192 zero columns), and the rows still give W's Gram matrix and singular
    values, in W's own column order."""
    import ctypes as C

    rng = np.random.default_rng(4)
    m = n = 256
    s = np.geomspace(1.0, 1e-2, 24)
    A = np.zeros((m, n), complex if cplx else float)
    A[:, 192:] = spectrum_matrix(rng, m, 64, s, cplx)
    kcap = n + 32
    dt = torch.complex128 if cplx else torch.float64
    Ad = torch.from_numpy(np.ascontiguousarray(A)).to("cuda")
    rows = torch.empty(kcap, n, dtype=dt, device="cuda")
    nrm = torch.empty(kcap, dtype=torch.float64, device="cuda")
    keff, sweeps = C.c_int(), C.c_int()
    _lib.check(_lib.load().sm_split_rows_f32(
        _lib.context(), 1 if cplx else 0, _lib.ptr(Ad), m, n, 0, 1e-14, 0.0, _lib.ptr(rows),
        C.cast(nrm.data_ptr(), C.POINTER(C.c_double)), kcap, C.byref(keff), C.byref(sweeps),
        _lib.stream_handle()))
    torch.cuda.synchronize()
    assert 24 <= keff.value <= 40, keff.value
    Y = rows.cpu().numpy()
    nv = nrm.cpu().numpy()
    assert np.abs(Y.conj().T @ Y - A.conj().T @ A).max() <= 1e-5 * np.linalg.norm(A) ** 2
    assert np.abs(Y[:, :192]).max() == 0.0  # the zero columns stay zero, in place
    sv = np.sort(nv)[::-1][:24]
    assert np.abs(sv - s).max() <= 2e-5 * np.linalg.norm(A)


def test_mixed_zero_matrix(mixed):
    AA = np.zeros((16, 2, 2, 16))
    L, R, err = core._left_orth_2site(AA, sg.Strategy(tolerance=1e-10))
    assert L.shape[-1] == 1 and err == 0.0
    assert torch.isfinite(L).all() and torch.isfinite(R).all()


def test_mixed_falls_back_when_fp32_cannot_meet_tolerance(mixed):
    """A tolerance below FP32 resolution: the exact discarded weight exceeds it,
    the split is redone in FP64 and then keeps the oracle's rank exactly."""
    rng = np.random.default_rng(3)
    s = np.geomspace(1.0, 1e-12, 90)
    A = spectrum_matrix(rng, 96, 96, s, False)
    AA = two_site(A, 48, 2, 2, 48)
    st = sg.Strategy(tolerance=1e-20, max_bond_dimension=10**6)
    L, R, err = core._left_orth_2site(AA, st)
    oL, oR, oerr = so.left_orth_2site(AA, so.Strategy(tolerance=1e-20, max_bond_dimension=10**6))
    stats = _lib.stats_read()
    assert stats["mixed_fallbacks"] >= 1
    assert L.shape[-1] == oL.shape[-1]


@pytest.mark.parametrize("qr", ["stop", "full"])
def test_mixed_split_of_a_graded_matrix(qr):
    """A matrix met while canonicalising the Laplacian product state (rows
    graded down to 1e-12 of the largest, a third exact zeros, numerical rank
    ~63 of 192; tests/golden/make_graded_split.py).  Its FP32 QR leaves rows of
    R far below FP32 resolution; the split must still give orthonormal rows,
    the oracle's rank and the exact discarded weight, with the QR stopped by the
    trailing weight ("stop") or run to the end ("full": a rank hint of 20 makes
    the first attempt miss weight, and its redo runs the whole QR)."""
    import os

    A = np.load(os.path.join(os.path.dirname(__file__), "golden",
                             "graded_split_192x250.npz"))["A"]
    a2 = float(np.sum(A ** 2))
    AA = two_site(A, 96, 2, 2, 125)
    st = sg.Strategy(tolerance=1e-12, max_bond_dimension=256)
    if qr == "full":
        sg.set_precision("mixed+learned", range_finder=True, rank_hint=20)
    else:
        sg.set_precision("mixed")
    _lib.stats_reset()
    try:
        US, V, err = core._right_orth_2site(AA, st)
        stats = _lib.stats_read()
    finally:
        sg.set_precision("fp64")
    oUS, oV, oerr = so.right_orth_2site(AA, so.Strategy(tolerance=1e-12, max_bond_dimension=256))
    D = V.shape[0]
    Vn = V.cpu().numpy().reshape(D, 250)
    USn = US.cpu().numpy().reshape(192, D)
    assert D == oV.shape[0]
    assert np.abs(Vn @ Vn.T - np.eye(D)).max() <= 1e-13
    assert abs(float(err) ** 2 - float(oerr) ** 2) <= 1e-10 * a2
    P, Po = USn @ Vn, oUS.reshape(192, D) @ oV.reshape(D, 250)
    assert product_fidelity_error(P, Po) <= 1e-10
    assert stats["mixed_splits"] >= 1
    if qr == "full":
        assert stats["mixed_cap_redone"] == 1


def laplacian_case(n, chi, seed=7):
    rng = np.random.default_rng(seed)
    raw = so.random_mps(2, n, chi, rng)
    mps, carry = [], np.eye(1)
    for i, A in enumerate(raw):
        A = np.tensordot(carry, A, axes=1)
        a, d, b = A.shape
        if i < n - 1:
            Q, R = np.linalg.qr(A.reshape(a * d, b))
            mps.append(np.ascontiguousarray(Q.reshape(a, d, Q.shape[1])))
            carry = R
        else:
            mps.append(A / np.linalg.norm(A))
    h = 2.0 ** (-n)
    return mps, so.tridiagonal_mpo(n, -2.0 / h**2, 1.0 / h**2, 1.0 / h**2)


def test_mixed_apply_laplacian_fidelity(mixed):
    """MPO.apply + simplify (tol 1e-12, max bond chi, 2 sweeps): the mixed state
    against the FP64 oracle, fidelity error below 1e-10."""
    n, chi = 14, 64
    mps, mpo = laplacian_case(n, chi)
    kw = dict(tolerance=1e-12, max_bond_dimension=chi, max_sweeps=2, simplification_tolerance=0.0)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    out = sg.MPO(mpo, st).apply(sg.MPS(mps), strategy=st)
    res = so.mpo_apply(mpo, mps, so.DEFAULT_STRATEGY.replace(**kw))
    stats = _lib.stats_read()
    assert stats["mixed_splits"] > 10
    fe = so.fidelity_error(mps_np(out), res.tensors)
    assert fe < 1e-10, fe
    assert abs(out.error() - res.error) <= 1e-10 + 1e-6 * res.error


def test_mixed_apply_random_complex(mixed):
    """The C1-shaped workload (complex MPS chi=32, random complex MPO D=4,
    tol 1e-10, max bond 64, 2 sweeps): fidelity error below 1e-10."""
    rng = np.random.default_rng(21)
    n = 12
    mps = so.random_mps(2, n, 32, rng, complex_=True)
    nrm = np.sqrt(so.norm_squared(mps).real)
    mps[0] = mps[0] / nrm
    mpo = so.random_mpo(2, n, 4, rng, complex_=True)
    kw = dict(tolerance=1e-10, max_bond_dimension=64, max_sweeps=2, simplification_tolerance=0.0)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    out = sg.MPO(mpo, st).apply(sg.MPS(mps), strategy=st)
    res = so.mpo_apply(mpo, mps, so.DEFAULT_STRATEGY.replace(**kw))
    assert _lib.stats_read()["mixed_splits"] > 5
    fe = so.fidelity_error(mps_np(out), res.tensors)
    assert fe < 1e-10, fe


def test_mixed_fp32_contractions_apply():
    """Mixed splits with FP32-arithmetic contractions (tol 1e-12, max bond chi,
    2 sweeps): fidelity error below 1e-10 against the FP64 oracle.  The error
    bound (a sum of sqrt(discarded weight) over all splits, which magnifies
    1e-7-level differences of tiny discarded weights) agrees to 1e-4 relative;
    the state norm and the final sweep estimate stay FP64."""
    n, chi = 14, 64
    mps, mpo = laplacian_case(n, chi)
    kw = dict(tolerance=1e-12, max_bond_dimension=chi, max_sweeps=2, simplification_tolerance=0.0)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    sg.set_precision("mixed", contractions="fp32")
    _lib.stats_reset()
    try:
        out = sg.MPO(mpo, st).apply(sg.MPS(mps), strategy=st)
        stats = _lib.stats_read()
    finally:
        sg.set_precision("fp64")
    res = so.mpo_apply(mpo, mps, so.DEFAULT_STRATEGY.replace(**kw))
    assert stats["gemm32_launches"] > 50
    assert stats["gemm_tc_launches"] > 0  # the larger contractions run on the tensor cores
    fe = so.fidelity_error(mps_np(out), res.tensors)
    assert fe < 1e-10, fe
    assert abs(out.error() - res.error) <= 1e-4 * res.error + 1e-12, (out.error(), res.error)
