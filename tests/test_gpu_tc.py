"""Tensor-core GEMM at FP32 accuracy (3xTF32 on tcgen05, sm_gemm_f32) against
an FP64 product: relative Frobenius error below 2e-6 for every op pair,
ragged sizes (M, N not multiples of the 128 x 128 tile, K not a multiple of
the 32-wide slice) and split-K; small shapes go to the FP32 SIMT kernel
instead (no tensor-core launch).  The two-term simplify checks the
accumulating (beta = 1) contractions of a sum under FP32 contractions."""

import ctypes as C

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

OPS = {"N": 0, "T": 1, "C": 2}


def _gemm_f32(opA, opB, A, B, M, N, K):
    Ad = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    Bd = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    Cd = torch.empty((M, N), dtype=torch.float64, device="cuda")
    _lib.check(_lib.load().sm_gemm_f32(
        _lib.context(), _lib.SM_FLOAT64, OPS[opA], OPS[opB], M, N, K, C.c_void_p(Ad.data_ptr()),
        A.shape[1], C.c_void_p(Bd.data_ptr()), B.shape[1], C.c_void_p(Cd.data_ptr()), N,
        _lib.stream_handle()))
    torch.cuda.synchronize()
    return Cd.cpu().numpy()


@pytest.mark.parametrize("M,N,K,opA,opB", [
    (128, 128, 256, "N", "N"),
    (256, 1536, 768, "N", "N"),   # left environment x product site (chi 256, D 3)
    (1536, 256, 768, "N", "T"),
    (512, 512, 768, "C", "N"),
    (300, 200, 100, "T", "T"),    # ragged in all three
    (64, 64, 1024, "N", "C"),     # one tile, deep K: split-K
    (1000, 130, 40, "T", "N"),
])
def test_tensor_core_gemm_matches_fp64(M, N, K, opA, opB):
    rng = np.random.default_rng(M + 7 * N + 13 * K)
    A = rng.normal(size=(M, K) if opA == "N" else (K, M))
    B = rng.normal(size=(K, N) if opB == "N" else (N, K))
    ref = (A if opA == "N" else A.T) @ (B if opB == "N" else B.T)
    _lib.stats_reset()
    out = _gemm_f32(opA, opB, A, B, M, N, K)
    st = _lib.stats_read()
    assert st["gemm_tc_launches"] == 1
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert rel < 2e-6, rel
    # better than a plain FP32 product of the rounded operands would allow by far
    assert np.isfinite(out).all()


def test_small_shapes_stay_on_simt():
    rng = np.random.default_rng(3)
    A = rng.normal(size=(40, 30))
    B = rng.normal(size=(30, 20))
    _lib.stats_reset()
    out = _gemm_f32("N", "N", A, B, 40, 20, 30)
    assert _lib.stats_read()["gemm_tc_launches"] == 0
    assert np.linalg.norm(out - A @ B) / np.linalg.norm(A @ B) < 1e-6


def test_fp32_contractions_of_a_sum():
    rng = np.random.default_rng(8)
    n, chi = 18, 128
    states = [so.random_mps(2, n, chi, rng) for _ in range(2)]
    kw = dict(tolerance=1e-12, max_bond_dimension=chi, max_sweeps=2, simplification_tolerance=0.0)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    sg.set_precision("mixed", contractions="fp32")
    _lib.stats_reset()
    try:
        out = sg.simplify(sg.MPSSum([0.6, -0.4], [sg.MPS(s) for s in states]), strategy=st)
        stats = _lib.stats_read()
    finally:
        sg.set_precision("fp64")
    res = so.simplify_mps_sum([0.6, -0.4], states, so.DEFAULT_STRATEGY.replace(**kw))
    assert stats["gemm_tc_launches"] > 10, stats["gemm_tc_launches"]
    fe = so.fidelity_error(mps_np(out), res.tensors)
    assert fe < 1e-10, fe


def _gemm_fp64(opA, opB, A, B, M, N, K):
    Ad = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    Bd = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    Cd = torch.empty((M, N), dtype=torch.float64, device="cuda")
    _lib.check(_lib.load().sm_gemm(
        _lib.context(), _lib.SM_FLOAT64, OPS[opA], OPS[opB], M, N, K, C.c_void_p(Ad.data_ptr()),
        A.shape[1], C.c_void_p(Bd.data_ptr()), B.shape[1], C.c_void_p(Cd.data_ptr()), N,
        _lib.stream_handle()))
    torch.cuda.synchronize()
    return Cd.cpu().numpy()


def _gemm_f64tc(opA, opB, A, B, M, N, K):
    Ad = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    Bd = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    Cd = torch.empty((M, N), dtype=torch.float64, device="cuda")
    _lib.check(_lib.load().sm_gemm_f64tc(
        _lib.context(), _lib.SM_FLOAT64, OPS[opA], OPS[opB], M, N, K, C.c_void_p(Ad.data_ptr()),
        A.shape[1], C.c_void_p(Bd.data_ptr()), B.shape[1], C.c_void_p(Cd.data_ptr()), N,
        _lib.stream_handle()))
    torch.cuda.synchronize()
    return Cd.cpu().numpy()


@pytest.mark.parametrize("M,N,K,opA,opB", [
    (128, 64, 256, "N", "N"),     # one tile, one exact chunk
    (512, 512, 768, "N", "T"),    # three chunks, split-K
    (225, 225, 512, "C", "N"),    # refinement Gram shape, ragged tiles
    (300, 200, 100, "T", "T"),    # K not a multiple of 32
    (64, 96, 1536, "N", "C"),     # deep K: six chunks over split-K
])
def test_fp64_tensor_core_gemm_has_fp64_accuracy(M, N, K, opA, opB):
    """Error against numpy's FP64 product, normalised by |A||B| (the scale of
    the FP64 GEMM error bound), within 8 sqrt(K) u and within twice the FP64
    SIMT GEMM's own error (at least sqrt(K) u) on the same inputs; rows and columns scaled over
    1e-8 .. 1e8, one zero row."""
    rng = np.random.default_rng(M + 3 * N + 5 * K)
    Aop = rng.normal(size=(M, K)) * np.exp(rng.uniform(-18, 18, size=(M, 1)))
    Bop = rng.normal(size=(K, N)) * np.exp(rng.uniform(-18, 18, size=(1, N)))
    Aop[M // 2] = 0.0
    A = Aop if opA == "N" else Aop.T.copy()
    B = Bop if opB == "N" else Bop.T.copy()
    _lib.stats_reset()
    out = _gemm_f64tc(opA, opB, A, B, M, N, K)
    assert _lib.stats_read()["gemm_oz_launches"] == 1
    native = _gemm_fp64(opA, opB, A, B, M, N, K)
    ref = Aop @ Bop
    scale = np.abs(Aop) @ np.abs(Bop)
    scale = np.where(scale > 0, scale, 1.0)
    err = np.max(np.abs(out - ref) / scale)
    err_native = np.max(np.abs(native - ref) / scale)
    assert err < 8 * np.sqrt(K) * 2.0**-53, err
    # as accurate as an FP64 GEMM (whose own error can be 0 when it sums in
    # numpy's order, hence the sqrt(K) u floor)
    assert err <= 2 * max(err_native, np.sqrt(K) * 2.0**-53), (err, err_native)
    assert np.all(out[M // 2] == 0.0)


def test_fp64_tensor_core_gemm_cancellation():
    """A product with heavy cancellation (result far below |A||B|): the error
    stays at the FP64 level of |A||B|, as for an FP64 GEMM."""
    rng = np.random.default_rng(11)
    M, N, K = 256, 128, 512
    A = rng.normal(size=(M, K))
    X = rng.normal(size=(K, N))
    B = X - A.T @ np.linalg.solve(A @ A.T + 1e-3 * np.eye(M), A @ X)  # nearly A-orthogonal
    out = _gemm_f64tc("N", "N", A, B, M, N, K)
    native = _gemm_fp64("N", "N", A, B, M, N, K)
    ref = A @ B
    scale = np.abs(A) @ np.abs(B)
    err = np.max(np.abs(out - ref) / scale)
    assert err < 8 * np.sqrt(K) * 2.0**-53
    assert err <= 2 * max(np.max(np.abs(native - ref) / scale), np.sqrt(K) * 2.0**-53)


def _gemm_c(fn, opA, opB, A, B, M, N, K):
    Ad = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    Bd = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    Cd = torch.empty((M, N), dtype=torch.complex128, device="cuda")
    _lib.check(getattr(_lib.load(), fn)(
        _lib.context(), _lib.SM_COMPLEX128, OPS[opA], OPS[opB], M, N, K,
        C.c_void_p(Ad.data_ptr()), A.shape[1], C.c_void_p(Bd.data_ptr()), B.shape[1],
        C.c_void_p(Cd.data_ptr()), N, _lib.stream_handle()))
    torch.cuda.synchronize()
    return Cd.cpu().numpy()


def _cplx_case(M, N, K, opA, opB, seed, scaled=False):
    rng = np.random.default_rng(seed)
    Aop = rng.normal(size=(M, K)) + 1j * rng.normal(size=(M, K))
    Bop = rng.normal(size=(K, N)) + 1j * rng.normal(size=(K, N))
    if scaled:
        Aop *= np.exp(rng.uniform(-18, 18, size=(M, 1)))
        Bop *= np.exp(rng.uniform(-18, 18, size=(1, N)))
    # the stored operands whose op() is Aop / Bop
    stored = {"N": lambda x: x, "T": lambda x: x.T.copy(), "C": lambda x: x.conj().T.copy()}
    return Aop, Bop, stored[opA](Aop), stored[opB](Bop)


@pytest.mark.parametrize("opB", ["N", "T", "C"])
@pytest.mark.parametrize("opA", ["N", "T", "C"])
@pytest.mark.parametrize("M,N,K", [(256, 192, 320), (130, 70, 120)])
def test_complex_tensor_core_gemm_3m(M, N, K, opA, opB):
    """Complex products on split real planes as three real 3xTF32 tensor-core products (the 3M
    form): relative Frobenius error against numpy's complex128 product below 4e-6, every op
    pair, ragged shapes."""
    Aop, Bop, A, B = _cplx_case(M, N, K, opA, opB, M + N + K + 3 * OPS[opA] + OPS[opB])
    _lib.stats_reset()
    out = _gemm_c("sm_gemm_f32", opA, opB, A, B, M, N, K)
    assert _lib.stats_read()["gemm_tc_launches"] == 3
    ref = Aop @ Bop
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert rel < 4e-6, rel


@pytest.mark.parametrize("opB", ["N", "T", "C"])
@pytest.mark.parametrize("opA", ["N", "T", "C"])
@pytest.mark.parametrize("M,N,K", [(128, 96, 256), (225, 100, 300)])
def test_complex_fp64_tensor_core_gemm_3m(M, N, K, opA, opB):
    """Complex products as three FP64-accurate real tensor-core products: error normalised by
    |A||B| within 16 sqrt(K) u and within four times the FP64 SIMT complex GEMM's own error
    (at least sqrt(K) u), rows and columns scaled over 1e-8 .. 1e8."""
    Aop, Bop, A, B = _cplx_case(M, N, K, opA, opB, 7 * M + N + K + OPS[opA], scaled=True)
    _lib.stats_reset()
    out = _gemm_c("sm_gemm_f64tc", opA, opB, A, B, M, N, K)
    assert _lib.stats_read()["gemm_oz_launches"] == 3
    native = _gemm_c("sm_gemm", opA, opB, A, B, M, N, K)
    ref = Aop @ Bop
    scale = np.abs(Aop) @ np.abs(Bop)
    err = np.max(np.abs(out - ref) / scale)
    err_native = np.max(np.abs(native - ref) / scale)
    assert err < 16 * np.sqrt(K) * 2.0**-53, err
    assert err <= 4 * max(err_native, np.sqrt(K) * 2.0**-53), (err, err_native)


def test_complex_mixed_form_uses_tensor_cores():
    """The complex MPO.apply + simplify of the first configuration (n=20, chi=32, D=4,
    complex128, tolerance 1e-10, max bond 64) in the mixed form with FP32 contractions: its
    complex contractions run as 3M tensor-core products, and the result stays within 1e-10
    fidelity of the FP64 oracle."""
    rng = np.random.default_rng(102)
    n, chi, D = 20, 32, 4
    mps = so.random_mps(2, n, chi, rng, complex_=True)
    mps = so.scale(mps, 1.0 / np.sqrt(so.norm_squared(mps)))
    mpo = so.random_mpo(2, n, D, rng, complex_=True)
    kw = dict(tolerance=1e-10, max_bond_dimension=64, max_sweeps=2)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    sg.set_precision("mixed", contractions="fp32")
    _lib.stats_reset()
    try:
        out = sg.MPO(mpo, st).apply(sg.MPS(mps), strategy=st)
        stats = _lib.stats_read()
    finally:
        sg.set_precision("fp64")
    ref = so.mpo_apply(mpo, mps, so.DEFAULT_STRATEGY.replace(**kw))
    assert stats["gemm_tc_launches"] > 0, stats
    fe = so.fidelity_error(mps_np(out), ref.tensors)
    assert fe < 1e-10, fe
