"""DMRG two-site effective-Hamiltonian matvec (sm_two_site_matvec and the prepared
sm_two_site_matvec_prepared) against the oracle's
restatement of QuadraticForm.two_site_operator._matvec, at every precision, and the Lanczos
solver against a dense eigensolver.  Bars (relative Frobenius error of the matvec): FP64 and
FP64-accurate tensor cores 1e-13, 3xTF32 1e-5, BF16 2e-2; Lanczos lowest eigenvalue 1e-10
(FP64) and 2e-2 (BF16)."""

import numpy as np
import pytest

from oracle import dmrg_oracle as do
from oracle import seemps_oracle as so

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from seemps2_gb300 import dmrg  # noqa: E402

BARS = {"fp64": 1e-13, "fp64tc": 1e-13, "tf32x3": 1e-5, "bf16": 2e-2}


def _random_block(a, c, b, p, e, g, f, rng, cplx=False):
    def r(*s):
        x = rng.normal(size=s)
        return x + 1j * rng.normal(size=s) if cplx else x
    L = r(a, c, b)
    O1 = r(c, p, p, 5)
    O2 = r(5, p, p, e)
    H = do.two_site_hamiltonian(O1, O2)
    R = r(g, e, f)
    v = r(b, p, p, f)
    return L, H, R, v


@pytest.mark.parametrize("precision", ["fp64", "fp64tc", "tf32x3", "bf16"])
@pytest.mark.parametrize("dims", [(64, 5, 64, 2, 5, 64, 64), (200, 3, 150, 2, 4, 130, 170),
                                  (256, 5, 256, 2, 5, 256, 256)])
def test_matvec_matches_oracle(precision, dims):
    a, c, b, p, e, g, f = dims
    rng = np.random.default_rng(sum(dims))
    L, H, R, v = _random_block(a, c, b, p, e, g, f, rng)
    out = dmrg.two_site_matvec(L, H, R, v, precision).cpu().numpy()
    ref = do.two_site_matvec(L, H, R, v)
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert rel < BARS[precision], rel


@pytest.mark.parametrize("precision", ["tf32x3", "bf16"])
@pytest.mark.parametrize("dims", [(64, 5, 64, 2, 5, 64, 64), (200, 3, 150, 2, 4, 130, 170),
                                  (256, 5, 256, 2, 5, 256, 256), (130, 5, 100, 2, 5, 70, 90)])
def test_prepared_matvec_matches_oracle(precision, dims):
    """The prepared operator (environments as tensor-core planes once, FP32 X1 and MPO step) at
    the same bars; several matvecs of one operator, and two operators alternating (each matvec
    after the other's prepares its own planes again)."""
    a, c, b, p, e, g, f = dims
    rng = np.random.default_rng(sum(dims) + 1)
    L, H, R, v = _random_block(a, c, b, p, e, g, f, rng)
    L2, H2, R2, v2 = _random_block(a, c, b, p, e, g, f, rng)
    op = dmrg.TwoSiteOperator(L, H, R, precision)
    op2 = dmrg.TwoSiteOperator(L2, H2, R2, precision)
    for _ in range(2):
        for o, (Lx, Hx, Rx, vx) in ((op, (L, H, R, v)), (op2, (L2, H2, R2, v2))):
            out = o.matvec(vx).cpu().numpy()
            ref = do.two_site_matvec(Lx, Hx, Rx, vx)
            rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
            assert rel < BARS[precision], rel


def test_prepared_rejects_fp64():
    rng = np.random.default_rng(5)
    L, H, R, v = _random_block(64, 5, 64, 2, 5, 64, 64, rng)
    with pytest.raises(ValueError):
        dmrg.TwoSiteOperator(L, H, R, "fp64")


def test_complex_matvec_fp64():
    rng = np.random.default_rng(3)
    L, H, R, v = _random_block(40, 4, 36, 2, 3, 44, 30, rng, cplx=True)
    out = dmrg.two_site_matvec(L, H, R, v, "fp64").cpu().numpy()
    ref = do.two_site_matvec(L, H, R, v)
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-13


def _heisenberg_block(n, site, chi, rng):
    """L, H, R of sites (site, site+1) of an n-site Heisenberg chain around a random real MPS."""
    W = do.heisenberg_mpo(n)
    psi = so.random_mps(2, n, chi, rng)
    L = do.begin_mpo_environment()
    for i in range(site):
        L = do.update_left_mpo_environment(L, psi[i], W[i], psi[i])
    R = do.begin_mpo_environment()
    for i in range(n - 1, site + 1, -1):
        R = do.update_right_mpo_environment(R, psi[i], W[i], psi[i])
    H = do.two_site_hamiltonian(W[site], W[site + 1])
    return L, H, R, psi


@pytest.mark.parametrize("precision,bar", [("fp64", 1e-10), ("bf16", 2e-2)])
def test_lanczos_lowest_eigenvalue(precision, bar):
    rng = np.random.default_rng(11)
    L, H, R, psi = _heisenberg_block(10, 4, 8, rng)
    M = do.dense_operator(L, H, R)
    M = 0.5 * (M + M.T)
    e0 = np.linalg.eigvalsh(M)[0]
    b, f = L.shape[2], R.shape[2]
    v0 = rng.normal(size=(b, 2, 2, f))
    ev, vec, steps = dmrg.lanczos_ground_state(L, H, R, v0, krylov=min(60, v0.size),
                                               precision=precision)
    assert abs(ev - e0) <= bar * abs(e0), (ev, e0)
    if precision == "fp64":
        x = vec.cpu().numpy().reshape(-1)
        r = M @ x - ev * x
        assert np.linalg.norm(r) <= 1e-6 * abs(ev)
