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


@pytest.mark.parametrize("cplx", [False, True])
def test_mpo_environments_match_oracle(cplx):
    rng = np.random.default_rng(21 + cplx)

    def r(*s):
        x = rng.normal(size=s)
        return x + 1j * rng.normal(size=s) if cplx else x

    for (a, j, d, c, e, b, f) in [(1, 2, 3, 1, 5, 1, 4), (9, 2, 12, 5, 5, 7, 10),
                                  (64, 2, 48, 3, 4, 40, 56)]:
        A, O, B = r(a, j, d), r(c, j, j, e), r(b, j, f)
        rho = r(a, c, b)
        got = dmrg.update_left_mpo_environment(rho, A, O, B).cpu().numpy()
        ref = do.update_left_mpo_environment(rho, A, O, B)
        assert np.allclose(got, ref, atol=1e-12 * np.abs(ref).max())
        rho = r(d, e, f)
        got = dmrg.update_right_mpo_environment(rho, A, O, B).cpu().numpy()
        ref = do.update_right_mpo_environment(rho, A, O, B)
        assert np.allclose(got, ref, atol=1e-12 * np.abs(ref).max())


def _fixture(name):
    import json
    import os

    z = np.load(os.path.join(os.path.dirname(__file__), "golden", f"{name}.npz"))
    W = [z[f"W{i}"] for i in range(sum(1 for k in z.files if k.startswith("W")))]
    return z, W, json.loads(bytes(z["meta"]).decode())["params"]


def test_matvec_and_environments_match_reference_fixture():
    """The reference's own QuadraticForm (HeisenbergHamiltonian(10).to_mpo(), a bond-8 state
    centred at site 4): its L, H12, R and one two_site_operator matvec, against the
    device's environments built from the same state and the device matvec."""
    import seemps2_gb300 as sg

    z, W, p = _fixture("dmrg_matvec_L10")
    i = p["site"]
    state = [z[f"A{k}"] for k in range(p["L"])]
    out = dmrg.two_site_matvec(z["L"], z["H12"], z["R"], z["v"], "fp64").cpu().numpy()
    assert np.allclose(out, z["out"], atol=1e-12 * np.abs(z["out"]).max())
    psi = sg.CanonicalMPS(state, center=i, is_canonical=True)
    QF = dmrg.QuadraticForm(sg.MPO(W), psi, start=i)
    L, H12, R = QF.two_site_block(i)
    assert np.allclose(L.cpu().numpy(), z["L"], atol=1e-12)
    assert np.allclose(R.cpu().numpy(), z["R"], atol=1e-12)
    assert np.allclose(H12.cpu().numpy(), z["H12"], atol=1e-14)


def test_dmrg_matches_reference_run():
    """Two DMRG sweeps of an L=10 Heisenberg chain from a seeded bond-4 guess (tolerance
    1e-10, max bond 32): the energy after each sweep within 1e-9 of the reference's run,
    the same bond dimensions, and the final state's overlap with the reference's to 1e-8."""
    import importlib.util
    import os

    import seemps2_gb300 as sg

    z, W, p = _fixture("dmrg_run_L10")
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(__file__), "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    guess = mg.make_dmrg_inputs(p)
    st = sg.DEFAULT_STRATEGY.replace(tolerance=p["tol"], max_bond_dimension=p["maxchi"])
    res = dmrg.dmrg(sg.MPO(W), guess=sg.MPS(guess), maxiter=p["maxiter"], tol=1e-14, strategy=st)
    traj = np.array(res.trajectory)
    assert traj.shape == z["trajectory"].shape
    assert np.max(np.abs(traj - z["trajectory"])) <= 1e-9 * max(1.0, abs(z["energy"]))
    assert abs(res.energy - float(z["energy"])) <= 1e-9 * max(1.0, abs(z["energy"]))
    assert res.state.bond_dimensions() == z["bonds"].tolist()
    v = res.state.to_vector().cpu().numpy().reshape(-1)
    ref = z["vector"].reshape(-1)
    ov = abs(np.vdot(ref, v)) / (np.linalg.norm(ref) * np.linalg.norm(v))
    assert 1.0 - ov <= 1e-8, 1.0 - ov


@pytest.mark.parametrize("precision", ["bf16", "tf32x3"])
def test_dmrg_reduced_precision_matches_fp64(precision):
    """The reduced-precision Lanczos (BF16 or 3xTF32 matvecs, FP64 polish of each eigenpair)
    reaches the FP64 run's energy."""
    import seemps2_gb300 as sg

    z, W, p = _fixture("dmrg_run_L10")
    rng = np.random.default_rng(7)
    guess = so.random_mps(2, p["L"], 4, rng)
    st = sg.DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=32)
    e64 = dmrg.dmrg(sg.MPO(W), guess=sg.MPS(guess), maxiter=2, tol=1e-14, strategy=st).energy
    er = dmrg.dmrg(sg.MPO(W), guess=sg.MPS(guess), maxiter=2, tol=1e-14, strategy=st,
                   precision=precision).energy
    assert abs(er - e64) <= 1e-8 * abs(e64), (er, e64)
