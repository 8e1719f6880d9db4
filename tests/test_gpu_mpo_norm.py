"""<O a|O b> from the MPO and MPS factors (sm_mpo_scprod) against the oracle's
scprod of the product states, and MPO.apply, whose state norm now comes from
the factors (sm_simplify_gram), against the oracle: the norm within 1e-13
relative, identical kept ranks, fidelity error below 1e-12."""

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
from seemps2_gb300 import state as sg_state  # noqa: E402


def _mpo(n, dout, din, D, rng, cplx):
    out = []
    for i in range(n):
        Dl = 1 if i == 0 else D
        Dr = 1 if i == n - 1 else D
        T = rng.normal(size=(Dl, dout, din, Dr))
        if cplx:
            T = T + 1j * rng.normal(size=T.shape)
        out.append(T / np.sqrt(D * din))
    return out


def _product(O, a):
    return [so.mpo_multiply_tensor(o, t) for o, t in zip(O, a)]


@pytest.mark.parametrize("n,dout,din,D,chi_a,chi_b,cplx", [
    (1, 2, 2, 1, 1, 1, False),
    (2, 2, 2, 3, 4, 2, False),
    (7, 2, 2, 3, 16, 16, False),
    (8, 3, 3, 4, 12, 5, True),
    (9, 2, 2, 2, 32, 24, True),
    (6, 3, 2, 3, 8, 8, False),   # rectangular MPO: output 3, input 2
])
def test_mpo_scprod_matches_product_scprod(n, dout, din, D, chi_a, chi_b, cplx):
    rng = np.random.default_rng(100 + n + D)
    a = so.random_mps(din, n, chi_a, rng, cplx)
    b = so.random_mps(din, n, chi_b, rng, cplx)
    O = _mpo(n, dout, din, D, rng, cplx)
    Oa, Ob = _product(O, a), _product(O, b)
    ref = so.scprod(Oa, Ob)
    got = sg.mpo_scprod(sg.MPO(O), sg.MPS(a), sg.MPS(b))
    scale = np.sqrt(so.norm_squared(Oa) * so.norm_squared(Ob))
    assert abs(got - ref) <= 1e-13 * scale, (got, ref)
    # the same state on both sides: the norm of the product
    nn = sg.mpo_scprod(sg.MPO(O), sg.MPS(a), sg.MPS(a))
    assert abs(nn - so.norm_squared(Oa)) <= 1e-13 * so.norm_squared(Oa)


def test_mpo_scprod_rejects_open_bonds():
    rng = np.random.default_rng(1)
    a = so.random_mps(2, 4, 4, rng)
    O = _mpo(4, 2, 2, 3, rng, False)
    O[0] = np.concatenate([O[0], O[0]], axis=0)  # left MPO bond 2
    with pytest.raises(Exception):
        sg.mpo_scprod(sg.MPO(O), sg.MPS(a), sg.MPS(a))


@pytest.mark.parametrize("cplx", [False, True])
def test_apply_state_norm_from_factors(cplx):
    rng = np.random.default_rng(21)
    n, chi = 12, 24
    mps = so.random_mps(2, n, chi, rng, cplx)
    mpo = so.random_mpo(2, n, 3, rng, cplx)
    kw = dict(tolerance=1e-10, max_bond_dimension=chi, max_sweeps=3, simplification_tolerance=0.0)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    with _lib.SplitTrace() as tr:
        out = sg.MPO(mpo, st).apply(sg.MPS(mps), strategy=st)
    norm_gpu = sg_state.last_report["norm_state_sqr"]
    rec = so.Recorder()
    res = so.mpo_apply(mpo, mps, so.DEFAULT_STRATEGY.replace(**kw), rec=rec)
    norm_ref = so.norm_squared(_product(mpo, mps))
    assert abs(norm_gpu - norm_ref) <= 1e-13 * norm_ref
    assert tr.ranks == [sp.rank for sp in rec.splits]
    assert so.fidelity_error(mps_np(out), res.tensors) < 1e-12
    e1, e2 = out.error() ** 2, res.error ** 2
    assert abs(e1 - e2) <= 1e-13 + 1e-8 * e2


def test_apply_to_sum_with_complex_and_zero_weights():
    rng = np.random.default_rng(22)
    n, chi = 10, 12
    states = [so.random_mps(2, n, chi, rng) for _ in range(3)]
    weights = [0.7, -0.3j, 0.0]
    mpo = so.random_mpo(2, n, 3, rng)
    kw = dict(tolerance=1e-10, max_bond_dimension=2 * chi, max_sweeps=3,
              simplification_tolerance=0.0)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    out = sg.MPO(mpo, st).apply(sg.MPSSum(weights, [sg.MPS(s) for s in states]), strategy=st)
    norm_gpu = sg_state.last_report["norm_state_sqr"]
    # the reference: sum_i (w_i O s_i) with the weight in the first tensor
    prods = [so.scale(_product(mpo, s), w) for w, s in zip(weights, states)]
    res = so.simplify_mps_sum([1.0] * 3, prods, so.DEFAULT_STRATEGY.replace(**kw))
    norm_ref = so.mpssum_norm_squared([1.0] * 3, prods)[0]
    assert abs(norm_gpu - norm_ref) <= 1e-13 * norm_ref
    assert out.bond_dimensions() == [A.shape[0] for A in res.tensors] + [1]
    assert so.fidelity_error(mps_np(out), res.tensors) < 1e-12
