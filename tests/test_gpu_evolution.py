"""ODE steppers (seemps2_gb300.evolution) on the GPU against the oracle: the same sequence of
products and sum simplifications as the reference's euler / euler2 / runge_kutta
(evolution/euler.py:10-98, runge_kutta.py:14-44), restated with the oracle's mpo_apply and
simplify_mps_sum (a scalar times a state scales its first tensor, as MPS.__mul__ does).  Bar:
fidelity error < 1e-10 and identical bonds after each run."""

import numpy as np
import pytest

from oracle import seemps_oracle as so

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import seemps2_gb300 as sg  # noqa: E402
from seemps2_gb300 import evolution  # noqa: E402

from tests.gpu_util import mps_np  # noqa: E402


def _setup(n=8, chi=8, seed=17):
    rng = np.random.default_rng(seed)
    psi = so.random_mps(2, n, chi, rng)
    psi = so.scale(psi, 1.0 / np.sqrt(so.norm_squared(psi)))
    mpo = so.tridiagonal_mpo(n, -2.0, 1.0, 1.0)
    kw = dict(tolerance=1e-12, max_bond_dimension=16, max_sweeps=2, simplification_tolerance=0.0)
    return psi, mpo, so.DEFAULT_STRATEGY.replace(**kw), sg.DEFAULT_STRATEGY.replace(**kw)


def _o_apply(mpo, x, st):
    return so.mpo_apply(mpo, x, st).tensors


def _o_sum(pairs, st):
    """simplify of sum_i states_i scaled by c_i (each scaling applied to the state's first
    tensor, the sum's weights all 1)."""
    states = [so.scale(x, c) if c != 1.0 else x for c, x in pairs]
    return so.simplify_mps_sum([1.0] * len(states), states, st).tensors


def _oracle(rule, mpo, x, dt, steps, st):
    for _ in range(steps):
        if rule == "euler":
            x = _o_sum([(1.0, x), (dt, _o_apply(mpo, x, st))], st)
        elif rule == "euler2":
            xi = _o_sum([(2.0, x), (dt, _o_apply(mpo, x, st))], st)
            x = _o_sum([(1.0, x), (0.5 * dt, _o_apply(mpo, xi, st))], st)
        else:
            h = dt
            k1 = _o_apply(mpo, x, st)
            k2 = _o_apply(mpo, _o_sum([(1.0, x), (0.5 * h, k1)], st), st)
            k3 = _o_apply(mpo, _o_sum([(1.0, x), (0.5 * h, k2)], st), st)
            k4 = _o_apply(mpo, _o_sum([(1.0, x), (h, k3)], st), st)
            # state + (h/6) (k1 + 2 k2 + 2 k3 + k4): k2, k3 scaled by 2 first, then the sum's
            # weights h/6 (the package's MPSSum keeps them as weights; here they scale)
            states = [x, so.scale(k1, h / 6), so.scale(so.scale(k2, 2), h / 6),
                      so.scale(so.scale(k3, 2), h / 6), so.scale(k4, h / 6)]
            x = so.simplify_mps_sum([1.0] * 5, states, st).tensors
    return x


@pytest.mark.parametrize("rule", ["euler", "euler2", "runge_kutta"])
def test_stepper_matches_oracle(rule):
    psi, mpo, ost, gst = _setup()
    dt, steps = 0.01, 2
    L = sg.MPO(mpo, gst)
    out = getattr(evolution, rule)(L, (0.0, dt * steps), sg.MPS(psi), steps=steps, strategy=gst)
    ref = _oracle(rule, mpo, psi, dt, steps, ost)
    got = mps_np(out)
    assert [A.shape[0] for A in got] == [A.shape[0] for A in ref]
    fe = so.fidelity_error(got, ref)
    assert fe < 1e-10, fe
