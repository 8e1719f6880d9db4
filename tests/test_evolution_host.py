"""Host logic of the ODE steppers (seemps2_gb300.evolution) without a GPU: the time-span rules
of ode_solver (evolution/common.py:32-73) and the stepping formulas of euler, euler2 and
runge_kutta (evolution/euler.py, runge_kutta.py), checked with stand-in vector states that follow
the package's arithmetic (a scalar times a state is a state, sums flatten) and an exact
``simplify`` against the same formulas in plain NumPy on dx/dt = A x."""

import numpy as np
import pytest

evolution = pytest.importorskip("seemps2_gb300.evolution")


class Vec:
    """Stand-in for an MPS: a scalar times it scales it; adding gives a Sum."""

    def __init__(self, x):
        self.x = np.asarray(x, dtype=float)

    def __add__(self, o):
        return Sum([(1.0, self)]) + o

    def __mul__(self, n):
        return Vec(n * self.x)

    __rmul__ = __mul__


class Sum:
    """Stand-in for an MPSSum: weighted terms, flattened on addition and scaling."""

    def __init__(self, terms):
        self.terms = list(terms)

    def __add__(self, o):
        if isinstance(o, Vec):
            return Sum(self.terms + [(1.0, o)])
        return Sum(self.terms + o.terms)

    def __mul__(self, n):
        return Sum([(n * w, s) for w, s in self.terms])

    __rmul__ = __mul__


class Op:
    def __init__(self, A):
        self.A = A

    def __matmul__(self, v):
        return Vec(self.A @ v.x)


def exact_simplify(state, strategy=None):
    if isinstance(state, Vec):
        return state
    return Vec(sum(w * s.x for w, s in state.terms))


@pytest.fixture
def system(monkeypatch):
    monkeypatch.setattr(evolution, "simplify", exact_simplify)
    rng = np.random.default_rng(3)
    A = rng.normal(size=(5, 5)) / 5
    x0 = rng.normal(size=5)
    return A, x0


def np_steps(A, x, dts, rule):
    for dt in dts:
        if rule == "euler":
            x = x + dt * (A @ x)
        elif rule == "euler2":
            xi = 2 * x + dt * (A @ x)
            x = x + 0.5 * dt * (A @ xi)
        else:
            k1 = A @ x
            k2 = A @ (x + 0.5 * dt * k1)
            k3 = A @ (x + 0.5 * dt * k2)
            k4 = A @ (x + dt * k3)
            x = x + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
    return x


@pytest.mark.parametrize("rule", ["euler", "euler2", "runge_kutta"])
def test_steppers_follow_the_formulas(system, rule):
    A, x0 = system
    if rule == "runge_kutta":
        out = evolution.runge_kutta(lambda t, s: Vec(A @ s.x), (0.0, 0.3), Vec(x0), steps=3)
        ref = np_steps(A, x0, [0.1] * 3, "rk4")
    else:
        out = getattr(evolution, rule)(Op(A), (0.0, 0.3), Vec(x0), steps=3)
        ref = np_steps(A, x0, [0.1] * 3, rule)
    assert np.allclose(out.x, ref, rtol=1e-13, atol=1e-14)


def test_time_span_forms_and_callback(system):
    A, x0 = system
    seen = []

    def cb(t, s):
        seen.append(t)
        return s.x.copy()

    # a final time: start at 0, `steps` equal steps, the callback at every time
    vals = evolution.euler(Op(A), 0.2, Vec(x0), steps=4, callback=cb)
    assert np.allclose(seen, np.linspace(0, 0.2, 5)) and len(vals) == 5
    assert np.allclose(vals[0], x0)
    assert np.allclose(vals[-1], np_steps(A, x0, [0.05] * 4, "euler"))
    # an explicit sequence of times, unequal steps
    times = [0.0, 0.1, 0.15, 0.3]
    out = evolution.euler(Op(A), times, Vec(x0))
    assert np.allclose(out.x, np_steps(A, x0, [0.1, 0.05, 0.15], "euler"))


def test_generalized_mpo_rejects_other_types():
    with pytest.raises(TypeError):
        evolution.make_generalized_MPO(3.0)
