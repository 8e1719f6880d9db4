"""Explicit ODE steppers for d|state>/dt = L|state> on the GPU path: the callers of the
MPO·MPS + simplify path in the reference's PDE workloads (evolution/common.py:17-76,
evolution/euler.py:10-98, evolution/runge_kutta.py:14-44).

Each step is the reference's sequence of ``MPO @ state`` products and ``simplify`` calls on
sums of states, written with this package's ``MPS`` / ``MPSSum`` arithmetic (a scalar times an
MPS scales its first tensor; a sum of states and sums flattens into one ``MPSSum``), so every
product and every simplification runs on the device through the library.
"""

from __future__ import annotations

from typing import Any, Callable

import numpy as np

from .core import DEFAULT_STRATEGY, Strategy
from .operators import MPO
from .state import MPS, simplify

ODEFunction = Callable[[float, MPS], MPS]
ODECallback = Callable[[float, MPS], Any]


def make_generalized_MPO(L) -> ODEFunction:
    """F(t, state) = L.apply(state) for an MPO, else L itself (evolution/common.py:18-29)."""
    if isinstance(L, MPO):
        def mpo_derivative(t: float, state: MPS) -> MPS:
            return L.apply(state)
        return mpo_derivative
    if callable(L):
        return L
    raise TypeError(f"expected an MPO or a callable (t, state) -> MPS, got {type(L).__name__}")


def ode_solver(evolve_for_dt, time, state, steps: int = 1000,
               strategy: Strategy = DEFAULT_STRATEGY, callback: ODECallback | None = None):
    """Common driver (evolution/common.py:32-73): ``time`` is a final time T (start 0), a pair
    (t0, t1) split into ``steps`` equal steps, or the sequence of times itself.  Calls
    ``evolve_for_dt(t, state, dt, strategy)`` for every new time and ``callback(t, state)`` at
    every time, the first included; returns the callback's values, or the final state."""
    if isinstance(time, (int, float)):
        time = (0.0, float(time))
    if isinstance(time, tuple):
        t_span = np.linspace(float(time[0]), float(time[1]), steps + 1, dtype=np.float64)
    else:
        t_span = np.asarray(time, dtype=np.float64)
    output = []
    last_t = t_span[0]
    for t in t_span:
        if t != last_t:
            state = evolve_for_dt(t, state, float(t - last_t), strategy)
        if callback:
            output.append(callback(t, state))
        last_t = t
    return output if callback else state


def euler(L: MPO, time, state: MPS, steps: int = 1000, strategy: Strategy = DEFAULT_STRATEGY,
          callback: ODECallback | None = None):
    """psi(t + dt) = psi(t) + dt L psi(t), simplified (evolution/euler.py:10-62)."""

    def evolve_for_dt(t, state, dt, strategy):
        return simplify(state + dt * (L @ state), strategy=strategy)

    return ode_solver(evolve_for_dt, time, state, steps, strategy, callback)


def euler2(L: MPO, time, state: MPS, steps: int = 1000, strategy: Strategy = DEFAULT_STRATEGY,
           callback: ODECallback | None = None):
    """Two-stage Euler (evolution/euler.py:65-98): xi = 2 psi + dt L psi, then
    psi(t + dt) = psi + (dt / 2) L xi, each simplified."""

    def evolve_for_dt(t, state, dt, strategy):
        xi = simplify(2.0 * state + dt * (L @ state), strategy=strategy)
        return simplify(state + (0.5 * dt) * (L @ xi), strategy=strategy)

    return ode_solver(evolve_for_dt, time, state, steps, strategy, callback)


def runge_kutta(L, time, state: MPS, steps: int = 1000, strategy: Strategy = DEFAULT_STRATEGY,
                callback: ODECallback | None = None):
    """Classical fourth-order Runge-Kutta (evolution/runge_kutta.py:14-44); ``L`` is an MPO or a
    callable F(t, state)."""
    GL = make_generalized_MPO(L)

    def evolve_for_dt(t, state, dt, strategy):
        h = dt
        k1 = GL(t, state)
        s2 = simplify(state + (0.5 * h) * k1, strategy=strategy)
        k2 = GL(t + dt / 2, s2)
        s3 = simplify(state + (0.5 * h) * k2, strategy=strategy)
        k3 = GL(t + dt / 2, s3)
        s4 = simplify(state + h * k3, strategy=strategy)
        k4 = GL(t + dt, s4)
        return simplify(state + (h / 6) * (k1 + 2 * k2 + 2 * k3 + k4), strategy=strategy)

    return ode_solver(evolve_for_dt, time, state, steps, strategy, callback)


__all__ = ["ode_solver", "make_generalized_MPO", "euler", "euler2", "runge_kutta"]
