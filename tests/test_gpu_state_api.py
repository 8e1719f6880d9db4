"""State utilities around the path, after the reference's state/mps.py and
state/mpssum.py: MPS.reverse / to_tensor / norm2, MPSSum.conj / reverse /
join_canonical and MPSSum.delete_zero_components (mpssum.py:204-228, the
term pruning that simplify applies to sums), checked against dense vectors."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import seemps2_gb300 as sg  # noqa: E402


def _vec(x):
    return x.to_vector().detach().cpu().numpy()


def _mps(n, D, cplx, seed):
    return sg.random_uniform_mps(2, n, D=D, complex=cplx, rng=np.random.default_rng(seed))


def test_mps_reverse_and_to_tensor():
    psi = _mps(6, 4, True, 1)
    t = psi.to_tensor().detach().cpu().numpy()
    assert t.shape == (2,) * 6
    r = psi.reverse()
    assert r.bond_dimensions() == psi.bond_dimensions()[::-1]
    assert np.allclose(r.to_tensor().detach().cpu().numpy(), t.transpose(tuple(range(5, -1, -1))),
                       rtol=1e-13, atol=1e-13 * np.abs(t).max())
    with pytest.warns(DeprecationWarning):
        assert psi.norm2() == psi.norm_squared()


def test_sum_conj_reverse_join_canonical():
    a, b = _mps(5, 3, True, 2), _mps(5, 2, False, 3)
    s = sg.MPSSum([0.5 + 1j, -2.0], [a, b])
    v = _vec(a) * (0.5 + 1j) - 2.0 * _vec(b)
    assert np.allclose(_vec(s.conj()), np.conj(v), atol=1e-13 * np.abs(v).max())
    vr = v.reshape((2,) * 5).transpose(tuple(range(4, -1, -1))).reshape(-1)
    assert np.allclose(_vec(s.reverse()), vr, atol=1e-13 * np.abs(v).max())
    c = s.join_canonical(center=2)
    assert isinstance(c, sg.CanonicalMPS) and c.center == 2
    assert np.allclose(_vec(c), v, atol=1e-12 * np.abs(v).max())


def test_delete_zero_components():
    a, b, c = _mps(5, 3, False, 4), _mps(5, 2, True, 5), _mps(5, 3, False, 6)
    s = sg.MPSSum([1.0, 0.0, 2.0 - 1j, 0.7], [a, b, c, a.zero_state()])
    v = _vec(a) + (2.0 - 1j) * _vec(c)
    n2 = s.delete_zero_components()
    assert len(s.states) == 2 and s.states[0] is a and s.states[1] is c
    assert s.weights == [1.0, 2.0 - 1j]
    assert abs(n2 - np.vdot(v, v).real) <= 1e-12 * np.vdot(v, v).real
    # nothing left: the sum becomes 0 * zero state
    z = sg.MPSSum([0.0, 1.0], [a, b.zero_state()])
    assert z.delete_zero_components() == 0.0
    assert z.weights == [0.0] and z.states[0].bond_dimensions() == [1] * 6
