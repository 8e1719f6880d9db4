"""The rest of the reference's kernel table on the GPU against the oracle: _canonicalize,
_recanonicalize, _update_in_canonical_form_right/left (cython/schmidt.pxi:18-120),
_contract_nrjl_ijk_klm (cython/contractions.pxi:102-127), AntilinearForm.tensor1site /
tensor2site (state/antilinear.py:59-98), simplify / simplify_mps_sum with a guess
(state/simplification.py:36,93-98,214-219), MPOList.apply and join (operators/mpo.py:585-711)
and simplify_mpo (operators/simplify_mpo.py:50-89).  Gauge-free comparisons: kept ranks,
errors, reconstructed products and fidelities."""

import numpy as np
import pytest

from oracle import seemps_oracle as so
from tests.gpu_util import mps_np, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import seemps2_gb300 as sg  # noqa: E402
from seemps2_gb300 import kernel_table as kt  # noqa: E402


def _state(n, chi, cplx, seed):
    rng = np.random.default_rng(seed)
    psi = so.random_mps(2, n, chi, rng, complex_=cplx)
    return so.scale(psi, 1.0 / np.sqrt(so.norm_squared(psi))), rng


def _dense(tensors):
    return so.to_vector([to_np(t) if isinstance(t, torch.Tensor) else np.asarray(t)
                         for t in tensors])


@pytest.mark.parametrize("cplx", [False, True])
@pytest.mark.parametrize("center", [0, 3, 7])
def test_canonicalize_and_recanonicalize_in_place(cplx, center):
    psi, _ = _state(8, 12, cplx, 31 + center)
    st = sg.DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=10)
    ost = so.DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=10)
    g = list(psi)
    o = [A.copy() for A in psi]
    err = kt._canonicalize(g, center, st)
    oerr = so.canonicalize(o, center, ost)
    assert [t.shape for t in g] == [A.shape for A in o]
    assert abs(err - oerr) <= 1e-10 * max(1.0, oerr)
    assert so.fidelity_error([to_np(t) for t in g], o) < 1e-12
    # move the centre to the other end and back
    for newc in (7 - center, center):
        err = kt._recanonicalize(g, center if newc != center else 7 - center, newc, st)
        oerr = so.recanonicalize(o, center if newc != center else 7 - center, newc, ost)
        assert [t.shape for t in g] == [A.shape for A in o]
        assert abs(err - oerr) <= 1e-10 * max(1.0, oerr)
        assert so.fidelity_error([to_np(t) for t in g], o) < 1e-12
    # the centre site holds the norm, the rest are isometries
    for i, t in enumerate(g):
        x = to_np(t)
        if i < center:
            m = x.reshape(-1, x.shape[2])
            assert np.allclose(m.conj().T @ m, np.eye(m.shape[1]), atol=1e-12)
        elif i > center:
            m = x.reshape(x.shape[0], -1)
            assert np.allclose(m @ m.conj().T, np.eye(m.shape[0]), atol=1e-12)


@pytest.mark.parametrize("cplx", [False, True])
def test_update_in_canonical_form(cplx):
    psi, rng = _state(6, 8, cplx, 41)
    st = sg.DEFAULT_STRATEGY.replace(tolerance=1e-6, max_bond_dimension=5)
    ost = so.DEFAULT_STRATEGY.replace(tolerance=1e-6, max_bond_dimension=5)
    g = list(psi)
    o = [A.copy() for A in psi]
    site, err = kt._update_in_canonical_form_right(g, psi[2], 2, st)
    oerr = so.update_canonical_right(o, psi[2], 2, ost)
    assert site == 3 and abs(err - oerr) <= 1e-10 * max(1.0, oerr)
    assert to_np(g[2]).shape == o[2].shape and to_np(g[3]).shape == o[3].shape
    assert np.allclose(_dense(g), _dense(o), atol=1e-12)
    site, err = kt._update_in_canonical_form_left(g, g[3], 3, st)
    oerr = so.update_canonical_left(o, o[3], 3, ost)
    assert site == 2 and abs(err - oerr) <= 1e-10 * max(1.0, oerr)
    assert np.allclose(_dense(g), _dense(o), atol=1e-12)
    # the ends store the tensor as given
    site, err = kt._update_in_canonical_form_right(g, g[5], 5, st)
    assert (site, err) == (5, 0.0)
    site, err = kt._update_in_canonical_form_left(g, g[0], 0, st)
    assert (site, err) == (0, 0.0)


@pytest.mark.parametrize("cplx", [False, True])
def test_contract_nrjl_ijk_klm(cplx):
    rng = np.random.default_rng(5)

    def r(*s):
        x = rng.normal(size=s)
        return x + 1j * rng.normal(size=s) if cplx else x

    for (a, d, b, e, c) in [(1, 2, 3, 2, 1), (7, 2, 9, 2, 5), (40, 2, 33, 3, 17)]:
        U, A, B = r(d * e, d * e), r(a, d, b), r(b, e, c)
        ref = np.einsum("ijk,klm,nrjl -> inrm", A, B, U.reshape(d, e, d, e))
        out = to_np(kt._contract_nrjl_ijk_klm(U, A, B))
        assert np.allclose(out, ref, atol=1e-12 * np.abs(ref).max())
        assert np.allclose(out, so.contract_nrjl_ijk_klm(U, A, B), atol=1e-12 * np.abs(ref).max())
    with pytest.raises(ValueError):
        kt._contract_nrjl_ijk_klm(r(3, 3), r(2, 2, 2), r(2, 2, 2))


@pytest.mark.parametrize("cplx", [False, True])
def test_antilinear_form_tensors(cplx):
    bra, rng = _state(7, 6, cplx, 51)
    ket = so.random_mps(2, 7, 9, rng, complex_=cplx)
    for center in (0, 3):
        g = sg.AntilinearForm(sg.MPS(bra), sg.MPS(ket), center=center)
        o = so.AntilinearForm(bra, ket, center=center)
        assert np.allclose(to_np(g.tensor1site()), o.tensor1site(), atol=1e-12)
        for direction in (+1, -1):
            if (direction < 0 and center == 0):
                continue
            assert np.allclose(to_np(g.tensor2site(direction)), o.tensor2site(direction),
                               atol=1e-12)
        g.update_right()
        o.update_right()
        assert np.allclose(to_np(g.tensor2site(+1)), o.tensor2site(+1), atol=1e-12)
        g.update_left()
        o.update_left()
        assert np.allclose(to_np(g.tensor1site()), o.tensor1site(), atol=1e-12)


@pytest.mark.parametrize("cplx", [False, True])
def test_simplify_with_guess(cplx):
    psi, rng = _state(10, 16, cplx, 61)
    guess = so.random_mps(2, 10, 5, rng, complex_=cplx)
    kw = dict(tolerance=1e-10, max_bond_dimension=12, max_sweeps=3, simplification_tolerance=0.0)
    st, ost = sg.DEFAULT_STRATEGY.replace(**kw), so.DEFAULT_STRATEGY.replace(**kw)
    out = sg.simplify(sg.MPS(psi), st, guess=sg.MPS(guess))
    ref = so.simplify(psi, ost, guess=[A.copy() for A in guess])
    assert out.bond_dimensions()[:-1] == [A.shape[0] for A in ref.tensors]
    assert so.fidelity_error(mps_np(out), ref.tensors) < 1e-12
    assert abs(out.error() ** 2 - ref.error ** 2) <= 1e-13 + 1e-8 * ref.error ** 2
    # a sum with a guess
    phi = so.random_mps(2, 10, 8, rng, complex_=cplx)
    w = [0.7, -0.3 + (0.2j if cplx else 0.0)]
    outs = sg.simplify(sg.MPSSum(w, [sg.MPS(psi), sg.MPS(phi)]), st, guess=sg.MPS(guess))
    refs = so.simplify_mps_sum(w, [psi, phi], ost, guess=[A.copy() for A in guess])
    assert outs.bond_dimensions()[:-1] == [A.shape[0] for A in refs.tensors]
    assert so.fidelity_error(mps_np(outs), refs.tensors) < 1e-12


def test_simplify_guess_larger_than_state():
    """A guess whose bonds exceed the state's: the buffers are sized for it."""
    psi, rng = _state(8, 4, False, 71)
    guess = so.random_mps(2, 8, 16, rng)
    st = sg.DEFAULT_STRATEGY.replace(tolerance=1e-12, max_bond_dimension=16, max_sweeps=2,
                                     simplification_tolerance=0.0)
    ost = so.DEFAULT_STRATEGY.replace(tolerance=1e-12, max_bond_dimension=16, max_sweeps=2,
                                      simplification_tolerance=0.0)
    out = sg.simplify(sg.MPS(psi), st, guess=sg.MPS(guess))
    ref = so.simplify(psi, ost, guess=[A.copy() for A in guess])
    assert out.bond_dimensions()[:-1] == [A.shape[0] for A in ref.tensors]
    assert so.fidelity_error(mps_np(out), ref.tensors) < 1e-12


@pytest.mark.parametrize("cplx", [False, True])
def test_mpolist_apply_and_join(cplx):
    psi, rng = _state(8, 8, cplx, 81)
    mpos = [so.random_mpo(2, 8, 3, rng, complex_=cplx), so.random_mpo(2, 8, 2, rng, complex_=cplx)]
    kw = dict(tolerance=1e-10, max_bond_dimension=20, max_sweeps=2, simplification_tolerance=0.0)
    st, ost = sg.DEFAULT_STRATEGY.replace(**kw), so.DEFAULT_STRATEGY.replace(**kw)
    ol = sg.MPOList([sg.MPO(m, st) for m in mpos], st)
    out = ol.apply(sg.MPS(psi))
    # the reference: each MPO applied with its own strategy (simplifying), then one simplify
    x = psi
    for m in mpos:
        x = so.mpo_apply(m, x, ost).tensors
    ref = so.simplify(x, ost)
    assert out.bond_dimensions()[:-1] == [A.shape[0] for A in ref.tensors]
    assert so.fidelity_error(mps_np(out), ref.tensors) < 1e-12
    # @ is apply
    assert so.fidelity_error(mps_np(ol @ sg.MPS(psi)), ref.tensors) < 1e-12
    # join: one MPO of bond 6 acting as the product
    J = ol.join()
    oj = so.mpo_join(mpos)
    for a, b in zip(J, oj):
        assert np.allclose(to_np(a), b, atol=1e-12)
    v = so.to_vector(psi)
    M0 = sg.MPO(mpos[0]).to_matrix().cpu().numpy()
    M1 = sg.MPO(mpos[1]).to_matrix().cpu().numpy()
    assert np.allclose(J.to_matrix().cpu().numpy() @ v, M1 @ (M0 @ v), atol=1e-11)


def test_simplify_mpo():
    rng = np.random.default_rng(91)
    n = 8
    m1 = so.random_mpo(2, n, 3, rng)
    m2 = so.random_mpo(2, n, 3, rng)
    st = sg.MPO_SIMPLIFICATION_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=6,
                                                max_sweeps=2, simplification_tolerance=0.0)
    ost = so.SIMPLIFICATION_STRATEGY.replace(normalize=False, tolerance=1e-10,
                                             max_bond_dimension=6, max_sweeps=2,
                                             simplification_tolerance=0.0)
    out = sg.simplify_mpo(sg.MPOList([sg.MPO(m1), sg.MPO(m2)]), st)
    ref, res = so.simplify_mpo(so.mpo_join([m1, m2]), ost)
    assert [int(t.shape[0]) for t in out] == [A.shape[0] for A in ref]
    as_vec = lambda ts: so.to_vector([np.asarray(t).reshape(t.shape[0], -1, t.shape[-1]) for t in ts])
    g = as_vec([to_np(t) for t in out])
    r = as_vec(ref)
    assert np.linalg.norm(g - r) <= 1e-10 * np.linalg.norm(r)
    # with a guess
    guess = so.random_mpo(2, n, 2, rng)
    out = sg.simplify_mpo(sg.MPO(m1), st, guess=sg.MPO(guess))
    ref, _ = so.simplify_mpo(m1, ost, guess=guess)
    assert [int(t.shape[0]) for t in out] == [A.shape[0] for A in ref]
    assert np.linalg.norm(as_vec([to_np(t) for t in out]) - as_vec(ref)) <= 1e-10 * np.linalg.norm(as_vec(ref))
