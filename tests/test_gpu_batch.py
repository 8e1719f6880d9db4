"""Batched MPO.apply + simplify (seemps2_gb300.batch) on instances of uneven length, bond and MPO
bond with complex64 storage: every result equals the FP64 oracle's (same bonds, fidelity error below
1e-12), results are bit-identical whatever the number of instances in flight, the stream autotuner
returns one of its candidates, and an instance's error reaches the caller."""

import numpy as np
import pytest

from oracle import seemps_oracle as so
from tests.gpu_util import mps_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import seemps2_gb300 as sg  # noqa: E402
from seemps2_gb300 import batch  # noqa: E402


def _instances(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(6, 13))
        chi = int(rng.choice([4, 8, 16]))
        D = int(rng.choice([2, 3]))
        mps = [t.astype(np.complex64) for t in so.random_mps(2, n, chi, rng, complex_=True)]
        nrm = np.sqrt(abs(so.scprod(mps, mps)))
        mps[0] = (mps[0] / nrm).astype(np.complex64)
        mpo = [t.astype(np.complex64) for t in so.random_mpo(2, n, D, rng, complex_=True)]
        out.append((mps, mpo, chi))
    return out


def _kw(chi):
    return dict(tolerance=1e-8, max_bond_dimension=chi, max_sweeps=2, simplification_tolerance=0.0)


def test_batch_matches_oracle():
    inst = _instances(10, 5)
    mpos = [sg.MPO(mpo, sg.DEFAULT_STRATEGY.replace(**_kw(chi))) for mps, mpo, chi in inst]
    states = [sg.MPS(mps) for mps, mpo, chi in inst]
    res, rep = batch.apply_batch(mpos, states, streams=4)
    assert len(rep.latencies_s) == 10 and rep.wall_s > 0
    for (mps, mpo, chi), out in zip(inst, res):
        ref = so.mpo_apply([t.astype(np.complex128) for t in mpo],
                           [t.astype(np.complex128) for t in mps],
                           so.DEFAULT_STRATEGY.replace(**_kw(chi)))
        assert out.bond_dimensions() == [A.shape[0] for A in ref.tensors] + [1]
        assert so.fidelity_error(mps_np(out), ref.tensors) < 1e-12


def test_batch_results_do_not_depend_on_streams():
    inst = _instances(8, 6)
    mpos = [sg.MPO(mpo, sg.DEFAULT_STRATEGY.replace(**_kw(chi))) for mps, mpo, chi in inst]
    states = [sg.MPS(mps) for mps, mpo, chi in inst]
    r1, _ = batch.apply_batch(mpos, states, streams=1)
    r8, _ = batch.apply_batch(mpos, states, streams=8)
    for a, b in zip(r1, r8):
        assert a.bond_dimensions() == b.bond_dimensions()
        for x, y in zip(mps_np(a), mps_np(b)):
            assert np.array_equal(x, y)


def test_stream_autotuner():
    inst = _instances(12, 7)
    mpos = [sg.MPO(mpo, sg.DEFAULT_STRATEGY.replace(**_kw(chi))) for mps, mpo, chi in inst]
    states = [sg.MPS(mps) for mps, mpo, chi in inst]
    best, table = batch.tune_streams(mpos, states, candidates=(1, 2, 4), sample=12)
    assert best in (1, 2, 4)
    assert set(table) == {1, 2, 4} and all(v > 0 for v in table.values())


def test_batch_reports_an_instance_error():
    inst = _instances(3, 8)
    mpos = [sg.MPO(mpo) for mps, mpo, chi in inst]
    states = [sg.MPS(mps) for mps, mpo, chi in inst]
    wrong = so.random_mps(2, len(inst[1][1]) + 1, 4, np.random.default_rng(9))
    states[1] = sg.MPS(wrong)  # one site longer than its MPO
    with pytest.raises(ValueError):
        batch.apply_batch(mpos, states, streams=2)
