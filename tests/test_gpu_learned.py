"""The learned rank predictor: GPU kernels against the CPU oracle, recording,
and what the trained network gains over the method without it.

Bars: forward within 1e-5 (relative, FP32 vs the FP64 oracle), gradients
within 1e-4 of the largest gradient entry, one Adam step within 1e-6, BF16
inference within 0.05 (relative) of the FP32 network; the trained network's
mean |error| in log2 rank below the no-network baseline's (the previous
split's rank); mixed+learned MPO.apply within 1e-10 fidelity of the FP64
oracle with the predicted-rank cap in use.
"""

import numpy as np
import pytest

from oracle import mlp_oracle as mo
from oracle import seemps_oracle as so
from tests.gpu_util import mps_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import seemps2_gb300 as sg  # noqa: E402
from seemps2_gb300 import _lib, learned  # noqa: E402

DIMS = (37, 64, 48, 1)


def _model(seed=3, dims=DIMS):
    p = mo.init_params(dims, np.random.default_rng(seed))
    return learned.RankModel(dims, params=p), p


def test_forward_matches_oracle():
    m, p = _model()
    X = np.random.default_rng(4).normal(size=(33, DIMS[0])).astype(np.float32)
    y_gpu, _ = m.forward(torch.from_numpy(X).cuda())
    y_ref, _ = mo.forward(p.astype(np.float32).astype(np.float64), DIMS, X.astype(np.float64))
    y_gpu = y_gpu.cpu().numpy()
    assert np.max(np.abs(y_gpu - y_ref.reshape(-1))) <= 1e-5 * max(1.0, np.abs(y_ref).max())


@pytest.mark.parametrize("batch", [1, 17, 256])
def test_gradients_match_oracle(batch):
    m, p = _model()
    rng = np.random.default_rng(5)
    X = rng.normal(size=(batch, DIMS[0])).astype(np.float32)
    y = rng.normal(size=batch).astype(np.float32)
    loss, g = m.loss_and_grad(torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda())
    p64 = p.astype(np.float32).astype(np.float64)
    yhat, cache = mo.forward(p64, DIMS, X.astype(np.float64))
    l_ref, dy = mo.mse(yhat, y.astype(np.float64))
    g_ref = mo.backward(p64, DIMS, X.astype(np.float64), cache, dy)
    assert abs(float(loss.item()) - l_ref) <= 1e-5 * max(1.0, l_ref)
    g = g.cpu().numpy()
    assert np.max(np.abs(g - g_ref)) <= 1e-4 * np.abs(g_ref).max()


def test_adam_step_matches_oracle():
    rng = np.random.default_rng(6)
    n = 1000
    p = rng.normal(size=n).astype(np.float32)
    g = rng.normal(size=n).astype(np.float32)
    m = (0.1 * rng.normal(size=n)).astype(np.float32)
    v = np.abs(rng.normal(size=n)).astype(np.float32)
    dev = [torch.from_numpy(x.copy()).cuda() for x in (p, g, m, v)]
    _lib.check(_lib.load().sm_adam_step(_lib.context(), dev[0].data_ptr(), dev[1].data_ptr(),
                                        dev[2].data_ptr(), dev[3].data_ptr(), n, 1e-3, 0.9, 0.999,
                                        1e-8, 7, _lib.stream_handle()))
    pr, mr, vr = (x.astype(np.float64) for x in (p, m, v))
    mo.adam_step(pr, g.astype(np.float64), mr, vr, 1e-3, 0.9, 0.999, 1e-8, 7)
    assert np.max(np.abs(dev[0].cpu().numpy() - pr)) <= 1e-6
    assert np.max(np.abs(dev[2].cpu().numpy() - mr)) <= 1e-6


def test_bf16_inference_matches_fp32_network():
    dims = learned.DIMS
    m, p = _model(seed=8, dims=dims)
    rng = np.random.default_rng(9)
    X = rng.normal(size=(64, dims[0])).astype(np.float32) * 3.0 + 1.0
    m.mean = X.mean(axis=0)
    m.std = X.std(axis=0) + 1e-3
    m.install()
    y = m.predict_log2(X)
    y_ref, _ = mo.forward(p.astype(np.float32).astype(np.float64), dims,
                          ((X - m.mean) / m.std).astype(np.float64))
    assert np.max(np.abs(y - y_ref.reshape(-1))) <= 0.05 * max(1.0, np.abs(y_ref).max())


def test_records_every_split_with_its_rank():
    rng = np.random.default_rng(2)
    mps = so.random_mps(2, 10, 16, rng)
    mpo = so.random_mpo(2, 10, 3, rng)
    st = sg.DEFAULT_STRATEGY.replace(tolerance=1e-8, max_bond_dimension=24, max_sweeps=2,
                                     simplification_tolerance=0.0)
    with _lib.SplitTrace() as tr, learned.record_truncations() as rec:
        sg.MPO(mpo, st).apply(sg.MPS(mps), strategy=st)
    assert rec.X.shape == (len(tr.ranks), 37)
    assert rec.D.tolist() == tr.ranks
    # the previous-rank feature is log2(1 + the previous split's rank) within a
    # sweep call (each call starts from 0)
    chained = rec.X[1:, 34] > 0
    assert chained.sum() >= len(tr.ranks) // 2
    assert np.allclose(rec.X[1:, 34][chained], np.log2(1.0 + rec.D[:-1][chained]))


@pytest.fixture(scope="module")
def trained():
    X, D = learned.record_dataset(count=45, seed=11)
    model = learned.RankModel.initial(seed=1)
    hist = model.fit(X, D, epochs=30)
    Xt, Dt = learned.record_dataset(count=15, seed=12)
    return model, hist, Xt, Dt


def test_trained_network_beats_the_baseline(trained):
    model, hist, Xt, Dt = trained
    assert hist[-1] < 0.25 * hist[0]
    model.install()
    y = np.log2(np.maximum(Dt, 1))
    err_net = np.mean(np.abs(model.predict_log2(Xt) - y))
    err_base = np.mean(np.abs(learned.baseline_log2(Xt) - y))
    assert err_net < err_base, (err_net, err_base)


def test_packaged_network_beats_the_baseline(trained):
    """The predictor shipped in seemps2_gb300/data (trained on ~200k truncations of
    the FP64 method) loads, and on held-out workloads its mean |error| in log2
    rank is below the no-network baseline's and below 0.1 (7 % in the rank)."""
    import os

    *_, Xt, Dt = trained
    assert os.path.exists(learned.PACKAGED_MODEL)
    z = np.load(learned.PACKAGED_MODEL)
    assert int(z["truncations"]) >= 200_000
    model = learned.RankModel.load(learned.PACKAGED_MODEL)
    model.install()
    y = np.log2(np.maximum(Dt, 1))
    err_net = np.mean(np.abs(model.predict_log2(Xt) - y))
    err_base = np.mean(np.abs(learned.baseline_log2(Xt) - y))
    assert err_net < err_base and err_net < 0.1, (err_net, err_base)


def test_mixed_learned_apply_matches_oracle(trained):
    model, *_ = trained
    model.install()
    rng = np.random.default_rng(7)
    n, chi = 14, 64
    mps, mpo = learned.laplacian_case(n, chi, rng)
    kw = dict(tolerance=1e-12, max_bond_dimension=chi, max_sweeps=2, simplification_tolerance=0.0)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    sg.set_precision("mixed+learned")
    _lib.stats_reset()
    try:
        out = sg.MPO(mpo, st).apply(sg.MPS(mps), strategy=st)
        stats = _lib.stats_read()
    finally:
        sg.set_precision("fp64")
    res = so.mpo_apply(mpo, mps, so.DEFAULT_STRATEGY.replace(**kw))
    info = {k: stats[k] for k in ("mixed_splits", "mixed_capped", "mixed_fallbacks",
                                  "mixed_cap_redone", "mixed_fallback_fp32",
                                  "mixed_fallback_cut", "rank_predicted_sum")}
    assert stats["mixed_capped"] > 5, info
    # caps that left weight behind are redone without the cap, not counted as FP64 fallbacks
    assert stats["mixed_fallbacks"] <= 0.3 * stats["mixed_capped"], info
    fe = so.fidelity_error(mps_np(out), res.tensors)
    assert fe < 1e-10, fe


def test_device_prediction_matches_host_features(trained):
    """The learned form predicts on the device (features from the previous
    split's values kept on the device, the network, the cap) with no host round
    trip.  Recording the same apply gives the host-side features of every
    split: the network on those (host side) must give the same ranks, summed
    over the splits that take the learned path (min(m, n) >= 24), as the device
    path reported."""
    model, *_ = trained
    model.install()
    rng = np.random.default_rng(8)
    n, chi = 14, 64
    mps, mpo = learned.laplacian_case(n, chi, rng)
    kw = dict(tolerance=1e-12, max_bond_dimension=chi, max_sweeps=2, simplification_tolerance=0.0)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    sg.set_precision("mixed+learned")
    _lib.stats_reset()
    try:
        with learned.record_truncations() as rec:
            sg.MPO(mpo, st).apply(sg.MPS(mps), strategy=st)
        stats = _lib.stats_read()
    finally:
        sg.set_precision("fp64")
    k = np.round(np.exp2(rec.X[:, 35].astype(np.float64)))  # log2 min(m, n), stored in float32
    take = k >= 24
    r = np.clip(np.ceil(np.exp2(model.predict_log2(rec.X[take]).astype(np.float64))), 1, k[take])
    assert stats["rank_predictions"] == int(take.sum()) > 5
    # the feature logarithms are taken on the device there and on the host here: a
    # last-bit difference may move a rank by one now and then
    assert abs(stats["rank_predicted_sum"] - int(r.sum())) <= max(2, 0.002 * r.sum()), (
        stats["rank_predicted_sum"], r.sum())


def _workload_split(rng, m, n):
    """A numerically rank-deficient m x n matrix with the spectrum of the n=30, chi=256
    workload's splits: 256 values from 1 to 3e-3, two more near 2.5e-3, then zeros."""
    s = np.concatenate([np.geomspace(1.0, 3e-3, 256), [2.5e-3, 2.4e-3]])
    Qa, _ = np.linalg.qr(rng.normal(size=(m, len(s))))
    Qb, _ = np.linalg.qr(rng.normal(size=(n, len(s))))
    return (Qa * s) @ Qb.T


@pytest.mark.parametrize("power_iters", [0, 1])
def test_range_finder_captures_the_numerical_range(power_iters):
    """sm_range_finder on a rank-258 512 x 480 matrix at k = 266: the 258 singular values of
    BH = W^T Q above the rounding level equal W's within 1e-7 s_max without subspace
    iterations (the Cholesky shift costs the sketch's worst-conditioned directions some
    orthonormality) and within 1e-9 s_max with one; the 8 directions beyond the rank stay
    below 1e-7 s_max; |BH|_F^2 = |W|_F^2 to 1e-8 relative.  The split refines its vectors
    against the exact matrix, so the sketch needs only this much."""
    import ctypes as C  # noqa: F401

    rng = np.random.default_rng(21)
    m, n, k = 512, 480, 266
    A = _workload_split(rng, m, n)
    Ad = torch.from_numpy(A).cuda()
    for want_u in (0, 1):
        W = A.T if want_u else A
        BH = torch.empty((W.shape[1], k), dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().sm_range_finder(_lib.context(), _lib.ptr(Ad), m, n, want_u, k,
                                               power_iters, _lib.ptr(BH), _lib.stream_handle()))
        sb = np.linalg.svd(BH.cpu().numpy(), compute_uv=False)
        sw = np.linalg.svd(W, compute_uv=False)[:k]
        bar = 1e-7 if power_iters == 0 else 1e-9
        assert np.max(np.abs(sb[:258] - sw[:258])) <= bar * sw[0], (power_iters, want_u)
        assert np.max(sb[258:]) <= 1e-7 * sw[0], (power_iters, want_u, sb[258:])
        assert abs(np.sum(sb**2) - np.sum(sw**2)) <= 1e-8 * np.sum(sw**2)


@pytest.mark.parametrize("shape", [(512, 512), (768, 512), (512, 768)])
def test_range_finder_split_matches_oracle(shape):
    """Two-site splits of workload-shaped matrices through the learned form's range finder
    (rank hint 256, k = 266): the kept rank, the discarded weight and the truncated product
    agree with the oracle's (relative-norm tolerance 1e-12, max bond 256; the product within
    1e-5 relative, i.e. fidelity 1e-10 as for the other mixed splits; sqrt(discarded weight)
    within 1e-8); the split runs the
    range finder and falls back to neither the full QR nor FP64."""
    from seemps2_gb300 import core

    rng = np.random.default_rng(sum(shape))
    m, n = shape
    AA = _workload_split(rng, m, n).reshape(m // 2, 2, 2, n // 2)
    st = sg.Strategy(tolerance=1e-12, max_bond_dimension=256)
    ost = so.Strategy(tolerance=1e-12, max_bond_dimension=256)
    for gpu_fn, ora_fn in [(core._left_orth_2site, so.left_orth_2site),
                           (core._right_orth_2site, so.right_orth_2site)]:
        sg.set_precision("mixed+learned", range_finder=True, rank_hint=256)
        _lib.stats_reset()
        try:
            L, R, err = gpu_fn(AA, st)
            stats = _lib.stats_read()
        finally:
            sg.set_precision("fp64")
        Lo, Ro, erro = ora_fn(AA, ost)
        info = {k: stats[k] for k in ("rf_splits", "mixed_fallbacks", "mixed_cap_redone",
                                      "mixed_fallback_cut", "mixed_fallback_over")}
        assert stats["rf_splits"] == 1 and stats["mixed_fallbacks"] == 0, info
        assert stats["mixed_cap_redone"] == 0, info
        D = L.shape[-1]
        assert D == Lo.shape[-1]
        rec = L.cpu().numpy().reshape(-1, D) @ R.cpu().numpy().reshape(D, -1)
        reco = Lo.reshape(-1, D) @ Ro.reshape(D, -1)
        assert np.linalg.norm(rec - reco) <= 1e-5 * np.linalg.norm(reco)
        assert abs(err - erro) <= 1e-8 * max(1.0, erro)


def test_range_finder_apply_matches_oracle(trained):
    """The learned form with the range finder sized by the trained predictor: MPO.apply of
    the Laplacian within 1e-10 fidelity of the FP64 oracle; splits whose subspace missed
    weight are redone with the full QR."""
    model, *_ = trained
    model.install()
    rng = np.random.default_rng(7)
    n, chi = 14, 64
    mps, mpo = learned.laplacian_case(n, chi, rng)
    kw = dict(tolerance=1e-12, max_bond_dimension=chi, max_sweeps=2, simplification_tolerance=0.0)
    st = sg.DEFAULT_STRATEGY.replace(**kw)
    sg.set_precision("mixed+learned", range_finder=True)
    _lib.stats_reset()
    try:
        out = sg.MPO(mpo, st).apply(sg.MPS(mps), strategy=st)
        stats = _lib.stats_read()
    finally:
        sg.set_precision("fp64")
    res = so.mpo_apply(mpo, mps, so.DEFAULT_STRATEGY.replace(**kw))
    assert stats["rf_splits"] > 5, stats
    fe = so.fidelity_error(mps_np(out), res.tensors)
    assert fe < 1e-10, fe
