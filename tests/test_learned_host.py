"""Host side of the learned rank predictor (no GPU): the training workloads
reach the benchmark's scale, and the packaged model file is complete.

A model trained only on small workloads (bond caps up to 128) predicted ranks
near 90 for the benchmark's rank-256 splits, whose bond-cap feature lay outside
its data; the generator therefore mixes in Laplacian steps of the benchmark's
own scale (n 16..30, chi 128..256), one in every 25 workloads.
"""

import os

import numpy as np

from seemps2_gb300 import learned


def test_training_workloads_reach_the_benchmark_scale():
    rng = np.random.default_rng(0)
    caps, large = [], 0
    for c, (mps, mpo, kw) in enumerate(learned.training_workloads(rng, 100)):
        caps.append(kw["max_bond_dimension"])
        bond = max(A.shape[2] for A in mps[:-1])
        if c % 25 == 24:
            large += 1
            assert kw["max_bond_dimension"] in (128, 192, 256)
            assert kw["tolerance"] == 1e-12 and 16 <= len(mps) <= 30
            assert bond <= kw["max_bond_dimension"]
            assert len(mpo) == len(mps) and mpo[0].shape[-1] == 3  # the Laplacian, bond 3
    assert large == 4
    assert max(caps) >= 192


def test_packaged_model_file():
    z = np.load(learned.PACKAGED_MODEL)
    dims = tuple(int(d) for d in z["dims"])
    assert dims == learned.DIMS
    n = sum(dims[k] * dims[k + 1] + dims[k + 1] for k in range(len(dims) - 1))
    assert z["params"].shape == (n,) and np.all(np.isfinite(z["params"]))
    assert z["mean"].shape == (dims[0],) and np.all(z["std"] > 0)
    assert int(z["truncations"]) >= 200_000 and int(z["workloads"]) >= 4000
    assert os.path.getsize(learned.PACKAGED_MODEL) < 2 * 1024 * 1024
