"""Helpers shared by the GPU tests (device <-> numpy, comparisons)."""

import numpy as np


def to_np(t):
    return t.detach().cpu().numpy()


def mps_np(mps):
    return [to_np(t) for t in mps._data]


def sv_close(s_gpu, s_ref, rel=1e-10):
    """Singular values within rel * s_max (the normwise relative accuracy of gesdd)."""
    s_gpu = np.asarray(s_gpu)
    s_ref = np.asarray(s_ref)
    assert s_gpu.shape == s_ref.shape, (s_gpu.shape, s_ref.shape)
    if s_ref.size == 0:
        return
    scale = max(float(s_ref[0]), 1e-300)
    assert np.max(np.abs(s_gpu - s_ref)) <= rel * scale, np.max(np.abs(s_gpu - s_ref)) / scale
