"""Learned kept-rank predictor for the mixed-precision splits.

A small MLP (``dims`` = SM_RANK_FEATURES -> 256 -> 256 -> 256 -> 1, GELU) maps
the features of a split (the previous split's leading singular values, the
site position, the tolerance, the previous kept rank, the split size and the
bond cap) to log2 of the rank the split keeps.  It is trained on the GPU with
the library's own kernels (``sm_mlp_forward`` / ``sm_mlp_backward`` /
``sm_mse_loss`` / ``sm_adam_step``) on truncations that the FP64 method records
(``sm_rank_features_record``).  Installed with :meth:`RankModel.install` and
``set_precision("mixed+learned")``, each mixed split stops its FP32
rank-revealing QR after ceil(1.15 r) + 10 steps (r the predicted rank) instead
of waiting for the trailing weight to fall below the noise-level threshold; a
split whose capped QR left weight behind is redone without the cap, and the
exact discarded weight still sends tolerance violations to the FP64 Jacobi
SVD.

Input standardisation is folded into the first layer when the model is
installed, so the device sees raw features.
"""

from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import _lib

DIMS = (_lib.RANK_FEATURES, 256, 256, 256, 1)

# The predictor shipped with the package: trained on the GPU with the library's
# kernels on truncations recorded by the FP64 method (``python -m
# seemps2_gb300.learned --out ... --count 4300``; its record counts are stored
# in the file).
PACKAGED_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "rank_model.npz")


def _torch():
    import torch

    return torch


def _dims_arr(dims):
    return (C.c_int * len(dims))(*dims)


class RankModel:
    """MLP parameters on the GPU (FP32) plus the feature standardisation."""

    def __init__(self, dims=DIMS, params: np.ndarray | None = None):
        torch = _torch()
        self.dims = tuple(int(d) for d in dims)
        self.L = len(self.dims) - 1
        n = _lib.load().sm_mlp_param_count(self.L, _dims_arr(self.dims))
        if n < 0:
            raise ValueError(_lib.load().sm_last_error().decode())
        if params is None:
            raise ValueError("RankModel needs parameters: use RankModel.initial() or RankModel.load()")
        self.params = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float32)).cuda()
        if self.params.numel() != n:
            raise ValueError(f"expected {n} parameters for dims {self.dims}")
        self.mean = np.zeros(self.dims[0], np.float32)
        self.std = np.ones(self.dims[0], np.float32)

    # -- construction ------------------------------------------------------------
    @classmethod
    def initial(cls, dims=DIMS, seed: int = 0) -> "RankModel":
        """Uniform(+-1/sqrt(fan_in)) initialisation from a seeded generator."""
        rng = np.random.default_rng(seed)
        parts = []
        for k in range(len(dims) - 1):
            bound = 1.0 / np.sqrt(dims[k])
            parts.append(rng.uniform(-bound, bound, size=dims[k + 1] * dims[k]))
            parts.append(rng.uniform(-bound, bound, size=dims[k + 1]))
        return cls(dims, params=np.concatenate(parts))

    @classmethod
    def load(cls, path: str) -> "RankModel":
        z = np.load(path)
        m = cls(tuple(int(d) for d in z["dims"]), params=z["params"])
        m.mean, m.std = z["mean"].astype(np.float32), z["std"].astype(np.float32)
        return m

    def save(self, path: str, **meta) -> None:
        np.savez(path, dims=np.array(self.dims), params=self.params.cpu().numpy(),
                 mean=self.mean, std=self.std, **meta)

    # -- kernels -----------------------------------------------------------------
    def forward(self, X):
        """Outputs (batch,) and the training cache for a standardised-feature
        batch X (torch, cuda, float32)."""
        torch = _torch()
        B = X.shape[0]
        lib = _lib.load()
        ncache = lib.sm_mlp_cache_count(self.L, _dims_arr(self.dims), B)
        cache = torch.empty(ncache, dtype=torch.float32, device="cuda")
        Y = torch.empty(B, self.dims[-1], dtype=torch.float32, device="cuda")
        _lib.check(lib.sm_mlp_forward(_lib.context(), self.L, _dims_arr(self.dims),
                                      self.params.data_ptr(), X.data_ptr(), B, Y.data_ptr(),
                                      cache.data_ptr(), _lib.stream_handle()))
        return Y.reshape(-1), cache

    def loss_and_grad(self, X, y):
        """(loss tensor[1], grads) of the mean squared error on (X, y)."""
        torch = _torch()
        lib = _lib.load()
        B = X.shape[0]
        Y, cache = self.forward(X)
        dY = torch.empty_like(Y)
        loss = torch.empty(1, dtype=torch.float32, device="cuda")
        _lib.check(lib.sm_mse_loss(_lib.context(), Y.data_ptr(), y.data_ptr(), B, dY.data_ptr(),
                                   loss.data_ptr(), _lib.stream_handle()))
        grads = torch.empty_like(self.params)
        _lib.check(lib.sm_mlp_backward(_lib.context(), self.L, _dims_arr(self.dims),
                                       self.params.data_ptr(), X.data_ptr(), B, cache.data_ptr(),
                                       dY.data_ptr(), grads.data_ptr(), _lib.stream_handle()))
        return loss, grads

    def fit(self, X: np.ndarray, D: np.ndarray, epochs: int = 60, batch: int = 512,
            lr: float = 1e-3, seed: int = 0):
        """Adam on log2(D); returns the per-epoch mean loss."""
        torch = _torch()
        lib = _lib.load()
        X = np.asarray(X, np.float32)
        self.mean = X.mean(axis=0)
        self.std = X.std(axis=0) + 1e-3
        Xs = torch.from_numpy((X - self.mean) / self.std).cuda()
        y = torch.from_numpy(
            np.log2(np.maximum(np.asarray(D, np.float64), 1.0)).astype(np.float32)).cuda()
        m = torch.zeros_like(self.params)
        v = torch.zeros_like(self.params)
        rng = np.random.default_rng(seed)
        n = Xs.shape[0]
        batch = min(batch, n)
        step, hist = 0, []
        for _ in range(epochs):
            perm = torch.from_numpy(rng.permutation(n)).cuda()
            tot = torch.zeros(1, dtype=torch.float32, device="cuda")
            nb = 0
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                loss, g = self.loss_and_grad(Xs[idx].contiguous(), y[idx].contiguous())
                step += 1
                _lib.check(lib.sm_adam_step(_lib.context(), self.params.data_ptr(), g.data_ptr(),
                                            m.data_ptr(), v.data_ptr(), self.params.numel(), lr,
                                            0.9, 0.999, 1e-8, step, _lib.stream_handle()))
                tot += loss
                nb += 1
            hist.append(float(tot.item()) / max(nb, 1))
        return hist

    # -- deployment ----------------------------------------------------------------
    def device_params(self):
        """Parameters with the standardisation folded into the first layer."""
        torch = _torch()
        p = self.params.detach().clone()
        n0, n1 = self.dims[0], self.dims[1]
        W = p[: n1 * n0].view(n1, n0)
        b = p[n1 * n0: n1 * n0 + n1]
        inv = torch.from_numpy(1.0 / self.std).cuda()
        mu = torch.from_numpy(self.mean).cuda()
        W.mul_(inv[None, :])
        b.sub_(W @ mu)
        return p

    def install(self) -> None:
        """Hand the model to the library for SM_PRECISION_MIXED_LEARNED."""
        p = self.device_params()
        _torch().cuda.synchronize()
        _lib.check(_lib.load().sm_rank_model_set(_lib.context(), self.L, _dims_arr(self.dims),
                                                 p.data_ptr()))

    def predict_log2(self, X: np.ndarray) -> np.ndarray:
        """log2 rank predicted for raw feature rows X by the installed (BF16) model."""
        X = np.ascontiguousarray(X, np.float32)
        out = np.empty(X.shape[0], np.float32)
        _lib.check(_lib.load().sm_rank_predict(_lib.context(), X.ctypes.data, X.shape[0],
                                               out.ctypes.data, _lib.stream_handle()))
        return out


class record_truncations:
    """Context manager: every split made inside records (features, kept rank)."""

    def __enter__(self):
        _lib.check(_lib.load().sm_rank_features_record(_lib.context(), 1))
        self.X = self.D = None
        return self

    def __exit__(self, *exc):
        lib = _lib.load()
        n = C.c_int()
        _lib.check(lib.sm_rank_features_read(_lib.context(), None, None, 0, C.byref(n)))
        X = np.empty((n.value, _lib.RANK_FEATURES), np.float32)
        D = np.empty(n.value, np.int32)
        _lib.check(lib.sm_rank_features_read(_lib.context(), X.ctypes.data, D.ctypes.data,
                                             n.value, C.byref(n)))
        _lib.check(lib.sm_rank_features_record(_lib.context(), 0))
        self.X, self.D = X, D
        return False


# ---- training workloads --------------------------------------------------------
def tridiagonal_mpo(n, a, b, c):
    """Bond-3 MPO of a x + b S x + c S^T x on n qubits, S the periodic shift
    (the table of analysis/derivatives/finite_differences.py:9-38, closed)."""
    A = np.zeros((3, 2, 2, 3))
    A[0, 0, 0, 0] = A[0, 1, 1, 0] = 1.0
    A[0, 1, 0, 1] = A[1, 0, 1, 1] = 1.0
    A[2, 1, 0, 2] = A[0, 0, 1, 2] = 1.0
    R = a * A[:, :, :, [0]] + b * A[:, :, :, [1]] + c * A[:, :, :, [2]]
    left = A[[0], :, :, :] + A[[1], :, :, :] + A[[2], :, :, :]
    return [np.ascontiguousarray(x) for x in [left] + [A] * (n - 2) + [R]]


def laplacian_case(n, chi, rng):
    """Random MPS of bond chi (QR-orthonormalised, normalised) and the
    second-difference MPO with h = 2^-n."""
    mps, carry, DR = [], np.eye(1), 1
    for i in range(n):
        DL, DR = DR, min(chi, 2 ** min(i + 1, n - 1 - i))
        A = np.tensordot(carry, rng.normal(size=(DL, 2, DR)), axes=1)
        a, d, b = A.shape
        if i < n - 1:
            Q, R = np.linalg.qr(A.reshape(a * d, b))
            mps.append(np.ascontiguousarray(Q.reshape(a, d, Q.shape[1])))
            carry = R
        else:
            mps.append(A / np.linalg.norm(A))
    h = 2.0 ** (-n)
    return mps, tridiagonal_mpo(n, -2.0 / h**2, 1.0 / h**2, 1.0 / h**2)


def random_case(n, chi, D, rng, cplx):
    """Random MPS (bond chi) and random MPO (bond D, entries N(0,1)/sqrt(2 D))."""
    def rnd(*shape):
        x = rng.normal(size=shape)
        return x + 1j * rng.normal(size=shape) if cplx else x
    mps, DR = [], 1
    for i in range(n):
        DL, DR = DR, min(chi, 2 ** min(i + 1, n - 1 - i))
        mps.append(rnd(DL, 2, DR))
    mpo = []
    for i in range(n):
        Dl = 1 if i == 0 else D
        Dr = 1 if i == n - 1 else D
        mpo.append(rnd(Dl, 2, 2, Dr) / np.sqrt(D * 2))
    return mps, mpo


def training_workloads(rng, count: int):
    """(mps, mpo, strategy kwargs) with the shapes the benchmarks use: Laplacian
    steps (tol 1e-12, max bond chi), random complex MPS x MPO (tol 1e-10, max
    bond 2 chi), random real (tol 1e-8), mostly small; every 25th workload is a
    Laplacian step of the benchmark's own scale (n 16..30, chi 128..256), so
    that the bond caps and ranks of the timed workload lie inside the data."""
    for c in range(count):
        kind = c % 3
        if c % 25 == 24:
            n = int(rng.integers(16, 31))
            chi = int(rng.choice([128, 192, 256]))
            mps, mpo = laplacian_case(n, chi, rng)
            kw = dict(tolerance=1e-12, max_bond_dimension=chi, max_sweeps=2,
                      simplification_tolerance=0.0)
        elif kind == 0:
            n = int(rng.integers(10, 24))
            chi = int(rng.choice([16, 32, 64, 96]))
            mps, mpo = laplacian_case(n, chi, rng)
            kw = dict(tolerance=1e-12, max_bond_dimension=chi, max_sweeps=2,
                      simplification_tolerance=0.0)
        elif kind == 1:
            n = int(rng.integers(10, 20))
            chi = int(rng.choice([8, 16, 32]))
            mps, mpo = random_case(n, chi, 4, rng, True)
            kw = dict(tolerance=1e-10, max_bond_dimension=2 * chi, max_sweeps=2,
                      simplification_tolerance=0.0)
        else:
            n = int(rng.integers(10, 30))
            chi = int(rng.choice([8, 16, 32, 64]))
            mps, mpo = random_case(n, chi, int(rng.choice([2, 4])), rng, False)
            kw = dict(tolerance=1e-8, max_bond_dimension=2 * chi, max_sweeps=2,
                      simplification_tolerance=0.0)
        yield mps, mpo, kw


def record_dataset(count: int = 60, seed: int = 1):
    """Run the FP64 method on ``count`` training workloads, recording every split."""
    from . import state
    from .operators import MPO

    rng = np.random.default_rng(seed)
    Xs, Ds = [], []
    for mps, mpo, kw in training_workloads(rng, count):
        st = state.DEFAULT_STRATEGY.replace(**kw)
        nrm = np.sqrt(state.MPS(mps).norm_squared())
        psi = state.MPS([mps[0] / nrm] + mps[1:]) if nrm > 0 else state.MPS(mps)
        with record_truncations() as rec:
            MPO(mpo, st).apply(psi, strategy=st)
        Xs.append(rec.X)
        Ds.append(rec.D)
    return np.concatenate(Xs), np.concatenate(Ds)


def baseline_log2(X: np.ndarray) -> np.ndarray:
    """The method without the network: predict the previous split's kept rank
    (feature 34 holds log2(1 + previous rank)), clamped to the split size."""
    prev = np.exp2(X[:, 34]) - 1.0
    k = np.exp2(X[:, 35])
    return np.log2(np.clip(prev, 1.0, k))


def train_default(count: int = 60, epochs: int = 40, seed: int = 1, verbose: bool = False):
    """Record, train and return (model, report)."""
    t0 = time.time()
    X, D = record_dataset(count, seed)
    t1 = time.time()
    model = RankModel.initial(seed=seed)
    hist = model.fit(X, D, epochs=epochs)
    _torch().cuda.synchronize()
    t2 = time.time()
    if verbose:
        print(f"recorded {len(D)} truncations in {t1 - t0:.1f} s; trained in {t2 - t1:.1f} s; "
              f"loss {hist[0]:.4f} -> {hist[-1]:.4f}")
    return model, {"truncations": int(len(D)), "workloads": int(count), "record_s": t1 - t0,
                   "train_s": t2 - t1, "loss_first": hist[0], "loss_last": hist[-1]}


def main():
    import argparse

    ap = argparse.ArgumentParser(description="record truncations, train the rank predictor")
    ap.add_argument("--out", required=True)
    ap.add_argument("--count", type=int, default=150)
    ap.add_argument("--epochs", type=int, default=60)
    args = ap.parse_args()
    model, rep = train_default(args.count, args.epochs, verbose=True)
    model.save(args.out, **{k: np.array(v) for k, v in rep.items()})


if __name__ == "__main__":
    main()
