"""ctypes binding of libseemps_gb300.so (the C ABI declared in include/seemps_gb300.h).

There is no CPU fallback: importing the compute entry points without the
built library, or calling them without a CUDA device, raises immediately.
Status codes are translated into the exceptions the reference raises
(ValueError, AssertionError, numpy.linalg.LinAlgError, RuntimeError).
"""

from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libseemps_gb300.so")

SM_OK, SM_ERR_VALUE, SM_ERR_CUDA, SM_ERR_LINALG, SM_ERR_TIMEOUT, SM_ERR_STRATEGY, SM_ERR_NOMEM = range(7)
SM_FLOAT64, SM_COMPLEX128 = 0, 1
SM_OP_N, SM_OP_T, SM_OP_C = 0, 1, 2


class sm_strategy(C.Structure):
    _fields_ = [
        ("method", C.c_int32),
        ("max_bond_dimension", C.c_int32),
        ("tolerance", C.c_double),
        ("simplification_tolerance", C.c_double),
        ("normalize", C.c_int32),
        ("simplify", C.c_int32),
        ("max_sweeps", C.c_int32),
        ("reserved", C.c_int32),
    ]


class sm_simplify_report(C.Structure):
    _fields_ = [
        ("error", C.c_double),
        ("norm_state_sqr", C.c_double),
        ("norm_mps_sqr", C.c_double),
        ("last_err", C.c_double),
        ("sweeps", C.c_int32),
        ("center", C.c_int32),
        ("splits", C.c_int32),
        ("zero_state", C.c_int32),
        ("sweep_err", C.c_double * 64),
    ]


class sm_stats(C.Structure):
    _fields_ = [
        ("launches", C.c_int64),
        ("jacobi_launches", C.c_int64),
        ("jacobi_sweeps", C.c_int64),
        ("gemm_launches", C.c_int64),
        ("splits", C.c_int64),
        ("jacobi_ms", C.c_double),
        ("jacobi_flops", C.c_double),
        ("gemm_ms", C.c_double),
        ("gemm_flops", C.c_double),
        ("mixed_splits", C.c_int64),
        ("mixed_fallbacks", C.c_int64),
        ("mixed_rows", C.c_int64),
        ("cluster_ms", C.c_double),
        ("cluster_qr_ms", C.c_double),
        ("cluster_jacobi_ms", C.c_double),
        ("mixed_fallback_cut", C.c_int64),
        ("mixed_fallback_fp32", C.c_int64),
        ("mixed_capped", C.c_int64),
        ("mixed_cap_redone", C.c_int64),
        ("rank_predicted_sum", C.c_int64),
        ("gemm32_launches", C.c_int64),
        ("gemm32_flops", C.c_double),
        ("gemm32_ms", C.c_double),
        ("gemm_tc_launches", C.c_int64),
        ("gemm_tc_flops", C.c_double),
        ("gemm_tc_ms", C.c_double),
        ("mixed_fallback_over", C.c_int64),
        ("mixed_fallback_unconverged", C.c_int64),
        ("gemm_oz_launches", C.c_int64),
        ("gemm_oz_flops", C.c_double),
        ("gemm_oz_ms", C.c_double),
        ("cluster_flops", C.c_double),
        ("cluster_alg_flops", C.c_double),
        ("cluster_bytes", C.c_double),
        ("rf_splits", C.c_int64),
        ("mixed_ns_steps", C.c_int64),
        ("rank_predictions", C.c_int64),
    ]


vp = C.c_void_p
ip = C.POINTER(C.c_int)
dp = C.POINTER(C.c_double)
i64p = C.POINTER(C.c_int64)
stp = C.POINTER(sm_strategy)

# name -> (restype, argtypes); every symbol declared in include/seemps_gb300.h
SIGNATURES = {
    "sm_abi_version": (C.c_int, []),
    "sm_last_error": (C.c_char_p, []),
    "sm_ctx_create": (C.c_int, [C.POINTER(vp), C.c_int]),
    "sm_ctx_destroy": (C.c_int, [vp]),
    "sm_ctx_set_precision": (C.c_int, [vp, C.c_int]),
    "sm_ctx_set_contraction_bits": (C.c_int, [vp, C.c_int]),
    "sm_split_rows_f32": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_double,
                                    C.c_double, vp, dp, C.c_int, ip, ip, vp]),
    "sm_truncate": (C.c_int, [vp, vp, C.c_int, stp, ip, dp, vp]),
    "sm_gemm": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_int,
                          vp, C.c_int, vp, C.c_int, vp]),
    "sm_gemm_f32": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp,
                              C.c_int, vp, C.c_int, vp, C.c_int, vp]),
    "sm_gemm_ex": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, dp, vp,
                             C.c_int, vp, C.c_int, dp, vp, C.c_int, vp]),
    "sm_gemm_f64tc": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp,
                                C.c_int, vp, C.c_int, vp, C.c_int, vp]),
    "sm_ctx_set_fp64_products": (C.c_int, [vp, C.c_int]),
    "sm_ctx_set_concurrent": (C.c_int, [vp, C.c_int]),
    "sm_ctx_set_range_finder": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
    "sm_range_finder": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp]),
    "sm_ctx_set_rank_cap": (C.c_int, [vp, C.c_double, C.c_int]),
    "sm_two_site_matvec": (C.c_int, [vp, C.c_int, ip, vp, vp, vp, vp, vp, C.c_int, vp]),
    "sm_two_site_prepare": (C.c_int, [vp, ip, vp, vp, C.c_int, vp]),
    "sm_two_site_matvec_prepared": (C.c_int, [vp, vp, vp, vp, vp]),
    "sm_svd": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, vp, vp, vp, vp]),
    "sm_left_orth_2site": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, stp, vp,
                                     vp, ip, dp, vp]),
    "sm_right_orth_2site": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, stp, vp,
                                      vp, ip, dp, vp]),
    "sm_left_orth_2site_noalloc": (C.c_int, [C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, stp,
                                             vp, vp, ip, dp, vp]),
    "sm_update_left_environment": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp, C.c_int,
                                             C.c_int, vp, vp, vp]),
    "sm_update_right_environment": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp,
                                              C.c_int, C.c_int, vp, vp, vp]),
    "sm_mpo_multiply_tensor": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp,
                                         C.c_int, C.c_int, vp, vp]),
    "sm_scprod": (C.c_int, [vp, C.c_int, C.c_int, ip, ip, C.POINTER(vp), ip, C.POINTER(vp), dp, vp]),
    "sm_canonicalize": (C.c_int, [vp, C.c_int, C.c_int, ip, ip, C.POINTER(vp), i64p, C.c_int, stp,
                                  dp, vp]),
    "sm_recanonicalize": (C.c_int, [vp, C.c_int, C.c_int, ip, ip, C.POINTER(vp), i64p, C.c_int,
                                    C.c_int, stp, dp, vp]),
    "sm_update_in_canonical_form_right": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp,
                                                    C.c_int, C.c_int, stp, vp, vp, ip, dp, vp]),
    "sm_update_in_canonical_form_left": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp,
                                                   C.c_int, C.c_int, stp, vp, vp, ip, dp, vp]),
    "sm_contract_nrjl_ijk_klm": (C.c_int, [vp, C.c_int, vp, C.c_int, vp, C.c_int, C.c_int, C.c_int,
                                           vp, C.c_int, C.c_int, vp, vp]),
    "sm_update_left_mpo_environment": (C.c_int, [vp, C.c_int, vp, vp, C.c_int, C.c_int, C.c_int, vp,
                                                 C.c_int, C.c_int, C.c_int, vp, C.c_int, C.c_int,
                                                 vp, vp]),
    "sm_update_right_mpo_environment": (C.c_int, [vp, C.c_int, vp, vp, C.c_int, C.c_int, C.c_int,
                                                  vp, C.c_int, C.c_int, C.c_int, vp, C.c_int,
                                                  C.c_int, vp, vp]),
    "sm_mpo_join": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_int,
                              C.c_int, C.c_int, vp, vp]),
    "sm_tensor2site": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int, vp, C.c_int, C.c_int, vp,
                                 C.c_int, C.c_int, vp, C.c_int, vp, vp]),
    "sm_select_svd_driver": (C.c_int, [C.c_char_p]),
    "sm_svd_driver": (C.c_int, []),
    "sm_simplify_guess": (C.c_int, [vp, C.c_int, C.c_int, ip, C.c_int, dp, ip, C.POINTER(vp), dp, dp,
                                    ip, C.POINTER(vp), stp, C.c_int, C.POINTER(vp), i64p, ip,
                                    C.POINTER(sm_simplify_report), vp]),
    "sm_simplify": (C.c_int, [vp, C.c_int, C.c_int, ip, C.c_int, dp, ip, C.POINTER(vp), dp, stp,
                              C.c_int, C.POINTER(vp), i64p, ip, C.POINTER(sm_simplify_report), vp]),
    "sm_simplify_gram": (C.c_int, [vp, C.c_int, C.c_int, ip, C.c_int, dp, ip, C.POINTER(vp), dp,
                                   dp, stp, C.c_int, C.POINTER(vp), i64p, ip,
                                   C.POINTER(sm_simplify_report), vp]),
    "sm_mpo_scprod": (C.c_int, [vp, C.c_int, C.c_int, ip, ip, ip, C.POINTER(vp), ip, C.POINTER(vp),
                                ip, C.POINTER(vp), dp, vp]),
    "sm_simplify_bond_caps": (C.c_int, [C.c_int, ip, C.c_int, ip, stp, ip]),
    "sm_trace_enable": (C.c_int, [vp, C.c_int]),
    "sm_trace_read": (C.c_int, [vp, ip, i64p, ip, ip, dp, dp]),
    "sm_stats_reset": (C.c_int, [vp, C.c_int]),
    "sm_stats_read": (C.c_int, [vp, C.POINTER(sm_stats)]),
    # rank predictor (device pointers as void*, dims as a host int array)
    "sm_mlp_param_count": (C.c_int64, [C.c_int, ip]),
    "sm_mlp_cache_count": (C.c_int64, [C.c_int, ip, C.c_int]),
    "sm_mlp_forward": (C.c_int, [vp, C.c_int, ip, vp, vp, C.c_int, vp, vp, vp]),
    "sm_mlp_backward": (C.c_int, [vp, C.c_int, ip, vp, vp, C.c_int, vp, vp, vp, vp]),
    "sm_mse_loss": (C.c_int, [vp, vp, vp, C.c_int, vp, vp, vp]),
    "sm_adam_step": (C.c_int, [vp, vp, vp, vp, vp, C.c_int64, C.c_float, C.c_float, C.c_float,
                               C.c_float, C.c_int, vp]),
    "sm_rank_model_set": (C.c_int, [vp, C.c_int, ip, vp]),
    "sm_rank_features_record": (C.c_int, [vp, C.c_int]),
    "sm_rank_features_read": (C.c_int, [vp, vp, vp, C.c_int, ip]),
    "sm_rank_predict": (C.c_int, [vp, vp, C.c_int, vp, vp]),
}

RANK_FEATURES = 37

_lib = None
_lock = threading.Lock()


def load(path: str | None = None):
    """Load the shared library (built by seemps2_gb300._build); raises if absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError(
                f"{p} is missing: build it with `python -m seemps2_gb300._build` "
                "(there is no CPU fallback for the MPO/MPS kernels)")
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


class LinAlgError(np.linalg.LinAlgError):
    pass


def check(status: int):
    if status == SM_OK:
        return
    msg = load().sm_last_error().decode(errors="replace")
    if status == SM_ERR_VALUE:
        raise ValueError(msg)
    if status == SM_ERR_STRATEGY:
        raise AssertionError(msg)
    if status == SM_ERR_LINALG:
        raise LinAlgError(msg)
    raise RuntimeError(f"seemps_gb300 status {status}: {msg}")


_ctx_local = threading.local()


def context(device: int = 0) -> int:
    """Per-thread, per-device library context (scratch memory and pinned words)."""
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("seemps2_gb300 needs a CUDA device (sm_103a); none is available")
    cache = getattr(_ctx_local, "ctx", None)
    if cache is None:
        cache = _ctx_local.ctx = {}
    if device not in cache:
        h = vp()
        lib = load()
        torch.cuda.init()
        with torch.cuda.device(device):
            check(lib.sm_ctx_create(C.byref(h), device))
        cache[device] = h
    return cache[device]


def stream_handle(device=None):
    import torch

    return vp(torch.cuda.current_stream(device).cuda_stream)


def ptr(t) -> vp:
    return vp(t.data_ptr())


def ptr_array(ts) -> C.Array:
    arr = (vp * len(ts))()
    for k, t in enumerate(ts):
        arr[k] = t.data_ptr()
    return arr


def int_array(xs) -> C.Array:
    return (C.c_int * len(xs))(*[int(x) for x in xs])


def i64_array(xs) -> C.Array:
    return (C.c_int64 * len(xs))(*[int(x) for x in xs])


def dbl_array(xs) -> C.Array:
    return (C.c_double * len(xs))(*[float(x) for x in xs])


class SplitTrace:
    """Context manager recording every SVD split (singular values, rank, err^2)."""

    def __init__(self, device: int = 0):
        self.device = device
        self.ranks, self.err2, self.s = [], [], []

    def __enter__(self):
        check(load().sm_trace_enable(context(self.device), 1))
        return self

    def __exit__(self, *exc):
        lib = load()
        ctx = context(self.device)
        n = C.c_int()
        tot = C.c_int64()
        check(lib.sm_trace_read(ctx, C.byref(n), C.byref(tot), None, None, None, None))
        ranks = (C.c_int * max(1, n.value))()
        lens = (C.c_int * max(1, n.value))()
        err2 = (C.c_double * max(1, n.value))()
        sv = (C.c_double * max(1, tot.value))()
        check(lib.sm_trace_read(ctx, None, None, ranks, lens, err2, sv))
        check(lib.sm_trace_enable(ctx, 0))
        self.ranks = [ranks[k] for k in range(n.value)]
        self.err2 = [err2[k] for k in range(n.value)]
        allv = np.frombuffer(sv, dtype=np.float64, count=tot.value).copy()
        offs = np.concatenate([[0], np.cumsum([lens[k] for k in range(n.value)])]).astype(int)
        self.s = [allv[offs[k]:offs[k + 1]] for k in range(n.value)]
        return False


PRECISIONS = {"fp64": 0, "mixed": 1, "mixed+learned": 2}


def set_precision(mode: str, device: int = 0, contractions: str = "fp64",
                  range_finder: bool = False, oversample: int = 10, power_iters: int = 0,
                  rank_hint: int = 0) -> None:
    """Arithmetic of the SVD splits: "fp64" (default, reference ranks), "mixed"
    (FP32 cluster factorisation refined by FP64 GEMMs) or "mixed+learned" (as
    "mixed", with the installed rank predictor capping the FP32 QR, or, with
    range_finder=True, sizing a randomized range finder of predicted rank +
    oversample columns and power_iters subspace iterations; rank_hint > 0 stands
    in for the prediction)."""
    if mode not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}, not {mode!r}")
    if contractions not in ("fp64", "fp32"):
        raise ValueError("contractions must be 'fp64' or 'fp32'")
    check(load().sm_ctx_set_precision(context(device), PRECISIONS[mode]))
    check(load().sm_ctx_set_contraction_bits(context(device), 32 if contractions == "fp32" else 64))
    check(load().sm_ctx_set_range_finder(context(device), int(bool(range_finder)), int(oversample),
                                         int(power_iters), int(rank_hint)))


def stats_reset(timing: bool = False, device: int = 0):
    check(load().sm_stats_reset(context(device), int(timing)))


def stats_read(device: int = 0) -> dict:
    st = sm_stats()
    check(load().sm_stats_read(context(device), C.byref(st)))
    return {name: getattr(st, name) for name, _ in sm_stats._fields_}
