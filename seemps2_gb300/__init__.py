"""seemps2_gb300 — SeeMPS's MPO·MPS + simplify path on one GB300 (sm_103a).

Drop-in for the reference API of that path: ``MPS``, ``CanonicalMPS``,
``MPSSum``, ``MPO``, ``MPOList``, ``Strategy``, ``Truncation``,
``Simplification``, ``simplify`` and ``MPO.apply`` / ``@``.  Site tensors live
in GPU memory; every numerical step runs in hand-written CUDA kernels of
``libseemps_gb300.so`` behind the C ABI of ``include/seemps_gb300.h``.
"""

from .core import (
    DEFAULT_STRATEGY,
    DEFAULT_TOLERANCE,
    MAX_BOND_DIMENSION,
    NO_TRUNCATION,
    GemmOrder,
    Simplification,
    Strategy,
    Truncation,
    _contract_last_and_first,
    _destructive_svd,
    _gemm,
    _left_orth_2site,
    _mpo_multiply_tensor,
    _right_orth_2site,
    _update_left_environment,
    _update_right_environment,
    destructively_truncate_vector,
)
from ._lib import set_precision
from .operators import MPO, MPOList, mpo_scprod
from .state import (
    SIMPLIFICATION_STRATEGY,
    CanonicalMPS,
    MPS,
    MPSSum,
    random_mps,
    random_uniform_mps,
    scprod,
    simplify,
    simplify_mps,
    simplify_mps_sum,
    vdot,
)

__all__ = [
    "DEFAULT_STRATEGY", "DEFAULT_TOLERANCE", "MAX_BOND_DIMENSION", "NO_TRUNCATION", "GemmOrder",
    "Simplification", "Strategy", "Truncation", "destructively_truncate_vector", "MPO", "MPOList",
    "SIMPLIFICATION_STRATEGY", "CanonicalMPS", "MPS", "MPSSum", "random_mps", "random_uniform_mps",
    "scprod", "simplify", "simplify_mps", "simplify_mps_sum", "vdot", "set_precision", "mpo_scprod",
]
