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
    _begin_environment,
    _canonicalize,
    _contract_last_and_first,
    _contract_nrjl_ijk_klm,
    _destructive_svd,
    _end_environment,
    _gemm,
    _join_environments,
    _left_orth_2site,
    _mpo_multiply_tensor,
    _recanonicalize,
    _right_orth_2site,
    _select_svd_driver,
    _tensor2site,
    _update_in_canonical_form_left,
    _update_in_canonical_form_right,
    _update_left_environment,
    _update_right_environment,
    destructively_truncate_vector,
)
from . import hdf5
from ._lib import set_precision
from .operators import (CANONICALIZE_MPO, MPO, MPO_SIMPLIFICATION_STRATEGY, MPOList,
                        mpo_as_mps, mpo_scprod, mps_as_mpo, simplify_mpo)
from .state import (
    SIMPLIFICATION_STRATEGY,
    AntilinearForm,
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
    "AntilinearForm", "simplify_mpo", "mpo_as_mps", "mps_as_mpo", "MPO_SIMPLIFICATION_STRATEGY",
    "CANONICALIZE_MPO",
]
