"""The reference's kernel table (``seemps.cython``, cython/__init__.py:25-54) served by this
library: the same eight configuration names and nineteen kernels, each running on the GPU
through the C ABI.  A SeeMPS installation can route its kernel table here (the binding is
shown in INTEGRATION.md); site tensors then come back as CUDA tensors.
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
    _recanonicalize,
    _right_orth_2site,
    _select_svd_driver,
    _update_in_canonical_form_left,
    _update_in_canonical_form_right,
    _update_left_environment,
    _update_right_environment,
    destructively_truncate_vector,
)
from .state import scprod, vdot

CONFIG_NAMES = ("DEFAULT_STRATEGY", "DEFAULT_TOLERANCE", "GemmOrder", "MAX_BOND_DIMENSION",
                "NO_TRUNCATION", "Simplification", "Strategy", "Truncation")
KERNEL_NAMES = ("_begin_environment", "_canonicalize", "_contract_last_and_first",
                "_contract_nrjl_ijk_klm", "_destructive_svd", "_end_environment", "_gemm",
                "_join_environments", "_left_orth_2site", "_right_orth_2site", "_recanonicalize",
                "_select_svd_driver", "_update_in_canonical_form_right",
                "_update_in_canonical_form_left", "_update_left_environment",
                "_update_right_environment", "destructively_truncate_vector", "scprod", "vdot")


def active_backend() -> str:
    """The name of this kernel table (the reference answers 'cython' or 'python')."""
    return "gb300"


__all__ = list(CONFIG_NAMES) + list(KERNEL_NAMES) + ["active_backend"]
