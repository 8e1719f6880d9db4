"""The C-ABI library loads and exports every entry point include/*.h declares (no GPU calls)."""

import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(sm_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from seemps2_gb300 import _build, _lib

    _build.build()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "sm_simplify" in names and "sm_truncate" in names and len(names) >= 15


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    from seemps2_gb300 import _lib

    assert sorted(_lib.SIGNATURES) == declared_functions()


def test_abi_version_and_no_gpu_needed_calls(lib):
    lib.sm_abi_version.restype = ctypes.c_int
    assert lib.sm_abi_version() == 1
    # pure host helper: bond caps
    from seemps2_gb300 import _lib
    from seemps2_gb300.core import Strategy

    l = _lib.load()
    caps = (ctypes.c_int * 5)()
    st = Strategy(max_bond_dimension=3).to_c()
    assert l.sm_simplify_bond_caps(4, _lib.int_array([2] * 4), 1, _lib.int_array([1, 2, 4, 2, 1]),
                                   ctypes.byref(st), caps) == 0
    assert list(caps) == [1, 2, 3, 2, 1]
    bad = Strategy().to_c()
    bad.max_bond_dimension = 0
    assert l.sm_simplify_bond_caps(4, _lib.int_array([2] * 4), 1, _lib.int_array([1, 2, 4, 2, 1]),
                                   ctypes.byref(bad), caps) == _lib.SM_ERR_STRATEGY


def test_strategy_mirrors_reference_semantics():
    from oracle import seemps_oracle as so
    from seemps2_gb300 import Strategy, Truncation, DEFAULT_STRATEGY, NO_TRUNCATION

    assert Strategy(tolerance=0.0).get_method() == Truncation.ABSOLUTE_SINGULAR_VALUE
    assert Strategy(method=0, tolerance=0.0).get_method() == Truncation.DO_NOT_TRUNCATE
    for bad in (dict(tolerance=-1), dict(tolerance=1.0), dict(max_bond_dimension=0),
                dict(max_sweeps=-1), dict(simplify=7), dict(method=9)):
        with pytest.raises(AssertionError):
            Strategy(**bad)
    s = DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=64, max_sweeps=2)
    o = so.DEFAULT_STRATEGY.replace(tolerance=1e-10, max_bond_dimension=64, max_sweeps=2)
    assert (s.get_method(), s.get_tolerance(), s.get_max_bond_dimension(), s.get_max_sweeps()) == \
        (o.method, o.tolerance, o.max_bond_dimension, o.max_sweeps)
    assert not NO_TRUNCATION.get_simplify_flag()
    assert "RelativeNorm" in str(DEFAULT_STRATEGY)


def test_no_cpu_fallback_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from seemps2_gb300 import _lib

    with pytest.raises(RuntimeError):
        _lib.context()


# The reference's kernel table, cython/__init__.py:25-54 (configuration names and kernels).
REFERENCE_CONFIG = ["DEFAULT_STRATEGY", "DEFAULT_TOLERANCE", "GemmOrder", "MAX_BOND_DIMENSION",
                    "NO_TRUNCATION", "Simplification", "Strategy", "Truncation"]
REFERENCE_KERNELS = ["_begin_environment", "_canonicalize", "_contract_last_and_first",
                     "_contract_nrjl_ijk_klm", "_destructive_svd", "_end_environment", "_gemm",
                     "_join_environments", "_left_orth_2site", "_right_orth_2site",
                     "_recanonicalize", "_select_svd_driver", "_update_in_canonical_form_right",
                     "_update_in_canonical_form_left", "_update_left_environment",
                     "_update_right_environment", "destructively_truncate_vector", "scprod",
                     "vdot"]


def test_kernel_table_has_every_reference_name():
    """Every configuration name and kernel of the reference's table has a mirror, both in
    seemps2_gb300.kernel_table and at the package top level."""
    import seemps2_gb300 as sg
    from seemps2_gb300 import kernel_table as kt

    for name in REFERENCE_CONFIG + REFERENCE_KERNELS:
        assert hasattr(kt, name), name
        assert hasattr(sg, name), name
    assert kt.active_backend() == "gb300"


def test_select_svd_driver_validates_like_the_reference():
    from seemps2_gb300 import _lib
    from seemps2_gb300.kernel_table import _select_svd_driver

    _select_svd_driver("gesvd")
    assert _lib.load().sm_svd_driver() == 1
    _select_svd_driver("gesdd")
    assert _lib.load().sm_svd_driver() == 0
    with pytest.raises(ValueError):
        _select_svd_driver("dgesvj")
