"""MPS and MPO storage in HDF5 groups (reference ``seemps/hdf5.py:39-173``).

The layout is the reference's, so files move between the two packages: an
MPS (MPO) named ``name`` is a subgroup of ``parent`` with the attributes
``type = "MPS"`` (``"MPO"``) and ``version = 1``, a scalar dataset ``length``
and one dataset per site, ``MPS[i]`` (``MPO[i]``), holding the site tensor
with its dtype (float64 or complex128 here; the device keeps no other).

The functions take any object with h5py's group interface: an open
``h5py.File`` or ``h5py.Group`` (h5py is imported only when a file name is
given, so the module loads without it), or the in-memory :class:`MemoryGroup`
below, which keeps the same tree in host memory.  Site tensors are copied from
the device on write and back to the device on read.

Errors follow the reference: writing anything but an MPS (MPO) raises
``TypeError``; reading a name that is absent, a dataset, or a group without the
right ``type``/``version`` attributes raises ``ValueError``.
"""

from __future__ import annotations

from typing import Any

import numpy as np

from .operators import MPO
from .state import MPS

__all__ = [
    "MemoryGroup",
    "read_full_hdf5",
    "read_full_hdf5_as_paths",
    "read_mpo",
    "read_mps",
    "write_mpo",
    "write_mps",
]


# ---------------------------------------------------------------------------
# In-memory tree with h5py's group interface
# ---------------------------------------------------------------------------


class _Dataset:
    """A dataset of a :class:`MemoryGroup`: a host array, read with ``d[()]``."""

    def __init__(self, name: str, data: np.ndarray):
        self.name = name
        self._data = data
        self.attrs: dict[str, Any] = {}

    @property
    def shape(self):
        return self._data.shape

    @property
    def dtype(self):
        return self._data.dtype

    def __getitem__(self, key):
        return self._data[key]


class MemoryGroup:
    """A group tree in host memory with the part of h5py's interface that
    the readers and writers use: ``create_group``, ``create_dataset(name,
    shape=None, data=None)``, ``attrs``, ``in``, ``[path]`` (relative or, from
    the root, absolute), ``keys/items/values`` and ``name``.  A new
    ``MemoryGroup()`` is a root, like an open ``h5py.File``.
    """

    def __init__(self, name: str = "/", root: "MemoryGroup | None" = None):
        self.name = name
        self.attrs: dict[str, Any] = {}
        self._items: dict[str, Any] = {}
        self._root = self if root is None else root

    def _child_path(self, key: str) -> str:
        return ("" if self.name == "/" else self.name) + "/" + key

    def _walk(self, path: str):
        node = self._root if path.startswith("/") else self
        for part in (p for p in path.split("/") if p):
            if not isinstance(node, MemoryGroup) or part not in node._items:
                return None
            node = node._items[part]
        return node

    def _parent_for_new(self, path: str):
        head, _, leaf = path.rstrip("/").rpartition("/")
        if not leaf:
            raise ValueError(f"invalid name {path!r}")
        parent = self._walk(head) if head else (self._root if path.startswith("/") else self)
        if not isinstance(parent, MemoryGroup):
            raise KeyError(f"no group {head!r}")
        if leaf in parent._items:
            raise ValueError(f"name {path!r} already exists")
        return parent, leaf

    def create_group(self, path: str) -> "MemoryGroup":
        parent, leaf = self._parent_for_new(path)
        g = MemoryGroup(parent._child_path(leaf), self._root)
        parent._items[leaf] = g
        return g

    def create_dataset(self, path: str, shape=None, dtype=None, data=None) -> _Dataset:
        parent, leaf = self._parent_for_new(path)
        if data is None:
            arr = np.zeros(shape, dtype=np.float64 if dtype is None else dtype)
        else:
            arr = np.array(data, dtype=dtype, copy=True)
            if shape is not None and tuple(shape) != arr.shape:
                raise ValueError(f"shape {tuple(shape)} does not match the data's {arr.shape}")
        d = _Dataset(parent._child_path(leaf), arr)
        parent._items[leaf] = d
        return d

    def __contains__(self, path: str) -> bool:
        return self._walk(path) is not None

    def __getitem__(self, path: str):
        node = self._walk(path)
        if node is None:
            raise KeyError(path)
        return node

    def __len__(self) -> int:
        return len(self._items)

    def keys(self):
        return self._items.keys()

    def items(self):
        return self._items.items()

    def values(self):
        return self._items.values()


# ---------------------------------------------------------------------------
# Whole-file readers (reference hdf5.py:9-36)
# ---------------------------------------------------------------------------


def _is_group(item) -> bool:
    return hasattr(item, "items") and hasattr(item, "create_group")


def _open(source):
    """An open root for ``source``: a file name (opened with h5py), or an
    object with the group interface, used as it is."""
    if isinstance(source, (str, bytes)) or hasattr(source, "__fspath__"):
        try:
            import h5py  # noqa: PLC0415
        except ImportError as exc:
            raise ImportError("reading an HDF5 file by name needs h5py, which is not installed; "
                              "pass an open group instead") from exc
        return h5py.File(source, "r"), True
    return source, False


def _paths(item, out: list) -> list:
    for sub in item.values():
        if _is_group(sub):
            _paths(sub, out)
        else:
            out.append((sub.name, sub[()]))
    return out


def _tree(item):
    if not _is_group(item):
        return item[()]
    out = {key: _tree(sub) for key, sub in item.items()}
    out["_attrs"] = list(item.attrs.items())
    return out


def read_full_hdf5_as_paths(source) -> dict[str, Any]:
    """Every dataset of a file (or group), keyed by its absolute path."""
    root, close = _open(source)
    try:
        return dict(_paths(root, []))
    finally:
        if close:
            root.close()


def read_full_hdf5(source) -> dict:
    """The tree of a file (or group) as nested dicts; each group's attributes
    go under ``"_attrs"`` as a list of (name, value) pairs."""
    root, close = _open(source)
    try:
        return _tree(root)
    finally:
        if close:
            root.close()


# ---------------------------------------------------------------------------
# MPS / MPO (reference hdf5.py:39-163)
# ---------------------------------------------------------------------------


def _host(A) -> np.ndarray:
    return A.detach().cpu().numpy() if hasattr(A, "detach") else np.asarray(A)


def _write_tensors(parent, name: str, kind: str, tensors) -> None:
    host = [_host(A) for A in tensors]  # all device reads before the group exists
    g = parent.create_group(name)
    g.attrs["type"] = kind
    g.attrs["version"] = 1
    g.create_dataset("length", data=len(host))
    for i, A in enumerate(host):
        g.create_dataset(f"{kind}[{i}]", shape=A.shape, data=A)


def _read_tensors(parent, name: str, kind: str) -> list | None:
    if name not in parent:
        return None
    g = parent[name]
    if not _is_group(g):
        return None
    attrs = g.attrs
    if "type" not in attrs or "version" not in attrs:
        return None
    if attrs["type"] != kind or attrs["version"] != 1:
        return None
    n = int(g["length"][()])
    return [g[f"{kind}[{i}]"][()] for i in range(n)]


def write_mps(parent, name: str, M) -> None:
    """Store the MPS ``M`` as the subgroup ``name`` of ``parent``."""
    if not isinstance(M, MPS):
        raise TypeError("write_mps() requires an MPS object")
    _write_tensors(parent, name, "MPS", M)


def read_mps(parent, name: str):
    """The MPS stored as the subgroup ``name`` of ``parent``, on the device."""
    tensors = _read_tensors(parent, name, "MPS")
    if tensors is None:
        raise ValueError(f"Unable to read MPS from HDF5 group {parent}")
    return MPS(tensors)


def write_mpo(parent, name: str, M) -> None:
    """Store the MPO ``M`` as the subgroup ``name`` of ``parent``."""
    if not isinstance(M, MPO):
        raise TypeError("write_mpo() requires an MPO object")
    _write_tensors(parent, name, "MPO", M)


def read_mpo(parent, name: str):
    """The MPO stored as the subgroup ``name`` of ``parent``, on the device."""
    tensors = _read_tensors(parent, name, "MPO")
    if tensors is None:
        raise ValueError(f"Unable to read MPO from HDF5 group {parent}")
    return MPO(tensors)
