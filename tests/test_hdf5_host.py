"""HDF5 storage without a GPU: the group tree, the whole-file readers and the
errors of the MPS/MPO readers and writers, following the reference's
tests/test_hdf5.py (read_whole_file, signals_errors_for_incorrect_data).
The round trips of device MPS/MPO live in test_gpu_hdf5.py."""

import importlib.util

import numpy as np
import pytest

from seemps2_gb300 import hdf5


def small_file():
    f = hdf5.MemoryGroup()
    f.create_dataset("A", data=1)
    f.create_dataset("B", data=2)
    f.create_group("C")
    f["C"].create_dataset("D", data=3)
    return f


def test_read_whole_tree():
    f = small_file()
    assert hdf5.read_full_hdf5_as_paths(f) == {"/A": 1, "/B": 2, "/C/D": 3}
    assert hdf5.read_full_hdf5(f) == {"A": 1, "B": 2, "C": {"D": 3, "_attrs": []}, "_attrs": []}


def test_memory_group_paths():
    f = small_file()
    assert "/C/D" in f and "C/D" in f and "D" in f["C"] and "/A" in f["C"]
    assert "E" not in f and "A/x" not in f
    assert f["/C/D"].name == "/C/D" and f["C"].name == "/C"
    g = f.create_group("C/E")
    g.create_dataset("F", data=np.arange(6.0).reshape(2, 3))
    assert f["/C/E/F"].shape == (2, 3) and f["/C/E/F"].dtype == np.float64
    with pytest.raises(ValueError):
        f.create_group("C")
    with pytest.raises(KeyError):
        f.create_dataset("Z/Y", data=1)
    with pytest.raises(ValueError):
        f.create_dataset("G", shape=(3,), data=np.zeros(2))


def test_dataset_keeps_its_own_copy_and_dtype():
    f = hdf5.MemoryGroup()
    a = (np.arange(8.0) * (1 + 2j)).reshape(1, 8, 1)
    f.create_dataset("a", shape=a.shape, data=a)
    a[0, 0, 0] = 99
    out = f["a"][()]
    assert out.dtype == np.complex128 and out[0, 0, 0] == 0


@pytest.mark.parametrize("read", [hdf5.read_mps, hdf5.read_mpo])
def test_readers_signal_incorrect_data(read):
    f = hdf5.MemoryGroup()
    f.create_dataset("A", data=2)
    f.create_group("B").create_dataset("C", data=3)
    wrong = f.create_group("W")
    wrong.attrs["type"] = "MPS" if read is hdf5.read_mpo else "MPO"
    wrong.attrs["version"] = 1
    wrong.create_dataset("length", data=0)
    old = f.create_group("V")
    old.attrs["type"] = "MPS" if read is hdf5.read_mps else "MPO"
    old.attrs["version"] = 2
    for name in ("A", "/A", "B", "/B", "W", "V", "missing"):
        with pytest.raises(ValueError):
            read(f, name)


def test_writers_reject_other_objects():
    f = hdf5.MemoryGroup()
    with pytest.raises(TypeError):
        hdf5.write_mps(f, "M", [np.zeros((1, 2, 1))])
    with pytest.raises(TypeError):
        hdf5.write_mpo(f, "M", [np.zeros((1, 2, 2, 1))])
    assert len(f) == 0


@pytest.mark.skipif(importlib.util.find_spec("h5py") is not None, reason="h5py is installed")
def test_file_name_without_h5py_says_so(tmp_path):
    with pytest.raises(ImportError, match="h5py"):
        hdf5.read_full_hdf5(str(tmp_path / "x.hdf5"))


def test_whole_file_readers_on_a_real_file(tmp_path):
    h5py = pytest.importorskip("h5py")
    name = str(tmp_path / "t.hdf5")
    with h5py.File(name, "w") as file:
        file.create_dataset("A", data=1)
        file.create_dataset("B", data=2)
        file.create_group("C").create_dataset("D", data=3)
    assert hdf5.read_full_hdf5_as_paths(name) == {"/A": 1, "/B": 2, "/C/D": 3}
    assert hdf5.read_full_hdf5(name) == {"A": 1, "B": 2, "C": {"D": 3, "_attrs": []}, "_attrs": []}
