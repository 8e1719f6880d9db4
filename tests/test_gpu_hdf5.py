"""Device MPS/MPO through HDF5 groups, after the reference's tests/test_hdf5.py:
attributes, real and complex round trips (bit-exact, dtypes kept), appending a
second state, and the readers' errors; written into the in-memory group tree,
and into a real HDF5 file where h5py is installed."""

import numpy as np
import pytest

from tests.gpu_util import mps_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import seemps2_gb300 as sg  # noqa: E402
from seemps2_gb300 import hdf5  # noqa: E402


def _mps(n, D, cplx, seed):
    rng = np.random.default_rng(seed)
    return sg.random_uniform_mps(2, n, D=D, complex=cplx, rng=rng)


def _mpo(n, D, cplx, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        A = rng.normal(size=(1 if i == 0 else D, 2, 2, 1 if i == n - 1 else D))
        out.append(A * (1.2 + 0.5j) if cplx else A)
    return sg.MPO(out)


def _check_layout(f, name, kind, obj):
    data = hdf5.read_full_hdf5_as_paths(f)
    assert len([k for k in data if k.startswith(f"/{name}/")]) == len(obj) + 1
    assert data[f"/{name}/length"] == len(obj)
    for i, A in enumerate(obj):
        stored = data[f"/{name}/{kind}[{i}]"]
        host = A.detach().cpu().numpy()
        assert stored.dtype == host.dtype and stored.shape == host.shape
        assert np.array_equal(stored, host)
    attrs = f[name].attrs
    assert len(attrs) == 2 and attrs["type"] == kind and attrs["version"] == 1


@pytest.mark.parametrize("cplx", [False, True])
def test_mps_round_trip(cplx):
    state = _mps(5, 3, cplx, 7)
    f = hdf5.MemoryGroup()
    hdf5.write_mps(f, "M", state)
    _check_layout(f, "M", "MPS", state)
    copy = hdf5.read_mps(f, "M")
    assert isinstance(copy, sg.MPS) and copy.size == state.size
    assert copy.dtype == state.dtype and copy[0].is_cuda
    assert all(np.array_equal(a, b) for a, b in zip(mps_np(state), mps_np(copy)))
    # the read state is a working device state: same norm through the device kernels
    assert abs(sg.scprod(copy, copy) - sg.scprod(state, state)) <= 1e-12 * abs(sg.scprod(state, state))


def test_append_a_second_state():
    state, aux = _mps(3, 3, False, 1), _mps(4, 2, True, 2)
    f = hdf5.MemoryGroup()
    hdf5.write_mps(f, "M", state)
    hdf5.write_mps(f, "X", aux)
    data = hdf5.read_full_hdf5_as_paths(f)
    assert len(data) == 4 + 5 and data["/X/length"] == 4
    with pytest.raises(ValueError):
        hdf5.write_mps(f, "X", aux)  # the name is taken
    assert all(np.array_equal(a, b) for a, b in zip(mps_np(aux), mps_np(hdf5.read_mps(f, "X"))))
    assert all(np.array_equal(a, b) for a, b in zip(mps_np(state), mps_np(hdf5.read_mps(f, "/M"))))


@pytest.mark.parametrize("cplx", [False, True])
def test_mpo_round_trip(cplx):
    mpo = _mpo(3, 10, cplx, 11)
    f = hdf5.MemoryGroup()
    hdf5.write_mpo(f, "M", mpo)
    _check_layout(f, "M", "MPO", mpo)
    copy = hdf5.read_mpo(f, "M")
    assert isinstance(copy, sg.MPO) and copy.size == mpo.size
    assert all(torch.equal(a, b) for a, b in zip(mpo, copy))
    with pytest.raises(ValueError):
        hdf5.read_mps(f, "M")  # an MPO group is not an MPS


def test_zero_mpo_attributes():
    f = hdf5.MemoryGroup()
    hdf5.write_mpo(f, "M", sg.MPO([np.zeros((1, 2, 2, 1))] * 3))
    attrs = f["M"].attrs
    assert len(attrs) == 2 and attrs["type"] == "MPO" and attrs["version"] == 1


def test_real_file_round_trip(tmp_path):
    h5py = pytest.importorskip("h5py")
    state, mpo = _mps(4, 3, True, 3), _mpo(4, 3, False, 4)
    name = str(tmp_path / "s.hdf5")
    with h5py.File(name, "w") as file:
        hdf5.write_mps(file, "M", state)
        hdf5.write_mpo(file, "O", mpo)
    with h5py.File(name, "r") as file:
        assert len(file["M"].attrs) == 2
        copy, op = hdf5.read_mps(file, "M"), hdf5.read_mpo(file, "O")
    assert len(hdf5.read_full_hdf5_as_paths(name)) == 5 + 5
    assert all(np.array_equal(a, b) for a, b in zip(mps_np(state), mps_np(copy)))
    assert all(torch.equal(a, b) for a, b in zip(mpo, op))
