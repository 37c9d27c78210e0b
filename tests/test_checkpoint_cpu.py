"""Checkpoint file naming and reading (host logic, no GPU): the reference's savefile pattern
<name>_t_<4 digits>.h5 (src/integrator.jl:260-264) and readMHDFlows's dataset order
(src/utils/IC.jl:245-257), for the HDF5 files and the .npz alternative."""
import numpy as np
import pytest

NAMES = ("i_velocity", "j_velocity", "k_velocity", "i_mag_field", "j_mag_field", "k_mag_field")


def test_checkpoint_path_pattern(pkg):
    assert pkg.checkpoint_path("out/run", 3) == "out/run_t_0003.h5"
    assert pkg.checkpoint_path("run", 12345) == "run_t_12345.h5"
    assert pkg.checkpoint_path("run", 3, fmt="npz") == "run_t_0003.npz"
    with pytest.raises(pkg.MHDError):
        pkg.checkpoint_path("run", 3, fmt="hdf")


def test_read_mhdflows_order_npz(pkg, tmp_path):
    rng = np.random.default_rng(0)
    data = {k: rng.standard_normal((4, 4, 4)).astype(np.float64) for k in NAMES}
    p = tmp_path / "x_t_0001.npz"
    np.savez(p, time=np.float64(0.25), **data)
    out = pkg.readMHDFlows(str(p))
    assert len(out) == 7 and out[-1] == 0.25
    for arr, k in zip(out[:6], NAMES):
        assert arr.dtype == np.float32
        assert np.array_equal(arr, data[k].astype(np.float32))


def test_read_mhdflows_order_h5(pkg, tmp_path):
    """Datasets written as HDF5.jl writes a Julia (nx, ny, nz) array: HDF5 dims (nz, ny, nx)."""
    from importlib import import_module

    hdf5 = import_module(pkg.__name__ + ".hdf5")
    rng = np.random.default_rng(1)
    julia = {k: np.asfortranarray(rng.standard_normal((4, 5, 6)).astype(np.float32)) for k in NAMES}
    p = tmp_path / "x_t_0002.h5"
    hdf5.write(str(p), {**{k: v.T for k, v in julia.items()}, "time": np.float32(0.5)})
    out = pkg.readMHDFlows(str(p))
    assert out[-1] == 0.5
    for arr, k in zip(out[:6], NAMES):
        assert arr.shape == (4, 5, 6) and arr.dtype == np.float32
        assert np.array_equal(arr, julia[k])
