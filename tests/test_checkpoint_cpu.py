"""Checkpoint file naming and reading (host logic, no GPU): the reference's savefile pattern
<name>_t_<4 digits> (src/integrator.jl:260-264) and readMHDFlows's dataset order
(src/utils/IC.jl:245-257)."""
import numpy as np


def test_checkpoint_path_pattern(pkg):
    assert pkg.checkpoint_path("out/run", 3) == "out/run_t_0003.npz"
    assert pkg.checkpoint_path("run", 12345) == "run_t_12345.npz"


def test_read_mhdflows_order(pkg, tmp_path):
    rng = np.random.default_rng(0)
    names = ("i_velocity", "j_velocity", "k_velocity", "i_mag_field", "j_mag_field", "k_mag_field")
    data = {k: rng.standard_normal((4, 4, 4)).astype(np.float64) for k in names}
    p = tmp_path / "x_t_0001.npz"
    np.savez(p, time=np.float64(0.25), **data)
    out = pkg.readMHDFlows(str(p))
    assert len(out) == 7 and out[-1] == 0.25
    for arr, k in zip(out[:6], names):
        assert arr.dtype == np.float32
        assert np.array_equal(arr, data[k].astype(np.float32))
