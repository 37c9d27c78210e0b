"""On-device diagnostics history (mhd_set_diag_history): the samples equal mhd_diagnostics of the
same states taken step by step on the host, bit for bit (same reduction order), per slot of a
batch, and with the on-device CFL clock."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _diag_row(d):
    return np.array([d.E_u, d.E_B, d.H_c, d.max_kdotu, d.max_kdotb, d.nonfinite])


def test_history_matches_host_diagnostics(pkg, mo):
    n, dt = 32, 1e-3
    s = mo.random_spectrum_state(mo.Grid(n), seed=91).astype(np.complex64)
    with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=2e-3, dt=dt) as a, \
            pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=2e-3, dt=dt) as b:
        a.set_sol(s.T)
        b.set_sol(s.T)
        a.record_diagnostics(2, capacity=8)
        pkg.stepforward(a, 7)  # samples after steps 2, 4 and 6
        h = a.diagnostic_history()
        ref = []
        for _ in range(3):
            pkg.stepforward(b, 2)
            ref.append(_diag_row(b.diagnostics()))
    assert h.shape == (3, 8)
    assert h[:, 0].tolist() == [2, 4, 6]
    dt32 = float(np.float32(dt))  # the clock advances by the FP32 dt the kernels use
    assert np.allclose(h[:, 1], [2 * dt32, 4 * dt32, 6 * dt32], rtol=0, atol=1e-12)
    assert np.array_equal(h[:, 2:], np.array(ref)), (h[:, 2:], ref)


def test_history_per_slot_of_a_batch(pkg, mo):
    n = 32
    s = mo.random_spectrum_state(mo.Grid(n), seed=92).astype(np.complex64)
    nus = (1e-3, 4e-3)
    b = pkg.Batch(n, 2)
    try:
        slots = [b.add(nu, nu, 1e-3) for nu in nus]
        for sl in slots:
            b.set_state(sl, s)
        b.record_diagnostics(3, capacity=4)
        b.step(6)
        hs = [b.diagnostic_history(sl) for sl in slots]
    finally:
        b.close()
    for nu, h in zip(nus, hs):
        with pkg.Problem(pkg.GPU(0), nx=n, nu=nu, eta=nu, dt=1e-3) as p:
            p.set_sol(s.T)
            rows = []
            for _ in range(2):
                pkg.stepforward(p, 3)
                rows.append(_diag_row(p.diagnostics()))
        assert h[:, 0].tolist() == [3, 6]
        assert np.array_equal(h[:, 2:], np.array(rows))
    assert not np.array_equal(hs[0][:, 2:], hs[1][:, 2:])


def test_history_with_on_device_cfl(pkg, mo):
    n = 32
    s = mo.random_spectrum_state(mo.Grid(n), seed=93).astype(np.complex64)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as p:
        p.set_sol(s.T)
        pkg.TimeIntegrator(p, math.inf, 9, diag_freq=5)  # 10 steps: samples after steps 5 and 10
        h = p.diagnostic_history()
        t_end = p.clock.t
    assert h[:, 0].tolist() == [5, 10]
    assert 0 < h[0, 1] < h[1, 1]
    assert h[1, 1] == pytest.approx(t_end, rel=1e-12)
    assert np.all(h[:, 7] == 0)


def test_history_off_and_capacity(pkg, mo):
    n = 32
    s = mo.random_spectrum_state(mo.Grid(n), seed=94).astype(np.complex64)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as p:
        p.set_sol(s.T)
        assert p.diagnostic_history().shape == (0, 8)
        p.record_diagnostics(1, capacity=2)
        pkg.stepforward(p, 4)
        assert p.diagnostic_history().shape == (2, 8)  # 4 recorded, 2 stored
        p.record_diagnostics(0)
        pkg.stepforward(p, 2)
        assert p.diagnostic_history().shape == (0, 8)
        with pytest.raises(pkg.MHDError):
            p.record_diagnostics(1, capacity=0)
