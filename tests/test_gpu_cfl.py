"""On-device getCFL! (TimeIntegrator with usr_dt = 0) against the oracle."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_cfl_dt_from_last_stage_fields(pkg, mo):
    n, coef = 32, 0.3
    g = mo.Grid(n)
    s0 = mo.random_spectrum_state(g, 21)
    nu, eta = 2e-3, 1e-3
    with pkg.Problem(pkg.GPU(0), nx=n, nu=nu, eta=eta, dt=1e-3) as prob:
        prob.set_sol(s0.astype(np.complex64).T)
        pkg._lib.check(prob._lib.mhd_set_cfl(prob.handle, 1, coef))
        dt0 = prob.clock.dt
        pkg.stepforward(prob, 1)
        dt1, t1 = prob.clock.dt, prob.clock.t
        pkg.stepforward(prob, 2)
        t3 = prob.clock.t
        assert prob.clock.step == 3
    dx = 2 * math.pi / n
    tdiff = coef * dx * dx / max(nu, eta)
    # first dt: from the current (initial) fields
    v0 = max(np.abs(g.irfft(s0[f])).max() for f in range(6))
    assert dt0 == pytest.approx(min(coef * dx / v0, tdiff), rel=1e-5)
    # after a step: from the physical fields of the step's last RK4 stage (the reference's vars)
    st = mo.Stepper(g, nu, eta, dt0, "RK4", literal=True)
    s = s0.astype(np.complex64).astype(np.complex128)
    st.stepforward(s)
    v1 = max(np.abs(st.vars[f]).max() for f in range(6))
    assert dt1 == pytest.approx(min(coef * dx / v1, tdiff), rel=1e-5)
    assert t1 == pytest.approx(dt0, rel=1e-6)
    assert t3 > t1 + dt1 * 0.99


def test_time_integrator_runs_n0_plus_one_steps(pkg, mo):
    n = 32
    g = mo.Grid(n)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-2, eta=1e-2, dt=1e-3) as prob:
        f = mo.taylor_green(g)
        for i in range(6):
            prob.set_physical_c(i, f[i].astype(np.float32))
        energy = pkg.Diagnostic(lambda p: p.diagnostics().E_u, prob, freq=2)
        rate = pkg.TimeIntegrator(prob, 10.0, 9, usr_dt=1e-3, diags=[energy])
        assert prob.clock.step == 10 and rate > 0
        assert energy.steps == [2, 4, 6, 8, 10]
        assert np.all(np.diff(energy.data) < 0)
        # CFL mode to a stopping time
        prob.clock.t = 0.0
        pkg.TimeIntegrator(prob, 0.3, 10 ** 6, usr_dt=0.0, CFL_Coef=0.3)
        assert prob.clock.t > 0.3 and prob.clock.step > 3
