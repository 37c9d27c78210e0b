"""A long decaying run at 256^3 (2000 RK4 steps, diagnostics recorded on the device every 100):
the total energy decreases monotonically, u and B stay solenoidal at roundoff, nothing goes
non-finite, and the first step's energy change matches the dissipation rate the state implies
(dE/dt = -2 nu sum k^2 |u|^2 dV - 2 eta sum k^2 |B|^2 dV; the nonlinear terms conserve energy)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, NU, ETA, DT = 256, 1e-3, 2e-3, 5e-4


def test_long_decaying_run(pkg, mo):
    from importlib import import_module

    s0 = import_module(pkg.__name__ + ".ic").random_spectrum_state(N, 121)
    g = mo.Grid(N)
    s = s0.astype(np.complex128)
    g.dealias(s)
    w = np.ones((1, 1, g.nkr))
    w[..., 1:] = 2.0
    w[..., -1] = 1.0
    scale = g.dx ** 3 / float(N) ** 3
    k2 = g.Krsq
    rate = -2 * scale * (NU * sum(np.sum(w * k2 * np.abs(s[f]) ** 2) for f in range(3))
                         + ETA * sum(np.sum(w * k2 * np.abs(s[f]) ** 2) for f in range(3, 6)))
    with pkg.Problem(pkg.GPU(0), nx=N, Lx=2 * math.pi, nu=NU, eta=ETA, dt=DT) as p:
        p.set_sol(s0.T)
        d0 = p.diagnostics()
        pkg.stepforward(p, 1)
        d1 = p.diagnostics()
        p.record_diagnostics(100, capacity=32)
        pkg.stepforward(p, 2000)
        h = p.diagnostic_history()
    e0, e1 = d0.E_u + d0.E_B, d1.E_u + d1.E_B
    measured = (e1 - e0) / DT
    print(f"dE/dt first step {measured:.6e}, dissipation rate {rate:.6e}")
    assert measured == pytest.approx(rate, rel=1e-2)
    assert h.shape == (20, 8)
    e = h[:, 2] + h[:, 3]
    assert np.all(np.diff(np.concatenate([[e1], e])) < 0)
    assert np.all(h[:, 7] == 0)
    # solenoidal at roundoff: max |k.u| against the largest k |u| the state holds
    kmax = math.sqrt(3) * (N // 3)
    amp_u = math.sqrt(e[-1] / scale)
    assert np.all(h[:, 5] < 1e-5 * kmax * amp_u) and np.all(h[:, 6] < 1e-5 * kmax * amp_u)
    print(f"E(0) {e0:.6f} -> E(2001 steps) {e[-1]:.6f}")


def test_ideal_invariants(pkg):
    """nu = eta = 0: the nonlinear terms conserve the total energy and the cross-helicity
    (ideal MHD invariants; dealiased Galerkin truncation keeps both).  200 RK4 steps at 128^3
    change them only by the scheme's O(dt^5) error and FP32 roundoff."""
    from importlib import import_module

    s0 = import_module(pkg.__name__ + ".ic").random_spectrum_state(128, 122)
    with pkg.Problem(pkg.GPU(0), nx=128, Lx=2 * math.pi, nu=0.0, eta=0.0, dt=2e-4) as p:
        p.set_sol(s0.T)
        d0 = p.diagnostics()
        pkg.stepforward(p, 200)
        d1 = p.diagnostics()
    e0, e1 = d0.E_u + d0.E_B, d1.E_u + d1.E_B
    print(f"ideal: dE/E {(e1 - e0) / e0:.3e}, dHc {d1.H_c - d0.H_c:.3e} (E {e0:.4f}, Hc {d0.H_c:.4f})")
    assert abs(e1 - e0) < 2e-5 * e0
    assert abs(d1.H_c - d0.H_c) < 2e-5 * e0
    assert abs(d1.E_u - d0.E_u) > 1e-4 * e0  # energy does move between u and B
