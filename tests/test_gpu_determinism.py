"""Determinism: the same input stepped twice on fresh handles gives bitwise equal states at 256^3
(the tuned kernel selection, RK4 and LSRK4) - no reduction or atomic feeds the data path."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("stepper", ["RK4", "LSRK4"])
def test_steps_are_bitwise_reproducible(pkg, stepper):
    from importlib import import_module

    s0 = import_module(pkg.__name__ + ".ic").random_spectrum_state(256, 111)
    out = []
    for _ in range(2):
        with pkg.Problem(pkg.GPU(0), nx=256, Lx=2 * math.pi, nu=1e-3, eta=1e-3, dt=5e-4, stepper=stepper) as p:
            p.set_sol(s0.T)
            pkg.autotune(p)
            pkg.stepforward(p, 3)
            out.append(p.sol_c())
    assert np.array_equal(out[0], out[1])
