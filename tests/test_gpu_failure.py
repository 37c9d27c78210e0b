"""Failure detection without a GPU fault: the bounded device wait the TMA-fed column passes use
gives up after its limit, records the timeout and returns, and the context stays usable."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(pkg, mo, lib):
    t, ms = C.c_int(-1), C.c_double(-1.0)
    pkg._lib.check(lib.mhd_check_bounded_wait(0, 5.0, C.byref(t), C.byref(ms)))
    assert t.value == 1
    assert 4.5 <= ms.value < 500.0, ms.value
    # the same process keeps stepping problems after the timed-out wait
    n = 32
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=81).astype(np.complex64)
    with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
        prob.set_sol(s.T)
        pkg.stepforward(prob, 2)
        prob.synchronize()
        assert prob.diagnostics().nonfinite == 0
