"""Memory safety without compute-sanitizer: every large device buffer of a handle ends in a guard
band of a fixed byte (mhd_check_guards).  Each configuration below runs the entry points that
write device memory (state and field transfers, steps, right-hand sides, diagnostics, the
autotuner's sweep over every kernel variant) and then requires every guard byte intact."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _guards(pkg, lib, h):
    bad = C.c_longlong(-1)
    pkg._lib.check(lib.mhd_check_guards(h, C.byref(bad)))
    return bad.value


def _exercise(pkg, prob, s, nf):
    prob.set_sol(s[:nf].T)
    pkg.stepforward(prob, 2)
    prob.rhs_c()
    prob.sol_c()
    f = prob.physical_c(0)
    prob.set_physical_c(0, f)
    prob.diagnostics()


@pytest.mark.parametrize("n,kw", [
    (16, {}),
    (48, dict(stepper="LSRK4")),
    (96, dict(B_field=False)),
    (64, dict(VP_method=True)),
    (48, dict(VP_method=True, B_field=False)),
    (128, dict(precision="split_fp16")),
    (256, {}),
])
def test_guards_intact(pkg, mo, lib, n, kw):
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=101).astype(np.complex64)
    nf = 3 if kw.get("B_field", True) is False else 6
    with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=1e-3, dt=5e-4, **kw) as prob:
        if kw.get("VP_method"):
            x, y, z = g.mesh()
            chi = (np.sqrt(x ** 2 + y ** 2 + z ** 2) < 1.0).astype(np.float32)
            prob.set_vp(chi.T, U0=(chi.T * 0.1,) * 3, B0=(chi.T * 0.2,) * 3)
        assert _guards(pkg, lib, prob.handle) == 0
        _exercise(pkg, prob, s, nf)
        pkg.autotune(prob, force=True, persist=False)  # every kernel variant of every class
        pkg.stepforward(prob, 1)
        assert _guards(pkg, lib, prob.handle) == 0


def test_guards_intact_in_a_batch(pkg, mo, lib):
    n = 32
    s = mo.random_spectrum_state(mo.Grid(n), seed=102).astype(np.complex64)
    b = pkg.Batch(n, 3)
    try:
        slots = [b.add(1e-3, 1e-3, 1e-3) for _ in range(3)]
        for sl in slots:
            b.set_state(sl, s)
        b.remove(slots[1])
        b.step(3)
        b.get_state(slots[2])
        assert _guards(pkg, lib, b.handle) == 0
    finally:
        b.close()
