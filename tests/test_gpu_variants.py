"""Every FFT pass kernel variant the autotuner can select computes the same right-hand side.

For each grid size with more than one candidate, each variant of each pass class is selected in
turn (the other classes at their defaults) and one RHS evaluation (mhd_compute_rhs) is compared
with the FP64 oracle's (calcN_fast) at the RHS parity tolerance, relative L2 <= 1e-5 on the
retained band.  At 512^3, where the FP64 oracle is too slow for a test, each variant is compared
with the default selection at the same tolerance.  Then mhd_autotune picks a variant per class,
and two steps with the tuned selection match two default steps to 1e-5.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("n", [32, 48, 64, 96, 128, 256, 512])
def test_variants_agree(pkg, mo, n):
    from importlib import import_module

    ic = import_module(pkg.__name__ + ".ic")
    s0 = ic.random_spectrum_state(n, seed=5)
    with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=2e-3, dt=1e-4, stepper="RK4") as prob:
        prob.set_sol(s0.T)
        var = pkg.variants(prob)
        defaults = {c: v[1].index(v[0]) for c, v in var.items()}
        if n <= 256:
            g = mo.Grid(n)
            ref = np.zeros(s0.shape, dtype=np.complex128)
            mo.calcN_fast(ref, s0.astype(np.complex128), g, 1e-3, 2e-3)
            mask = g.retained_mask()
            err0 = mo.rel_l2(prob.rhs_c(), ref, mask)
            assert err0 < TOL, f"default selection: rel L2 {err0:.2e}"
            rel = lambda a: mo.rel_l2(a, ref, mask)  # noqa: E731
        else:
            ref = prob.rhs_c()
            rel = lambda a: _rel(a, ref)  # noqa: E731
        checked = 0
        for cls, (_, names) in var.items():
            for i, name in enumerate(names):
                if i == defaults[cls]:
                    continue
                try:
                    pkg.select_variant(prob, cls, i)
                except pkg.MHDError:
                    continue  # does not fit on this device
                err = rel(prob.rhs_c())
                assert err < TOL, f"{cls} {name}: rel L2 {err:.2e}"
                checked += 1
            pkg.select_variant(prob, cls, defaults[cls])
        if n in (128, 256, 512):
            assert checked >= 3


@pytest.mark.parametrize("n", [64, 256])
def test_autotune_selects_and_steps_alike(pkg, n):
    from importlib import import_module

    ic = import_module(pkg.__name__ + ".ic")
    s0 = ic.random_spectrum_state(n, seed=9)
    kw = dict(nx=n, Lx=2 * math.pi, nu=1e-3, eta=1e-3, dt=5e-4, stepper="RK4")
    with pkg.Problem(pkg.GPU(0), **kw) as a:
        a.set_sol(s0.T)
        pkg.stepforward(a, 2)
        ref = a.sol_c()
    with pkg.Problem(pkg.GPU(0), **kw) as b:
        b.set_sol(s0.T)
        chosen = pkg.autotune(b, force=True, persist=False)
        assert set(chosen) == set(pkg.TUNED_CLASSES)
        assert all(chosen.values())
        pkg.stepforward(b, 2)
        got = b.sol_c()
        assert pkg.autotune(b, persist=False) == chosen  # known result: applied without timing
    assert _rel(got, ref) < TOL


def test_x_variants_give_the_same_cfl_dt(pkg):
    """The x-row kernels also reduce max|u| and max|B| for the on-device CFL step: every x
    variant at 256^3 (the paired-transform ones included) yields the default variant's dt."""
    from importlib import import_module

    ic = import_module(pkg.__name__ + ".ic")
    n = 256
    s0 = ic.random_spectrum_state(n, seed=13)
    with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-4, eta=1e-4, dt=1e-3, stepper="RK4") as prob:
        names = pkg.variants(prob)["x_fused"][1]
        dts = {}
        for i, name in enumerate(names):
            try:
                pkg.select_variant(prob, "x_fused", i)
            except pkg.MHDError:
                continue
            prob.set_sol(s0.T)
            prob.clock.t, prob.clock.step, prob.clock.dt = 0.0, 0, 1e-3
            pkg._lib.check(prob._lib.mhd_set_cfl(prob.handle, 1, 0.3))
            pkg.stepforward(prob, 1)
            dts[name] = prob.clock.dt
            pkg._lib.check(prob._lib.mhd_set_cfl(prob.handle, 0, 0.3))
        ref = dts[names[0]]
        assert len(dts) >= 3
        for name, dt in dts.items():
            assert dt == pytest.approx(ref, rel=1e-5), name
