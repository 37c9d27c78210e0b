"""A99 random forcing (SetUpFk! / A99ForceDriving!, src/pgen/A99ForceDriving_GPU.jl) against the
oracle's restatement, both driven by the same counter-based generator (seed, 8*step + stage).

Tolerance: relative L2 on the retained band 1e-5 (FP32 kernels, FP64 oracle), for one RHS, one
RK4 step and two LSRK4 steps (the second step checks the device step counter of the generator).
P = 1e-5 keeps the forcing comparable to the advection terms at these sizes.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

P, KF, SIGMA, B, SEED = 1e-5, 2.0, 1.0, 1.0, 1234


def _forcing_dict(mo, g):
    A = mo.a99_amplitude(g, KF, P, SIGMA)
    return dict(A=A, kf_used=B, sigma2=SIGMA ** 2, b=B, seed=SEED)


def test_forcing_amplitude_matches_setupfk(pkg, mo):
    n = 32
    g = mo.Grid(n)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
        pkg.SetUpFk(prob, kf=KF, P=P, sigma=SIGMA, b=B, seed=SEED)
        A, kf_used = pkg.forcing_amplitude(prob)
    assert A == pytest.approx(mo.a99_amplitude(g, KF, P, SIGMA), rel=1e-6)
    assert kf_used == B


def test_forced_rhs_matches_oracle(pkg, mo):
    n = 32
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=41).astype(np.complex64)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=2e-3, dt=1e-3) as prob:
        prob.set_sol(s.T)
        pkg.SetUpFk(prob, kf=KF, P=P, sigma=SIGMA, b=B, seed=SEED)
        got = prob.rhs_c()
    N = np.zeros(s.shape, dtype=np.complex128)
    mo.calcN_literal(N, s.astype(np.complex128), g, 1e-3, 2e-3)
    N0 = N.copy()
    mo.add_a99_forcing(N, g, _forcing_dict(mo, g), 8 * 0 + 7)
    m = g.retained_mask()
    assert mo.rel_l2(N, N0, m) > 1e-2  # the forcing is a visible part of the right-hand side
    err = mo.rel_l2(got, N, m)
    assert err < 1e-5, err
    assert np.all(got[:3, :, :, 0].imag == 0)  # kx = 0 plane: real right-hand side


@pytest.mark.parametrize("scheme,steps", [("RK4", 1), ("LSRK4", 2)])
def test_forced_steps_match_oracle(pkg, mo, scheme, steps):
    n = 32
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=42).astype(np.complex64)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3, stepper=scheme) as prob:
        prob.set_sol(s.T)
        pkg.SetUpFk(prob, kf=KF, P=P, sigma=SIGMA, b=B, seed=SEED)
        pkg.stepforward(prob, steps)
        got = prob.sol_c()
    st = mo.Stepper(g, 1e-3, 1e-3, 1e-3, scheme, literal=False)
    st.forcing = _forcing_dict(mo, g)
    ref = s.astype(np.complex128)
    for _ in range(steps):
        st.stepforward(ref)
    g.dealias(ref)
    err = mo.rel_l2(got, ref, g.retained_mask())
    assert err < 1e-5, err


def test_forcing_reproducible_by_seed(pkg, mo):
    n = 32
    s = mo.random_spectrum_state(mo.Grid(n), seed=43).astype(np.complex64)

    def run(seed, off=False):
        with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
            prob.set_sol(s.T)
            pkg.SetUpFk(prob, kf=KF, P=P, sigma=SIGMA, b=B, seed=seed)
            if off:
                pkg.SetUpFk(prob, P=0.0)
            pkg.stepforward(prob, 3)
            return prob.sol_c()

    a, b, c, d = run(5), run(5), run(6), run(5, off=True)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
        prob.set_sol(s.T)
        pkg.stepforward(prob, 3)
        assert np.array_equal(prob.sol_c(), d)


def test_hydrodynamic_problem_stays_unforced(pkg, mo):
    """HDcalcN! (src/pgen.jl:176-182) adds the forcing before HDcalcN_advection!, whose UᵢUpdate!
    zeroes the velocity right-hand side (src/Solver/HDSolver.jl:55): SetUpFk! leaves an HD run
    unchanged, bit for bit."""
    n = 32
    s = mo.random_spectrum_state(mo.Grid(n), seed=44).astype(np.complex64)[:3]

    def run(forced):
        with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, dt=1e-3, B_field=False) as prob:
            prob.set_sol(s.T)
            if forced:
                pkg.SetUpFk(prob, kf=KF, P=P, sigma=SIGMA, b=B, seed=SEED)
            pkg.stepforward(prob, 2)
            return prob.sol_c()

    assert np.array_equal(run(True), run(False))
