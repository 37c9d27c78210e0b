"""GPU parity of the CUDA path against the CPU oracle, through the C ABI.

Tolerances (relative L2 on the retained band, FP32 kernels vs FP64 oracle):
  transforms 2e-6, one RHS 1e-5, one RK4/LSRK4 step 1e-5, 100 RK4 steps 1e-4;
  max|k.u|, max|k.B| at FP32 roundoff: <= 1e-5 * max|k| * max|u_hat|.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [16, 32, 48, 64, 96, 128]


def make_problem(pkg, n, nu=1e-3, eta=1e-3, dt=5e-4, stepper="RK4"):
    return pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=nu, eta=eta, dt=dt, stepper=stepper)


@pytest.mark.parametrize("n", SIZES + [256])
def test_physical_roundtrip(pkg, mo, n):
    g = mo.Grid(n)
    rng = np.random.default_rng(n)
    phys = rng.standard_normal((n, n, n)).astype(np.float32)
    with make_problem(pkg, n) as prob:
        prob.set_physical_c(2, phys)
        got = prob.sol_c()[2]
        ref = g.rfft(phys.astype(np.float64))
        m = g.retained_mask()
        assert mo.rel_l2(got, ref, m) < 2e-6
        assert np.all(got[~m] == 0)
        back = prob.physical_c(2)
        expect = g.irfft(g.dealias(ref.copy()))
        assert np.linalg.norm(back - expect) / np.linalg.norm(expect) < 2e-6


@pytest.mark.parametrize("n", [32, 96])
def test_state_roundtrip_exact(pkg, mo, n):
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=3).astype(np.complex64)
    s[:, 1, 1, 1] += 1.0 + 2.0j  # arbitrary retained content
    with make_problem(pkg, n) as prob:
        prob.set_sol(s.T)
        got = prob.sol_c()
    expect = g.dealias(s.copy())
    assert np.array_equal(got, expect)


@pytest.mark.parametrize("n", SIZES)
def test_rhs_parity(pkg, mo, n):
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=11)
    s32 = s.astype(np.complex64)
    with make_problem(pkg, n, nu=2e-3, eta=3e-3) as prob:
        prob.set_sol(s32.T)
        got = prob.rhs_c()
    N = np.zeros_like(s)
    mo.calcN_literal(N, s32.astype(np.complex128), g, 2e-3, 3e-3)
    m = g.retained_mask()
    err = mo.rel_l2(got, N, m)
    assert err < 1e-5, err
    assert np.all(got[:, ~m] == 0)


def _run_oracle(mo, g, s0, nu, eta, dt, steps, scheme):
    st = mo.Stepper(g, nu, eta, dt, scheme, literal=False)
    s = s0.astype(np.complex128).copy()
    for _ in range(steps):
        st.stepforward(s)
    g.dealias(s)
    return s


def test_tg32_rk4_1_and_100_steps(pkg, mo):
    n = 32
    g = mo.Grid(n)
    fields = mo.taylor_green(g)
    s0 = mo.physical_to_state(g, fields)
    with make_problem(pkg, n, nu=1e-2, eta=1e-2, dt=1e-3) as prob:
        for f in range(6):
            prob.set_physical_c(f, fields[f].astype(np.float32))
        pkg.stepforward(prob, 1)
        one = prob.sol_c()
        pkg.stepforward(prob, 99)
        hundred = prob.sol_c()
        assert prob.clock.step == 100
    m = g.retained_mask()
    ref1 = _run_oracle(mo, g, s0, 1e-2, 1e-2, 1e-3, 1, "RK4")
    ref100 = _run_oracle(mo, g, ref1, 1e-2, 1e-2, 1e-3, 99, "RK4")
    e1 = mo.rel_l2(one, ref1, m)
    e100 = mo.rel_l2(hundred, ref100, m)
    assert e1 < 1e-5, e1
    assert e100 < 1e-4, e100


@pytest.mark.parametrize("n,scheme", [(32, "LSRK4"), (48, "RK4"), (64, "LSRK4"), (96, "RK4")])
def test_random_steps(pkg, mo, n, scheme):
    g = mo.Grid(n)
    s0 = mo.random_spectrum_state(g, seed=5).astype(np.complex64)
    dt = 0.2 * (2 * math.pi / n)
    with make_problem(pkg, n, nu=1e-3, eta=2e-3, dt=dt, stepper=scheme) as prob:
        prob.set_sol(s0.T)
        pkg.stepforward(prob, 5)
        got = prob.sol_c()
    ref = _run_oracle(mo, g, s0, 1e-3, 2e-3, dt, 5, scheme)
    err = mo.rel_l2(got, ref, g.retained_mask())
    assert err < 2e-5, err


def test_diagnostics(pkg, mo):
    n = 48
    g = mo.Grid(n)
    s0 = mo.random_spectrum_state(g, seed=9).astype(np.complex64)
    with make_problem(pkg, n) as prob:
        prob.set_sol(s0.T)
        d = prob.diagnostics()
        ke, me = pkg.ProbDiagnostic(prob)
    ref = mo.spectral_diagnostics(g, s0)
    assert abs(d.E_u - ref["E_u"]) / ref["E_u"] < 1e-6
    assert abs(d.E_B - ref["E_B"]) / ref["E_B"] < 1e-6
    assert abs(d.H_c - ref["H_c"]) < 1e-6 * math.sqrt(ref["E_u"] * ref["E_B"])
    assert d.nonfinite == 0
    assert ke == float(f"{ref['E_u']:.3g}") and me == float(f"{ref['E_B']:.3g}")
    kmax = math.sqrt(3) * n / 3
    umax = np.abs(s0).max()
    assert d.max_kdotu <= 1e-5 * kmax * umax
    assert d.max_kdotb <= 1e-5 * kmax * umax
    assert d.max_divb < 1e-4


def test_updatevars_matches_oracle(pkg, mo):
    n = 32
    g = mo.Grid(n)
    s0 = mo.random_spectrum_state(g, seed=2).astype(np.complex64)
    with make_problem(pkg, n) as prob:
        prob.set_sol(s0.T)
        pkg.updatevars(prob)
        ux = prob.vars.ux.copy()
    expect = g.irfft(s0[0].astype(np.complex128))  # (nz, ny, nx)
    assert np.linalg.norm(ux.T - expect) / np.linalg.norm(expect) < 2e-6


def test_256_one_step_vs_oracle(pkg, mo):
    n = 256
    g = mo.Grid(n)
    s0 = mo.random_spectrum_state(g, seed=1).astype(np.complex64)
    with make_problem(pkg, n, nu=1e-3, eta=1e-3, dt=5e-4) as prob:
        prob.set_sol(s0.T)
        pkg.stepforward(prob, 1)
        got = prob.sol_c()
        d = prob.diagnostics()
    ref = _run_oracle(mo, g, s0, 1e-3, 1e-3, 5e-4, 1, "RK4")
    err = mo.rel_l2(got, ref, g.retained_mask())
    assert err < 1e-5, err
    assert d.max_divb < 1e-3
