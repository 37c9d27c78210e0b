"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from the FP64 oracle).

CPU tests pin the oracle to its own committed outputs; GPU tests compare the CUDA path with them
through the C ABI (tolerances as in test_gpu_parity: 1e-5 one step / one RHS, 1e-4 after 100).
"""
import math
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(HERE, name)))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def compact(mo, g, s):
    kxs, kfs = mo.kept_wavenumbers(g.n)
    idx = kfs % g.n
    return s[:, idx][:, :, idx][:, :, :, : len(kxs)]


def test_oracle_reproduces_tg32(mo):
    d = load("tg32_rk4.npz")
    g = mo.Grid(32)
    s = mo.physical_to_state(g, mo.taylor_green(g))
    st = mo.Stepper(g, 1e-2, 1e-2, 1e-3, "RK4", literal=True)
    assert rel(compact(mo, g, g.dealias(s.copy())), d["s0"]) < 1e-14
    st.stepforward(s)
    assert rel(compact(mo, g, g.dealias(s.copy())), d["s1"]) < 1e-13
    assert abs(mo.spectral_diagnostics(g, s)["E_u"] - d["E_u"][0]) < 1e-12 * d["E_u"][0]
    # energy decays monotonically for Taylor-Green MHD with nu = eta = 1e-2
    assert np.all(np.diff(d["E_u"] + d["E_B"]) < 0)


def test_oracle_reproduces_rhs32(mo):
    d = load("rhs32.npz")
    g = mo.Grid(32)
    s = mo.random_spectrum_state(g, 11)
    assert rel(compact(mo, g, s), d["s"]) < 1e-14
    N = np.zeros_like(s)
    mo.calcN_literal(N, s.copy(), g, 2e-3, 3e-3)
    assert rel(compact(mo, g, N), d["rhs"]) < 1e-12


def test_oracle_reproduces_rand48_initial(mo):
    d = load("rand48_lsrk4.npz")
    g = mo.Grid(48)
    assert rel(compact(mo, g, mo.random_spectrum_state(g, 7)), d["s0"]) < 1e-14


def _problem(pkg, n, nu, eta, dt, stepper):
    return pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=nu, eta=eta, dt=dt, stepper=stepper)


@pytest.mark.gpu
def test_gpu_tg32_against_golden(pkg, mo):
    d = load("tg32_rk4.npz")
    g = mo.Grid(32)
    with _problem(pkg, 32, 1e-2, 1e-2, 1e-3, "RK4") as prob:
        prob.set_sol(mo.expand_compact(32, d["s0"], np.complex64).T)
        pkg.stepforward(prob)
        e1 = rel(compact(mo, g, prob.sol_c()), d["s1"])
        eu = [prob.diagnostics().E_u]
        for _ in range(99):
            pkg.stepforward(prob)
            eu.append(prob.diagnostics().E_u)
        e100 = rel(compact(mo, g, prob.sol_c()), d["s100"])
    assert e1 < 1e-5, e1
    assert e100 < 1e-4, e100
    assert np.max(np.abs(np.array(eu) - d["E_u"]) / d["E_u"]) < 1e-5


@pytest.mark.gpu
def test_gpu_rand48_lsrk4_against_golden(pkg, mo):
    d = load("rand48_lsrk4.npz")
    g = mo.Grid(48)
    with _problem(pkg, 48, 1e-3, 2e-3, float(d["dt"]), "LSRK4") as prob:
        prob.set_sol(mo.expand_compact(48, d["s0"], np.complex64).T)
        pkg.stepforward(prob, 10)
        err = rel(compact(mo, g, prob.sol_c()), d["s10"])
    assert err < 3e-5, err


@pytest.mark.gpu
def test_gpu_rhs32_against_golden(pkg, mo):
    d = load("rhs32.npz")
    g = mo.Grid(32)
    with _problem(pkg, 32, 2e-3, 3e-3, 1e-3, "RK4") as prob:
        prob.set_sol(mo.expand_compact(32, d["s"], np.complex64).T)
        got = prob.rhs_c()
    assert rel(compact(mo, g, got), d["rhs"]) < 1e-5
