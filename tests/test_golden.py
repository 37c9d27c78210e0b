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


def _make_golden():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def test_oracle_reproduces_vp_and_hd_fixtures(mo):
    mg = _make_golden()
    g32, g48 = mo.Grid(32), mo.Grid(48)
    d = load("vp32_rhs.npz")
    s = mo.random_spectrum_state(g32, 13)
    N = np.zeros_like(s)
    mo.calcN_literal(N, s.copy(), g32, 2e-3, 3e-3, vp=mg._vp(g32, 1e-3))
    assert rel(compact(mo, g32, N), d["rhs"]) < 1e-12
    d = load("hd48_rk4.npz")
    s = mo.random_spectrum_state(g48, 17)
    s[3:] = 0
    st = mo.Stepper(g48, 1e-3, 0.0, 1e-3, "RK4", literal=False)
    for _ in range(3):
        st.stepforward(s)
    assert rel(compact(mo, g48, g48.dealias(s))[:3], d["s3"]) < 1e-12


def _vp_arrays(mg, g, walls_b=True):
    chi, U0, B0 = mg.vp_inputs(g)
    return chi.T, tuple(a.T for a in U0), (tuple(a.T for a in B0) if walls_b else None)


@pytest.mark.gpu
def test_gpu_vp32_rhs_against_golden(pkg, mo):
    mg = _make_golden()
    d = load("vp32_rhs.npz")
    g = mo.Grid(32)
    chi, U0, B0 = _vp_arrays(mg, g)
    with pkg.Problem(pkg.GPU(0), nx=32, Lx=2 * math.pi, nu=2e-3, eta=3e-3, dt=1e-3, VP_method=True) as prob:
        prob.set_sol(mo.expand_compact(32, d["s"], np.complex64).T)
        prob.set_vp(chi, U0=U0, B0=B0)
        got = prob.rhs_c()
    assert rel(compact(mo, g, got), d["rhs"]) < 1e-5


@pytest.mark.gpu
def test_gpu_hd_fixtures(pkg, mo):
    mg = _make_golden()
    d = load("hd48_rk4.npz")
    g = mo.Grid(48)
    full = np.zeros((6,) + d["s0"].shape[1:], np.complex128)
    full[:3] = d["s0"]
    with pkg.Problem(pkg.GPU(0), nx=48, Lx=2 * math.pi, nu=1e-3, dt=1e-3, B_field=False) as prob:
        prob.set_sol(mo.expand_compact(48, full, np.complex64)[:3].T)
        pkg.stepforward(prob, 3)
        err = rel(compact(mo, g, prob.sol_c()), d["s3"])
    assert err < 1e-5, err
    d = load("hdvp32_rk4.npz")
    g = mo.Grid(32)
    full = np.zeros((6,) + d["s0"].shape[1:], np.complex128)
    full[:3] = d["s0"]
    chi, U0, _ = _vp_arrays(mg, g, walls_b=False)
    with pkg.Problem(pkg.GPU(0), nx=32, Lx=2 * math.pi, nu=2e-3, dt=1e-3, B_field=False, VP_method=True) as prob:
        prob.set_sol(mo.expand_compact(32, full, np.complex64)[:3].T)
        prob.set_vp(chi, U0=U0)
        pkg.stepforward(prob, 2)
        err = rel(compact(mo, g, prob.sol_c()), d["s2"])
    assert err < 1e-5, err


def test_oracle_reproduces_forced32(mo):
    d = load("forced32_rk4.npz")
    g = mo.Grid(32)
    s = mo.random_spectrum_state(g, 23)
    assert rel(compact(mo, g, s), d["s0"]) < 1e-14
    st = mo.Stepper(g, 1e-3, 1e-3, 1e-3, "RK4", literal=False)
    st.forcing = dict(A=mo.a99_amplitude(g, 2.0, 1e-5, 1.0), kf_used=1.0, sigma2=1.0, b=1.0, seed=1234)
    for _ in range(2):
        st.stepforward(s)
    assert rel(compact(mo, g, g.dealias(s)), d["s2"]) < 1e-12


@pytest.mark.gpu
def test_gpu_forced32_against_golden(pkg, mo):
    d = load("forced32_rk4.npz")
    g = mo.Grid(32)
    with _problem(pkg, 32, 1e-3, 1e-3, 1e-3, "RK4") as prob:
        prob.set_sol(mo.expand_compact(32, d["s0"], np.complex64).T)
        pkg.SetUpFk(prob, kf=2.0, P=1e-5, sigma=1.0, b=1.0, seed=1234)
        pkg.stepforward(prob, 2)
        err = rel(compact(mo, g, prob.sol_c()), d["s2"])
    assert err < 1e-5, err
