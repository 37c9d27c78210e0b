"""Volume penalisation (VP_method = true, src/Solver/VPSolver.jl) and the divergence corrections
through the C ABI, against the oracle's restatement (oracle.mhd_oracle.vp_update / div_correct).

Tolerances (relative L2 on the retained band, FP32 kernels against the FP64 oracle): RHS 1e-5,
RK4 / LSRK4 steps 1e-5, divergence corrections 1e-6.  The penalty factor 1/eta = 7 / (13 dt) makes
the penalty the largest term of these right-hand sides, so they test it directly.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mask(g, r=1.2):
    x, y, z = g.mesh()
    d = np.sqrt(x ** 2 + (y - 0.3) ** 2 + z ** 2)
    return (0.5 * (1 - np.tanh((d - r) / 0.25))).astype(np.float32)


def _walls(g, seed):
    rng = np.random.default_rng(seed)
    x, y, z = g.mesh()
    return tuple((rng.uniform(0.2, 1.0) * np.sin(x + rng.uniform(0, 6)) * np.cos(y - z)).astype(np.float32)
                 for _ in range(3))


def _state(mo, g, seed, hydro=False):
    s = mo.random_spectrum_state(g, seed=seed).astype(np.complex64)
    if hydro:
        s[3:] = 0
    return s


def _T(t):
    return None if t is None else tuple(a.T for a in t)


@pytest.mark.parametrize("walls", [False, True])
def test_vp_rhs_matches_oracle(pkg, mo, walls):
    n, dt = 32, 1e-3
    g = mo.Grid(n)
    s = _state(mo, g, 61)
    chi = _mask(g)
    U0, B0 = (_walls(g, 1), _walls(g, 2)) if walls else (None, None)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=2e-3, dt=dt, VP_method=True) as prob:
        prob.set_sol(s.T)
        prob.set_vp(chi.T, U0=_T(U0), B0=_T(B0))
        got = prob.rhs_c()
    N = np.zeros(s.shape, dtype=np.complex128)
    vp = dict(chi=chi.astype(np.float64), dt=dt,
              U0=None if U0 is None else tuple(a.astype(np.float64) for a in U0),
              B0=None if B0 is None else tuple(a.astype(np.float64) for a in B0))
    mo.calcN_literal(N, s.astype(np.complex128), g, 1e-3, 2e-3, vp=vp)
    N0 = np.zeros_like(N)
    mo.calcN_literal(N0, s.astype(np.complex128), g, 1e-3, 2e-3)
    m = g.retained_mask()
    assert mo.rel_l2(N0, N, m) > 0.5  # the penalty dominates
    err = mo.rel_l2(got, N, m)
    print(f"VP RHS walls={walls} rel L2 vs FP64 oracle: {err:.3e}")
    assert err < 1e-5, err


@pytest.mark.parametrize("scheme,steps", [("RK4", 2), ("LSRK4", 2)])
def test_vp_steps_match_oracle(pkg, mo, scheme, steps):
    n, dt = 48, 1e-3
    g = mo.Grid(n)
    s = _state(mo, g, 62)
    chi = _mask(g)
    U0 = _walls(g, 3)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=dt, stepper=scheme, VP_method=True) as prob:
        prob.set_sol(s.T)
        prob.set_vp(chi.T, U0=_T(U0))
        pkg.stepforward(prob, steps)
        got = prob.sol_c()
    st = mo.Stepper(g, 1e-3, 1e-3, dt, scheme, literal=False)
    st.vp = dict(chi=chi.astype(np.float64), U0=tuple(a.astype(np.float64) for a in U0))
    ref = s.astype(np.complex128)
    for _ in range(steps):
        st.stepforward(ref)
    g.dealias(ref)
    err = mo.rel_l2(got, ref, g.retained_mask())
    print(f"VP {scheme} {steps} steps rel L2 vs FP64 oracle: {err:.3e}")
    assert err < 1e-5, err


@pytest.mark.parametrize("n,walls,scheme", [(32, True, "RK4"), (48, False, "LSRK4"), (128, True, "RK4")])
def test_vp_hydrodynamic(pkg, mo, n, walls, scheme):
    """VP on the hydrodynamic passes: the velocity penalty fields ride in the spare product slots."""
    dt = 1e-3
    g = mo.Grid(n)
    s = _state(mo, g, 63, hydro=True)
    chi = _mask(g)
    U0 = _walls(g, 4) if walls else None
    with pkg.Problem(pkg.GPU(0), nx=n, nu=2e-3, dt=dt, B_field=False, VP_method=True, stepper=scheme) as prob:
        prob.set_sol(s[:3].T)
        prob.set_vp(chi.T, U0=_T(U0))
        got_rhs = prob.rhs_c()
        pkg.stepforward(prob, 2)
        got = prob.sol_c()
        d = prob.diagnostics()
    vp = dict(chi=chi.astype(np.float64), U0=None if U0 is None else tuple(a.astype(np.float64) for a in U0))
    N = np.zeros(s.shape, dtype=np.complex128)
    mo.calcN_fast(N, s.astype(np.complex128), g, 2e-3, 0.0, vp=dict(vp, dt=dt))
    m = g.retained_mask()
    e_rhs = mo.rel_l2(got_rhs, N[:3], m)
    print(f"VP HD n={n} walls={walls} RHS rel L2 vs FP64 oracle: {e_rhs:.3e}")
    assert e_rhs < 1e-5, e_rhs
    st = mo.Stepper(g, 2e-3, 0.0, dt, scheme, literal=False)
    st.vp = vp
    ref = s.astype(np.complex128)
    for _ in range(2):
        st.stepforward(ref)
    g.dealias(ref)
    err = mo.rel_l2(got, ref[:3], m)
    print(f"VP HD n={n} two {scheme} steps rel L2 vs FP64 oracle: {err:.3e}")
    assert err < 1e-5, err
    assert d.E_B == 0.0


def test_div_corrections_match_oracle(pkg, mo):
    n = 32
    g = mo.Grid(n)
    s = _state(mo, g, 64).astype(np.complex128)
    rng = np.random.default_rng(65)
    phi = rng.standard_normal(s.shape[1:]) + 1j * rng.standard_normal(s.shape[1:])
    phi[~g.retained_mask()] = 0
    bad = (s + np.stack([1j * k * phi for k in g.ks] * 2)).astype(np.complex64)
    m = g.retained_mask()
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3, VP_method=True) as prob:
        prob.set_sol(bad.T)
        pkg.DivVCorrection(prob)
        got_u = prob.sol_c()
        pkg.DivBCorrection(prob)
        got = prob.sol_c()
    ref_u = mo.div_correct(g, bad.astype(np.complex128), 1)
    ref = mo.div_correct(g, bad.astype(np.complex128), 3)
    e_u, e_b = mo.rel_l2(got_u, ref_u, m), mo.rel_l2(got, ref, m)
    print(f"DivVCorrection / DivBCorrection rel L2 vs FP64 oracle: {e_u:.3e} / {e_b:.3e}")
    assert e_u < 1e-6 and e_b < 1e-6
    assert mo.rel_l2(got, s, m) < 1e-6


def test_time_integrator_with_vp(pkg, mo):
    """TimeIntegrator! with VP (src/integrator.jl:84-88,118-122): divergence corrections before the
    loop and after every step, fixed dt."""
    n, dt, N0 = 32, 1e-3, 2
    g = mo.Grid(n)
    s = _state(mo, g, 66)
    chi = _mask(g)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=dt, VP_method=True) as prob:
        prob.set_sol(s.T)
        prob.set_vp(chi.T)
        pkg.TimeIntegrator(prob, math.inf, N0, usr_dt=dt)
        got = prob.sol_c()
        assert prob.clock.step == N0 + 1
    st = mo.Stepper(g, 1e-3, 1e-3, dt, "RK4", literal=False)
    st.vp = dict(chi=chi.astype(np.float64))
    ref = mo.div_correct(g, s.astype(np.complex128), 3)
    for _ in range(N0 + 1):
        st.stepforward(ref)
        g.dealias(ref)
        mo.div_correct(g, ref, 3)
    err = mo.rel_l2(got, ref, g.retained_mask())
    print(f"VP TimeIntegrator ({N0 + 1} steps) rel L2 vs FP64 oracle: {err:.3e}")
    assert err < 1e-5, err


def test_vp_cfl_reads_corrected_fields(pkg, mo):
    """With the on-device CFL, the dt after a corrected step comes from the corrected state's
    physical maxima (getCFL! reads the vars DivVCorrection! / DivBCorrection! refreshed)."""
    n, coef = 32, 0.3
    g = mo.Grid(n)
    s = _state(mo, g, 67)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3, VP_method=True) as prob:
        prob.set_sol(s.T)
        prob.set_vp(_mask(g).T)
        pkg.TimeIntegrator(prob, math.inf, 1, CFL_Coef=coef)
        state = prob.sol_c().astype(np.complex128)
        dt = prob.clock.dt
    vmax = max(np.abs(g.irfft(state[f])).max() for f in range(6))
    dl = 2 * math.pi / n
    expect = min(coef * dl / vmax, coef * dl * dl / 1e-3)
    assert dt == pytest.approx(expect, rel=2e-5)


def test_vp_batch_slots_are_independent(pkg, mo):
    n, dt = 32, 1e-3
    g = mo.Grid(n)
    s = _state(mo, g, 68)
    chis = [_mask(g, 1.0), _mask(g, 1.6)]
    single = []
    for chi in chis:
        with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=dt, VP_method=True) as prob:
            prob.set_sol(s.T)
            prob.set_vp(chi.T)
            pkg.stepforward(prob, 2)
            single.append(prob.sol_c())
    b = pkg.Batch(n, 2, VP_method=True)
    try:
        slots = [b.add(1e-3, 1e-3, dt) for _ in chis]
        for sl, chi in zip(slots, chis):
            b.set_state(sl, s)
            b.set_vp(sl, chi.T)
        b.step(2)
        for sl, ref in zip(slots, single):
            assert np.array_equal(b.get_state(sl), ref)
    finally:
        b.close()


def test_vp_errors(pkg):
    with pkg.Problem(pkg.GPU(0), nx=32, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
        with pytest.raises(pkg.MHDError):
            prob.set_vp(np.zeros((32, 32, 32), np.float32))
    with pytest.raises(pkg.MHDError):
        pkg.Problem(pkg.GPU(0), nx=128, nu=1e-3, eta=1e-3, dt=1e-3, VP_method=True, precision="split_fp16")
    with pkg.Problem(pkg.GPU(0), nx=32, nu=1e-3, eta=1e-3, dt=1e-3, VP_method=True) as prob:
        with pytest.raises(pkg.MHDError):
            prob.set_vp(np.zeros((16, 16, 16), np.float32))
