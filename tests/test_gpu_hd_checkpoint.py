"""Hydrodynamics (B_field=false) and checkpoint / restart through the C ABI.

HD: HDcalcN! (src/pgen.jl:176-182, src/Solver/HDSolver.jl) is the MHD momentum equation with
B = 0; the library runs it with a zero induction right-hand side, so B stays exactly zero.  Tolerances as in test_gpu_parity.py
(relative L2 on the retained band): RHS 1e-5, one RK4 step 1e-5.
Checkpoint: savefile -> Restart round trip, physical fields to 2e-6 (one c2r + r2c in FP32).
"""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _hd_state(mo, g, seed):
    s = mo.random_spectrum_state(g, seed=seed)
    s[3:] = 0
    return s


def test_hd_rhs_matches_oracle(pkg, mo):
    n = 32
    g = mo.Grid(n)
    s = _hd_state(mo, g, 31)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=2e-3, dt=1e-3, B_field=False) as prob:
        assert prob.nfields == 3
        prob.set_sol(s[:3].astype(np.complex64).T)
        got = prob.rhs_c()
    N = np.zeros_like(s)
    mo.calcN_literal(N, s.astype(np.complex64).astype(np.complex128), g, 2e-3, 0.0)
    m = g.retained_mask()
    err = mo.rel_l2(got, N[:3], m)
    assert err < 1e-5, err
    assert np.all(N[3:] == 0)


def test_hd_steps_keep_b_zero_and_match_oracle(pkg, mo):
    n = 48
    g = mo.Grid(n)
    s = _hd_state(mo, g, 32)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, dt=1e-3, B_field=False, stepper="RK4") as prob:
        prob.set_sol(s[:3].astype(np.complex64).T)
        pkg.stepforward(prob, 3)
        got = prob.sol_c()
        d = prob.diagnostics()
    st = mo.Stepper(g, 1e-3, 0.0, 1e-3, "RK4", literal=False)
    ref = s.astype(np.complex64).astype(np.complex128)
    for _ in range(3):
        st.stepforward(ref)
    g.dealias(ref)
    err = mo.rel_l2(got, ref[:3], g.retained_mask())
    assert err < 1e-5, err
    assert d.E_B == 0.0 and d.H_c == 0.0 and d.max_kdotb == 0.0


@pytest.mark.parametrize("n,scheme", [(128, "RK4"), (96, "LSRK4")])
def test_hd_dedicated_passes_match_oracle(pkg, mo, n, scheme):
    """The hydrodynamic passes (three fields in, five products out) at larger sizes: the RHS and
    one step against the FP64 oracle with B = 0."""
    g = mo.Grid(n)
    s = _hd_state(mo, g, 33)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, dt=5e-4, B_field=False, stepper=scheme) as prob:
        prob.set_sol(s[:3].astype(np.complex64).T)
        rhs = prob.rhs_c()
        pkg.stepforward(prob, 1)
        got = prob.sol_c()
    m = g.retained_mask()
    N = np.zeros_like(s)
    mo.calcN_fast(N, s.astype(np.complex64).astype(np.complex128), g, 1e-3, 0.0)
    e_rhs = mo.rel_l2(rhs, N[:3], m)
    st = mo.Stepper(g, 1e-3, 0.0, 5e-4, scheme, literal=False)
    ref = s.astype(np.complex64).astype(np.complex128)
    st.stepforward(ref)
    g.dealias(ref)
    e_step = mo.rel_l2(got, ref[:3], m)
    print(f"HD n={n} {scheme}: RHS {e_rhs:.3e}, one step {e_step:.3e} rel L2 vs FP64 oracle")
    assert e_rhs < 1e-5 and e_step < 1e-5


def test_hd_rejects_magnetic_fields(pkg):
    with pkg.Problem(pkg.GPU(0), nx=16, nu=1e-3, dt=1e-3, B_field=False) as prob:
        with pytest.raises(pkg.MHDError):
            pkg.SetUpProblemIC(prob, bx=np.zeros((16, 16, 16), np.float32))


def test_savefile_restart_round_trip(pkg, mo, tmp_path):
    n = 32
    g = mo.Grid(n)
    fields = mo.taylor_green(g)
    kw = dict(nx=n, Lx=2 * math.pi, nu=1e-2, eta=1e-2, dt=1e-3)
    with pkg.Problem(pkg.GPU(0), **kw) as a:
        pkg.SetUpProblemIC(a, **{k: fields[i].astype(np.float32).T for i, k in enumerate(pkg.FIELDS)})
        pkg.stepforward(a, 5)
        path = pkg.savefile(a, 7, file_path_and_name=str(tmp_path / "run"))
        assert os.path.basename(path) == "run_t_0007.h5"
        sol_a = a.sol_c()
        t_a = a.clock.t
    iv, jv, kv, ib, jb, kb, t = pkg.readMHDFlows(path)
    assert iv.shape == (n, n, n) and iv.dtype == np.float32 and t == pytest.approx(t_a)
    with pkg.Problem(pkg.GPU(0), **kw) as b:
        pkg.Restart(b, path)
        assert b.clock.t == pytest.approx(t_a)
        sol_b = b.sol_c()
    err = mo.rel_l2(sol_b, sol_a, g.retained_mask())
    assert err < 2e-6, err
