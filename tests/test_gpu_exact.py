"""The CUDA path against exact solutions of the MHD equations, with no oracle in between.

MHDFlows.jl ships no tests and no golden vectors, so besides the oracle the solver is pinned to
solutions known in closed form, stepped on the GPU through the C ABI:
  * ABC (Beltrami) flow, B = 0: u x (curl u) = 0, so the stress divergence is a gradient that the
    projection removes, and u(t) = u0 exp(-nu k^2 t) (k = 1);
  * two-dimensional Taylor-Green flow u = (sin x cos y, -cos x sin y, 0), B = 0: an exact
    Navier-Stokes solution, u(t) = u0 exp(-2 nu t);
  * Alfven wave on a uniform field: B = B0 x + b, u = -b, b = eps (0, sin(x - B0 t), 0) solves the
    ideal equations exactly; with nu = eta both u and b also decay as exp(-nu t).
Tolerances: relative L2 of the state (retained band) or max error of the wave, FP32 kernels, after
hundreds of RK4 / LSRK4 steps: 1e-5 (time-discretisation error of these smooth solutions is far
below FP32 roundoff at these dt).  The on-device kinetic energy follows exp(-2 nu k^2 t) to 1e-5.
Fields that are zero in the exact solution stay at roundoff relative to the flow, 1e-6: the row
transforms carry two real fields in one complex transform (u_z with B_x, B_y with B_z), so FP32
roundoff of the partner leaks into a zero field and the equations carry it along.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(pkg, n, nu, eta, dt, stepper):
    return pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=nu, eta=eta, dt=dt, stepper=stepper)


def _set_fields(prob, fields):
    for f, a in enumerate(fields):
        prob.set_physical_c(f, np.asarray(a, dtype=np.float32))


@pytest.mark.parametrize("n,stepper,steps", [(64, "RK4", 200), (64, "LSRK4", 200), (256, "RK4", 50)])
def test_abc_flow_decays_exactly(pkg, mo, n, stepper, steps):
    nu, dt = 0.02, 0.005
    g = mo.Grid(n)
    x, y, z = g.mesh()
    A, B, C = 1.0, 0.7, 0.4
    ux = A * np.sin(z) + C * np.cos(y)
    uy = B * np.sin(x) + A * np.cos(z)
    uz = C * np.sin(y) + B * np.cos(x)
    zero = np.zeros_like(x)
    with _problem(pkg, n, nu, 0.0, dt, stepper) as prob:
        _set_fields(prob, [ux, uy, uz, zero, zero, zero])
        s0 = prob.sol_c().astype(np.complex128)
        e0 = prob.diagnostics().E_u
        pkg.stepforward(prob, steps)
        got = prob.sol_c()
        e1 = prob.diagnostics().E_u
    t = dt * steps
    expect = s0 * math.exp(-nu * t)
    m = g.retained_mask()
    err_u = mo.rel_l2(got[:3], expect[:3], m)
    print(f"ABC {n}^3 {stepper}: u rel L2 {err_u:.2e} after {steps} steps; B max {np.abs(got[3:]).max():.1e}")
    assert err_u < 1e-5
    assert np.abs(got[3:]).max() < 1e-6 * np.abs(got[:3]).max()
    assert e1 / e0 == pytest.approx(math.exp(-2 * nu * t), rel=1e-5)


def test_taylor_green_2d_is_an_exact_solution(pkg, mo):
    n, nu, dt, steps = 32, 0.05, 0.004, 250
    g = mo.Grid(n)
    x, y, z = g.mesh()
    zero = np.zeros_like(x)
    with _problem(pkg, n, nu, nu, dt, "RK4") as prob:
        _set_fields(prob, [np.sin(x) * np.cos(y), -np.cos(x) * np.sin(y), zero, zero, zero, zero])
        s0 = prob.sol_c().astype(np.complex128)
        pkg.stepforward(prob, steps)
        got = prob.sol_c()
    expect = s0 * math.exp(-2 * nu * dt * steps)
    err = mo.rel_l2(got[:2], expect[:2], g.retained_mask())
    print(f"2D Taylor-Green: rel L2 {err:.2e} after {steps} steps")
    assert err < 1e-5
    assert np.abs(got[2:]).max() < 1e-6 * np.abs(got[:2]).max()


@pytest.mark.parametrize("nu", [0.0, 0.02])
def test_alfven_wave_travels_exactly(pkg, mo, nu):
    n, B0, eps, dt, steps = 32, 1.0, 0.1, 0.005, 400
    g = mo.Grid(n)
    x, y, z = g.mesh()
    zero = np.zeros_like(x)
    b_y = eps * np.sin(x)
    with _problem(pkg, n, nu, nu, dt, "LSRK4") as prob:
        _set_fields(prob, [zero, -b_y, zero, B0 + zero, b_y, zero])
        pkg.stepforward(prob, steps)
        got_b = prob.physical_c(4).astype(np.float64)
        got_u = prob.physical_c(1).astype(np.float64)
    t = dt * steps
    decay = math.exp(-nu * t)
    # the wave's direction of travel follows the sign convention of the induction term
    err = min(np.abs(got_b - decay * eps * np.sin(x - s * B0 * t)).max() for s in (1.0, -1.0))
    print(f"Alfven wave nu={nu}: max |b_y - exact| / eps = {err / eps:.2e} after {steps} steps")
    assert err < 1e-5 * eps * 10
    assert np.abs(got_u + got_b).max() < 1e-5 * eps * 10
