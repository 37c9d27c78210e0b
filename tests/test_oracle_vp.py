"""CPU tests of the oracle's volume penalisation (src/Solver/VPSolver.jl) and divergence
corrections, from identities the mathematics gives:
  * the literal (reference-ordered) and compact right-hand sides agree with VP on;
  * with a constant mask c and zero walls the penalty of a solenoidal state is exactly
    -(c / eta) times the state (eta = 13 dt / 7);
  * the penalty's energy rate is 2 Re sum conj(s) dN = -(2 n^3 / eta) sum_x chi (|u|^2 + |B|^2);
  * DivVCorrection! / DivBCorrection! remove exactly the gradient part: k.X = 0 afterwards, a
    solenoidal field is unchanged, a gradient field vanishes, the map is idempotent.
"""
import numpy as np


def _mask(mo, g, r=1.0):
    """Smoothed ball obstacle of radius r at the box centre, (nz, ny, nx)."""
    x, y, z = g.mesh()
    d = np.sqrt(x ** 2 + y ** 2 + z ** 2)
    return 0.5 * (1 - np.tanh((d - r) / 0.2))


def _walls(g, seed):
    rng = np.random.default_rng(seed)
    x, y, z = g.mesh()
    return tuple(rng.standard_normal() * np.sin(x + rng.uniform(0, 6)) * np.cos(y - z) for _ in range(3))


def test_vp_literal_equals_fast(mo):
    for n in (16, 24):
        g = mo.Grid(n)
        s = mo.random_spectrum_state(g, seed=51)
        vp = dict(chi=_mask(mo, g), U0=_walls(g, 1), B0=_walls(g, 2), dt=1e-3)
        a, b = np.zeros_like(s), np.zeros_like(s)
        mo.calcN_literal(a, s.copy(), g, 1e-3, 2e-3, vp=vp)
        mo.calcN_fast(b, s.copy(), g, 1e-3, 2e-3, vp=vp)
        assert mo.rel_l2(a, b, g.retained_mask()) < 1e-13


def test_constant_mask_is_a_uniform_damping(mo):
    n, c, dt = 16, 0.7, 2e-3
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=52)
    g.dealias(s)
    plain, pen = np.zeros_like(s), np.zeros_like(s)
    mo.calcN_fast(plain, s.copy(), g, 1e-3, 1e-3)
    mo.calcN_fast(pen, s.copy(), g, 1e-3, 1e-3, vp=dict(chi=np.full((n, n, n), c), dt=dt))
    eta = dt * 13 / 7
    d = pen - plain + (c / eta) * s
    assert np.abs(d).max() < 1e-9 * (c / eta) * np.abs(s).max()


def test_penalty_energy_rate(mo):
    n, dt = 24, 1e-3
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=53)
    g.dealias(s)
    chi = _mask(mo, g)
    plain, pen = np.zeros_like(s), np.zeros_like(s)
    mo.calcN_fast(plain, s.copy(), g, 0.0, 0.0)
    mo.calcN_fast(pen, s.copy(), g, 0.0, 0.0, vp=dict(chi=chi, dt=dt))
    w = np.ones((1, 1, g.nkr))
    w[..., 1:] = 2
    w[..., -1] = 1  # Nyquist column of the half spectrum counted once
    rate = 2 * np.sum(w * (np.conj(s) * (pen - plain)).real)
    v = [g.irfft(s[f]) for f in range(6)]
    expect = -(2 * n ** 3 / (dt * 13 / 7)) * np.sum(chi * sum(f ** 2 for f in v))
    assert expect < 0
    assert abs(rate - expect) < 1e-9 * abs(expect)


def test_div_correct_removes_gradient_part(mo):
    n = 16
    g = mo.Grid(n)
    sol = mo.random_spectrum_state(g, seed=54)  # solenoidal u and B
    g.dealias(sol)
    rng = np.random.default_rng(55)
    phi = (rng.standard_normal(sol.shape[1:]) + 1j * rng.standard_normal(sol.shape[1:]))
    phi[~g.retained_mask()] = 0
    grad = np.stack([1j * k * phi for k in g.ks] * 2)  # i k phi in both triples
    both = sol + grad
    out = mo.div_correct(g, both.copy(), 3)
    ks = g.ks
    for off in (0, 3):
        assert np.abs(sum(ks[i] * out[off + i] for i in range(3))).max() < 1e-12 * np.abs(out).max()
    assert np.abs(out - sol).max() < 1e-12 * np.abs(sol).max()
    assert np.abs(mo.div_correct(g, out.copy(), 3) - out).max() < 1e-14 * np.abs(out).max()  # idempotent
    only_u = mo.div_correct(g, both.copy(), 1)
    assert np.abs(only_u[3:] - both[3:]).max() == 0
    assert np.abs(only_u[:3] - sol[:3]).max() < 1e-12 * np.abs(sol).max()
