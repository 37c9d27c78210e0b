"""CPU tests of the oracle: conventions, known answers from the mathematics, FP32/FP64 agreement.

The reference ships no tests or golden vectors, so these pin the restatement itself:
  * alias ranges and grid conventions (FourierFlows ThreeDGrid / getaliasedwavenumbers);
  * the literal reference-ordered RHS equals the compact form;
  * exact solutions: an ABC (Beltrami) flow with B = 0 decays as exp(-nu k^2 t) (its nonlinear
    term is a pure gradient), and a uniform B0 with a transverse Alfven wave u = -b/sqrt(1)
    travels exactly (ideal limit) with viscous/resistive decay;
  * solenoidality is preserved and the energy budget dE/dt = -2 nu <|w|^2> - 2 eta <|J|^2>;
  * Taylor-Green symmetries.
"""
import math

import numpy as np
import pytest


def test_alias_ranges_known_sizes(mo):
    # kept counts (kx, kp, kn) of the 1/3 rule
    assert mo.kept_counts(32) == (10, 10, 10)
    assert mo.kept_counts(48) == (16, 16, 16)
    assert mo.kept_counts(64) == (21, 21, 21)
    assert mo.kept_counts(96) == (32, 32, 32)
    assert mo.kept_counts(256) == (85, 85, 85)
    assert mo.kept_counts(512) == (170, 170, 170)
    g = mo.Grid(32)
    m = g.retained_mask()
    # kept kx 0..9, ky/kz in -10..9
    assert m[0, 0, :10].all() and not m[0, 0, 10:].any()
    ky = np.fft.fftfreq(32, 1 / 32).astype(int)
    kept_ky = sorted(ky[m[0, :, 0]])
    assert kept_ky == list(range(-10, 10))


def test_grid_conventions(mo):
    g = mo.Grid(16, L=2 * math.pi)
    assert np.isclose(g.x[0], -math.pi) and np.isclose(g.x[1] - g.x[0], 2 * math.pi / 16)
    assert g.kr.ravel().tolist() == list(range(9))
    assert g.l.ravel()[:3].tolist() == [0, 1, 2] and g.l.ravel()[-1] == -1 and g.l.ravel()[8] == -8
    assert g.invKrsq[0, 0, 0] == 0


def test_literal_equals_fast(mo):
    for n in (16, 24):
        g = mo.Grid(n)
        s = mo.random_spectrum_state(g, seed=4)
        a, b = np.zeros_like(s), np.zeros_like(s)
        mo.calcN_literal(a, s.copy(), g, 1e-3, 2e-3)
        mo.calcN_fast(b, s.copy(), g, 1e-3, 2e-3)
        assert mo.rel_l2(a, b, g.retained_mask()) < 1e-13


def test_literal_dealiases_state_in_place(mo):
    g = mo.Grid(16)
    s = (np.random.default_rng(0).standard_normal((6, 16, 16, 9))
         + 1j * np.random.default_rng(1).standard_normal((6, 16, 16, 9)))
    N = np.zeros_like(s)
    mo.calcN_literal(N, s, g, 0.0, 0.0)
    assert np.all(s[:, ~g.retained_mask()] == 0)


def abc_state(g, A=1.0, B=0.7, C_=0.4, k=1):
    x, y, z = g.mesh()
    ux = A * np.sin(k * z) + C_ * np.cos(k * y)
    uy = B * np.sin(k * x) + A * np.cos(k * z)
    uz = C_ * np.sin(k * y) + B * np.cos(k * x)
    zero = np.zeros_like(x)
    return mo_state(g, [ux, uy, uz, zero, zero, zero])


def mo_state(g, fields):
    from oracle import mhd_oracle

    return mhd_oracle.physical_to_state(g, fields)


def test_abc_flow_exact_decay(mo):
    g = mo.Grid(16)
    nu, dt, steps = 0.05, 0.01, 20
    s = abc_state(g)
    s0 = s.copy()
    st = mo.Stepper(g, nu, 0.0, dt, "RK4", literal=True)
    for _ in range(steps):
        st.stepforward(s)
    expect = s0 * math.exp(-nu * 1 * dt * steps)
    assert mo.rel_l2(s, expect, g.retained_mask()) < 1e-8


def test_alfven_wave_exact(mo):
    # B = B0 x_hat + b(x, t), u = -b, b = eps (0, sin(x - B0 t), 0) is an exact ideal solution
    g = mo.Grid(16)
    B0, eps, nu, dt, steps = 1.0, 0.1, 0.0, 0.005, 40
    x, y, z = g.mesh()
    b_y = eps * np.sin(x)
    zero = np.zeros_like(x)
    s = mo_state(g, [zero, -b_y, zero, B0 + zero, b_y, zero])
    st = mo.Stepper(g, nu, nu, dt, "LSRK4", literal=True)
    for _ in range(steps):
        st.stepforward(s)
    t = dt * steps
    b_t = eps * np.sin(x + B0 * t)  # u = -b travels in -x for this sign convention
    b_t2 = eps * np.sin(x - B0 * t)
    got = g.irfft(s[4])
    err = min(np.abs(got - b_t).max(), np.abs(got - b_t2).max())
    assert err < 1e-8


def test_solenoidal_and_energy_budget(mo):
    n = 24
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=8)
    nu = eta = 2e-2
    N = np.zeros_like(s)
    mo.calcN_fast(N, s.copy(), g, nu, eta)
    ks = g.ks
    kdotN = sum(ks[i] * N[i] for i in range(3))
    kdotNb = sum(ks[i] * N[3 + i] for i in range(3))
    scale = np.abs(N).max() * n
    assert np.abs(kdotN).max() < 1e-10 * scale and np.abs(kdotNb).max() < 1e-10 * scale
    # dE/dt = 2 Re sum conj(s) N  (Parseval weights) = -2 nu sum k^2|u|^2 - 2 eta sum k^2|b|^2
    w = np.ones((1, 1, g.nkr)); w[..., 1:] = 2
    m = g.retained_mask()
    dE = 2 * np.sum((w * (np.conj(s) * N).real)[:, m])
    diss = -2 * (nu * np.sum((w * g.Krsq * np.abs(s[:3]) ** 2)[:, m])
                 + eta * np.sum((w * g.Krsq * np.abs(s[3:]) ** 2)[:, m]))
    assert abs(dE - diss) < 1e-9 * abs(diss)


def test_fp32_literal_close_to_fp64(mo):
    g64 = mo.Grid(32)
    g32 = mo.Grid(32, dtype=np.float32)
    f = mo.taylor_green(g64)
    s64 = mo.physical_to_state(g64, f)
    s32 = mo.physical_to_state(g32, [a.astype(np.float32) for a in f])
    a = mo.Stepper(g64, 1e-2, 1e-2, 1e-3, "RK4")
    b = mo.Stepper(g32, 1e-2, 1e-2, 1e-3, "RK4")
    for _ in range(3):
        a.stepforward(s64)
        b.stepforward(s32)
    assert mo.rel_l2(s32, s64, g64.retained_mask()) < 1e-6


def test_taylor_green_symmetries(mo):
    g = mo.Grid(16)
    f = mo.taylor_green(g)
    s = mo.physical_to_state(g, f)
    d = mo.spectral_diagnostics(g, s)
    # <u.B> vanishes for Taylor-Green u and B; both divergence free
    assert abs(d["H_c"]) < 1e-12
    assert d["max_divb"] < 1e-12 and d["max_kdotu"] < 1e-9
    # E_u of TG on the periodic cube: sum |u|^2 dV = (2pi)^3 / 4
    assert abs(d["E_u"] - (2 * math.pi) ** 3 / 4) < 1e-9


def test_random_spectrum_properties(mo):
    n = 32
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=17)
    d = mo.spectral_diagnostics(g, s)
    vol = (2 * math.pi) ** 3
    # E_u = 1/2 <|u|^2> = 0.5 -> sum |u|^2 dV = vol; B at 0.3 of u's rms amplitude
    assert abs(d["E_u"] / vol - 1.0) < 1e-10
    assert abs(d["E_B"] / vol - 0.09) < 1e-10
    assert d["max_kdotu"] < 1e-8 and d["max_kdotb"] < 1e-8
    # real field: the irfft of the spectrum reproduces it on the retained band
    back = g.rfft(g.irfft(s[0]))
    assert mo.rel_l2(back, s[0], g.retained_mask()) < 1e-12
    # mode-indexed: 48^3 shares its common modes with 32^3 up to normalisation
    g2 = mo.Grid(48)
    s2 = mo.random_spectrum_state(g2, seed=17)
    a = s[0, 1, 2, 3] / s[0, 2, 1, 3]
    b = s2[0, 1, 2, 3] / s2[0, 2, 1, 3]
    assert abs(a - b) < 1e-9 * abs(a)


def test_mode_phases_uniform(mo):
    ph = mo.mode_phases(5, 0, np.arange(4000), 3, 7)
    assert ph.min() >= 0 and ph.max() < 2 * math.pi
    hist, _ = np.histogram(ph, bins=8, range=(0, 2 * math.pi))
    assert hist.min() > 400


def test_lsrk4_coefficients_order4(mo):
    # the 2N-storage scheme integrates y' = y with 4th-order accuracy
    def run(dt, steps):
        y, du = 1.0, 0.0
        for _ in range(steps):
            for i in range(5):
                r = y
                du = (mo.LSRK4_A[i] * du if i else 0.0) + dt * r
                y += mo.LSRK4_B[i] * du
        return y

    e1 = abs(run(0.1, 10) - math.e)
    e2 = abs(run(0.05, 20) - math.e)
    assert 12 < e1 / e2 < 20


def test_prob_diagnostic_matches_spectral(mo):
    g = mo.Grid(16)
    s = mo.random_spectrum_state(g, seed=3)
    v = [g.irfft(s[f]) for f in range(6)]
    ke, me = mo.prob_diagnostic(g, v)
    d = mo.spectral_diagnostics(g, s)
    assert abs(ke - d["E_u"]) < 1e-10 * ke and abs(me - d["E_B"]) < 1e-10 * me


def test_literal_equals_fast_over_steps(mo):
    # the kx = 0 edge modes (partner in the alias band) become non-Hermitian under time stepping;
    # the reference's diffusion sees only their Hermitian part (rfft(irfft(.)))
    g = mo.Grid(24)
    s0 = mo.random_spectrum_state(g, seed=21)
    dt = 0.2 * (2 * math.pi / 24)
    a, b = s0.copy(), s0.copy()
    sa = mo.Stepper(g, 1e-2, 2e-2, dt, "LSRK4", literal=True)
    sb = mo.Stepper(g, 1e-2, 2e-2, dt, "LSRK4", literal=False)
    for _ in range(4):
        sa.stepforward(a)
        sb.stepforward(b)
    m = g.retained_mask()
    assert mo.rel_l2(b, a, m) < 1e-12
    # and the edge modes really are non-Hermitian by now
    kfs = np.fft.fftfreq(24, 1 / 24).astype(int)
    edge = np.where(kfs == -kfs[m[:, 0, 0]].max() - 1)[0]
    assert edge.size == 1
