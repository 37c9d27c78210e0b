"""Generate the committed golden fixtures from the CPU oracle (FP64, literal reference-ordered RHS).

Fixtures (retained band only, complex128, compressed npz):
  tg32_rk4.npz       Taylor-Green 32^3 on the centred grid, nu = eta = 1e-2, dt = 1e-3:
                     state after 0, 1 and 100 RK4 steps and E_u, E_B every step
  rand48_lsrk4.npz   seeded k^4 exp(-2(k/4)^2) spectrum at 48^3 (seed 7), nu = 1e-3, eta = 2e-3,
                     dt = 0.2*dx: state after 0 and 10 LSRK4 steps
  rhs32.npz          one calcN! evaluation of the 32^3 random state (seed 11), nu = 2e-3, eta = 3e-3
  vp32_rhs.npz       one calcN! evaluation with volume penalisation (VP_UᵢUpdate! / VP_BᵢUpdate!) of
                     the 32^3 random state (seed 13), nu = 2e-3, eta = 3e-3, dt = 1e-3, mask and
                     walls from vp_inputs()
  hd48_rk4.npz       hydrodynamics (B = 0) at 48^3 (seed 17), nu = 1e-3, dt = 1e-3: 0 and 3 RK4 steps
  hdvp32_rk4.npz     hydrodynamics with volume penalisation at 32^3 (seed 19), nu = 2e-3, dt = 1e-3,
                     mask and velocity walls from vp_inputs(): 0 and 2 RK4 steps
  forced32_rk4.npz   A99 forcing (SetUpFk! kf = 2, P = 1e-5, sigma = 1, b = 1, seed 1234) on the 32^3
                     random state (seed 23), nu = eta = 1e-3, dt = 1e-3: 0 and 2 RK4 steps

Run from the repository root:  python tests/golden/make_golden.py
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import mhd_oracle as mo  # noqa: E402


def compact(g, s):
    """(6, K2, K2, Kx) retained band in kept-index order."""
    kxs, kfs = mo.kept_wavenumbers(g.n)
    idx = kfs % g.n
    return np.ascontiguousarray(s[:, idx][:, :, idx][:, :, :, : len(kxs)])


def tg32():
    g = mo.Grid(32)
    s = mo.physical_to_state(g, mo.taylor_green(g))
    st = mo.Stepper(g, 1e-2, 1e-2, 1e-3, "RK4", literal=True)
    out = {"s0": compact(g, g.dealias(s.copy()))}
    eu, eb = [], []
    for k in range(1, 101):
        st.stepforward(s)
        d = mo.spectral_diagnostics(g, s)
        eu.append(d["E_u"])
        eb.append(d["E_B"])
        if k in (1, 100):
            out[f"s{k}"] = compact(g, g.dealias(s.copy()))
    np.savez_compressed(os.path.join(HERE, "tg32_rk4.npz"), E_u=np.array(eu), E_B=np.array(eb), **out)


def rand48():
    g = mo.Grid(48)
    s = mo.random_spectrum_state(g, 7)
    dt = 0.2 * (2 * math.pi / 48)
    st = mo.Stepper(g, 1e-3, 2e-3, dt, "LSRK4", literal=True)
    s0 = compact(g, s)
    for _ in range(10):
        st.stepforward(s)
    np.savez_compressed(os.path.join(HERE, "rand48_lsrk4.npz"), s0=s0, s10=compact(g, g.dealias(s.copy())),
                        dt=dt)


def rhs32():
    g = mo.Grid(32)
    s = mo.random_spectrum_state(g, 11)
    N = np.zeros_like(s)
    mo.calcN_literal(N, s.copy(), g, 2e-3, 3e-3)
    np.savez_compressed(os.path.join(HERE, "rhs32.npz"), s=compact(g, s), rhs=compact(g, N))


def vp_inputs(g):
    """Mask chi (a smoothed ball of radius 1.2 off the box centre) and wall fields U0, B0 as FP32
    physical arrays (nz, ny, nx), analytic in the grid coordinates."""
    x, y, z = g.mesh()
    chi = (0.5 * (1 - np.tanh((np.sqrt(x ** 2 + (y - 0.3) ** 2 + z ** 2) - 1.2) / 0.25))).astype(np.float32)
    U0 = tuple((a * np.sin(x + p) * np.cos(y - z)).astype(np.float32) for a, p in ((0.6, 0.3), (0.4, 1.1), (0.8, 2.0)))
    B0 = tuple((a * np.cos(x - p) * np.sin(y + z)).astype(np.float32) for a, p in ((0.2, 0.5), (0.3, 1.7), (0.1, 2.9)))
    return chi, U0, B0


def _vp(g, dt, walls_b=True):
    chi, U0, B0 = vp_inputs(g)
    return dict(chi=chi.astype(np.float64), dt=dt, U0=tuple(a.astype(np.float64) for a in U0),
                B0=tuple(a.astype(np.float64) for a in B0) if walls_b else None)


def vp32():
    g = mo.Grid(32)
    s = mo.random_spectrum_state(g, 13)
    N = np.zeros_like(s)
    mo.calcN_literal(N, s.copy(), g, 2e-3, 3e-3, vp=_vp(g, 1e-3))
    np.savez_compressed(os.path.join(HERE, "vp32_rhs.npz"), s=compact(g, s), rhs=compact(g, N))


def hd48():
    g = mo.Grid(48)
    s = mo.random_spectrum_state(g, 17)
    s[3:] = 0
    st = mo.Stepper(g, 1e-3, 0.0, 1e-3, "RK4", literal=True)
    s0 = compact(g, s)
    for _ in range(3):
        st.stepforward(s)
    np.savez_compressed(os.path.join(HERE, "hd48_rk4.npz"), s0=s0[:3], s3=compact(g, g.dealias(s.copy()))[:3])


def hdvp32():
    g = mo.Grid(32)
    s = mo.random_spectrum_state(g, 19)
    s[3:] = 0
    st = mo.Stepper(g, 2e-3, 0.0, 1e-3, "RK4", literal=True)
    v = _vp(g, 1e-3, walls_b=False)
    st.vp = dict(chi=v["chi"], U0=v["U0"])
    s0 = compact(g, s)
    for _ in range(2):
        st.stepforward(s)
    np.savez_compressed(os.path.join(HERE, "hdvp32_rk4.npz"), s0=s0[:3], s2=compact(g, g.dealias(s.copy()))[:3])


def forced32():
    g = mo.Grid(32)
    s = mo.random_spectrum_state(g, 23)
    st = mo.Stepper(g, 1e-3, 1e-3, 1e-3, "RK4", literal=True)
    st.forcing = dict(A=mo.a99_amplitude(g, 2.0, 1e-5, 1.0), kf_used=1.0, sigma2=1.0, b=1.0, seed=1234)
    s0 = compact(g, s)
    for _ in range(2):
        st.stepforward(s)
    np.savez_compressed(os.path.join(HERE, "forced32_rk4.npz"), s0=s0, s2=compact(g, g.dealias(s.copy())))


if __name__ == "__main__":
    tg32()
    rand48()
    rhs32()
    vp32()
    hd48()
    hdvp32()
    forced32()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
