"""Generate the committed golden fixtures from the CPU oracle (FP64, literal reference-ordered RHS).

Fixtures (retained band only, complex128, compressed npz):
  tg32_rk4.npz       Taylor-Green 32^3 on the centred grid, nu = eta = 1e-2, dt = 1e-3:
                     state after 0, 1 and 100 RK4 steps and E_u, E_B every step
  rand48_lsrk4.npz   seeded k^4 exp(-2(k/4)^2) spectrum at 48^3 (seed 7), nu = 1e-3, eta = 2e-3,
                     dt = 0.2*dx: state after 0 and 10 LSRK4 steps
  rhs32.npz          one calcN! evaluation of the 32^3 random state (seed 11), nu = 2e-3, eta = 3e-3

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


if __name__ == "__main__":
    tg32()
    rand48()
    rhs32()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
