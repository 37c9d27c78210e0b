"""FP64 comparator on the GPU: the oracle's compact right-hand side and RK4 / LSRK4, in torch.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only the tests use it,
as the checker at grid sizes where the CPU oracle in float64 would take too long (256^3 and
512^3).  torch.fft (cuFFT, a library called here purely as a comparator) does the transforms;
every other step restates ``mhd_oracle.calcN_fast`` and ``mhd_oracle.Stepper`` line for line, so
the two agree to float64 roundoff (checked at 32^3 and 64^3 against the CPU oracle in the same
test file).  Parity status follows the CPU oracle's: unpinned against the reference itself.

What it restates (file:line into MHDFlows.jl), through ``mhd_oracle``:

* ``calcN``: ``MHDcalcN!`` (src/pgen.jl:153-162) = ``dealias!`` of the state in place, then the
  stress-form ``UᵢUpdate!`` / ``BᵢUpdate!`` (src/Solver/MHDSolver.jl:27-103, 106-177) with each
  unique product transformed once, the Leray projection ``δ_aj − k_a k_j / k²`` and the diffusion
  ``−ν k² û``, ``−η k² B̂`` acting on the Hermitian part of the kx = 0 plane (what the
  reference's rfft(irfft(·)) does there, src/Solver/MHDSolver.jl:91-94,166-168).
* ``step``: FourierFlows' RK4 as restated in-repo at src/DyeModule.jl:62-89, and LSRK4, the
  Carpenter & Kennedy (1994) five-stage 2N-storage scheme (coefficients from ``mhd_oracle``).

Layout as the CPU oracle: a state is (6, nz, ny, nkr) complex128, C order, the memory of Julia's
``sol[i, j, k, f]``.
"""
from __future__ import annotations

import math

import torch

from oracle import mhd_oracle as mo


class TorchGrid:
    """ThreeDGrid conventions (src/utils/utils.jl:14-38) on a torch device, float64."""

    def __init__(self, n: int, L: float = 2 * math.pi, device="cuda"):
        self.n, self.L, self.nkr = n, L, n // 2 + 1
        self.device = torch.device(device)
        self.dx = L / n
        f64 = dict(dtype=torch.float64, device=self.device)
        kr = torch.arange(self.nkr, **f64) * (2 * math.pi / L)
        kf = torch.fft.fftfreq(n, 1.0 / n, **f64) * (2 * math.pi / L)
        self.kx = kr.reshape(1, 1, self.nkr)
        self.ky = kf.reshape(1, n, 1)
        self.kz = kf.reshape(n, 1, 1)
        self.ks = (self.kx, self.ky, self.kz)
        self.Krsq = self.kx ** 2 + self.ky ** 2 + self.kz ** 2
        self.invKrsq = torch.where(self.Krsq > 0, 1.0 / torch.where(self.Krsq > 0, self.Krsq, 1.0),
                                   torch.zeros((), **f64))
        (self.a0, self.a1), (self.r0, _) = mo.alias_ranges(n)
        self.herm_idx = (-torch.arange(n, device=self.device)) % n

    def dealias_(self, fh):
        fh[..., :, :, self.r0:] = 0
        fh[..., :, self.a0:self.a1, :] = 0
        fh[..., self.a0:self.a1, :, :] = 0
        return fh

    def retained_mask(self):
        m = torch.ones((self.n, self.n, self.nkr), dtype=torch.bool, device=self.device)
        return self.dealias_(m)

    def rfft(self, a):
        return torch.fft.rfftn(a, dim=(0, 1, 2))

    def irfft(self, ah):
        return torch.fft.irfftn(ah, s=(self.n,) * 3, dim=(0, 1, 2))

    def hermitian_kx0(self, p):
        """(p + conj p(-k)) / 2 of one kx = 0 plane (nz, ny)."""
        i = self.herm_idx
        return 0.5 * (p + torch.conj(p[i][:, i]))


def calcN(g: TorchGrid, sol, nu: float, eta: float, out=None):
    """``mhd_oracle.calcN_fast`` in torch; dealiases ``sol`` in place, returns the right-hand side."""
    g.dealias_(sol)
    N = torch.empty_like(sol) if out is None else out
    u = [g.irfft(sol[f]) for f in range(3)]
    b = [g.irfft(sol[f]) for f in range(3, 6)]
    ks = g.ks
    V = [torch.zeros_like(sol[0]) for _ in range(3)]
    for i in range(3):
        for j in range(i, 3):
            T = g.rfft(b[i] * b[j] - u[i] * u[j])
            V[j] += ks[i] * T
            if i != j:
                V[i] += ks[j] * T
            del T
    kV = (ks[0] * V[0] + ks[1] * V[1] + ks[2] * V[2]) * g.invKrsq
    for a in range(3):
        N[a] = 1j * (V[a] - ks[a] * kV)
    del V, kV
    for a in range(3):
        N[3 + a] = 0
    for a in range(3):
        for j in range(a + 1, 3):
            E = g.rfft(u[a] * b[j] - b[a] * u[j])
            N[3 + a] += 1j * ks[j] * E
            N[3 + j] -= 1j * ks[a] * E
            del E
    del u, b
    for f in range(6):
        c = nu if f < 3 else eta
        H = sol[f].clone()
        H[:, :, 0] = g.hermitian_kx0(sol[f][:, :, 0])
        N[f] -= g.Krsq * c * H
        del H
    return N


class Stepper:
    """RK4 / LSRK4 of ``mhd_oracle.Stepper`` (compact right-hand side) in torch float64."""

    def __init__(self, g: TorchGrid, nu: float, eta: float, dt: float, scheme: str = "RK4"):
        self.g, self.nu, self.eta, self.dt = g, nu, eta, dt
        self.scheme = scheme.upper()
        if self.scheme not in ("RK4", "LSRK4"):
            raise ValueError(f"unknown stepper {scheme!r}")
        self.t, self.step = 0.0, 0

    def stepforward(self, sol):
        g, dt = self.g, self.dt
        if self.scheme == "RK4":
            R = calcN(g, sol, self.nu, self.eta)
            acc = R / 6
            s1 = sol + (dt / 2) * R
            calcN(g, s1, self.nu, self.eta, out=R)
            acc += R / 3
            torch.add(sol, R, alpha=dt / 2, out=s1)
            calcN(g, s1, self.nu, self.eta, out=R)
            acc += R / 3
            torch.add(sol, R, alpha=dt, out=s1)
            calcN(g, s1, self.nu, self.eta, out=R)
            acc += R / 6
            del s1, R
            sol += dt * acc
            del acc
        else:
            S2 = None
            R = torch.empty_like(sol)
            for i in range(5):
                calcN(g, sol, self.nu, self.eta, out=R)
                S2 = dt * R if i == 0 else mo.LSRK4_A[i] * S2 + dt * R
                sol += mo.LSRK4_B[i] * S2
            del S2, R
        self.t += dt
        self.step += 1
        return sol


def diagnostics(g: TorchGrid, sol):
    """``mhd_oracle.spectral_diagnostics`` (E_u, E_B, H_c, max|k.u|, max|k.B|) of a state, float64."""
    s = g.dealias_(sol.clone())
    w = torch.full((1, 1, g.nkr), 2.0, dtype=torch.float64, device=g.device)
    w[..., 0] = 1.0
    if g.n % 2 == 0:
        w[..., -1] = 1.0
    scale = g.dx ** 3 / float(g.n) ** 3
    e_u = float(sum((w * s[f].abs() ** 2).sum() for f in range(3))) * scale
    e_b = float(sum((w * s[f].abs() ** 2).sum() for f in range(3, 6))) * scale
    h_c = float(sum((w * (s[f] * torch.conj(s[f + 3])).real).sum() for f in range(3))) * scale
    ku = sum(g.ks[i] * s[i] for i in range(3))
    kb = sum(g.ks[i] * s[3 + i] for i in range(3))
    return {"E_u": e_u, "E_B": e_b, "H_c": h_c, "max_kdotu": float(ku.abs().max()),
            "max_kdotb": float(kb.abs().max())}


def run(n: int, state, nu: float, eta: float, dt: float, steps: int, scheme: str = "RK4", L: float = 2 * math.pi,
        device="cuda", keep=()):
    """Step a host state (6, n, n, nkr) ``steps`` times in float64 on ``device``; returns the
    dealiased final state (torch, on the device) and the dealiased states after the step counts
    in ``keep`` ({count: state})."""
    g = TorchGrid(n, L, device)
    s = torch.as_tensor(state).to(device=g.device, dtype=torch.complex128).contiguous()
    st = Stepper(g, nu, eta, dt, scheme)
    kept = {}
    for k in range(1, steps + 1):
        st.stepforward(s)
        if k in keep:
            kept[k] = g.dealias_(s.clone())
    return g.dealias_(s), kept, g
