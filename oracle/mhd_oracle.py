"""CPU oracle for the 3D incompressible MHD right-hand side and RK4 / LSRK4 step.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module: only the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline / reference legs of
``bench.py`` use it, and only as the checker or as the timed CPU restatement.

Parity status: UNPINNED against the reference.  MHDFlows.jl ships no tests, no
golden vectors and no fixtures, and Julia + FourierFlows cannot run here, so
this restatement is pinned only by known-answer tests derived from the
mathematics (exact decaying Beltrami flows, the exact Alfven wave, energy
identities, symmetries) and by its own FP64 / FP32 agreement.

What it restates (file:line into MHDFlows.jl):

* ``calcN_literal``: ``MHDcalcN!`` (src/pgen.jl:153-162) = ``dealias!`` of the
  state in place, then ``MHDcalcN_advection!`` (src/Solver/MHDSolver.jl:330-351):
  six normalised inverse rffts of the state into ``vars``, ``UiUpdate!`` x3
  (src/Solver/MHDSolver.jl:27-103; the i<=j product loop at :63-83, diffusion at
  :90-99) and ``BiUpdate!`` x3 (src/Solver/MHDSolver.jl:106-177; the j!=a loop at
  :147-158, resistivity at :165-173).  Same term order, same products, same
  number of forward transforms (30 r2c + 6 c2r per RHS).
* ``rk4_step``: FourierFlows' RK4 as restated in-repo at src/DyeModule.jl:62-89
  (stage 1 evaluates the RHS on ``sol`` itself, so ``sol`` is dealiased in place
  once per step; update ``sol += dt*(R1/6 + R2/3 + R3/3 + R4/6)``).
* ``lsrk4_step``: FourierFlows' "LSRK4" = Carpenter & Kennedy (1994, NASA
  TM-109112) five-stage fourth-order 2N-storage scheme, ``dU = A_i dU + dt R(U);
  U += B_i dU``, RHS evaluated on ``sol`` itself (dealiased in place every stage).
  FourierFlows itself is not vendored; the coefficients are the published ones.
* ``Grid``: FourierFlows ``ThreeDGrid`` conventions mirrored in-repo at
  src/utils/utils.jl:14-38,42-98 (``kr = rfftfreq``, ``l, m = fftfreq`` scaled by
  2*pi/L*n, ``invKrsq[0,0,0] = 0``, centred ``x = -L/2 + i*dx``) and the alias
  ranges of ``getaliasedwavenumbers`` (``iL = floor((1-a)/2*n)+1``,
  ``iR = ceil((1+a)/2*n)``, 1-based, rfft axis ``iL:nkr``; recollection of
  FourierFlows 0.10.1, unverified, same double arithmetic as Julia).
* ``prob_diagnostic``: ``ProbDiagnostic`` (src/utils/UserInterface.jl:29,65-86),
  KE = ME = sum(|.|^2)*dV with no 1/2, and ``Div`` (src/utils/VectorCalculus.jl:72-94).
* ``vp_update`` / ``add_vp``: ``VP_UᵢUpdate!`` / ``VP_BᵢUpdate!`` (src/Solver/VPSolver.jl:20-58),
  called from src/Solver/MHDSolver.jl:85-88,160-163 (and HDSolver.jl:76-79): eta = dt*13/7,
  out += -(delta_aj - k_j k_a / k^2) rfft(chi/eta (f_j - W_j)).  ``div_correct``:
  ``DivVCorrection!`` / ``DivBCorrection!`` (src/Solver/VPSolver.jl:60-138).
* Hydrodynamics (``HDcalcN!``, src/pgen.jl:176-182): the MHD right-hand side with B = 0 and
  eta = 0 (the induction terms vanish identically); HDcalcN! applies addforcing! before the
  advection step zeroes the velocity right-hand side, so a forced HD run is unforced.
* ``add_a99_forcing`` / ``a99_force``: SetUpFk! and A99ForceDriving!
  (src/pgen/A99ForceDriving_GPU.jl:18-130) with a counter-based generator in place of the
  device rand().

Array layout: numpy C order ``(nz, ny, nx)`` for physical fields and
``(nz, ny, nkr)`` for half spectra, which is the same memory as Julia's
column-major ``(nx, ny, nz)`` / ``(nkr, ny, nz)``.  A state is ``(6, nz, ny, nkr)``
== Julia ``sol[i, j, k, f]`` with f = ux, uy, uz, bx, by, bz.
"""
from __future__ import annotations

import math
import os

import numpy as np
import scipy.fft as sfft

FIELDS = ("ux", "uy", "uz", "bx", "by", "bz")

# Carpenter & Kennedy (1994) LSRK(5,4) 2N-storage coefficients.
LSRK4_A = (0.0,
           -567301805773.0 / 1357537059087.0,
           -2404267990393.0 / 2016746695238.0,
           -3550918686646.0 / 2091501179385.0,
           -1275806237668.0 / 842570457699.0)
LSRK4_B = (1432997174477.0 / 9575080441755.0,
           5161836677717.0 / 13612068292357.0,
           1720146321549.0 / 2090206949498.0,
           3134564353537.0 / 4481467310338.0,
           2277821191437.0 / 14882151754819.0)
LSRK4_C = (0.0,
           1432997174477.0 / 9575080441755.0,
           2526269341429.0 / 6820363962896.0,
           2006345519317.0 / 3224310063776.0,
           2802321613138.0 / 2924317926251.0)


def _workers() -> int:
    return int(os.environ.get("MHD_ORACLE_WORKERS", os.cpu_count() or 1))


def alias_ranges(n: int, aliased_fraction: float = 1.0 / 3.0):
    """0-based half-open alias ranges (full axis, rfft axis) for length n.

    Mirrors getaliasedwavenumbers (FourierFlows 0.10.1; used by dealias! at
    src/pgen.jl:155 and rebuilt in-repo at src/utils/utils.jl:82-84).
    """
    lo = (1 - aliased_fraction) / 2
    hi = (1 + aliased_fraction) / 2
    i_l = math.floor(lo * n) + 1          # 1-based first aliased index
    i_r = math.ceil(hi * n)               # 1-based last aliased index
    if not aliased_fraction < 1:
        i_l += 1
    nkr = n // 2 + 1
    return (i_l - 1, i_r), (i_l - 1, nkr)


def kept_counts(n: int):
    """(Kx, Kpos, Kneg): kept rfft-axis modes, kept non-negative / negative full-axis modes."""
    (a0, a1), (r0, _) = alias_ranges(n)
    return r0, a0, n - a1


class Grid:
    """Periodic cube of side L with n points per axis (FourierFlows ThreeDGrid conventions)."""

    def __init__(self, n: int, L: float = 2 * math.pi, dtype=np.float64, centred: bool = True):
        self.n = n
        self.L = L
        self.nkr = n // 2 + 1
        self.dtype = np.dtype(dtype)
        self.cdtype = np.result_type(self.dtype, np.complex64)
        self.dx = L / n
        x0 = -L / 2 if centred else 0.0
        self.x = (x0 + self.dx * np.arange(n)).astype(dtype)
        # rfftfreq(n, 2pi/L*n) and fftfreq(n, 2pi/L*n), computed in float64 then cast (utils.jl:23-26)
        kr = np.arange(self.nkr, dtype=np.float64) * (2 * math.pi / L)
        kf = np.fft.fftfreq(n, 1.0 / n) * (2 * math.pi / L)
        self.kr = kr.astype(dtype).reshape(1, 1, self.nkr)
        self.l = kf.astype(dtype).reshape(1, n, 1)
        self.m = kf.astype(dtype).reshape(n, 1, 1)
        self.Krsq = self.kr ** 2 + self.l ** 2 + self.m ** 2
        with np.errstate(divide="ignore"):
            self.invKrsq = (1 / self.Krsq).astype(dtype)
        self.invKrsq[0, 0, 0] = 0
        (self.a0, self.a1), (self.r0, _) = alias_ranges(n)
        self.ks = (self.kr, self.l, self.m)

    # --- transforms (FourierFlows rfftplan: mul! unnormalised r2c, ldiv! normalised c2r)
    def rfft(self, a):
        return sfft.rfftn(a, axes=(0, 1, 2), workers=_workers())

    def irfft(self, ah):
        return sfft.irfftn(ah, s=(self.n,) * 3, axes=(0, 1, 2), workers=_workers())

    def dealias(self, fh):
        """In-place per-axis cube truncation of ``fh`` (..., nz, ny, nkr)."""
        fh[..., :, :, self.r0:] = 0
        fh[..., :, self.a0:self.a1, :] = 0
        fh[..., self.a0:self.a1, :, :] = 0
        return fh

    def retained_mask(self):
        m = np.ones((self.n, self.n, self.nkr), dtype=bool)
        self.dealias(m)
        return m

    def mesh(self):
        z, y, x = np.meshgrid(self.x, self.x, self.x, indexing="ij")
        return x, y, z


def _delta(a, b):
    return 1 if a == b else 0


def calcN_literal(N, sol, grid: Grid, nu, eta, nnu=0, neta=0, vars_out=None, vp=None):
    """Literal restatement of MHDcalcN! (src/pgen.jl:153-162); dealiases ``sol`` in place.
    ``vp``: None or the volume-penalisation inputs (``add_vp``)."""
    g = grid
    g.dealias(sol)
    # MHDcalcN_advection! (src/Solver/MHDSolver.jl:333-338): vars <- ldiv!(rfftplan, copy(sol[f]))
    v = [g.irfft(sol[f].copy()).astype(g.dtype) for f in range(6)]
    if vars_out is not None:
        for f in range(6):
            vars_out[f][...] = v[f]
    u = v[0:3]
    b = v[3:6]
    ks = g.ks
    nu_s = np.float64(nu)
    eta_s = np.float64(eta)
    # UiUpdate! (src/Solver/MHDSolver.jl:27-103)
    for a in range(3):
        ka = ks[a]
        out = N[a]
        out[...] = 0
        for i in range(3):
            for j in range(3):
                if j >= i:
                    nl = b[i] * b[j] - u[i] * u[j]
                    nlh = g.rfft(nl)
                    out += 1j * ks[i] * (_delta(a, j) - ka * ks[j] * g.invKrsq) * nlh
                    if i != j:
                        out += 1j * ks[j] * (_delta(a, i) - ka * ks[i] * g.invKrsq) * nlh
        if vp is not None:  # src/Solver/MHDSolver.jl:85-88
            vp_update(out, a, u, vp["chi"], vp.get("U0"), vp["dt"], g)
        uh = g.rfft(u[a])
        out += (-g.Krsq * nu_s * uh).astype(out.dtype)
        if nnu > 1:
            out += (-g.Krsq ** nnu * nu_s * uh).astype(out.dtype)
    # BiUpdate! (src/Solver/MHDSolver.jl:106-177)
    for a in range(3):
        out = N[3 + a]
        out[...] = 0
        for j in range(3):
            if a != j:
                nl = u[a] * b[j] - b[a] * u[j]
                nlh = g.rfft(nl)
                out += 1j * ks[j] * nlh
        if vp is not None:  # src/Solver/MHDSolver.jl:160-163
            vp_update(out, a, b, vp["chi"], vp.get("B0"), vp["dt"], g)
        bh = g.rfft(b[a])
        out += (-g.Krsq * eta_s * bh).astype(out.dtype)
        if neta > 1:
            out += (-g.Krsq ** neta * eta_s * bh).astype(out.dtype)
    return N


def vp_update(out, a, fields, chi, walls, dt, grid: Grid):
    """VP_UᵢUpdate! / VP_BᵢUpdate! (src/Solver/VPSolver.jl:20-58) for component a:
    out += -(δ_aj - k_j k_a / k^2) rfft(chi / eta (f_j - W_j)), eta = dt 13 / 7, summed over j.
    ``walls`` is None (zero) or the three wall fields; physical arrays are (nz, ny, nx)."""
    g = grid
    eta_vp = dt * 13 / 7
    ks = g.ks
    for j in range(3):
        w = 0.0 if walls is None else walls[j]
        F = g.rfft(chi / eta_vp * (fields[j] - w))
        out += (-(_delta(a, j) - ks[j] * ks[a] * g.invKrsq) * F).astype(out.dtype)


def add_vp(N, sol_dealiased, grid: Grid, vp: dict):
    """The penalty terms of both equations added to a right-hand side N, from the physical fields
    of a dealiased state (``vp``: chi, dt and optional U0, B0)."""
    v = [grid.irfft(sol_dealiased[f]) for f in range(6)]
    for a in range(3):
        vp_update(N[a], a, v[0:3], vp["chi"], vp.get("U0"), vp["dt"], grid)
        vp_update(N[3 + a], a, v[3:6], vp["chi"], vp.get("B0"), vp["dt"], grid)
    return N


def div_correct(grid: Grid, sol, fields: int = 3):
    """DivVCorrection! (fields & 1) and DivBCorrection! (fields & 2), src/Solver/VPSolver.jl:60-138:
    phi = -i (k.X) / k^2, X -= i k phi, i.e. X loses k (k.X) / k^2 (1/k^2 = 0 at k = 0)."""
    ks = grid.ks
    for bit, off in ((1, 0), (2, 3)):
        if fields & bit:
            phi = (ks[0] * sol[off] + ks[1] * sol[off + 1] + ks[2] * sol[off + 2]) * grid.invKrsq
            for a in range(3):
                sol[off + a] -= ks[a] * phi
    return sol


def hermitian_kx0(grid: Grid, X):
    """X with its kx = 0 plane replaced by the Hermitian part (X(k) + conj X(-k))/2.

    This is what rfft(irfft(X)) does to a dealiased state: the reference computes its diffusion
    term from the re-transformed physical field (src/Solver/MHDSolver.jl:91-94, 166-168), so on
    the kx = 0 plane it acts on the Hermitian part.  It matters on the edge modes ky or kz = -Kn,
    whose partner +Kn is in the alias band (there the effective diffusion is halved).
    """
    Y = X.copy()
    n = grid.n
    iz = (-np.arange(n)) % n
    p = X[..., :, :, 0]
    Y[..., :, :, 0] = 0.5 * (p + np.conj(p[..., iz, :][..., :, iz]))
    return Y


def calcN_fast(N, sol, grid: Grid, nu, eta, vp=None):
    """Same RHS as ``calcN_literal`` with the six unique stress products transformed once.

    Used for larger FP64 checks; mathematically identical to the literal form (the diffusion
    acts on the Hermitian part of the kx = 0 plane, as rfft(irfft(.)) makes it do there).
    """
    g = grid
    g.dealias(sol)
    H = hermitian_kx0(g, sol)
    v = [g.irfft(sol[f]) for f in range(6)]
    u, b = v[0:3], v[3:6]
    ks = g.ks
    T = {}
    for i in range(3):
        for j in range(i, 3):
            T[(i, j)] = g.rfft(b[i] * b[j] - u[i] * u[j])
            T[(j, i)] = T[(i, j)]
    V = [sum(ks[i] * T[(i, j)] for i in range(3)) for j in range(3)]
    kV = sum(ks[j] * V[j] for j in range(3)) * g.invKrsq
    for a in range(3):
        N[a] = 1j * (V[a] - ks[a] * kV) - g.Krsq * nu * H[a]
    E = {}
    for a in range(3):
        for j in range(a + 1, 3):
            E[(a, j)] = g.rfft(u[a] * b[j] - b[a] * u[j])
            E[(j, a)] = -E[(a, j)]
    for a in range(3):
        acc = 0
        for j in range(3):
            if j != a:
                acc = acc + ks[j] * E[(a, j)]
        N[3 + a] = 1j * acc - g.Krsq * eta * H[3 + a]
    if vp is not None:
        add_vp(N, sol, g, vp)
    return N


class Stepper:
    """RK4 / LSRK4 on the full half-spectrum state, as FourierFlows does it."""

    def __init__(self, grid: Grid, nu, eta, dt, scheme="RK4", literal=True, nnu=0, neta=0):
        self.g = grid
        self.nu, self.eta, self.dt = nu, eta, dt
        self.nnu, self.neta = nnu, neta
        self.scheme = scheme.upper()
        self.literal = literal
        self.t = 0.0
        self.step = 0
        shape = (6, grid.n, grid.n, grid.nkr)
        z = lambda: np.zeros(shape, dtype=grid.cdtype)
        if self.scheme == "RK4":
            self.R = [z() for _ in range(4)]
            self.sol1 = z()
        elif self.scheme == "LSRK4":
            self.S2 = z()
            self.RHS = z()
        else:
            raise ValueError(f"unknown stepper {scheme!r}")
        self.vars = [np.zeros((grid.n,) * 3, dtype=grid.dtype) for _ in range(6)]

    # A99 forcing (add_a99_forcing): None or dict(A, kf_used, sigma2, b, seed)
    forcing = None
    # volume penalisation (add_vp): None or dict(chi, U0=None, B0=None); eta uses the step's dt
    vp = None

    def calcN(self, N, X, stage=0):
        vp = None if self.vp is None else dict(self.vp, dt=self.dt)
        if self.literal:
            calcN_literal(N, X, self.g, self.nu, self.eta, self.nnu, self.neta, self.vars, vp=vp)
        else:
            calcN_fast(N, X, self.g, self.nu, self.eta, vp=vp)
        if self.forcing is not None:
            add_a99_forcing(N, self.g, self.forcing, 8 * self.step + stage)
        return N

    def stepforward(self, sol):
        dt = self.dt
        if self.scheme == "RK4":
            R1, R2, R3, R4 = self.R
            s1 = self.sol1
            self.calcN(R1, sol, 0)
            np.add(sol, (dt / 2) * R1, out=s1)
            self.calcN(R2, s1, 1)
            np.add(sol, (dt / 2) * R2, out=s1)
            self.calcN(R3, s1, 2)
            np.add(sol, dt * R3, out=s1)
            self.calcN(R4, s1, 3)
            sol += dt * (R1 / 6 + R2 / 3 + R3 / 3 + R4 / 6)
        else:
            S2, R = self.S2, self.RHS
            for i in range(5):
                self.calcN(R, sol, i)
                if i == 0:
                    S2[...] = dt * R
                else:
                    S2[...] = LSRK4_A[i] * S2 + dt * R
                sol += LSRK4_B[i] * S2
        self.t += dt
        self.step += 1
        return sol


# ----------------------------------------------------------------------------------------------
# Initial conditions
# ----------------------------------------------------------------------------------------------

def taylor_green(grid: Grid, b_amp=0.5):
    """Taylor-Green u and B on the grid points (centred by default, as the reference's grid)."""
    x, y, z = grid.mesh()
    ux = np.sin(x) * np.cos(y) * np.cos(z)
    uy = -np.cos(x) * np.sin(y) * np.cos(z)
    uz = np.zeros_like(x)
    bx = b_amp * np.cos(x) * np.sin(y) * np.sin(z)
    by = -b_amp * np.sin(x) * np.cos(y) * np.sin(z)
    bz = np.zeros_like(x)
    return [a.astype(grid.dtype) for a in (ux, uy, uz, bx, by, bz)]


def physical_to_state(grid: Grid, fields):
    """SetUpProblemIC! (src/utils/IC.jl:41-109): forward r2c of each physical field into ``sol``."""
    sol = np.zeros((6, grid.n, grid.n, grid.nkr), dtype=grid.cdtype)
    for f in range(6):
        sol[f] = grid.rfft(np.asarray(fields[f], dtype=grid.dtype))
    return sol


def _splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    return z ^ (z >> np.uint64(31))


def mode_phases(seed: int, field: int, kx, ky, kz):
    """Uniform [0, 2pi) phase per (seed, field, integer wavevector), independent of n.

    Counter-based (splitmix64 of a packed key) so the same mode gets the same phase on
    every grid size: a 512^3 and a 128^3 spectrum share their common modes exactly.
    """
    kx = np.asarray(kx, dtype=np.int64) & 0xFFFF
    ky = np.asarray(ky, dtype=np.int64) & 0xFFFF
    kz = np.asarray(kz, dtype=np.int64) & 0xFFFF
    key = (kx.astype(np.uint64) | (ky.astype(np.uint64) << np.uint64(16))
           | (kz.astype(np.uint64) << np.uint64(32)) | (np.uint64(field & 0xFF) << np.uint64(48)))
    with np.errstate(over="ignore"):
        h = _splitmix64(key ^ _splitmix64(np.uint64(seed & 0xFFFFFFFFFFFFFFFF)))
        h = _splitmix64(h)
    return (h >> np.uint64(11)).astype(np.float64) * (2.0 ** -53) * (2 * math.pi)


def kept_wavenumbers(n: int):
    """Integer wavenumbers of the kept rfft-axis modes and of the kept full-axis modes (kept-index order)."""
    kx, kp, kn = kept_counts(n)
    full = np.concatenate([np.arange(kp), np.arange(-kn, 0)]).astype(np.int64)
    return np.arange(kx, dtype=np.int64), full


def random_spectrum_compact(n: int, seed: int, L: float = 2 * math.pi, e_u: float = 0.5,
                            b_ratio: float = 0.3, kpeak: float = 4.0):
    """Retained band (6, K2, K2, Kx) [f, kz', ky', kx] of ``random_spectrum_state`` (float64)."""
    kxs, kfs = kept_wavenumbers(n)
    K2, Kx = len(kfs), len(kxs)
    KZ, KY, KX = np.meshgrid(kfs, kfs, kxs, indexing="ij")
    s2p = 2 * math.pi / L
    kx, ky, kz = KX * s2p, KY * s2p, KZ * s2p
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    k = np.sqrt(k2)
    with np.errstate(divide="ignore", invalid="ignore"):
        amp = np.sqrt(k ** 4 * np.exp(-2 * (k / kpeak) ** 2) / (4 * math.pi * k2))
    amp[k2 == 0] = 0.0
    sol = np.empty((6, K2, K2, Kx), dtype=np.complex128)
    for f in range(6):
        sol[f] = amp * np.exp(1j * mode_phases(seed, f, KX, KY, KZ))
    # Hermitian kx = 0 plane: F(0,-ky,-kz) = conj(F(0,ky,kz)); partner outside the band -> 0
    pos = {int(v): i for i, v in enumerate(kfs)}
    partner = np.array([pos.get(int(-v), -1) for v in kfs])
    has = partner >= 0
    pz, py = np.meshgrid(partner, partner, indexing="ij")
    both = has[:, None] & has[None, :]
    for f in range(6):
        p = sol[f, :, :, 0]
        herm = np.zeros_like(p)
        herm[both] = 0.5 * (p[both] + np.conj(p[pz[both], py[both]]))
        sol[f, :, :, 0] = herm
    inv = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    kv = (kx, ky, kz)
    for base in (0, 3):
        dot = (kv[0] * sol[base] + kv[1] * sol[base + 1] + kv[2] * sol[base + 2]) * inv
        for i in range(3):
            sol[base + i] -= kv[i] * dot
    w = np.where(KX == 0, 1.0, 2.0)

    def mean_sq(fs):
        return float(sum(np.sum(w * (sol[f].real ** 2 + sol[f].imag ** 2)) for f in fs)) / float(n) ** 6

    mu, mb = mean_sq((0, 1, 2)), mean_sq((3, 4, 5))
    su = math.sqrt(2 * e_u / mu) if mu > 0 else 0.0
    sb = math.sqrt((b_ratio ** 2) * (2 * e_u) / mb) if mb > 0 else 0.0
    sol[0:3] *= su
    sol[3:6] *= sb
    return sol


def expand_compact(n: int, compact, dtype=np.complex128):
    """Full half-spectrum state (6, n, n, nkr) from a retained-band array (alias band zero)."""
    kxs, kfs = kept_wavenumbers(n)
    idx = kfs % n
    out = np.zeros((compact.shape[0], n, n, n // 2 + 1), dtype=dtype)
    for f in range(compact.shape[0]):
        out[f][np.ix_(idx, idx, np.arange(len(kxs)))] = compact[f]
    return out


def random_spectrum_state(grid: Grid, seed: int, e_u: float = 0.5, b_ratio: float = 0.3,
                          kpeak: float = 4.0):
    """Seeded random-phase solenoidal u, B with shell spectrum E(k) ~ k^4 exp(-2 (k/kpeak)^2).

    Every retained mode of the rfft half space gets amplitude sqrt(E(|k|)/(4 pi |k|^2)) and a
    mode-indexed random phase per field component; the kx = 0 plane is made Hermitian (modes
    whose partner lies in the alias band are zeroed), each triple is projected solenoidal
    (F - k (k.F)/k^2), u is normalised to E_u = <|u|^2>/2 = e_u and B to b_ratio times u's rms.
    Built in float64 and returned in the grid's complex dtype.
    """
    c = random_spectrum_compact(grid.n, seed, grid.L, e_u, b_ratio, kpeak)
    return expand_compact(grid.n, c, dtype=grid.cdtype)


# ----------------------------------------------------------------------------------------------
# Diagnostics
# ----------------------------------------------------------------------------------------------

def prob_diagnostic(grid: Grid, vars6):
    """ProbDiagnostic (src/utils/UserInterface.jl:65-86) without the 3-digit rounding: KE, ME."""
    dV = grid.dx ** 3
    ke = float(sum(np.sum(np.asarray(vars6[i], dtype=np.float64) ** 2) for i in range(3))) * dV
    me = float(sum(np.sum(np.asarray(vars6[i], dtype=np.float64) ** 2) for i in range(3, 6))) * dV
    if math.isnan(ke) or math.isnan(me):
        raise FloatingPointError("detected NaN! Quit the simulation right now.")
    return ke, me


def spectral_diagnostics(grid: Grid, sol):
    """Diagnostics of a (dealiased) state in float64.

    Returns dict: E_u, E_B = sum(|u|^2) dV and sum(|B|^2) dV (the reference's KE / ME, no 1/2),
    H_c = sum(u.B) dV, max|k.u_hat|, max|k.B_hat| (unnormalised spectra, like the state), and
    max|div B| in physical space (Div, src/utils/VectorCalculus.jl:72-94).
    """
    g = Grid(grid.n, grid.L, np.float64)
    s = np.asarray(sol, dtype=np.complex128).copy()
    g.dealias(s)
    n = g.n
    w = np.ones((1, 1, g.nkr))
    w[..., 1:] = 2.0
    if n % 2 == 0:
        w[..., -1] = 1.0
    dV = g.dx ** 3
    scale = dV / float(n) ** 3
    e_u = float(sum(np.sum(w * np.abs(s[f]) ** 2) for f in range(3))) * scale
    e_b = float(sum(np.sum(w * np.abs(s[f]) ** 2) for f in range(3, 6))) * scale
    h_c = float(sum(np.sum(w * (s[f] * np.conj(s[f + 3])).real) for f in range(3))) * scale
    ku = sum(g.ks[i] * s[i] for i in range(3))
    kb = sum(g.ks[i] * s[3 + i] for i in range(3))
    divb = g.irfft(1j * kb)
    return {
        "E_u": e_u, "E_B": e_b, "H_c": h_c,
        "max_kdotu": float(np.max(np.abs(ku))), "max_kdotb": float(np.max(np.abs(kb))),
        "max_divb": float(np.max(np.abs(divb))),
        "nan": bool(not np.all(np.isfinite(s))),
    }


def rel_l2(a, b, mask=None):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    if mask is not None:
        a = a[..., mask]
        b = b[..., mask]
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


# ----------------------------------------------------------------------------------------------
# A99 random solenoidal forcing (src/pgen/A99ForceDriving_GPU.jl of MHDFlows.jl), restated.
# SetUpFk! (:24-48) computes the amplitude A from the forcing spectrum over the whole (nkr, n, n)
# grid; A99Force_Driving_CUDA! (:76-130) adds A*Fk*(e^{i th1} gi e1 + e^{i th2} gj e2) to the
# velocity right-hand side at every call with fresh random numbers, then keeps only the real part
# of the whole right-hand side on the kx = 0 (and Nyquist) planes.  Restated as the reference
# does it, including two of its quirks: SetUpFk! stores kf = b (:46), so the kernel's spectrum
# peaks at k = b; and Fk already carries the factor A, so the amplitude is A^2 Fk/A.
# The reference draws its random numbers with the device rand(); here they come from a
# counter-based generator (SplitMix64 finaliser) keyed by (seed, call, mode, draw), which the
# GPU kernels evaluate identically: call = 8 * step + stage, mode = x + nkr * (y + n * z) in the
# reference's (nkr, n, n) layout, draws 0, 1, 2 = th1 / 2pi, phi / pi, th2 / 2pi.
# ----------------------------------------------------------------------------------------------
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix64(z):
    """SplitMix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = np.asarray(z, dtype=np.uint64) + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def a99_uniform(seed: int, call: int, index, draw: int):
    """Uniform numbers in [0, 1) with 24 bits, float32, for mode indices ``index``."""
    key = _mix64(np.uint64(seed) ^ _mix64(np.uint64(call)))
    with np.errstate(over="ignore"):
        z = _mix64(key ^ (np.asarray(index, dtype=np.uint64) * np.uint64(4) + np.uint64(draw)))
    return ((z >> np.uint64(40)).astype(np.float64) * (1.0 / 16777216.0)).astype(np.float32)


def a99_amplitude(grid: Grid, kf: float = 2.0, P: float = 1.0, sigma: float = 1.0) -> float:
    """A of SetUpFk! (src/pgen/A99ForceDriving_GPU.jl:24-48), in float64."""
    g = grid
    k = np.sqrt(g.Krsq.astype(np.float64))
    integral = float(np.sum(np.exp(-(k - kf) ** 2 / sigma ** 2) / (k + 1) ** 2))
    return math.sqrt(P * 3 * g.n ** 3 / integral * (1 / g.dx ** 3))


def a99_force(grid: Grid, A: float, kf_used: float, sigma2: float, b: float, seed: int, call: int):
    """Forcing of the three velocity components, (3, n, n, nkr) complex128, of one call."""
    g = grid
    kx = np.broadcast_to(g.kr.astype(np.float64), g.Krsq.shape)
    ky = np.broadcast_to(g.l.astype(np.float64), g.Krsq.shape)
    kz = np.broadcast_to(g.m.astype(np.float64), g.Krsq.shape)
    k = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    kp = np.sqrt(kx ** 2 + kz ** 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        kinv = np.where(k > 0, 1 / k, 0.0)
        pinv = np.where(kp > 0, 1 / kp, 0.0)
    Fk = A * np.sqrt(np.exp(-(k - kf_used) ** 2 / sigma2) / 2 / math.pi) * kinv
    e1x, e1z = kz * pinv, -kx * pinv
    e2x, e2y, e2z = kx * ky * pinv * kinv, -kp * kinv, kz * ky * pinv * kinv
    index = np.arange(k.size, dtype=np.uint64).reshape(k.shape)
    th1 = a99_uniform(seed, call, index, 0).astype(np.float64) * 2 * math.pi
    phi = a99_uniform(seed, call, index, 1).astype(np.float64) * math.pi
    th2 = a99_uniform(seed, call, index, 2).astype(np.float64) * 2 * math.pi
    gi = -np.tanh(b * (phi - math.pi / 2)) / math.tanh(b * math.pi / 2)
    gi = np.where(np.abs(gi) >= 1.0, np.sign(gi), gi)
    gj = np.sqrt(1 - gi ** 2)
    p1, p2 = np.exp(1j * th1), np.exp(1j * th2)
    amp = A * Fk
    F = np.empty((3,) + k.shape, dtype=np.complex128)
    F[0] = amp * (p1 * gi * e1x + p2 * gj * e2x)
    F[1] = amp * p2 * gj * e2y
    F[2] = amp * (p1 * gi * e1z + p2 * gj * e2z)
    return F


def add_a99_forcing(N, grid: Grid, forcing: dict, call: int):
    """addforcing! with the A99 hook: N[u] += F, then the kx = 0 and Nyquist planes of the whole
    velocity right-hand side keep only their real parts (src/pgen/A99ForceDriving_GPU.jl:121-127)."""
    F = a99_force(grid, forcing["A"], forcing["kf_used"], forcing["sigma2"], forcing["b"], forcing["seed"], call)
    N[0:3] += F.astype(N.dtype)
    for c in range(3):
        N[c, :, :, 0] = N[c, :, :, 0].real
        N[c, :, :, -1] = N[c, :, :, -1].real
    return N
