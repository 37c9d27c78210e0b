"""Initial conditions of the benchmark and serving workloads (host side, numpy).

The reference builds initial fields on the host and uploads them with SetUpProblemIC!
(src/utils/IC.jl:41-109); its own random field helper is DivFreeSpectraMap
(src/utils/IC.jl:122-179).  The workloads here use a seeded random-phase solenoidal field with
shell spectrum E(k) ~ k^4 exp(-2 (k/kpeak)^2), built directly on the retained (2/3-rule) band of
the rfft half spectrum:

* every retained mode gets amplitude sqrt(E(|k|) / (4 pi |k|^2));
* each field component gets a phase per integer wavevector from a counter-based hash of
  (seed, component, kx, ky, kz), so a mode has the same phase on every grid size;
* the kx = 0 plane is made Hermitian (modes whose partner is in the alias band are zeroed);
* each triple (u, B) is projected solenoidal, F - k (k.F)/k^2;
* u is scaled to E_u = <|u|^2>/2 = e_u and B to b_ratio times u's rms amplitude.

All arithmetic is float64; the result is returned as the complex64 state the solver consumes.
"""
from __future__ import annotations

import math

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def kept_counts(n: int):
    """(Kx, Kp, Kn): kept rfft-axis modes, kept non-negative / negative full-axis modes (1/3 rule)."""
    a = 1.0 / 3.0
    i_l = math.floor((1 - a) / 2 * n) + 1
    i_r = math.ceil((1 + a) / 2 * n)
    return i_l - 1, i_l - 1, n - i_r


def kept_wavenumbers(n: int):
    kx, kp, kn = kept_counts(n)
    full = np.concatenate([np.arange(kp), np.arange(-kn, 0)]).astype(np.int64)
    return np.arange(kx, dtype=np.int64), full


def _mix(x):
    # splitmix64 finaliser (Steele, Lea & Flood 2014), vectorised over uint64 arrays
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    x = ((x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    x = ((x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return x ^ (x >> np.uint64(31))


def mode_phases(seed: int, field: int, kx, ky, kz):
    """Uniform phases in [0, 2 pi) keyed by (seed, field, integer wavevector)."""
    key = ((np.asarray(kx, dtype=np.int64) & 0xFFFF).astype(np.uint64)
           | ((np.asarray(ky, dtype=np.int64) & 0xFFFF).astype(np.uint64) << np.uint64(16))
           | ((np.asarray(kz, dtype=np.int64) & 0xFFFF).astype(np.uint64) << np.uint64(32))
           | (np.uint64(field & 0xFF) << np.uint64(48)))
    with np.errstate(over="ignore"):
        h = _mix(_mix(key ^ _mix(np.uint64(seed & 0xFFFFFFFFFFFFFFFF))))
    return (h >> np.uint64(11)).astype(np.float64) * (2.0 ** -53) * (2 * math.pi)


def random_spectrum_compact(n: int, seed: int, L: float = 2 * math.pi, e_u: float = 0.5,
                            b_ratio: float = 0.3, kpeak: float = 4.0):
    """Retained band (6, K2, K2, Kx) of the random state, [field, kz', ky', kx], float64."""
    kxs, kfs = kept_wavenumbers(n)
    KZ, KY, KX = np.meshgrid(kfs, kfs, kxs, indexing="ij")
    s2p = 2 * math.pi / L
    kx, ky, kz = KX * s2p, KY * s2p, KZ * s2p
    k2 = kx ** 2 + ky ** 2 + kz ** 2
    k = np.sqrt(k2)
    with np.errstate(divide="ignore", invalid="ignore"):
        amp = np.sqrt(k ** 4 * np.exp(-2 * (k / kpeak) ** 2) / (4 * math.pi * k2))
    amp[k2 == 0] = 0.0
    sol = np.empty((6, len(kfs), len(kfs), len(kxs)), dtype=np.complex128)
    for f in range(6):
        sol[f] = amp * np.exp(1j * mode_phases(seed, f, KX, KY, KZ))
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


def random_spectrum_state(n: int, seed: int, L: float = 2 * math.pi, **kw):
    """Full half-spectrum state (6, n, n, n/2+1) complex64, zero in the alias band."""
    c = random_spectrum_compact(n, seed, L, **kw)
    kxs, kfs = kept_wavenumbers(n)
    idx = kfs % n
    out = np.zeros((6, n, n, n // 2 + 1), dtype=np.complex64)
    for f in range(6):
        out[f][np.ix_(idx, idx, np.arange(len(kxs)))] = c[f]
    return out


def taylor_green_fields(n: int, L: float = 2 * math.pi, b_amp: float = 0.5, centred: bool = True):
    """Taylor-Green u and B on the grid points, C-ordered (nz, ny, nx) float32 arrays."""
    dx = L / n
    x0 = -L / 2 if centred else 0.0
    x = x0 + dx * np.arange(n)
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    ux = np.sin(xx) * np.cos(y) * np.cos(z)
    uy = -np.cos(xx) * np.sin(y) * np.cos(z)
    bx = b_amp * np.cos(xx) * np.sin(y) * np.sin(z)
    by = -b_amp * np.sin(xx) * np.cos(y) * np.sin(z)
    zero = np.zeros_like(xx)
    return [a.astype(np.float32) for a in (ux, uy, zero, bx, by, zero)]
