"""GB300-native drop-in for MHDFlows.jl's 3D incompressible MHD RHS + RK4/LSRK4 step.

Host-side mirror of the reference's interface for this path, over the C ABI in
``include/mhdgb.h`` (libmhdgb.so, hand-written sm_103a CUDA):

    prob = Problem(GPU(); nx=256, Lx=2pi, nu=1e-3, eta=1e-3, B_field=True, stepper="RK4",
                   T=np.float32, dt=5e-4)                 # src/pgen.jl:64-127
    SetUpProblemIC(prob, ux=..., uy=..., uz=..., bx=..., by=..., bz=...)   # src/utils/IC.jl:41-109
    prob.set_vp(chi, U0=(...), B0=(...))   # with VP_method=True: params.χ, U₀, B₀ (VPSolver.jl)
    stepforward(prob)                                      # stepforward!(prob.sol, prob.clock, ...)
    updatevars(prob)                                       # vars <- irfft(sol)
    KE, ME = ProbDiagnostic(prob)                          # src/utils/UserInterface.jl:65-86
    TimeIntegrator(prob, t0, N0, usr_dt=...)               # src/integrator.jl:31-156 (stepping part)

Arrays use the reference's index order: ``prob.sol[i, j, k, f]`` is a complex64 array of shape
(nkr, ny, nz, 6) and ``prob.vars.ux[i, j, k]`` a float32 array of shape (nx, ny, nz), both
Fortran-ordered (the memory of a Julia Array).  There is no CPU fallback: ``Problem(CPU())``
raises, and a missing CUDA library raises at import of the first problem.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import MHDError, MHD_LSRK4, MHD_RK4

__all__ = [
    "GPU", "CPU", "Problem", "SetUpProblemIC", "stepforward", "updatevars", "ProbDiagnostic",
    "Diagnostics", "TimeIntegrator", "MHDError", "kept_modes", "supported_sizes", "footprint_bytes",
    "Batch", "Ensemble", "slot_bytes", "Diagnostic", "autotune", "variants", "select_variant",
    "TUNED_CLASSES", "PRECISIONS", "savefile", "Restart", "readMHDFlows", "checkpoint_path", "FIELDS",
    "SetUpFk", "forcing_amplitude", "DivVCorrection", "DivBCorrection", "HISTORY_COLUMNS",
]

FIELDS = ("ux", "uy", "uz", "bx", "by", "bz")


class GPU:
    """Device tag (FourierFlows ``GPU()``)."""

    def __init__(self, device: int = 0):
        self.device = device

    def __repr__(self):
        return f"GPU({self.device})"


class CPU:
    """Device tag (FourierFlows ``CPU()``); this library has no CPU path."""


def supported_sizes():
    lib = _lib.load()
    return [n for n in (16, 32, 48, 64, 96, 128, 256, 512) if lib.mhd_supported_n(n)]


def kept_modes(n: int):
    """(kx, kp, kn) kept modes of the 2/3 rule (FourierFlows getaliasedwavenumbers, 1/3)."""
    lib = _lib.load()
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    _lib.check(lib.mhd_kept_modes(n, C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


PRECISIONS = {"fp32": 0, "split_fp16": 1, "split_bf16": 2, "split_tf32": 3}


def _precision(precision) -> int:
    """Precision form: "fp32" (plain), "split_fp16" / "split_bf16" (mma.sync tensor-core x-row DFTs) or
    "split_tf32" (tcgen05 tensor-core x-row DFTs, n = 256)."""
    if isinstance(precision, int) and precision in PRECISIONS.values():
        return precision
    key = str(precision).lower()
    if key not in PRECISIONS:
        raise MHDError(_lib.MHD_ERR_INVALID, f"unknown precision {precision!r} (fp32, split_fp16, split_bf16, split_tf32)")
    return PRECISIONS[key]


def _params(n, L, nu, eta, nnu, neta, dt, scheme, device, precision=0, hydro_only=False, vp=False):
    return _lib.MhdParams(n, L, nu, eta, nnu, neta, dt, scheme, _precision(precision), device, int(bool(hydro_only)),
                          int(bool(vp)))


def _vp_arrays(n, chi, U0, B0):
    """Host buffers of set_vp: chi and the wall triples as float32 in the reference's (nx, ny, nz)
    column-major order (arrays indexed [x, y, z], like prob.vars.ux)."""
    def field(a, what):
        a = np.asarray(a, dtype=np.float32)
        if a.shape != (n, n, n):
            raise MHDError(_lib.MHD_ERR_INVALID, f"{what} must be an (n, n, n) array indexed [x, y, z]")
        return np.asfortranarray(a)

    def triple(t, what):
        if t is None:
            return None
        if len(t) != 3:
            raise MHDError(_lib.MHD_ERR_INVALID, f"{what} must be three (n, n, n) arrays (x, y, z components)")
        return np.concatenate([field(c, what).ravel(order="F") for c in t])

    c = None if chi is None else field(chi, "chi")
    return c, triple(U0, "U0"), triple(B0, "B0")


def _ptr(a):
    return None if a is None else a.ctypes.data


HISTORY_COLUMNS = ("step", "t", "E_u", "E_B", "H_c", "max_kdotu", "max_kdotb", "nonfinite")


def _history(lib, h, slot):
    n = C.c_int()
    _lib.check(lib.mhd_get_diag_history(h, int(slot), None, 0, C.byref(n)))
    out = np.zeros((max(n.value, 1), 8), dtype=np.float64)
    _lib.check(lib.mhd_get_diag_history(h, int(slot), out.ctypes.data, n.value, C.byref(n)))
    return out[: min(n.value, out.shape[0])] if n.value else out[:0]


def footprint_bytes(n: int, L: float = 2 * math.pi, stepper: str = "RK4") -> int:
    """Device bytes one problem of size n holds (admission control of the serving loop)."""
    lib = _lib.load()
    p = _params(n, L, 0.0, 0.0, 0, 0, 0.0, MHD_RK4 if stepper.upper() == "RK4" else MHD_LSRK4, 0)
    out = C.c_longlong()
    _lib.check(lib.mhd_footprint_bytes(C.byref(p), C.byref(out)))
    return out.value


class Clock:
    """FourierFlows Clock: t, step, dt (kept by the library, mirrored here)."""

    def __init__(self, prob):
        self._p = prob

    def _read(self):
        t, s, dt = C.c_double(), C.c_longlong(), C.c_double()
        _lib.check(self._p._lib.mhd_get_clock(self._p._h, C.byref(t), C.byref(s), C.byref(dt)))
        return t.value, s.value, dt.value

    @property
    def t(self):
        return self._read()[0]

    @t.setter
    def t(self, v):
        _, s, dt = self._read()
        _lib.check(self._p._lib.mhd_set_clock(self._p._h, float(v), s, dt))

    @property
    def step(self):
        return self._read()[1]

    @step.setter
    def step(self, v):
        t, _, dt = self._read()
        _lib.check(self._p._lib.mhd_set_clock(self._p._h, t, int(v), dt))

    @property
    def dt(self):
        return self._read()[2]

    @dt.setter
    def dt(self, v):
        t, s, _ = self._read()
        _lib.check(self._p._lib.mhd_set_clock(self._p._h, t, s, float(v)))


class Vars:
    """Physical fields ux..bz (MVars, src/Structure/MHDVars.jl:1-24), filled by updatevars."""

    def __init__(self, n, nfields=6):
        for f in FIELDS[:nfields]:
            setattr(self, f, np.zeros((n, n, n), dtype=np.float32, order="F"))


class Params:
    def __init__(self, nu, eta, nnu, neta):
        self.nu, self.eta, self.nnu, self.neta = nu, eta, nnu, neta
        self.ν, self.η, self.nν, self.nη = nu, eta, nnu, neta
        self.ux_ind, self.uy_ind, self.uz_ind, self.bx_ind, self.by_ind, self.bz_ind = 1, 2, 3, 4, 5, 6


class Grid:
    """Grid quantities the host needs (ThreeDGrid conventions: centred x, kr, l, m)."""

    def __init__(self, n, L):
        self.nx = self.ny = self.nz = n
        self.Lx = self.Ly = self.Lz = L
        self.nkr = n // 2 + 1
        self.dx = self.dy = self.dz = L / n
        self.x = (-L / 2 + self.dx * np.arange(n)).astype(np.float32)
        self.y = self.x.copy()
        self.z = self.x.copy()
        self.kr = (2 * math.pi / L) * np.arange(self.nkr, dtype=np.float32)
        self.l = ((2 * math.pi / L) * np.fft.fftfreq(n, 1.0 / n)).astype(np.float32)
        self.m = self.l.copy()


class Problem:
    """``Problem(GPU(); nx, Lx, ν/nu, η/eta, nν, nη, B_field=True, VP_method=False, stepper, T=Float32, dt)``.

    The MHD and HD branches of src/pgen.jl:64-127, with or without volume penalisation
    (``VP_method``; the mask and walls are set with ``set_vp``).  EMHD, compressibility, shear
    and the dye module are not on this path; forcing is set with ``SetUpFk``.
    """

    def __init__(self, dev=None, *, nx=64, ny=None, nz=None, Lx=2 * math.pi, Ly=None, Lz=None,
                 dt=0.0, nu=None, eta=None, nnu=0, neta=0, B_field=True, EMHD=False,
                 Compressibility=False, Shear=False, VP_method=False, Dye_Module=False,
                 stepper="RK4", calcF=None, T=np.float32, aliased_fraction=1 / 3, precision="fp32", **kw):
        nu = kw.pop("ν", nu)
        eta = kw.pop("η", eta)
        nnu = kw.pop("nν", nnu)
        neta = kw.pop("nη", neta)
        if kw:
            raise TypeError(f"unexpected keyword arguments: {sorted(kw)}")
        if dev is None:
            dev = GPU()
        if isinstance(dev, CPU) or dev is CPU:
            raise MHDError(_lib.MHD_ERR_INVALID, "this library runs on the GPU only: use Problem(GPU(); ...)")
        if EMHD or Compressibility or Shear or Dye_Module or calcF is not None:
            raise MHDError(_lib.MHD_ERR_INVALID, "EMHD, compressibility, shear, dye and calcF hooks are not on this path")
        if (ny not in (None, nx)) or (nz not in (None, nx)) or (Ly not in (None, Lx)) or (Lz not in (None, Lx)):
            raise MHDError(_lib.MHD_ERR_INVALID, "only cubic boxes (nx = ny = nz, Lx = Ly = Lz) are provided")
        if np.dtype(T) != np.float32:
            raise MHDError(_lib.MHD_ERR_INVALID, "the plain form computes in Float32 (T=Float32)")
        if abs(aliased_fraction - 1 / 3) > 1e-12:
            raise MHDError(_lib.MHD_ERR_INVALID, "aliased_fraction is fixed at 1/3 (the reference does not forward it)")
        scheme = {"RK4": MHD_RK4, "LSRK4": MHD_LSRK4}.get(str(stepper).upper())
        if scheme is None:
            raise MHDError(_lib.MHD_ERR_INVALID, f"unknown stepper {stepper!r} (RK4 or LSRK4)")
        self._lib = _lib.load()
        self.n = int(nx)
        self.L = float(Lx)
        self.stepper = str(stepper).upper()
        self.precision = _precision(precision)
        self.B_field = bool(B_field)
        self.VP = bool(VP_method)
        self.nfields = 6 if self.B_field else 3
        if not self.B_field:  # HDcalcN! (src/pgen.jl:176-182): the three velocity fields only
            eta, neta = 0.0, 0
        p = _params(self.n, self.L, float(nu or 0.0), float(eta or 0.0), int(nnu), int(neta), float(dt),
                    scheme, dev.device, self.precision, hydro_only=not self.B_field, vp=self.VP)
        h = C.c_void_p()
        _lib.check(self._lib.mhd_create(C.byref(p), C.byref(h)))
        self._h = h
        self.grid = Grid(self.n, self.L)
        self.params = Params(float(nu or 0.0), float(eta or 0.0), int(nnu), int(neta))
        self.vars = Vars(self.n, self.nfields)
        self.clock = Clock(self)
        self.device = dev

    # -- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            self._lib.mhd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    # -- state
    @property
    def sol(self):
        """Copy of prob.sol, complex64 (nkr, n, n, 6) Fortran order ((nkr, n, n, 3) for a hydrodynamic
        problem); alias band is zero."""
        out = np.empty((self.nfields, self.n, self.n, self.grid.nkr), dtype=np.complex64)
        _lib.check(self._lib.mhd_get_state(self._h, out.ctypes.data))
        return out.T

    @sol.setter
    def sol(self, value):
        self.set_sol(value)

    def set_sol(self, value):
        a = np.asarray(value)
        nf = self.nfields
        if a.shape == (self.grid.nkr, self.n, self.n, nf):
            a = a.T
        if a.shape != (nf, self.n, self.n, self.grid.nkr):
            raise MHDError(_lib.MHD_ERR_INVALID, f"sol must have shape (nkr, n, n, {nf}) = {(self.grid.nkr, self.n, self.n, nf)}")
        a = np.ascontiguousarray(a, dtype=np.complex64)
        _lib.check(self._lib.mhd_set_state(self._h, a.ctypes.data))

    def record_diagnostics(self, freq: int, capacity: int = 1024):
        """Record the spectral diagnostics on the device every ``freq`` steps (0: off) into up to
        ``capacity`` samples, without host synchronisation; read them with diagnostic_history."""
        _lib.check(self._lib.mhd_set_diag_history(self._h, int(freq), int(capacity)))

    def diagnostic_history(self):
        """(samples, 8) float64: step, t, E_u, E_B, H_c, max|k.u|, max|k.B|, non-finite count."""
        return _history(self._lib, self._h, 0)

    def set_vp(self, chi, U0=None, B0=None):
        """The volume-penalisation mask and walls, in place of writing params.χ, params.U₀x..U₀z and
        params.B₀x..B₀z (src/Structure/datastructure.jl:79-95): ``chi`` an (n, n, n) array indexed
        [x, y, z] (like prob.vars.ux), ``U0`` / ``B0`` None (zero) or three such arrays.  Needs
        ``VP_method=True``."""
        c, u, b = _vp_arrays(self.n, chi, U0, B0)
        _lib.check(self._lib.mhd_set_vp(self._h, _ptr(c), _ptr(u), _ptr(b)))

    def sol_c(self):
        """prob.sol as a C-ordered (nfields, nz, ny, nkr) array (same memory order as the Julia array)."""
        out = np.empty((self.nfields, self.n, self.n, self.grid.nkr), dtype=np.complex64)
        _lib.check(self._lib.mhd_get_state(self._h, out.ctypes.data))
        return out

    def rhs_c(self):
        """calcN!(N, sol, ...) of the current state, C-ordered (nfields, nz, ny, nkr)."""
        out = np.empty((self.nfields, self.n, self.n, self.grid.nkr), dtype=np.complex64)
        _lib.check(self._lib.mhd_compute_rhs(self._h, out.ctypes.data))
        return out

    def physical_c(self, field: int):
        out = np.empty((self.n, self.n, self.n), dtype=np.float32)
        _lib.check(self._lib.mhd_get_physical(self._h, int(field), out.ctypes.data))
        return out

    def set_physical_c(self, field: int, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        if a.shape != (self.n, self.n, self.n):
            raise MHDError(_lib.MHD_ERR_INVALID, "physical fields are (n, n, n)")
        _lib.check(self._lib.mhd_set_physical(self._h, int(field), a.ctypes.data))

    def synchronize(self):
        _lib.check(self._lib.mhd_synchronize(self._h))

    def memory_bytes(self):
        b = C.c_longlong()
        _lib.check(self._lib.mhd_memory_bytes(self._h, C.byref(b)))
        return b.value

    def diagnostics(self):
        out = (C.c_double * 8)()
        rc = self._lib.mhd_diagnostics(self._h, out, 8)
        d = Diagnostics(*list(out))
        if rc == _lib.MHD_ERR_NONFINITE:
            raise MHDError(rc, self._lib.mhd_last_error().decode())
        _lib.check(rc)
        return d

    def __repr__(self):
        return (f"MHDFlows Problem (GB300)\n  grid: {self.n}^3, L = {self.L:.6g}\n  stepper: {self.stepper}\n"
                f"  nu = {self.params.nu}, eta = {self.params.eta}, dt = {self.clock.dt}")


class Diagnostics:
    """Result of mhd_diagnostics (FP64 accumulation on the device)."""

    __slots__ = ("E_u", "E_B", "H_c", "max_kdotu", "max_kdotb", "max_divb", "nonfinite", "t")

    def __init__(self, E_u, E_B, H_c, max_kdotu, max_kdotb, max_divb, nonfinite, t):
        self.E_u, self.E_B, self.H_c = E_u, E_B, H_c
        self.max_kdotu, self.max_kdotb, self.max_divb = max_kdotu, max_kdotb, max_divb
        self.nonfinite, self.t = nonfinite, t

    def as_dict(self):
        return {k: getattr(self, k) for k in self.__slots__}


def _to_c_phys(a, n):
    a = np.asarray(a)
    if a.shape != (n, n, n):
        raise MHDError(_lib.MHD_ERR_INVALID, f"initial fields must be (nx, ny, nz) = {(n, n, n)}")
    # Julia (nx, ny, nz) column-major == C-ordered (nz, ny, nx): transpose the index order
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).T)


def SetUpProblemIC(prob: Problem, *, ux=None, uy=None, uz=None, bx=None, by=None, bz=None):
    """SetUpProblemIC!(prob; ux, ..., bz) (src/utils/IC.jl:41-109): host field -> device -> r2c."""
    for f, arr in enumerate((ux, uy, uz, bx, by, bz)):
        if arr is None:
            continue
        if f >= prob.nfields:
            raise MHDError(_lib.MHD_ERR_INVALID, "a hydrodynamic problem (B_field=false) has no magnetic field")
        c = _to_c_phys(arr, prob.n)
        prob.set_physical_c(f, c)
        getattr(prob.vars, FIELDS[f])[...] = c.T
    return None


def DivVCorrection(prob):
    """DivVCorrection!(prob) (src/Solver/VPSolver.jl:100-138): u loses its gradient part."""
    _lib.check(prob._lib.mhd_div_correct(prob._h, _lib.MHD_DIV_U))


def DivBCorrection(prob):
    """DivBCorrection!(prob) (src/Solver/VPSolver.jl:60-98): B loses its gradient part."""
    _lib.check(prob._lib.mhd_div_correct(prob._h, _lib.MHD_DIV_B))


def stepforward(prob: Problem, nsteps: int = 1):
    """stepforward!(prob.sol, prob.clock, prob.timestepper, ...): advance nsteps (default 1)."""
    _lib.check(prob._lib.mhd_step(prob._h, int(nsteps)))
    return None


def updatevars(prob: Problem):
    """updatevars!(prob): vars.ux..bz <- normalised c2r of the current sol."""
    for f, name in enumerate(FIELDS[: prob.nfields]):
        getattr(prob.vars, name)[...] = prob.physical_c(f).T
    return None


def ProbDiagnostic(prob: Problem):
    """(KE, ME) = (sum |u|^2 dV, sum |B|^2 dV) of the current state, rounded to 3 significant
    digits like src/utils/UserInterface.jl:65-86; NaN raises."""
    d = prob.diagnostics()

    def r3(x):
        return float(f"{x:.3g}")

    return r3(d.E_u), r3(d.E_B)


class Diagnostic:
    """Diagnostic{T,N} (src/DiagnosticWrapper.jl:14-105): ``calc(prob)`` evaluated every ``freq``
    steps by ``increment``; ``data``, ``t`` and ``steps`` hold the samples."""

    def __init__(self, calc, prob, freq: int = 1):
        self.calc, self.prob, self.freq = calc, prob, int(freq)
        self.data, self.t, self.steps = [], [], []

    def update(self):
        self.data.append(self.calc(self.prob))
        self.t.append(self.prob.clock.t)
        self.steps.append(self.prob.clock.step)

    def increment(self):
        if self.prob.clock.step % self.freq == 0:
            self.update()

    __call__ = increment


def TimeIntegrator(prob: Problem, t0: float, N0: int, *, usr_dt: float = 0.0, CFL_Coef: float = 0.25,
                   diags=(), diag_freq: int = 0):
    """Stepping part of TimeIntegrator! (src/integrator.jl:31-156): runs while N0 >= step and
    t0 >= t, i.e. N0+1 steps from step 0 like the reference.  With usr_dt > 0 the step is fixed;
    with usr_dt = 0 getCFL! runs on the device before every step (dt = min(CFL_Coef dx / vmax,
    t_diff), src/integrator.jl:158-198) without host synchronisation.  Diagnostics are
    incremented after every step (increment!(diags), src/integrator.jl:116).  With diag_freq > 0
    the spectral diagnostics are recorded on the device every diag_freq steps instead, with no host
    round trip (prob.diagnostic_history() reads them).  Returns the zone updates per second, the
    reference's own throughput figure (src/integrator.jl:150-153)."""
    import time

    vp = getattr(prob, "VP", False)
    if vp:  # src/integrator.jl:84-88: clean the divergence before the loop
        DivVCorrection(prob)
        if prob.B_field:
            DivBCorrection(prob)
    if usr_dt > 0:
        _lib.check(prob._lib.mhd_set_cfl(prob._h, 0, CFL_Coef))
        prob.clock.dt = usr_dt
    else:
        _lib.check(prob._lib.mhd_set_cfl(prob._h, 1, CFL_Coef))
    prob.clock.step = 0
    if diag_freq > 0:
        prob.record_diagnostics(diag_freq, (N0 + 1) // diag_freq + 1)
    if vp:  # src/integrator.jl:118-122: and after every step
        _lib.check(prob._lib.mhd_set_div_correction(prob._h, 1))
    start = time.perf_counter()
    try:
        if math.isinf(t0) and not diags:
            stepforward(prob, N0 + 1)  # no stopping time to test: one call, no host round trips
        else:
            while N0 >= prob.clock.step and t0 >= prob.clock.t:
                stepforward(prob)
                for d in diags:
                    d.increment()
        prob.synchronize()
    finally:
        if vp:
            _lib.check(prob._lib.mhd_set_div_correction(prob._h, 0))
    el = time.perf_counter() - start
    return prob.clock.step * prob.n ** 3 / el if el > 0 else float("inf")


# ---------------------------------------------------------------------------------------------
# Batched solves (no counterpart in the reference): size classes of resident problems stepped
# together, and ensembles of size classes stepped concurrently in one CUDA graph per step.
# ---------------------------------------------------------------------------------------------

def slot_bytes(n: int, L: float = 2 * math.pi):
    """(bytes per slot, bytes per size class) on the device for grid size n."""
    lib = _lib.load()
    p = _params(n, L, 0.0, 0.0, 0, 0, 0.0, MHD_RK4, 0)
    a, b = C.c_longlong(), C.c_longlong()
    _lib.check(lib.mhd_slot_bytes(C.byref(p), C.byref(a), C.byref(b)))
    return a.value, b.value


class Batch:
    """A size class: up to ``capacity`` problems of grid size n (one scheme) resident in HBM.

    ``step`` advances every active slot by one time step in the same kernel launches; each slot
    has its own nu, eta, dt and clock.  Slot arrays use the C-ordered reference layout
    (6, n, n, nkr) complex64 for states and (n, n, n) float32 for physical fields.
    """

    def __init__(self, n: int, capacity: int, stepper: str = "RK4", L: float = 2 * math.pi, device: int = 0,
                 precision="fp32", VP_method=False):
        scheme = {"RK4": MHD_RK4, "LSRK4": MHD_LSRK4}.get(str(stepper).upper())
        if scheme is None:
            raise MHDError(_lib.MHD_ERR_INVALID, f"unknown stepper {stepper!r}")
        self._lib = _lib.load()
        self.n, self.L, self.stepper = int(n), float(L), str(stepper).upper()
        self.nkr = self.n // 2 + 1
        p = _params(self.n, self.L, 0.0, 0.0, 0, 0, 0.0, scheme, device, precision, vp=VP_method)
        h = C.c_void_p()
        _lib.check(self._lib.mhd_batch_create(C.byref(p), int(capacity), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mhd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self):
        cap, act = C.c_int(), C.c_int()
        _lib.check(self._lib.mhd_batch_info(self._h, C.byref(cap), C.byref(act)))
        return cap.value, act.value

    def add(self, nu: float, eta: float, dt: float) -> int:
        s = C.c_int()
        _lib.check(self._lib.mhd_batch_add(self._h, float(nu), float(eta), float(dt), C.byref(s)))
        return s.value

    def remove(self, slot: int):
        _lib.check(self._lib.mhd_batch_remove(self._h, int(slot)))

    def set_state(self, slot: int, sol_c):
        a = np.ascontiguousarray(sol_c, dtype=np.complex64)
        if a.shape != (6, self.n, self.n, self.nkr):
            raise MHDError(_lib.MHD_ERR_INVALID, "state must be (6, n, n, nkr)")
        _lib.check(self._lib.mhd_slot_set_state(self._h, int(slot), a.ctypes.data))

    def get_state(self, slot: int):
        out = np.empty((6, self.n, self.n, self.nkr), dtype=np.complex64)
        _lib.check(self._lib.mhd_slot_get_state(self._h, int(slot), out.ctypes.data))
        return out

    def set_physical(self, slot: int, field: int, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32)
        _lib.check(self._lib.mhd_slot_set_physical(self._h, int(slot), int(field), a.ctypes.data))

    def record_diagnostics(self, freq: int, capacity: int = 1024):
        """On-device diagnostics of every active slot every ``freq`` steps (Problem.record_diagnostics)."""
        _lib.check(self._lib.mhd_set_diag_history(self._h, int(freq), int(capacity)))

    def diagnostic_history(self, slot: int):
        """(samples, 8) float64 of a slot, columns HISTORY_COLUMNS."""
        return _history(self._lib, self._h, slot)

    def set_vp(self, slot: int, chi, U0=None, B0=None):
        """Volume-penalisation mask and walls of a slot (Problem.set_vp); needs VP_method=True."""
        c, u, b = _vp_arrays(self.n, chi, U0, B0)
        _lib.check(self._lib.mhd_slot_set_vp(self._h, int(slot), _ptr(c), _ptr(u), _ptr(b)))

    def get_physical(self, slot: int, field: int):
        out = np.empty((self.n, self.n, self.n), dtype=np.float32)
        _lib.check(self._lib.mhd_slot_get_physical(self._h, int(slot), int(field), out.ctypes.data))
        return out

    def diagnostics(self, slot: int):
        out = (C.c_double * 8)()
        rc = self._lib.mhd_slot_diagnostics(self._h, int(slot), out, 8)
        if rc == _lib.MHD_ERR_NONFINITE:
            raise MHDError(rc, self._lib.mhd_last_error().decode())
        _lib.check(rc)
        return Diagnostics(*list(out))

    def clock(self, slot: int):
        t, s, dt = C.c_double(), C.c_longlong(), C.c_double()
        _lib.check(self._lib.mhd_slot_get_clock(self._h, int(slot), C.byref(t), C.byref(s), C.byref(dt)))
        return t.value, s.value, dt.value

    def step(self, nsteps: int = 1):
        _lib.check(self._lib.mhd_step(self._h, int(nsteps)))

    def synchronize(self):
        _lib.check(self._lib.mhd_synchronize(self._h))

    def memory_bytes(self):
        b = C.c_longlong()
        _lib.check(self._lib.mhd_memory_bytes(self._h, C.byref(b)))
        return b.value


class Ensemble:
    """Size classes stepped together: one CUDA graph per step forks every member onto its own
    stream, so boxes of different sizes advance concurrently."""

    def __init__(self, batches):
        self._lib = _lib.load()
        self.batches = list(batches)
        arr = (C.c_void_p * len(self.batches))(*[b.handle.value for b in self.batches])
        e = C.c_void_p()
        _lib.check(self._lib.mhd_ensemble_create(arr, len(self.batches), C.byref(e)))
        self._e = e

    def step(self, nsteps: int = 1):
        _lib.check(self._lib.mhd_ensemble_step(self._e, int(nsteps)))

    def synchronize(self):
        for b in self.batches:
            b.synchronize()

    def close(self):
        if getattr(self, "_e", None):
            self._lib.mhd_ensemble_destroy(self._e)
            self._e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- autotuner (FFT pass kernel variants) --------------------------------------------------
TUNED_CLASSES = ("z_inverse", "y_inverse", "x_fused", "y_forward", "z_forward")


def autotune(obj, force: bool = False, persist: bool = True):
    """Time the kernel variants of each FFT pass on ``obj`` (a Problem or Batch) and keep the
    fastest; returns the selected variant names.  A result already known for this device and
    grid size is applied without timing unless ``force``."""
    lib = _lib.load()
    flags = (_lib.MHD_TUNE_FORCE if force else 0) | (0 if persist else _lib.MHD_TUNE_NO_FILE)
    _lib.check(lib.mhd_autotune(obj.handle, flags))
    return {c: v[0] for c, v in variants(obj).items()}


def variants(obj):
    """{class: (selected variant name, [all variant names])} of a Problem or Batch."""
    lib = _lib.load()
    out = {}
    buf = C.create_string_buffer(256)
    for i, cname in enumerate(TUNED_CLASSES):
        cnt = C.c_int()
        _lib.check(lib.mhd_variant_count(obj.handle, i, C.byref(cnt)))
        names = []
        for j in range(cnt.value):
            _lib.check(lib.mhd_variant_name(obj.handle, i, j, buf, 256))
            names.append(buf.value.decode())
        _lib.check(lib.mhd_variant_name(obj.handle, i, -1, buf, 256))
        out[cname] = (buf.value.decode(), names)
    return out


def select_variant(obj, cls, idx: int):
    """Select variant ``idx`` of FFT pass class ``cls`` (index or name in TUNED_CLASSES)."""
    lib = _lib.load()
    ci = TUNED_CLASSES.index(cls) if isinstance(cls, str) else int(cls)
    _lib.check(lib.mhd_select_variant(obj.handle, ci, int(idx)))


# ---- checkpoint / restart (src/integrator.jl:208-288, src/utils/IC.jl:245-257) ----------------
# The reference writes one HDF5 file per snapshot through HDF5.jl, <name>_t_<4-digit number>.h5,
# holding i_velocity, j_velocity, k_velocity, i_mag_field, j_mag_field, k_mag_field (Float32,
# Julia (nx, ny, nz)) and time.  The same files are written and read here by ``hdf5.py``, a small
# implementation of the HDF5 file format (no HDF5 library exists on this system); ``fmt="npz"``
# keeps a NumPy archive with the same datasets instead.
_DATASETS = ("i_velocity", "j_velocity", "k_velocity", "i_mag_field", "j_mag_field", "k_mag_field")


def checkpoint_path(file_path_and_name: str, file_number: int, fmt: str = "h5") -> str:
    """<name>_t_0001.h5: the number zero-padded to four digits like savefile."""
    if fmt not in ("h5", "npz"):
        raise MHDError(_lib.MHD_ERR_INVALID, "checkpoint format must be 'h5' or 'npz'")
    return f"{file_path_and_name}_t_{int(file_number):04d}.{fmt}"


def savefile(prob: Problem, file_number: int, file_path_and_name: str = "", fmt: str = "h5") -> str:
    """savefile(prob, file_number; file_path_and_name) (src/integrator.jl:260-288): the physical
    fields of the current state and the time, in the reference's HDF5 layout (or ``fmt="npz"``).
    The time is stored in float64 (the library's clock); the reference's Restart! and
    readMHDFlows read either width.  Returns the path written."""
    from . import hdf5

    updatevars(prob)
    fields = {name: np.asarray(getattr(prob.vars, FIELDS[f]), dtype=np.float32)
              for f, name in enumerate(_DATASETS[: prob.nfields])}
    t = np.float64(prob.clock.t)
    path = checkpoint_path(file_path_and_name, file_number, fmt)
    if fmt == "h5":
        # a Julia (nx, ny, nz) array is stored with HDF5 dimensions (nz, ny, nx), the same bytes
        hdf5.write(path, {**{k: np.ascontiguousarray(v.T) for k, v in fields.items()}, "time": t})
    else:
        with open(path, "wb") as fh:
            np.savez(fh, time=t, **fields)
    return path


def _read_checkpoint(path: str, names):
    """{name: array in the reference's (nx, ny, nz) index order} and the time, from .h5 or .npz."""
    from . import hdf5

    with open(path, "rb") as fh:
        head = fh.read(8)
    if head == hdf5.SIGNATURE:
        d = hdf5.read(path, list(names) + ["time"])
        return {k: d[k].T for k in names}, float(d["time"])
    with np.load(path) as f:
        return {k: np.asarray(f[k]) for k in names}, float(f["time"])


def readMHDFlows(path: str):
    """readMHDFlows(FileName) (src/utils/IC.jl:245-257): (iv, jv, kv, ib, jb, kb, t), Float32
    fields in the reference's (nx, ny, nz) index order."""
    fields, t = _read_checkpoint(path, _DATASETS)
    return (*[np.asarray(fields[k], dtype=np.float32) for k in _DATASETS], t)


def Restart(prob: Problem, path: str):
    """Restart!(prob, file_path_and_name) (src/integrator.jl:208-258): fields -> r2c into sol,
    clock.t <- time."""
    fields, t = _read_checkpoint(path, _DATASETS[: prob.nfields])
    SetUpProblemIC(prob, **{FIELDS[i]: fields[k] for i, k in enumerate(_DATASETS[: prob.nfields])})
    prob.clock.t = t
    return None


# ---- A99 random forcing (src/pgen/A99ForceDriving_GPU.jl) ----------------------------------
def SetUpFk(prob, kf: float = 2.0, P: float = 1.0, sigma: float = 1.0, b: float = 1.0, seed: int = 0, slot: int = 0):
    """SetUpFk!(prob; kf, P, σ, b) (src/pgen/A99ForceDriving_GPU.jl:24-48) plus the A99ForceDriving!
    hook: the velocity right-hand side of every stage gets the A99 random forcing.  P = 0 turns
    it off.  ``prob`` is a Problem (slot 0) or a Batch (``slot``).  Random numbers come from a
    counter-based generator keyed by ``seed`` (the reference draws them with the device rand()).
    A hydrodynamic problem stays unforced, as in the reference: HDcalcN! (src/pgen.jl:176-182)
    adds the forcing before HDcalcN_advection!, which zeroes the velocity right-hand side."""
    lib = _lib.load()
    _lib.check(lib.mhd_slot_set_forcing(prob.handle, int(slot), float(P), float(kf), float(sigma), float(b),
                                        int(seed) & 0xFFFFFFFFFFFFFFFF))
    return None


def forcing_amplitude(prob, slot: int = 0):
    """(A, kf the forcing kernel uses) of a slot (A = 0: no forcing)."""
    lib = _lib.load()
    a, k = C.c_double(), C.c_double()
    _lib.check(lib.mhd_get_forcing(prob.handle, int(slot), C.byref(a), C.byref(k)))
    return a.value, k.value

