"""Parity at the benchmark configurations, against an FP64 comparator on the GPU.

The CPU oracle in float64 is too slow for 50 steps at 256^3 or 20 steps at 512^3, so these tests
use ``oracle/mhd_fp64_torch.py``: the oracle's compact right-hand side and RK4 restated in torch
float64 (cuFFT as a library comparator only).  The first test pins that comparator to the CPU
oracle at 32^3 and 64^3.  Every stepped case starts the GPU (FP32) and the comparator (FP64) from
the same complex64 state and reports, on the retained band:

  relative L2 error of the u and B spectra (separately);
  E_u, E_B (relative) and H_c (relative to sqrt(E_u E_B)) errors of the GPU diagnostics against
  the FP64 state's, and max|k.u_hat|, max|k.B_hat| of the GPU state against FP32 roundoff.

Tolerances (the configurations' stated bounds): one step 1e-5, 50 or 20 steps 1e-4; energies
and cross-helicity 1e-5; max|k.u_hat|, max|k.B_hat| <= 1e-5 max|k| max|u_hat| (FP32 roundoff).
The split forms are held to the bounds of tests/test_gpu_precision.py (FP16 1e-5, BF16 3e-4).

Configurations:
  256^3: the seeded k^4 exp(-2(k/4)^2) spectrum (seed 1), nu = eta = 1e-3, dt = 5e-4, 50 RK4 steps.
  512^3: the same spectrum, nu = eta = 5e-4, dt = 2.5e-4, 20 RK4 steps; the plain form against
         FP64 at 512^3, and the plain and split forms against FP64 run at 128^3 from the same
         seed's truncated spectrum (the generator keys each mode's phase by its wavevector, so the
         shared modes are identical).  A separate test shows that truncation itself moves the
         shared modes by far less than the tolerances.
"""
import math
from importlib import import_module

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SEED = 1


@pytest.fixture(scope="module")
def ft():
    from oracle import mhd_fp64_torch

    return mhd_fp64_torch


@pytest.fixture(scope="module")
def ic(pkg):
    return import_module(pkg.__name__ + ".ic")


def _cuda(a):
    return torch.as_tensor(a).to("cuda")


def _errors(g, got, ref):
    """Relative L2 of u and B on the retained band: got (GPU state, numpy complex64) vs ref (torch)."""
    m = g.retained_mask()
    got_t = _cuda(got).to(torch.complex128)
    out = {}
    for name, sl in (("u", slice(0, 3)), ("B", slice(3, 6))):
        a, b = got_t[sl][:, m], ref[sl][:, m]
        out[name] = float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
    del got_t
    return out


def _energy_errors(d, ref):
    scale = math.sqrt(ref["E_u"] * ref["E_B"])
    return {"E_u": abs(d.E_u - ref["E_u"]) / ref["E_u"], "E_B": abs(d.E_B - ref["E_B"]) / ref["E_B"],
            "H_c": abs(d.H_c - ref["H_c"]) / scale}


def _check(label, g, got, ref, d, tol, ft, n):
    err = _errors(g, got, ref)
    rd = ft.diagnostics(g, ref)
    en = _energy_errors(d, rd)
    kmax = math.sqrt(3) * n / 3
    umax = float(np.abs(got[:3]).max())
    bmax = float(np.abs(got[3:]).max())
    print(f"{label}: rel L2 u {err['u']:.3e}  B {err['B']:.3e} | E_u err {en['E_u']:.2e}  E_B err {en['E_B']:.2e}  "
          f"H_c err {en['H_c']:.2e} | max|k.u| {d.max_kdotu:.3e} (bound {1e-5 * kmax * umax:.3e})  "
          f"max|k.B| {d.max_kdotb:.3e} (bound {1e-5 * kmax * bmax:.3e})")
    assert err["u"] <= tol and err["B"] <= tol, (label, err)
    assert en["E_u"] <= 1e-5 and en["E_B"] <= 1e-5 and en["H_c"] <= 1e-5, (label, en)
    assert d.max_kdotu <= 1e-5 * kmax * umax and d.max_kdotb <= 1e-5 * kmax * bmax
    assert d.nonfinite == 0
    return err, en


@pytest.mark.parametrize("n,scheme", [(32, "RK4"), (64, "RK4"), (64, "LSRK4")])
def test_fp64_comparator_matches_cpu_oracle(mo, ft, n, scheme):
    """The torch FP64 comparator against the CPU oracle (FP64, compact form): RHS and 3 steps."""
    g = mo.Grid(n)
    s0 = mo.random_spectrum_state(g, 7).astype(np.complex64)
    N = np.zeros(s0.shape, dtype=np.complex128)
    mo.calcN_fast(N, s0.astype(np.complex128), g, 1e-3, 2e-3)
    tg = ft.TorchGrid(n)
    Nt = ft.calcN(tg, _cuda(s0).to(torch.complex128), 1e-3, 2e-3).cpu().numpy()
    e_rhs = mo.rel_l2(Nt, N)
    st = mo.Stepper(g, 1e-3, 2e-3, 0.01, scheme, literal=False)
    ref = s0.astype(np.complex128).copy()
    for _ in range(3):
        st.stepforward(ref)
    g.dealias(ref)
    out, _, _ = ft.run(n, s0, 1e-3, 2e-3, 0.01, 3, scheme)
    e_step = mo.rel_l2(out.cpu().numpy(), ref)
    print(f"comparator vs CPU oracle n={n} {scheme}: RHS {e_rhs:.2e}, 3 steps {e_step:.2e}")
    assert e_rhs < 1e-12 and e_step < 1e-12


@pytest.fixture(scope="module")
def fp64_256(ft, ic):
    """FP64 256^3, nu = eta = 1e-3, dt = 5e-4: the states after 1 and 50 RK4 steps."""
    s0 = ic.random_spectrum_state(256, SEED)
    ref, kept, g = ft.run(256, s0, 1e-3, 1e-3, 5e-4, 50, "RK4", keep=(1,))
    yield {"s0": s0, "ref": ref, "one": kept[1], "g": g}
    torch.cuda.empty_cache()


@pytest.mark.parametrize("prec", ["fp32", "split_tf32"])
def test_256_rk4_50_steps_vs_fp64(pkg, ft, fp64_256, prec):
    """256^3, nu = eta = 1e-3, dt = 5e-4: 1 step <= 1e-5 and 50 RK4 steps <= 1e-4 against FP64, for
    the plain form and the tcgen05 TF32 form."""
    n = 256
    s0, ref, g = fp64_256["s0"], fp64_256["ref"], fp64_256["g"]
    kept = {1: fp64_256["one"]}
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=5e-4, precision=prec) as prob:
        prob.set_sol(s0.T)
        pkg.stepforward(prob, 1)
        one, d1 = prob.sol_c(), prob.diagnostics()
        pkg.stepforward(prob, 49)
        fifty, d50 = prob.sol_c(), prob.diagnostics()
    _check(f"256^3 {prec} RK4 1 step", g, one, kept[1], d1, 1e-5, ft, n)
    _check(f"256^3 {prec} RK4 50 steps", g, fifty, ref, d50, 1e-4, ft, n)


@pytest.fixture(scope="module")
def fp64_512(ft, ic):
    """FP64 512^3, nu = eta = 5e-4, dt = 2.5e-4, 20 RK4 steps from the seeded state, and the same at
    128^3 from the seed's truncated spectrum."""
    s512 = ic.random_spectrum_state(512, SEED)
    ref512, _, g512 = ft.run(512, s512, 5e-4, 5e-4, 2.5e-4, 20, "RK4")
    s128 = ic.random_spectrum_state(128, SEED)
    ref128, _, g128 = ft.run(128, s128, 5e-4, 5e-4, 2.5e-4, 20, "RK4")
    yield {"s512": s512, "ref512": ref512, "g512": g512, "ref128": ref128, "g128": g128}
    torch.cuda.empty_cache()


def _band128(ic, a, n):
    """The 128^3 retained band (6, K2, K2, Kx) of an n^3 state, rescaled to 128^3 amplitudes (the
    unnormalised spectra carry a factor n^3)."""
    kxs, kfs = ic.kept_wavenumbers(128)
    idx = torch.as_tensor(kfs % n, device="cuda")
    t = a if torch.is_tensor(a) else _cuda(a)
    t = t.to(torch.complex128)
    return t[:, idx][:, :, idx][..., : len(kxs)] * (128.0 / n) ** 3


def _rel(a, b):
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


def test_truncated_128_comparator_is_exact_enough(fp64_512, ic):
    """FP64 at 128^3 from the truncated spectrum against FP64 at 512^3 on the shared modes: the
    truncation error of the 128^3 comparator, far below the split forms' tolerances."""
    a = _band128(ic, fp64_512["ref512"], 512)
    b = _band128(ic, fp64_512["ref128"], 128)
    e = _rel(b, a)
    print(f"FP64 128^3 (truncated spectrum) vs FP64 512^3 on the 128^3 band after 20 steps: {e:.3e}")
    assert e < 1e-7


def test_512_plain_20_steps_vs_fp64(pkg, ft, fp64_512):
    n = 512
    with pkg.Problem(pkg.GPU(0), nx=n, nu=5e-4, eta=5e-4, dt=2.5e-4) as prob:
        prob.set_sol(fp64_512["s512"].T)
        pkg.stepforward(prob, 20)
        got, d = prob.sol_c(), prob.diagnostics()
    _check("512^3 plain FP32 RK4 20 steps", fp64_512["g512"], got, fp64_512["ref512"], d, 1e-4, ft, n)


@pytest.mark.parametrize("prec,tol", [("fp32", 1e-5), ("split_fp16", 1e-5), ("split_bf16", 3e-4)])
def test_512_forms_20_steps_vs_truncated_128_fp64(pkg, ic, ft, fp64_512, prec, tol):
    """The precision configuration: each form at 512^3 for 20 RK4 steps, compared on the 128^3 band
    with FP64 run at 128^3 from the same seed's truncated spectrum, and on the whole band with
    FP64 at 512^3; energies against the FP64 512^3 state."""
    n = 512
    with pkg.Problem(pkg.GPU(0), nx=n, nu=5e-4, eta=5e-4, dt=2.5e-4, precision=prec) as prob:
        prob.set_sol(fp64_512["s512"].T)
        pkg.stepforward(prob, 20)
        got, d = prob.sol_c(), prob.diagnostics()
    e128 = _rel(_band128(ic, got, n), _band128(ic, fp64_512["ref128"], 128))
    g = fp64_512["g512"]
    err = _errors(g, got, fp64_512["ref512"])
    en = _energy_errors(d, ft.diagnostics(g, fp64_512["ref512"]))
    print(f"512^3 {prec} 20 RK4 steps: rel L2 vs FP64 128^3 (truncated) {e128:.3e}; vs FP64 512^3 u {err['u']:.3e} "
          f"B {err['B']:.3e}; E_u err {en['E_u']:.2e} E_B err {en['E_B']:.2e} H_c err {en['H_c']:.2e}")
    assert e128 <= tol
    assert err["u"] <= tol and err["B"] <= tol
    assert max(en.values()) <= max(tol, 1e-5)
    assert d.nonfinite == 0
