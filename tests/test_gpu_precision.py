"""Split-precision tensor-core forms (precision="split_fp16" / "split_bf16") against the oracle.

The x-row transforms run as dense complex DFT matrix products on the tensor cores with 16-bit
hi+lo operands and FP32 accumulation; everything else is the plain FP32 path.  Tolerances
(relative L2 on the retained band):
  split FP16  RHS 1e-5 and one RK4 step 1e-5 against the FP64 oracle (FP32-level accuracy);
  split BF16  RHS 3e-4 and one RK4 step 3e-4 (8-bit mantissas: hi+lo carries 16 bits, so the
              form sits near 1e-4 and cannot reach FP32-level accuracy);
  512^3       RHS of each split form against the plain FP32 RHS, 1e-5 (FP16) / 3e-4 (BF16).
  split TF32  (tcgen05, n = 256) RHS 1e-5 against the FP64 oracle and one RK4 step 1e-5 against FP64.
Each test prints the measured error.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"split_fp16": 1e-5, "split_bf16": 3e-4, "split_tf32": 1e-5}


def _state(pkg, n, seed):
    from importlib import import_module

    return import_module(pkg.__name__ + ".ic").random_spectrum_state(n, seed)


@pytest.mark.parametrize("n", [128, 256])
@pytest.mark.parametrize("prec", ["split_fp16", "split_bf16"])
def test_split_rhs_vs_fp64_oracle(pkg, mo, n, prec):
    s0 = _state(pkg, n, 21)
    g = mo.Grid(n)
    ref = np.zeros(s0.shape, dtype=np.complex128)
    mo.calcN_fast(ref, s0.astype(np.complex128), g, 1e-3, 2e-3)
    with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=2e-3, dt=5e-4, precision=prec) as prob:
        prob.set_sol(s0.T)
        got = prob.rhs_c()
    err = mo.rel_l2(got, ref, g.retained_mask())
    print(f"{prec} n={n} RHS rel L2 vs FP64 oracle: {err:.3e}")
    assert err < TOL[prec], err


@pytest.mark.parametrize("prec", ["split_fp16", "split_bf16"])
def test_split_step_vs_fp64_oracle(pkg, mo, prec):
    n = 128
    s0 = _state(pkg, n, 22)
    g = mo.Grid(n)
    st = mo.Stepper(g, 1e-3, 1e-3, 5e-4, "RK4", literal=False)
    ref = s0.astype(np.complex128).copy()
    st.stepforward(ref)
    g.dealias(ref)
    with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=1e-3, dt=5e-4, precision=prec) as prob:
        prob.set_sol(s0.T)
        pkg.stepforward(prob, 1)
        got = prob.sol_c()
        d = prob.diagnostics()
    err = mo.rel_l2(got, ref, g.retained_mask())
    print(f"{prec} n={n} one RK4 step rel L2 vs FP64 oracle: {err:.3e}")
    assert err < TOL[prec], err
    assert d.nonfinite == 0


@pytest.mark.parametrize("prec", ["split_fp16", "split_bf16"])
def test_split_512_rhs_vs_plain(pkg, prec):
    n = 512
    s0 = _state(pkg, n, 23)
    kw = dict(nx=n, Lx=2 * math.pi, nu=5e-4, eta=5e-4, dt=2.5e-4)
    with pkg.Problem(pkg.GPU(0), **kw) as a:
        a.set_sol(s0.T)
        ref = a.rhs_c()
    with pkg.Problem(pkg.GPU(0), precision=prec, **kw) as b:
        b.set_sol(s0.T)
        got = b.rhs_c()
    err = float(np.linalg.norm((got - ref).ravel()) / np.linalg.norm(ref.ravel()))
    print(f"{prec} n=512 RHS rel L2 vs plain FP32: {err:.3e}")
    assert err < TOL[prec], err


def test_split_rejected_where_absent(pkg):
    with pytest.raises(pkg.MHDError):
        pkg.Problem(pkg.GPU(0), nx=64, nu=1e-3, eta=1e-3, dt=1e-3, precision="split_fp16")


@pytest.mark.parametrize("prec", ["split_fp16", "split_bf16"])
def test_split_512_twenty_steps_vs_plain(pkg, prec):
    """The precision configuration: 512^3, nu = eta = 5e-4, dt = 2.5e-4, 20 RK4 steps; the split
    form against the plain FP32 form from the same state (relative L2 of the final spectra)."""
    n = 512
    s0 = _state(pkg, n, 24)
    kw = dict(nx=n, Lx=2 * math.pi, nu=5e-4, eta=5e-4, dt=2.5e-4)
    out = {}
    for form in ("fp32", prec):
        with pkg.Problem(pkg.GPU(0), precision=form, **kw) as p:
            p.set_sol(s0.T)
            pkg.stepforward(p, 20)
            out[form] = p.sol_c()
            d = p.diagnostics()
            assert d.nonfinite == 0
    ref, got = out["fp32"], out[prec]
    err = float(np.linalg.norm((got - ref).ravel()) / np.linalg.norm(ref.ravel()))
    print(f"{prec} n=512 20 RK4 steps rel L2 vs plain FP32: {err:.3e}")
    assert err < TOL[prec], err


def test_tf32_rhs_vs_fp64_oracle(pkg, mo):
    """The tcgen05 x rows (TF32 hi + lo, data operand in tensor memory) at 256^3: one RHS."""
    n = 256
    s0 = _state(pkg, n, 25)
    g = mo.Grid(n)
    ref = np.zeros(s0.shape, dtype=np.complex128)
    mo.calcN_fast(ref, s0.astype(np.complex128), g, 1e-3, 2e-3)
    with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=2e-3, dt=5e-4, precision="split_tf32") as prob:
        prob.set_sol(s0.T)
        got = prob.rhs_c()
        prob.synchronize()
    err = mo.rel_l2(got, ref, g.retained_mask())
    print(f"split_tf32 n=256 RHS rel L2 vs FP64 oracle: {err:.3e}")
    assert err < TOL["split_tf32"], err


def test_tf32_rejected_off_256(pkg):
    for n in (128, 512):
        with pytest.raises(pkg.MHDError):
            pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3, precision="split_tf32")
