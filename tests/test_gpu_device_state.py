"""prob.sol as a device array: mhd_set_state_device / mhd_get_state_device.

MHDFlows' Problem(GPU(); ...) keeps prob.sol in a CuArray that stepforward! updates in place
(src/timestepper/timestepper.jl:4-6), and TimeIntegrator! reads and edits it between steps
(src/integrator.jl:112-122).  A drop-in stepper therefore pushes the caller's device array in,
steps, and writes it back, every step, at device-copy cost.  These tests pass torch device
buffers through the C ABI on torch's stream and require results bit-identical to mhd_step on the
library's own state, including when the caller edits the array between steps.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    import torch

    assert torch.cuda.is_available()
    return torch


def _state(mo, n, seed):
    return mo.random_spectrum_state(mo.Grid(n), seed).astype(np.complex64)


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.float32)).cuda()


def _host(t, shape):
    return t.cpu().numpy().view(np.complex64).reshape(shape)


@pytest.mark.parametrize("n,scheme", [(48, "RK4"), (64, "LSRK4")])
@pytest.mark.parametrize("side_stream", [False, True])
def test_device_state_loop_matches_library_steps(pkg, mo, lib, n, scheme, side_stream):
    """torch's current stream: the legacy default stream (0), or a side stream of torch's."""
    torch = _torch()
    s0 = _state(mo, n, 61)
    dt = 0.2 * (2 * math.pi / n)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=2e-3, dt=dt, stepper=scheme) as ref:
        ref.set_sol(s0.T)
        pkg.stepforward(ref, 3)
        want = ref.sol_c()
    sol = _dev(torch, s0)
    side = torch.cuda.Stream() if side_stream else torch.cuda.current_stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side), pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=2e-3, dt=dt, stepper=scheme) as prob:
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        h = prob.handle
        for _ in range(3):  # the Julia stepforward!(sol::CuArray, ...) of the binding
            pkg._lib.check(lib.mhd_set_state_device(h, C.c_void_p(sol.data_ptr()), stream))
            pkg._lib.check(lib.mhd_step(h, 1))
            pkg._lib.check(lib.mhd_get_state_device(h, C.c_void_p(sol.data_ptr()), stream))
        got = _host(sol, s0.shape)  # a copy on the same stream: ordered after the write-back
        assert np.array_equal(got, prob.sol_c())
    assert np.array_equal(got, want)


def test_edit_between_steps_is_seen(pkg, mo, lib):
    """An edit of the device array between steps (what DivVCorrection! or user code does to
    prob.sol) reaches the next step; the alias band comes back zero."""
    torch = _torch()
    n = 32
    s0 = _state(mo, n, 62)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as ref:
        ref.set_sol(s0.T)
        pkg.stepforward(ref, 1)
        mid = ref.sol_c()
        mid[:, 1, 2, 3] *= 0.5
        ref.set_sol(mid.T)
        pkg.stepforward(ref, 1)
        want = ref.sol_c()
    garbage = s0.copy()
    garbage[...] = 7.0 + 7.0j  # every element, alias band included, must be overwritten
    sol = _dev(torch, s0)
    out = _dev(torch, garbage)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
        h = prob.handle
        pkg._lib.check(lib.mhd_set_state_device(h, C.c_void_p(sol.data_ptr()), stream))
        pkg._lib.check(lib.mhd_step(h, 1))
        pkg._lib.check(lib.mhd_get_state_device(h, C.c_void_p(sol.data_ptr()), stream))
        v = sol.view(torch.complex64).reshape(s0.shape)
        v[:, 1, 2, 3] *= 0.5  # on torch's stream, ordered before the next set
        pkg._lib.check(lib.mhd_set_state_device(h, C.c_void_p(sol.data_ptr()), stream))
        pkg._lib.check(lib.mhd_step(h, 1))
        own = C.c_void_p(lib.mhd_get_stream(h))  # the handle's own stream
        pkg._lib.check(lib.mhd_get_state_device(h, C.c_void_p(out.data_ptr()), own))
        prob.synchronize()
        got = _host(out, s0.shape)
    assert np.array_equal(got, want)
    assert np.all(got[:, ~mo.Grid(n).retained_mask()] == 0)


def test_device_state_rejects_host_and_misaligned_pointers(pkg, mo, lib):
    torch = _torch()
    n = 16
    s0 = _state(mo, n, 63)
    with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
        rc = lib.mhd_set_state_device(prob.handle, C.c_void_p(s0.ctypes.data), None)
        assert rc == pkg._lib.MHD_ERR_INVALID and "device memory" in lib.mhd_last_error().decode()
        buf = torch.zeros(s0.size * 2 + 2, dtype=torch.float32, device="cuda")
        rc = lib.mhd_get_state_device(prob.handle, C.c_void_p(buf.data_ptr() + 8), None)
        assert rc == pkg._lib.MHD_ERR_INVALID and "aligned" in lib.mhd_last_error().decode()
