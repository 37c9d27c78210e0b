"""The allocation-free diagnostics entry point (mhd_diagnostics_noalloc) against mhd_diagnostics.

The entry point is for callers that cannot allocate device memory themselves: a Julia program
whose prob.sol is a CuArray from CUDA.jl's pool, a Python program on PyTorch's caching
allocator, or a real-time loop that must not block on the allocator.  Its only scratch is a
fixed array inside the library.  Here the caller-owned device buffers come from the CUDA runtime
through ctypes, so the test needs nothing beyond the toolkit.  Each case makes two calls in a
row on different states and both must agree with the allocating entry point, which also shows
that the shared scratch left by the first call does not leak into the second.  n = 256 needs
33,024 partial-sum blocks, more than the array holds (1216), so it runs the grid-stride path.

This file is collected last, so a run that stops at the first failure has run every other test.
"""
import ctypes as C
import ctypes.util
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H2D, D2H = 1, 2  # cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost


def _cudart():
    names = ["libcudart.so", "libcudart.so.13"]
    found = ctypes.util.find_library("cudart")
    if found:
        names.insert(0, found)
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    names += [os.path.join(home, "lib64", "libcudart.so"), os.path.join(home, "lib64", "libcudart.so.13")]
    for name in names:
        try:
            rt = C.CDLL(name)
        except OSError:
            continue
        rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        rt.cudaFree.argtypes = [C.c_void_p]
        rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        rt.cudaDeviceSynchronize.argtypes = []
        rt.cudaSetDevice.argtypes = [C.c_int]
        return rt
    raise AssertionError("the CUDA runtime library (libcudart.so) was not found")


class DeviceBuffer:
    def __init__(self, rt, nbytes):
        self.rt, self.ptr = rt, C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), nbytes) == 0
        self.nbytes = nbytes

    def upload(self, a):
        a = np.ascontiguousarray(a)
        assert a.nbytes == self.nbytes
        assert self.rt.cudaMemcpy(self.ptr, a.ctypes.data, a.nbytes, H2D) == 0

    def download(self, dtype, count):
        out = np.empty(count, dtype=dtype)
        assert self.rt.cudaMemcpy(out.ctypes.data, self.ptr, out.nbytes, D2H) == 0
        return out

    def free(self):
        if self.ptr:
            self.rt.cudaFree(self.ptr)
            self.ptr = C.c_void_p()


def _states(mo, n):
    g = mo.Grid(n)
    a = mo.random_spectrum_state(g, 5).astype(np.complex64)
    b = (0.5 * mo.random_spectrum_state(g, 6)).astype(np.complex64)
    b[3, 2, 1, 4] += 1.0 + 1.0j  # the second state differs beyond a scale factor
    return [a, b]


@pytest.mark.parametrize("n", [48, 256])
def test_noalloc_matches_diagnostics_twice(pkg, mo, lib, n):
    rt = _cudart()
    assert rt.cudaSetDevice(0) == 0
    states = _states(mo, n)
    sol_dev = DeviceBuffer(rt, states[0].nbytes)
    out_dev = DeviceBuffer(rt, 6 * 8)
    try:
        with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
            for s in states:
                prob.set_sol(s.T)
                ref = prob.diagnostics()
                sol_dev.upload(s)
                out_dev.upload(np.full(6, np.nan))
                rc = lib.mhd_diagnostics_noalloc(sol_dev.ptr, n, 2 * math.pi, out_dev.ptr, None)
                assert rc == 0, lib.mhd_last_error().decode()
                assert rt.cudaDeviceSynchronize() == 0
                out = out_dev.download(np.float64, 6)
                print(f"n={n}: noalloc E_u={out[0]:.12e} E_B={out[1]:.12e} H_c={out[2]:.6e}")
                for i, name in enumerate(("E_u", "E_B", "H_c")):
                    want = getattr(ref, name)
                    assert abs(out[i] - want) <= 1e-12 * max(abs(want), abs(ref.E_u)), (name, out[i], want)
                assert out[3] == pytest.approx(ref.max_kdotu, rel=1e-12, abs=1e-12)
                assert out[4] == pytest.approx(ref.max_kdotb, rel=1e-12, abs=1e-12)
                assert out[5] == ref.nonfinite == 0
    finally:
        sol_dev.free()
        out_dev.free()


def test_noalloc_rejects_bad_sizes(pkg, lib):
    rc = lib.mhd_diagnostics_noalloc(C.c_void_p(16), 1024, 2 * math.pi, C.c_void_p(16), None)
    assert rc == pkg._lib.MHD_ERR_INVALID
    assert "beyond" in lib.mhd_last_error().decode()
