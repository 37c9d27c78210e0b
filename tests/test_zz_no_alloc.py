"""The allocation-free diagnostics entry point (mhd_diagnostics_noalloc) against mhd_diagnostics.

It exists for callers that cannot allocate device memory (graph capture, stream callbacks,
real-time loops, hosts whose device memory belongs to another allocator); its only scratch is a
fixed array inside the library.  Here the caller-owned device buffers come from torch.  Two calls
in a row must both agree with the allocating entry point, which also shows that the shared
scratch left by the first call does not leak into the second.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_diagnostics_twice(pkg, mo, lib):
    torch = pytest.importorskip("torch")
    n = 48
    g = mo.Grid(n)
    states = [mo.random_spectrum_state(g, 5).astype(np.complex64),
              (0.5 * mo.random_spectrum_state(g, 6)).astype(np.complex64)]
    states[1][3, 2, 1, 4] += 1.0 + 1.0j  # change the second state beyond a scale factor
    for s in states:
        with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
            prob.set_sol(s.T)
            ref = prob.diagnostics()
        sol_dev = torch.from_numpy(s.view(np.float32)).cuda()
        out_dev = torch.full((6,), float("nan"), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.mhd_diagnostics_noalloc(C.c_void_p(sol_dev.data_ptr()), n, 2 * math.pi,
                                         C.c_void_p(out_dev.data_ptr()), C.c_void_p(stream))
        assert rc == 0, lib.mhd_last_error().decode()
        torch.cuda.synchronize()
        out = out_dev.cpu().numpy()
        for i, name in enumerate(("E_u", "E_B", "H_c")):
            want = getattr(ref, name)
            assert abs(out[i] - want) <= 1e-12 * max(abs(want), abs(ref.E_u)), (name, out[i], want)
        assert out[3] == pytest.approx(ref.max_kdotu, rel=1e-12, abs=1e-12)
        assert out[4] == pytest.approx(ref.max_kdotb, rel=1e-12, abs=1e-12)
        assert out[5] == ref.nonfinite == 0


def test_noalloc_rejects_bad_sizes(pkg, lib):
    rc = lib.mhd_diagnostics_noalloc(C.c_void_p(16), 1024, 2 * math.pi, C.c_void_p(16), None)
    assert rc == pkg._lib.MHD_ERR_INVALID
    assert "beyond" in lib.mhd_last_error().decode()
