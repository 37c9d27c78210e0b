"""State transfer through page-locked host buffers (mhd_host_alloc): the gather / scatter kernels
read and write the mapped buffer directly.  Results must equal the pageable-memory path bit for
bit; a pageable buffer goes through the staging copy.  From 16 MB up, get_state into mapped
memory writes only the retained band from the device, the copy engine writes the zeros of the
alias z-planes, and host threads zero the alias row blocks and row tails (n = 96 and the HD
n = 128 case); smaller buffers are written whole by the device (n = 32).
MHDGB_HOST_TRANSFER=copy selects the copy-engine path for mapped buffers too (checked in a child
process)."""
import ctypes as C
import math
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pinned(lib, pkg, nbytes):
    p = C.c_void_p()
    pkg._lib.check(lib.mhd_host_alloc(nbytes, C.byref(p)))
    return p


@pytest.mark.parametrize("n", [32, 96])
def test_pinned_state_roundtrip_equals_pageable(pkg, mo, lib, n):
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=51).astype(np.complex64)
    s[:, 3, 2, 1] += 0.5 - 0.25j
    nbytes = s.nbytes
    pin_in, pin_out = _pinned(lib, pkg, nbytes), _pinned(lib, pkg, nbytes)
    try:
        C.memmove(pin_in, s.ctypes.data, nbytes)
        with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
            pkg._lib.check(lib.mhd_set_state(prob.handle, pin_in))
            pageable = prob.sol_c()
            C.memset(pin_out, 0x7f, nbytes)  # garbage: every element must be overwritten
            pkg._lib.check(lib.mhd_get_state(prob.handle, pin_out))
            got = np.frombuffer((C.c_char * nbytes).from_address(pin_out.value), dtype=np.complex64).reshape(s.shape).copy()
            pkg.stepforward(prob, 2)
            after_pageable = prob.sol_c()
            pkg._lib.check(lib.mhd_get_state(prob.handle, pin_out))
            after_pinned = np.frombuffer((C.c_char * nbytes).from_address(pin_out.value), dtype=np.complex64).reshape(s.shape).copy()
        assert np.array_equal(got, pageable)
        assert np.array_equal(got, g.dealias(s.copy()))
        assert np.array_equal(after_pinned, after_pageable)
    finally:
        lib.mhd_host_free(pin_in)
        lib.mhd_host_free(pin_out)


def test_pageable_buffer_uses_staging(pkg, mo, lib):
    n = 32
    g = mo.Grid(n)
    s = mo.random_spectrum_state(g, seed=52).astype(np.complex64)
    buf = np.ascontiguousarray(s)  # pageable host array
    with pkg.Problem(pkg.GPU(0), nx=n, Lx=2 * math.pi, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
        pkg._lib.check(lib.mhd_set_state(prob.handle, buf.ctypes.data))
        assert np.array_equal(prob.sol_c(), g.dealias(s.copy()))


def test_pinned_hydrodynamic_state_overwrites_every_element(pkg, mo, lib):
    """get_state into mapped memory: the device writes the rows with kept ky and kz, host threads
    zero the rest; a (nkr, n, n, 3) HD buffer full of garbage comes back exact."""
    n = 128
    g = mo.Grid(n)
    s = np.ascontiguousarray(mo.random_spectrum_state(g, seed=53).astype(np.complex64)[:3])
    nbytes = s.nbytes
    pin = _pinned(lib, pkg, nbytes)
    try:
        with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, dt=1e-3, B_field=False) as prob:
            prob.set_sol(s.T)
            C.memset(pin, 0x7f, nbytes)
            pkg._lib.check(lib.mhd_get_state(prob.handle, pin))
            got = np.frombuffer((C.c_char * nbytes).from_address(pin.value), dtype=np.complex64).reshape(s.shape).copy()
            assert np.array_equal(got, prob.sol_c())
        full = np.zeros((6,) + s.shape[1:], np.complex64)
        full[:3] = s
        assert np.array_equal(got, g.dealias(full)[:3])
    finally:
        lib.mhd_host_free(pin)


def _child_roundtrip(env_extra, tag):
    """A mapped-buffer round trip at n = 96 (21.7 MB: the split zero path) in a child process with
    extra environment variables (the library reads them once per process)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = textwrap.dedent("""
        import ctypes as C, sys
        import numpy as np
        sys.path.insert(0, %r)
        import __graft_entry__ as ge
        from oracle import mhd_oracle as mo
        pkg = ge.load_package(); lib = pkg._lib.load()
        n = 96
        g = mo.Grid(n)
        s = mo.random_spectrum_state(g, seed=54).astype(np.complex64)
        nb = s.nbytes
        pin = C.c_void_p(); pkg._lib.check(lib.mhd_host_alloc(nb, C.byref(pin)))
        C.memmove(pin, s.ctypes.data, nb)
        with pkg.Problem(pkg.GPU(0), nx=n, nu=1e-3, eta=1e-3, dt=1e-3) as prob:
            pkg._lib.check(lib.mhd_set_state(prob.handle, pin))
            pkg.stepforward(prob, 2)
            ref = prob.sol_c()
            C.memset(pin, 0x7f, nb)
            pkg._lib.check(lib.mhd_get_state(prob.handle, pin))
            got = np.frombuffer((C.c_char * nb).from_address(pin.value), dtype=np.complex64).reshape(s.shape).copy()
        lib.mhd_host_free(pin)
        assert np.array_equal(got, ref)
        assert np.array_equal(np.where(g.retained_mask(), 0, got), np.zeros_like(got))
        print("%s ok")
    """) % (root, tag)
    env = dict(os.environ, **env_extra)
    res = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and f"{tag} ok" in res.stdout, res.stdout + res.stderr


def test_copy_engine_transfer_mode():
    """The same round trip with MHDGB_HOST_TRANSFER=copy."""
    _child_roundtrip({"MHDGB_HOST_TRANSFER": "copy"}, "copy mode")


@pytest.mark.parametrize("zeros,threads", [("ce", "16"), ("host", "16"), ("split", "3")])
def test_alias_zero_paths(zeros, threads):
    """get_state's alias-band zeros from each path (MHDGB_HOST_ZEROS) and a small host pool
    (MHDGB_HOST_THREADS): a garbage-filled mapped buffer comes back exact."""
    _child_roundtrip({"MHDGB_HOST_ZEROS": zeros, "MHDGB_HOST_THREADS": threads}, f"zeros {zeros}")
