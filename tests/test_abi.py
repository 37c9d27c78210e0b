"""CPU tests of the C ABI library and the host mirror (no device compute)."""
import ctypes as C
import math
import os
import re
import subprocess

import numpy as np
import pytest


def test_library_exports_every_header_symbol(pkg, lib):
    names = pkg._lib.header_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    # and the binding table covers the header exactly
    assert sorted(pkg._lib._SIGS) == names


def test_nm_dynamic_symbols(pkg):
    path = pkg._lib.load()._name
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (mhd_\w+)", out))
    assert set(pkg._lib.header_functions()) <= exported


@pytest.mark.parametrize("n", [16, 32, 48, 64, 96, 128, 256, 512])
def test_kept_modes_match_oracle(pkg, mo, n):
    assert pkg.kept_modes(n) == mo.kept_counts(n)


def test_supported_sizes(pkg, lib):
    assert pkg.supported_sizes() == [16, 32, 48, 64, 96, 128, 256, 512]
    assert lib.mhd_supported_n(33) == 0


def _params(pkg, **kw):
    d = dict(n=32, L=2 * math.pi, nu=1e-3, eta=1e-3, nnu=0, neta=0, dt=1e-3, scheme=0, precision=0, device=0)
    d.update(kw)
    return pkg._lib.MhdParams(**d)


@pytest.mark.parametrize("bad", [dict(n=33), dict(n=1000), dict(L=-1.0), dict(nu=-1.0), dict(nnu=2),
                                 dict(scheme=7), dict(precision=3), dict(dt=float("nan"))])
def test_create_rejects_invalid_params(pkg, lib, bad):
    h = C.c_void_p()
    rc = lib.mhd_create(C.byref(_params(pkg, **bad)), C.byref(h))
    assert rc == pkg._lib.MHD_ERR_INVALID
    assert h.value is None
    assert lib.mhd_last_error().decode()


def test_footprint(pkg, lib):
    out = C.c_longlong()
    assert lib.mhd_footprint_bytes(C.byref(_params(pkg, n=256)), C.byref(out)) == 0
    assert 1.0e9 < out.value < 2.0e9
    assert pkg.footprint_bytes(512) > 7 * pkg.footprint_bytes(256)


def test_bounded_wait_check_validates_arguments(pkg, lib):
    import ctypes as C

    t, ms = C.c_int(), C.c_double()
    assert lib.mhd_check_bounded_wait(0, 0.0, C.byref(t), C.byref(ms)) == pkg._lib.MHD_ERR_INVALID
    assert lib.mhd_check_bounded_wait(0, 2000.0, C.byref(t), C.byref(ms)) == pkg._lib.MHD_ERR_INVALID
    assert lib.mhd_check_bounded_wait(0, 5.0, None, None) == pkg._lib.MHD_ERR_INVALID


def test_native_server_host_logic(pkg, lib):
    """The C++ scheduler's validation and, with no GPU here, its rejection path: the size class of
    an admitted request cannot be allocated, so that request alone is rejected."""
    import ctypes as C

    L = pkg._lib
    p = L.MhdServerParams()
    p.budget_bytes, p.steps_per_tick, p.scheme = 0.0, 4, L.MHD_RK4
    h = C.c_void_p()
    assert lib.mhd_server_create(C.byref(p), C.byref(h)) == L.MHD_ERR_INVALID
    p.budget_bytes = 1e9
    assert lib.mhd_server_create(C.byref(p), C.byref(h)) == L.MHD_OK
    try:
        r = L.MhdRequest()
        r.n, r.L, r.nu, r.eta, r.steps = 17, 6.283, 1e-3, 1e-3, 5
        rid = C.c_longlong()
        assert lib.mhd_server_submit(h, C.byref(r), C.byref(rid)) == L.MHD_ERR_INVALID
        a, q = C.c_int(), C.c_int()
        assert lib.mhd_server_tick(h, C.byref(a), C.byref(q)) == L.MHD_OK and (a.value, q.value) == (0, 0)
        r.n = 32
        assert lib.mhd_server_submit(h, C.byref(r), C.byref(rid)) == L.MHD_OK
        st, done = C.c_int(), C.c_longlong()
        assert lib.mhd_server_poll(h, rid, C.byref(st), C.byref(done)) == L.MHD_OK and st.value == 0  # queued
        if not __import__("torch").cuda.is_available():
            assert lib.mhd_server_tick(h, C.byref(a), C.byref(q)) == L.MHD_OK
            assert lib.mhd_server_poll(h, rid, C.byref(st), C.byref(done)) == L.MHD_OK
            assert st.value == 4  # rejected: the size class could not be allocated
            assert lib.mhd_server_result(h, rid, None, None) == L.MHD_ERR_OOM
            assert b"allocation failed" in lib.mhd_last_error()
        assert lib.mhd_server_poll(h, 999, C.byref(st), C.byref(done)) == L.MHD_ERR_INVALID
    finally:
        lib.mhd_server_destroy(h)


def test_null_handle_errors(pkg, lib):
    assert lib.mhd_step(None, 1) == pkg._lib.MHD_ERR_INVALID
    assert lib.mhd_destroy(None) == 0
    assert lib.mhd_get_clock(None, None, None, None) == pkg._lib.MHD_ERR_INVALID
    assert lib.mhd_kernel_class_count() == 7
    assert lib.mhd_kernel_class_name(2).decode() == "x_fused"


def test_problem_host_validation(pkg):
    with pytest.raises(pkg.MHDError):
        pkg.Problem(pkg.CPU(), nx=32, nu=1e-3, eta=1e-3, dt=1e-3)
    with pytest.raises(pkg.MHDError):
        pkg.Problem(pkg.GPU(), nx=32, B_field=False)
    with pytest.raises(pkg.MHDError):
        pkg.Problem(pkg.GPU(), nx=32, stepper="AB3")
    with pytest.raises(pkg.MHDError):
        pkg.Problem(pkg.GPU(), nx=32, T=np.float64)
    with pytest.raises(pkg.MHDError):
        pkg.Problem(pkg.GPU(), nx=32, ny=64)
    with pytest.raises(TypeError):
        pkg.Problem(pkg.GPU(), nx=32, bogus=1)


def test_build_is_in_tree(pkg):
    from importlib import import_module

    b = import_module("mhdflows_gb300.build")
    assert b.LIB_PATH.startswith(b.PKG_DIR)
    assert "arch=compute_103a,code=sm_103a" in b.ARCH_FLAGS


def test_missing_library_fails_loudly(pkg, tmp_path):
    """No CPU fallback: pointing the loader at a library that does not exist raises."""
    saved = pkg._lib._lib
    pkg._lib._lib = None
    try:
        with pytest.raises(pkg.MHDError):
            pkg._lib.load(str(tmp_path / "libmhdgb_missing.so"))
    finally:
        pkg._lib._lib = saved


def test_product_does_not_import_oracle():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    pkgdir = os.path.join(root, "mhdflows.jl_gb300")
    for dirpath, _, files in os.walk(pkgdir):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".jl")):
                text = open(os.path.join(dirpath, f)).read()
                assert not re.search(r"^\s*(from|import)\s+oracle", text, re.M), f


def test_package_initial_conditions_match_oracle(pkg, mo):
    from importlib import import_module

    ic = import_module("mhdflows_gb300.ic")
    for n in (16, 32, 48):
        a = ic.random_spectrum_state(n, 12)
        b = mo.random_spectrum_state(mo.Grid(n, dtype=np.float32), 12)
        assert np.array_equal(a, b)
    assert ic.kept_counts(96) == mo.kept_counts(96)
    g = mo.Grid(16, dtype=np.float32)
    for x, y in zip(ic.taylor_green_fields(16), mo.taylor_green(g)):
        assert np.allclose(x, y, atol=1e-6)
