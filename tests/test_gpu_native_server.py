"""The C++ serving scheduler (mhd_server_*, serving.NativeServer): every request's result equals
the same solve alone, bit for bit; failures, rejections and cancellations stay with their request."""
import copy
from importlib import import_module

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _serving():
    return import_module("mhdflows_gb300.serving")


def test_native_server_results_equal_alone(pkg):
    serving = _serving()
    reqs = serving.poisson_requests(14, 400.0, [32, 48, 64], [0.4, 0.3, 0.3], (4, 18), (5e-4, 5e-3), seed=7)
    alone = copy.deepcopy(reqs)
    srv = serving.NativeServer(pkg, budget_bytes=20e9, steps_per_tick=3, keep_states=True,
                               capacity={32: 3, 48: 3, 64: 2})
    try:
        rep = srv.run(reqs, realtime=False)
        reserved, peak = srv.memory()
    finally:
        srv.close()
    assert rep["done"] == len(reqs) and rep["failed"] == 0
    assert rep["peak_active"] > 1
    assert 0 < peak <= 20e9
    seq = serving.run_sequential(pkg, alone, realtime=False, keep_states=True)
    assert seq["done"] == len(alone)
    for a, b in zip(reqs, alone):
        assert a.steps_done == b.steps_done == a.steps
        assert np.array_equal(a.final_state, b.final_state), a.rid
        assert a.diagnostics["E_u"] == b.diagnostics["E_u"]


def test_native_server_failures_stay_with_their_request(pkg):
    serving = _serving()
    ic = import_module("mhdflows_gb300.ic")
    bad = ic.random_spectrum_state(32, 3)
    bad[0, 1, 1, 1] = np.nan
    srv = serving.NativeServer(pkg, budget_bytes=2e9, steps_per_tick=4, capacity={32: 4})
    try:
        r_bad = srv.submit(32, 1e-3, 1e-3, 5, bad)
        r_big = srv.submit(512, 1e-3, 1e-3, 5)           # a 512^3 class can never fit 2 GB
        r_ok = srv.submit(32, 1e-3, 1e-3, 5, ic.random_spectrum_state(32, 4))
        r_cancel = srv.submit(32, 1e-3, 1e-3, 40, ic.random_spectrum_state(32, 5))
        srv.tick()
        assert srv.poll(r_bad)[0] == "failed"
        assert srv.poll(r_big)[0] == "rejected"
        assert srv.poll(r_cancel)[0] == "active"
        srv.cancel(r_cancel)
        assert srv.poll(r_cancel)[0] == "cancelled"
        while srv.tick() != (0, 0):
            pass
        assert srv.poll(r_ok) == ("done", 5)
        d, _ = srv.result(r_ok)
        assert d["nonfinite"] == 0 and d["E_u"] > 0
        with pytest.raises(pkg.MHDError):
            srv.result(r_bad)
        with pytest.raises(pkg.MHDError):
            srv.result(r_big)
    finally:
        srv.close()
