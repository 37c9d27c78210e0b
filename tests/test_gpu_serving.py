"""Serving loop on the GPU: every request's result is the same alone and in the mix."""
import copy
from importlib import import_module

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_serving_results_equal_alone(pkg):
    serving = import_module("mhdflows_gb300.serving")
    reqs = serving.poisson_requests(14, 400.0, [32, 48, 64], [0.4, 0.3, 0.3], (4, 18), (5e-4, 5e-3), seed=5)
    alone = copy.deepcopy(reqs)
    srv = serving.Server(serving.GpuBackend(pkg, "RK4"), budget_bytes=20e9, capacity={32: 3, 48: 3, 64: 2},
                         steps_per_tick=3, keep_states=True)
    rep = srv.run(reqs, realtime=False)
    assert rep["done"] == len(reqs) and rep["failed"] == 0
    assert srv.peak_active > 1
    seq = serving.run_sequential(pkg, alone, realtime=False, keep_states=True)
    assert seq["done"] == len(alone)
    for a, b in zip(reqs, alone):
        assert a.steps_done == b.steps_done == a.steps
        assert np.array_equal(a.final_state, b.final_state), a.rid
        assert a.diagnostics["E_u"] == b.diagnostics["E_u"]


def test_serving_rejects_nonfinite_on_gpu(pkg):
    serving = import_module("mhdflows_gb300.serving")
    ic = import_module("mhdflows_gb300.ic")
    bad = ic.random_spectrum_state(32, 3)
    bad[0, 1, 1, 1] = np.nan
    R = serving.SolveRequest
    reqs = [R(0, 32, 1e-3, 1e-3, 5, arrival=0.0, init_state=bad), R(1, 32, 1e-3, 1e-3, 5, seed=4, arrival=0.0)]
    srv = serving.Server(serving.GpuBackend(pkg), budget_bytes=5e9, capacity={32: 2})
    srv.run(reqs, realtime=False)
    assert reqs[0].status == "failed" and reqs[1].status == "done"
