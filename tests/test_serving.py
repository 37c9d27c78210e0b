"""Serving loop host logic on the CPU: a fake backend (deterministic per-slot arithmetic, virtual
clock) exercises admission, the memory budget, continuous batching, retirement, cancellation and
the host-side failure paths (non-finite input, allocation failure, oversize request)."""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def serving(pkg):
    from importlib import import_module

    return import_module("mhdflows_gb300.serving")


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, s):
        self.t += s


class FakeBatch:
    def __init__(self, n, cap, clock):
        self.n, self.cap, self.clock = n, cap, clock
        self.states, self.params = {}, {}

    def info(self):
        return self.cap, len(self.states)

    def add(self, nu, eta, dt):
        s = next(i for i in range(self.cap) if i not in self.states)
        self.states[s] = np.zeros(4)
        self.params[s] = (nu, eta, dt)
        return s

    def remove(self, s):
        self.states.pop(s)
        self.params.pop(s)

    def set_state(self, s, x):
        self.states[s] = np.asarray(x, dtype=np.float64).ravel()[:4].copy()

    def get_state(self, s):
        return self.states[s].copy()

    def step_all(self, k):
        for s, x in self.states.items():
            nu = self.params[s][0]
            for _ in range(k):
                x *= (1.0 - nu)

    def diagnostics(self, s):
        x = self.states[s]
        if not np.all(np.isfinite(x)):
            raise FloatingPointError("detected NaN! Quit the simulation right now.")

        class D:
            def as_dict(self_):
                return {"E_u": float(np.sum(x * x))}

        return D()


class FakeBackend:
    def __init__(self, clock, slot_bytes=1.0, fail_sizes=()):
        self.clock, self.slot_b, self.fail = clock, slot_bytes, set(fail_sizes)
        self.created = []

    def class_bytes(self, n, cap):
        return self.slot_b * cap * (n / 32.0) ** 3

    def new_class(self, n, cap):
        if n in self.fail:
            raise MemoryError("simulated device allocation failure")
        b = FakeBatch(n, cap, self.clock)
        self.created.append(b)
        return b

    def initial_state(self, req):
        return np.full(4, 1.0 + req.seed % 7)

    def step(self, classes, nsteps):
        for c in classes:
            c.step_all(nsteps)
        # simulated device time: proportional to the work of the active slots
        self.clock.t += nsteps * sum(len(c.states) * c.n ** 3 for c in classes) * 1e-9


def make(serving, clock, **kw):
    return serving.Server(FakeBackend(clock, **{k: v for k, v in kw.items() if k in ("slot_bytes", "fail_sizes")}),
                          budget_bytes=kw.get("budget", 1e9), steps_per_tick=kw.get("tick", 4),
                          capacity=kw.get("capacity"), keep_states=True, clock=clock, sleep=clock.sleep)


def test_poisson_stream_is_seeded(serving):
    a = serving.poisson_requests(50, 20.0, [32, 64], [0.5, 0.5], (10, 20), (5e-4, 5e-3), seed=3)
    b = serving.poisson_requests(50, 20.0, [32, 64], [0.5, 0.5], (10, 20), (5e-4, 5e-3), seed=3)
    assert [(r.n, r.steps, r.arrival, r.seed) for r in a] == [(r.n, r.steps, r.arrival, r.seed) for r in b]
    assert all(5e-4 <= r.nu <= 5e-3 and 10 <= r.steps <= 20 for r in a)
    assert np.all(np.diff([r.arrival for r in a]) > 0)


def test_all_requests_complete_and_match_alone(serving):
    clock = FakeClock()
    reqs = serving.poisson_requests(40, 50.0, [32, 48, 64], [0.5, 0.3, 0.2], (5, 30), (1e-3, 1e-2), seed=1)
    srv = make(serving, clock, capacity={32: 4, 48: 4, 64: 2})
    rep = srv.run(reqs, realtime=True)
    assert rep["done"] == 40 and rep["failed"] == 0
    assert srv.peak_active > 1  # continuous batching: several solves in flight
    for r in reqs:
        assert r.completed_at >= r.admitted_at >= r.arrival - 1e-12
        alone = np.full(4, 1.0 + r.seed % 7)
        for _ in range(r.steps):
            alone *= (1.0 - r.nu)
        assert np.array_equal(r.final_state, alone)
    assert rep["p99_latency_s"] >= rep["p50_latency_s"] > 0


def test_late_arrivals_join_running_batch(serving):
    clock = FakeClock()
    R = serving.SolveRequest
    reqs = [R(0, 64, 1e-3, 1e-3, 400, seed=1, arrival=0.0), R(1, 64, 1e-3, 1e-3, 8, seed=2, arrival=0.01)]
    srv = make(serving, clock, capacity={64: 2}, tick=4)
    srv.run(reqs)
    assert reqs[1].admitted_at < reqs[0].completed_at  # admitted while the first one ran
    assert reqs[1].completed_at < reqs[0].completed_at


def test_budget_limits_classes_and_queues(serving):
    clock = FakeClock()
    reqs = serving.poisson_requests(30, 100.0, [32], [1.0], (20, 40), (1e-3, 1e-3), seed=2)
    # one class of capacity 2 fits the budget, a second does not: at most 2 solves at once
    srv = make(serving, clock, capacity={32: 2}, budget=2.5, slot_bytes=1.0)
    rep = srv.run(reqs)
    assert rep["done"] == 30
    assert srv.peak_active == 2 and srv.peak_reserved <= 2.5


def test_oversize_request_rejected_others_served(serving):
    clock = FakeClock()
    R = serving.SolveRequest
    reqs = [R(0, 32, 1e-3, 1e-3, 10, arrival=0.0), R(1, 512, 1e-3, 1e-3, 10, arrival=0.0),
            R(2, 32, 1e-3, 1e-3, 10, arrival=0.1)]
    srv = make(serving, clock, capacity={32: 2, 512: 1}, budget=100.0, slot_bytes=1.0)
    rep = srv.run(reqs)
    assert reqs[1].status == "rejected" and "budget" in reqs[1].error
    assert rep["done"] == 2


def test_nonfinite_input_fails_alone(serving):
    clock = FakeClock()
    R = serving.SolveRequest
    bad = np.full(4, np.nan)
    reqs = [R(0, 32, 1e-3, 1e-3, 10, arrival=0.0, init_state=bad), R(1, 32, 1e-3, 1e-3, 10, arrival=0.0)]
    rep = make(serving, clock, capacity={32: 4}).run(reqs)
    assert reqs[0].status == "failed" and "non-finite" in reqs[0].error
    assert reqs[1].status == "done" and rep["done"] == 1


def test_allocation_failure_rejects_that_size(serving):
    clock = FakeClock()
    R = serving.SolveRequest
    reqs = [R(0, 128, 1e-3, 1e-3, 10, arrival=0.0), R(1, 32, 1e-3, 1e-3, 10, arrival=0.0)]
    rep = make(serving, clock, capacity={32: 2, 128: 2}, fail_sizes=(128,)).run(reqs)
    assert reqs[0].status == "rejected" and "allocation failed" in reqs[0].error
    assert reqs[1].status == "done"


def test_cancel_frees_slot(serving):
    clock = FakeClock()
    R = serving.SolveRequest
    reqs = [R(0, 32, 1e-3, 1e-3, 1000, arrival=0.0), R(1, 32, 1e-3, 1e-3, 10, arrival=0.0),
            R(2, 32, 1e-3, 1e-3, 10, arrival=0.0)]
    srv = make(serving, clock, capacity={32: 2}, budget=3.0, slot_bytes=1.0)

    def on_tick(s, active):
        if reqs[0].status == "active" and reqs[0].steps_done >= 8:
            s.cancel(reqs[0])

    rep = srv.run(reqs, on_tick=on_tick)
    assert reqs[0].status == "cancelled"
    assert rep["done"] == 2  # the third request got the cancelled slot
