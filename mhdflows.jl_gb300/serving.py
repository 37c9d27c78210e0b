"""Continuous-batching serving loop for independent MHD solves (no counterpart in the reference,
which runs one problem per Julia process).

Requests (n, nu, eta, steps, seed, arrival time) arrive over time.  The server keeps every
admitted solve's state resident in HBM in a size class (a Batch: slots of one grid size), admits
a request when its size class has a free slot or a new class fits in the memory budget (the
budget is charged with the measured device bytes of each class), and advances all active solves
together: one CUDA graph per tick steps every non-empty class, each on its own stream.  Requests
that arrive while others run join at the next tick; finished ones free their slot at once.
Results do not depend on what else is in the batch (no reduction crosses slots).

Host-side failure handling: a request whose state turns non-finite is reported as failed and its
slot is freed; a request that can never fit the budget is rejected; a size class whose creation
fails (device allocation) rejects the requests that needed it; cancel() removes a request.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class SolveRequest:
    rid: int
    n: int
    nu: float
    eta: float
    steps: int
    seed: int = 0
    arrival: float = 0.0          # seconds after the start of the run
    dt: float | None = None       # default 0.2 * dx / u_rms with u_rms = 1
    init_state: np.ndarray | None = None  # (6, n, n, n/2+1) complex64; built from seed if None
    # results
    status: str = "queued"        # queued, active, done, failed, rejected, cancelled
    error: str = ""
    admitted_at: float = math.nan
    completed_at: float = math.nan
    steps_done: int = 0
    diagnostics: dict = field(default_factory=dict)
    final_state: np.ndarray | None = None

    @property
    def latency(self):
        return self.completed_at - self.arrival

    @property
    def work(self):
        return float(self.n) ** 3 * self.steps


def poisson_requests(count: int, rate: float, sizes, probs, steps_range, visc_range, seed: int = 0):
    """Seeded request stream: exponential inter-arrival times, N from `sizes` with `probs`,
    steps uniform in steps_range, nu = eta log-uniform in visc_range."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += rng.exponential(1.0 / rate)
        n = int(rng.choice(sizes, p=probs))
        steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
        v = float(math.exp(rng.uniform(math.log(visc_range[0]), math.log(visc_range[1]))))
        out.append(SolveRequest(rid=i, n=n, nu=v, eta=v, steps=steps, seed=int(rng.integers(1 << 31)), arrival=t))
    return out


class GpuBackend:
    """Size classes on the GPU through the C ABI."""

    def __init__(self, pkg, stepper="RK4", device=0):
        self.pkg = pkg
        self.stepper = stepper
        self.device = device
        self._ens = {}

    def class_bytes(self, n, capacity):
        per_slot, per_class = self.pkg.slot_bytes(n)
        return per_class + capacity * per_slot

    def new_class(self, n, capacity):
        return self.pkg.Batch(n, capacity, stepper=self.stepper, device=self.device)

    def initial_state(self, req):
        from . import ic

        return ic.random_spectrum_state(req.n, req.seed)

    def step(self, classes, nsteps):
        key = tuple(id(c) for c in classes)
        ens = self._ens.get(key)
        if ens is None:
            ens = self.pkg.Ensemble(classes)
            self._ens[key] = ens
        ens.step(nsteps)
        for c in classes:
            c.synchronize()

    def forget(self, cls):
        for key in [k for k in self._ens if id(cls) in k]:
            self._ens.pop(key).close()


class Server:
    """Admission, continuous batching and accounting over a backend of size classes."""

    DEFAULT_CAPACITY = {16: 32, 32: 32, 48: 24, 64: 16, 96: 8, 128: 8, 256: 4, 512: 1}

    def __init__(self, backend, budget_bytes=150e9, capacity=None, steps_per_tick=8, keep_states=False,
                 clock=None, sleep=None):
        self.backend = backend
        self.budget = float(budget_bytes)
        self.capacity = dict(self.DEFAULT_CAPACITY)
        if capacity:
            self.capacity.update(capacity)
        self.steps_per_tick = int(steps_per_tick)
        self.keep_states = keep_states
        self.clock = clock or time.perf_counter
        self.sleep = sleep or time.sleep
        self.classes = {}      # n -> list of (batch, reserved bytes)
        self.slots = {}        # rid -> (batch, slot)
        self.reserved = 0.0
        self.peak_reserved = 0.0
        self.peak_active = 0
        self.ticks = 0

    # -- capacity management
    def _free_slot_class(self, n):
        for b, _ in self.classes.get(n, []):
            cap, act = b.info()
            if act < cap:
                return b
        return None

    def _admit(self, req, now):
        b = self._free_slot_class(req.n)
        if b is None:
            cap = self.capacity.get(req.n, 1)
            need = self.backend.class_bytes(req.n, cap)
            if self.reserved + need > self.budget:
                if not self.classes.get(req.n) and self.backend.class_bytes(req.n, 1) > self.budget:
                    req.status, req.error = "rejected", "request does not fit the memory budget"
                return False
            try:
                b = self.backend.new_class(req.n, cap)
            except Exception as e:  # device allocation failure: reject what needed this class
                req.status, req.error = "rejected", f"size class allocation failed: {e}"
                return False
            self.classes.setdefault(req.n, []).append((b, need))
            self.reserved += need
            self.peak_reserved = max(self.peak_reserved, self.reserved)
        dt = req.dt if req.dt is not None else 0.2 * (2 * math.pi / req.n)
        slot = b.add(req.nu, req.eta, dt)
        state = req.init_state if req.init_state is not None else self.backend.initial_state(req)
        if not np.all(np.isfinite(state)):
            b.remove(slot)
            req.status, req.error = "failed", "non-finite initial state"
            req.completed_at = now
            return True
        b.set_state(slot, state)
        self.slots[req.rid] = (b, slot)
        req.status = "active"
        req.admitted_at = now
        return True

    def _retire(self, req, now, status="done", error=""):
        b, slot = self.slots.pop(req.rid)
        try:
            d = b.diagnostics(slot)
            req.diagnostics = d.as_dict()
            if self.keep_states:
                req.final_state = b.get_state(slot)
        except Exception as e:  # non-finite state or device error
            status, error = "failed", str(e)
        b.remove(slot)
        req.status, req.error = status, error
        req.completed_at = now

    def cancel(self, req, now=None):
        if req.rid in self.slots:
            b, slot = self.slots.pop(req.rid)
            b.remove(slot)
        req.status = "cancelled"
        req.completed_at = self.clock() if now is None else now

    # -- main loop
    def run(self, requests, realtime=True, on_tick=None):
        reqs = sorted(requests, key=lambda r: r.arrival)
        pending, active = [], []
        i = 0
        t0 = self.clock()
        now = lambda: self.clock() - t0  # noqa: E731
        while i < len(reqs) or pending or active:
            t = now()
            while i < len(reqs) and reqs[i].arrival <= t:
                pending.append(reqs[i])
                i += 1
            still = []
            for r in pending:  # first fit in arrival order
                if r.status == "queued" and self._admit(r, now()):
                    if r.status == "active":
                        active.append(r)
                elif r.status == "queued":
                    still.append(r)
            pending = [r for r in still if r.status == "queued"]
            if not active:
                if pending and i >= len(reqs):
                    for r in pending:  # nothing running and nothing fits: cannot ever run
                        r.status, r.error = "rejected", "request does not fit the memory budget"
                    pending = []
                    continue
                if i < len(reqs):
                    wait = reqs[i].arrival - now()
                    if wait > 0:
                        if realtime:
                            self.sleep(wait)
                        else:
                            t0 -= wait  # virtual clock: jump to the next arrival
                continue
            self.peak_active = max(self.peak_active, len(active))
            nsteps = min(self.steps_per_tick, min(r.steps - r.steps_done for r in active))
            classes = []
            for r in active:
                b = self.slots[r.rid][0]
                if all(b is not c for c in classes):
                    classes.append(b)
            self.backend.step(classes, nsteps)
            self.ticks += 1
            if on_tick:
                on_tick(self, active)
            t = now()
            keep = []
            for r in active:
                if r.status != "active":
                    continue
                r.steps_done += nsteps
                if r.steps_done >= r.steps:
                    self._retire(r, t)
                else:
                    keep.append(r)
            active = keep
        return report(requests, self)


def report(requests, server=None):
    done = [r for r in requests if r.status == "done"]
    lat = np.array([r.latency for r in done]) if done else np.array([np.nan])
    work = sum(r.work for r in done)
    start = min((r.arrival for r in requests), default=0.0)
    end = max((r.completed_at for r in done), default=0.0)
    span = end - min(start, 0.0) if done else float("nan")
    out = {
        "requests": len(requests),
        "done": len(done),
        "failed": sum(r.status == "failed" for r in requests),
        "rejected": sum(r.status == "rejected" for r in requests),
        "cancelled": sum(r.status == "cancelled" for r in requests),
        "p50_latency_s": float(np.percentile(lat, 50)),
        "p99_latency_s": float(np.percentile(lat, 99)),
        "mean_latency_s": float(np.mean(lat)),
        "makespan_s": float(span),
        "grid_pt_steps": work,
        "grid_pt_steps_per_s": work / span if span and span > 0 else float("nan"),
    }
    if server is not None:
        out.update({"peak_reserved_bytes": server.peak_reserved, "peak_active": server.peak_active,
                    "ticks": server.ticks})
    return out


def run_sequential(pkg, requests, stepper="RK4", device=0, realtime=True, clock=None, sleep=None, keep_states=False):
    """Plain one-solve-at-a-time service of the same requests (FIFO, one problem on the GPU)."""
    from . import ic

    clock = clock or time.perf_counter
    sleep = sleep or time.sleep
    probs = {}
    t0 = clock()
    for r in sorted(requests, key=lambda q: q.arrival):
        t = clock() - t0
        if t < r.arrival:
            if realtime:
                sleep(r.arrival - t)
            else:
                t0 -= r.arrival - t
        p = probs.get(r.n)
        if p is None:
            p = pkg.Batch(r.n, 1, stepper=stepper, device=device)
            probs[r.n] = p
        dt = r.dt if r.dt is not None else 0.2 * (2 * math.pi / r.n)
        slot = p.add(r.nu, r.eta, dt)
        p.set_state(slot, r.init_state if r.init_state is not None else ic.random_spectrum_state(r.n, r.seed))
        r.admitted_at = clock() - t0
        p.step(r.steps)
        p.synchronize()
        r.steps_done = r.steps
        try:
            r.diagnostics = p.diagnostics(slot).as_dict()
            if keep_states:
                r.final_state = p.get_state(slot)
            r.status = "done"
        except Exception as e:
            r.status, r.error = "failed", str(e)
        p.remove(slot)
        r.completed_at = clock() - t0
    for p in probs.values():
        p.close()
    return report(requests)


_NATIVE_STATUS = ("queued", "active", "done", "failed", "rejected", "cancelled")
_SIZES = (16, 32, 48, 64, 96, 128, 256, 512)


class NativeServer:
    """The library's own continuous-batching scheduler (mhd_server_* of the C ABI): the same
    policy as Server (first-fit admission in arrival order under a device-memory budget, size
    classes stepped together, min(steps_per_tick, smallest remaining) steps per tick), with the
    scheduling loop in C++.  ``submit`` copies the request; ``tick`` runs one round."""

    def __init__(self, pkg, budget_bytes=150e9, steps_per_tick=8, stepper="RK4", device=0, keep_states=False,
                 capacity=None):
        from . import _lib

        self._L = _lib
        self.lib = _lib.load()
        p = _lib.MhdServerParams()
        p.budget_bytes = float(budget_bytes)
        p.steps_per_tick = int(steps_per_tick)
        p.scheme = _lib.MHD_RK4 if str(stepper).upper() == "RK4" else _lib.MHD_LSRK4
        p.device = int(device)
        p.keep_states = int(bool(keep_states))
        for i, n in enumerate(_SIZES):
            p.capacity[i] = int((capacity or {}).get(n, 0))
        h = C.c_void_p()
        _lib.check(self.lib.mhd_server_create(C.byref(p), C.byref(h)))
        self._h = h
        self.keep_states = bool(keep_states)
        self.ticks = 0
        self.peak_active = 0

    def close(self):
        if getattr(self, "_h", None):
            self.lib.mhd_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, n, nu, eta, steps, sol=None, dt=None, L=2 * math.pi):
        """Queue a solve; sol is the (6, n, n, n/2+1) complex64 initial state (None: zero)."""
        r = self._L.MhdRequest()
        r.n, r.L, r.nu, r.eta = int(n), float(L), float(nu), float(eta)
        r.dt = 0.0 if dt is None else float(dt)
        r.steps = int(steps)
        buf = None
        if sol is not None:
            buf = np.ascontiguousarray(sol, dtype=np.complex64)
            if buf.shape != (6, n, n, n // 2 + 1):
                raise ValueError("sol must be (6, n, n, n/2+1)")
            r.sol = buf.ctypes.data
        rid = C.c_longlong()
        self._L.check(self.lib.mhd_server_submit(self._h, C.byref(r), C.byref(rid)))
        return rid.value

    def tick(self):
        a, q = C.c_int(), C.c_int()
        self._L.check(self.lib.mhd_server_tick(self._h, C.byref(a), C.byref(q)))
        self.ticks += 1
        self.peak_active = max(self.peak_active, a.value)
        return a.value, q.value

    def poll(self, rid):
        st, done = C.c_int(), C.c_longlong()
        self._L.check(self.lib.mhd_server_poll(self._h, int(rid), C.byref(st), C.byref(done)))
        return _NATIVE_STATUS[st.value], done.value

    def result(self, rid, n=None):
        """(diagnostics dict, final state or None) of a done request; raises MHDError otherwise."""
        d = (C.c_double * 8)()
        out = None
        if self.keep_states and n is not None:
            out = np.empty((6, n, n, n // 2 + 1), dtype=np.complex64)
        self._L.check(self.lib.mhd_server_result(self._h, int(rid), d, None if out is None else out.ctypes.data))
        keys = ("E_u", "E_B", "H_c", "max_kdotu", "max_kdotb", "max_divb", "nonfinite", "t")
        return dict(zip(keys, list(d))), out

    def cancel(self, rid):
        self._L.check(self.lib.mhd_server_cancel(self._h, int(rid)))

    def memory(self):
        r, p = C.c_double(), C.c_double()
        self._L.check(self.lib.mhd_server_memory(self._h, C.byref(r), C.byref(p)))
        return r.value, p.value

    def run(self, requests, realtime=True, clock=None, sleep=None):
        """Serve SolveRequest objects arriving at their `arrival` times (seconds from the start);
        fills each request's status, latency, diagnostics (and final state with keep_states).
        realtime=False jumps a virtual clock to the next arrival when nothing runs."""
        from . import ic

        clock = clock or time.perf_counter
        sleep = sleep or time.sleep
        reqs = sorted(requests, key=lambda r: r.arrival)
        ids = {}
        i = 0
        t0 = clock()
        now = lambda: clock() - t0  # noqa: E731
        live = []
        while i < len(reqs) or live:
            t = now()
            while i < len(reqs) and reqs[i].arrival <= t:
                r = reqs[i]
                st = r.init_state if r.init_state is not None else ic.random_spectrum_state(r.n, r.seed)
                ids[r.rid] = self.submit(r.n, r.nu, r.eta, r.steps, st, r.dt)
                live.append(r)
                i += 1
            if not live:
                wait = reqs[i].arrival - now()
                if wait > 0:
                    if realtime:
                        sleep(wait)
                    else:
                        t0 -= wait
                continue
            active, queued = self.tick()
            t = now()
            keep = []
            for r in live:
                status, done = self.poll(ids[r.rid])
                r.steps_done = done
                if status == "active" and math.isnan(r.admitted_at):
                    r.admitted_at = t
                if status in ("queued", "active"):
                    keep.append(r)
                    continue
                r.status = status
                r.completed_at = t
                if status == "done":
                    r.diagnostics, r.final_state = self.result(ids[r.rid], r.n)
                else:
                    try:
                        self.result(ids[r.rid])
                    except Exception as e:  # the request's failure message
                        r.error = str(e)
            live = keep
            if active == 0 and queued:
                if i >= len(reqs):
                    for r in live:  # nothing runs and nothing fits: cannot ever run
                        self.cancel(ids[r.rid])
                        r.status, r.error = "rejected", "request does not fit the memory budget"
                    live = []
                else:  # nothing fits until later arrivals change the mix: wait for the next one
                    wait = reqs[i].arrival - now()
                    if wait > 0:
                        if realtime:
                            sleep(wait)
                        else:
                            t0 -= wait
        out = report(requests)
        out.update({"peak_reserved_bytes": self.memory()[1], "peak_active": self.peak_active, "ticks": self.ticks})
        return out
