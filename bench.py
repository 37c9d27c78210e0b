"""Benchmark: MHD RK4 step, 256^3, FP32 (plain form), on N GPUs as independent replicas.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--grid 256]

A step is one RK4 step (4 right-hand-side evaluations, 24 kernel launches) of the seeded random
k^4 exp(-2(k/4)^2) problem with nu = eta = 1e-3, dt = 5e-4.  `value` is whole-job grid-point
steps per second with the state resident in HBM; `e2e` is the same metric through the C ABI with
host buffers (state uploaded from pinned host memory, stepped once and downloaded every step).
The working set of a step (1.5 GB at 256^3) is larger than L2, so no flush is needed between steps.
Multi-GPU runs are replicas (one independent problem per rank, no collectives on the data path);
rank 0 prints one JSON line.  `--impl reference` times the CPU restatement of the reference path
(oracle/, scipy FP32, all host cores) on the same workload instead.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per RK4 MHD step at 256³/512³ & grid-pt·steps/s vs plain; p50/p99 latency"
UNIT = "grid-pt·steps/s"
NU = ETA = 1e-3
DT = 5e-4
SEED = 1
# README.md:78 of the reference: MHD RK4 256^3 on an RTX 3080, 0.271 s per step
PUBLISHED_256_S_PER_STEP = 0.271


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Host-side control plane (gloo): barrier and max over ranks; no data-path collective."""

    def __init__(self, world):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockMonitor:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9 and parts[1].replace(".", "").isdigit():
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [float(r[1]) for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][2]), "reasons": sorted(reasons),
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3].replace(".", "").isdigit()) if rows else None}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(cls_name: str, n: int, form: str = ""):
    """Per-launch DRAM bytes of a kernel class from a committed ncu summary of the same form
    (plain MHD FP32: profiles/<class>_<n>.txt; others: profiles/<class>_<n>_<form>.txt), if any."""
    path = os.path.join(ROOT, "profiles", f"{cls_name}_{n}{'_' + form if form else ''}.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def initial_state(n: int, seed: int = SEED):
    """Seeded k^4 exp(-2(k/4)^2) state from the package's initial-condition module."""
    import __graft_entry__ as ge
    from importlib import import_module

    ge.load_package()
    return import_module(ge.PKG_NAME + ".ic").random_spectrum_state(n, seed)


def run_ensemble(args):
    """Batched ensemble: 24x32^3 + 20x48^3 + 12x64^3 + 8x96^3 LSRK4 boxes stepped together (one
    CUDA graph per step, one stream per size class) against the same boxes one at a time."""
    import __graft_entry__ as ge

    pkg = ge.load_package()
    spec = [(32, 24), (48, 20), (64, 12), (96, 8)]
    rng = np.random.default_rng(2024)
    boxes, batches = [], []
    for n, count in spec:
        b = pkg.Batch(n, count, stepper="LSRK4")
        dt = 0.2 * (2 * math.pi / n)  # dt = 0.2 dx / u_rms with u_rms = 1
        for _ in range(count):
            v = float(math.exp(rng.uniform(math.log(5e-4), math.log(5e-3))))
            seed = int(rng.integers(1 << 31))
            x = initial_state(n, seed)
            slot = b.add(v, v, dt)
            b.set_state(slot, x)
            boxes.append((n, v, dt, seed, x))
        pkg.autotune(b)
        batches.append(b)
    ens = pkg.Ensemble(batches)
    K = args.steps
    ens.step(args.warmup)
    ens.synchronize()
    t0 = time.perf_counter()
    ens.step(K)
    ens.synchronize()
    el = time.perf_counter() - t0
    pts = sum(float(n) ** 3 * c for n, c in spec)
    batched = pts * K / el
    finite = all(b.diagnostics(s).nonfinite == 0 for b in batches for s in range(b.info()[0]))
    ens.close()
    for b in batches:
        b.close()
    # plain: one box at a time, each K steps (CUDA-graph steps too), same boxes and parameters
    seq_el = 0.0
    singles = {}
    for n, v, dt, seed, x in boxes:
        p = singles.get(n) or pkg.Batch(n, 1, stepper="LSRK4")
        singles[n] = p
        slot = p.add(v, v, dt)
        p.set_state(slot, x)
        p.step(args.warmup)
        p.synchronize()
        t0 = time.perf_counter()
        p.step(K)
        p.synchronize()
        seq_el += time.perf_counter() - t0
        p.remove(slot)
    for p in singles.values():
        p.close()
    seq = pts * K / seq_el
    return {"metric": "batched ensemble grid-pt·steps/s (24x32^3+20x48^3+12x64^3+8x96^3, LSRK4)",
            "value": batched, "unit": UNIT, "steps": K, "warmup": args.warmup, "higher_is_better": True,
            "ms_per_ensemble_step": el / K * 1e3, "plain_one_at_a_time": seq, "speedup_vs_plain": batched / seq,
            "boxes": len(boxes), "grid_points": pts, "finite": finite, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batched ensemble: 24x32^3 + 20x48^3 + 12x64^3 + 8x96^3 boxes, one graph per step",
                       "scheme": "LSRK4", "dt": "0.2*dx/u_rms"}}


def run_serve(args):
    """Serving loop: Poisson arrivals of independent solves, continuous batching, 150 GB budget,
    against the plain one-solve-at-a-time service of the same request stream."""
    import __graft_entry__ as ge
    from importlib import import_module

    pkg = ge.load_package()
    serving = import_module(ge.PKG_NAME + ".serving")
    lo, hi = max(1, int(100 * args.serve_scale)), max(2, int(2000 * args.serve_scale))
    mk = lambda: serving.poisson_requests(args.serve_count, 20.0, [32, 48, 64, 128, 256],  # noqa: E731
                                         [0.3, 0.25, 0.2, 0.15, 0.1], (lo, hi), (5e-4, 5e-3), seed=11)
    reqs = mk()
    # inputs are built before the clock starts, on host threads (numpy releases the GIL in the
    # array work)
    from concurrent.futures import ThreadPoolExecutor

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        for r, st in zip(reqs, ex.map(lambda q: initial_state(q.n, q.seed), reqs)):
            r.init_state = st
    srv = serving.Server(serving.GpuBackend(pkg, "RK4"), budget_bytes=150e9, steps_per_tick=8)
    rep = srv.run(reqs, realtime=True)
    nrep = None
    if getattr(args, "native", True):
        nat_reqs = mk()  # the same stream through the C++ scheduler (mhd_server_*)
        for r, q in zip(nat_reqs, reqs):
            r.init_state = q.init_state
        nat = serving.NativeServer(pkg, budget_bytes=150e9, steps_per_tick=8)
        try:
            nrep = nat.run(nat_reqs, realtime=True)
        finally:
            nat.close()
    seq_reqs = mk()
    for r, q in zip(seq_reqs, reqs):
        r.init_state = q.init_state
    seq = serving.run_sequential(pkg, seq_reqs, realtime=True)
    return {"metric": "serving grid-pt·steps/s and p50/p99 completion latency (continuous batching)",
            "value": rep["grid_pt_steps_per_s"], "unit": UNIT, "higher_is_better": True,
            "p50_latency_s": rep["p50_latency_s"], "p99_latency_s": rep["p99_latency_s"],
            "makespan_s": rep["makespan_s"], "done": rep["done"], "failed": rep["failed"],
            "peak_active": rep.get("peak_active"), "peak_reserved_gb": rep.get("peak_reserved_bytes", 0) / 1e9,
            "plain_one_at_a_time": {"grid_pt_steps_per_s": seq["grid_pt_steps_per_s"],
                                    "p50_latency_s": seq["p50_latency_s"], "p99_latency_s": seq["p99_latency_s"],
                                    "makespan_s": seq["makespan_s"]},
            "speedup_vs_plain": rep["grid_pt_steps_per_s"] / seq["grid_pt_steps_per_s"],
            "native_scheduler": None if nrep is None else {
                "grid_pt_steps_per_s": nrep["grid_pt_steps_per_s"], "p50_latency_s": nrep["p50_latency_s"],
                "p99_latency_s": nrep["p99_latency_s"], "makespan_s": nrep["makespan_s"], "done": nrep["done"],
                "peak_active": nrep.get("peak_active"), "peak_reserved_gb": nrep.get("peak_reserved_bytes", 0) / 1e9},
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "serving loop: Poisson requests for N in {32,48,64,128,256}, continuous batching",
                       "requests": args.serve_count,
                       "rate_per_s": 20.0, "steps": [lo, hi], "budget_gb": 150}}


def run_gpu(args, rank, world, local, dist: Dist):
    import __graft_entry__ as ge

    pkg = ge.load_package()
    lib = pkg._lib.load()
    n = args.n
    s0 = initial_state(n)
    prob = pkg.Problem(pkg.GPU(local), nx=n, Lx=2 * math.pi, nu=NU, eta=ETA, dt=DT, stepper=args.scheme,
                       precision=args.precision, B_field=not args.hydro, VP_method=args.vp)
    if args.hydro:
        s0 = s0[:3]
    if args.vp:  # a smoothed ball obstacle of radius L/5 at the box centre, walls at rest
        x = (np.arange(n, dtype=np.float32) - n / 2) * (2 * math.pi / n)
        r = np.sqrt(x[:, None, None] ** 2 + x[None, :, None] ** 2 + x[None, None, :] ** 2)
        prob.set_vp((0.5 * (1 - np.tanh((r - 2 * math.pi / 5) / (4 * 2 * math.pi / n)))).astype(np.float32))
    if args.forcing:  # A99 forcing with SetUpFk!'s defaults (kf = 2, sigma = 1, b = 1), small P
        pkg.SetUpFk(prob, kf=2.0, P=1e-6, sigma=1.0, b=1.0, seed=7)
    h = prob.handle
    chk = pkg._lib.check
    prob.set_sol(s0.T)
    stream = lib.mhd_get_stream(h)
    # kernel variants: the autotuner's choice for this device and size (timed once, then cached)
    variants = pkg.autotune(prob)

    # warm-up
    pkg.stepforward(prob, args.warmup)
    prob.synchronize()

    nc = lib.mhd_kernel_class_count()
    names = [lib.mhd_kernel_class_name(c).decode() for c in range(nc)]
    mon = ClockMonitor(local)
    dist.barrier()
    prob.synchronize()
    mon.start()
    # timed region: K steps back to back on the library's stream (each step one CUDA-graph
    # launch); an event between consecutive steps gives the per-step latency
    arr = (C.c_double * args.steps)()
    chk(lib.mhd_step_timed(h, args.steps, arr))
    per_step = list(arr)
    clocks = mon.stop()
    # per-kernel window: the next K steps with CUDA events around every launch (direct launches;
    # the events would perturb the timed region, so they run right after it)
    chk(lib.mhd_profile_enable(h, 1))
    prof = (C.c_double * args.steps)()
    chk(lib.mhd_step_timed(h, args.steps, prof))
    L = (C.c_longlong * nc)()
    T = (C.c_double * nc)()
    chk(lib.mhd_profile_read(h, L, T, nc))
    chk(lib.mhd_profile_enable(h, 0))
    prof_ms = sum(prof) / args.steps
    dist.barrier()
    local_ms = sum(per_step)
    max_ms = dist.max(local_ms)
    total_pts = dist.sum(float(n) ** 3 * args.steps)
    value = total_pts / (max_ms / 1e3)
    ms_per_step = max_ms / args.steps
    p50 = float(np.percentile(per_step, 50))
    p99 = float(np.percentile(per_step, 99))
    launches = int(sum(L[c] for c in range(nc)))  # the profiled window runs the same K steps

    # dominant kernel roofline
    shares = {names[c]: T[c] for c in range(nc) if L[c] > 0}
    top = max(shares, key=shares.get)
    ci = names.index(top)
    b = C.c_double()
    chk(lib.mhd_kernel_class_bytes(h, ci, C.byref(b)))
    avg_s = T[ci] / L[ci] / 1e3
    achieved = b.value / avg_s / 1e9
    peak, peak_kind = measured_peaks()
    kernels = {}
    for c in range(nc):
        if L[c] == 0:
            continue
        bb = C.c_double()
        lib.mhd_kernel_class_bytes(h, c, C.byref(bb))
        avg = T[c] / L[c] / 1e3
        kernels[names[c]] = {"launches": int(L[c]), "avg_us": round(avg * 1e6, 2),
                             "share": round(T[c] / sum(T), 4),
                             "gbs": round(bb.value / avg / 1e9, 1) if bb.value else None,
                             "frac_of_peak": round(bb.value / avg / 1e9 / peak, 3) if bb.value else None}

    # e2e through the C ABI with pinned host buffers: upload state, one step, download state
    nbytes = s0.nbytes
    pin_in = C.c_void_p()
    pin_out = C.c_void_p()
    chk(lib.mhd_host_alloc(nbytes, C.byref(pin_in)))
    chk(lib.mhd_host_alloc(nbytes, C.byref(pin_out)))
    C.memmove(pin_in, s0.ctypes.data, nbytes)
    ke = max(3, min(args.steps, 30))
    for _ in range(2):
        chk(lib.mhd_set_state(h, pin_in)); chk(lib.mhd_step(h, 1)); chk(lib.mhd_get_state(h, pin_out))
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        chk(lib.mhd_set_state(h, pin_in))
        chk(lib.mhd_step(h, 1))
        chk(lib.mhd_get_state(h, pin_out))
    el = time.perf_counter() - t0
    el_max = dist.max(el)
    e2e_value = dist.sum(float(n) ** 3 * ke) / el_max

    # the e2e step's pieces, each call timed on its own (host clock, synchronised): set_state,
    # step, get_state after an idle device, and step + get_state back to back
    def piece(f, k=5):
        f()
        chk(lib.mhd_synchronize(h))
        a = time.perf_counter()
        for _ in range(k):
            f()
        chk(lib.mhd_synchronize(h))
        return round((time.perf_counter() - a) / k * 1e3, 3)

    e2e_pieces = {
        "set_state_ms": piece(lambda: chk(lib.mhd_set_state(h, pin_in))),
        "step_ms": piece(lambda: chk(lib.mhd_step(h, 1))),
        "get_state_ms": piece(lambda: chk(lib.mhd_get_state(h, pin_out))),
        "step_then_get_state_ms": piece(lambda: (chk(lib.mhd_step(h, 1)), chk(lib.mhd_get_state(h, pin_out)))),
    }
    out_arr = np.frombuffer((C.c_char * nbytes).from_address(pin_out.value), dtype=np.complex64)
    finite = bool(np.isfinite(out_arr).all())
    chk(lib.mhd_host_free(pin_in))
    chk(lib.mhd_host_free(pin_out))

    # optional secondary size (512^3 ms per step)
    secondary = None
    if args.secondary and rank == 0:
        n2 = 512
        s2 = initial_state(n2)
        p2 = pkg.Problem(pkg.GPU(local), nx=n2, Lx=2 * math.pi, nu=5e-4, eta=5e-4, dt=2.5e-4, stepper="RK4",
                         precision=args.precision)
        p2.set_sol(s2.T)
        variants2 = pkg.autotune(p2)
        pkg.stepforward(p2, 3)
        p2.synchronize()
        ms2 = C.c_double()
        chk(lib.mhd_time_steps(p2.handle, 10, C.byref(ms2)))
        chk(lib.mhd_profile_enable(p2.handle, 1))
        prof2 = (C.c_double * 10)()
        chk(lib.mhd_step_timed(p2.handle, 10, prof2))
        L2 = (C.c_longlong * nc)()
        T2 = (C.c_double * nc)()
        chk(lib.mhd_profile_read(p2.handle, L2, T2, nc))
        chk(lib.mhd_profile_enable(p2.handle, 0))
        kernels2 = {}
        for c in range(nc):
            if L2[c] == 0:
                continue
            bb = C.c_double()
            lib.mhd_kernel_class_bytes(p2.handle, c, C.byref(bb))
            avg = T2[c] / L2[c] / 1e3
            gbs = bb.value / avg / 1e9 if bb.value else None
            kernels2[names[c]] = {"launches": int(L2[c]), "avg_us": round(avg * 1e6, 2), "share": round(T2[c] / sum(T2), 4),
                                  "gbs": round(gbs, 1) if gbs else None,
                                  "frac_of_peak": round(gbs / measured_peaks()[0], 3) if gbs else None}
        secondary = {"n": n2, "ms_per_step": round(ms2.value / 10, 3),
                     "grid_pt_steps_per_s": n2 ** 3 / (ms2.value / 10 / 1e3), "variants": variants2,
                     "kernels": kernels2, "workload": "512^3 RK4, nu = eta = 5e-4, dt = 2.5e-4, same seeded spectrum"}
        p2.close()
    forms = None
    if args.extras and rank == 0:
        forms = run_forms(args, pkg, lib, local)
    prob.close()
    return {
        "value": value, "ms_per_step": ms_per_step, "p50_ms": p50, "p99_ms": p99, "launches": launches,
        "clocks": clocks, "top": top, "achieved": achieved, "bytes": b.value, "peak": peak, "peak_kind": peak_kind,
        "kernels": kernels, "e2e": e2e_value, "e2e_bytes": nbytes, "e2e_steps": ke, "e2e_pieces": e2e_pieces, "finite": finite,
        "secondary": secondary, "prof_ms": prof_ms, "variants": variants, "forms": forms,
    }


def _cpu_steps(n, fields_or_state, nu, eta, dt, steps, warmup):
    """Whole RK4 steps of the CPU restatement of the reference path (oracle literal form: 30 r2c +
    6 c2r per right-hand side, scipy.fft float32 on every host core); per-step seconds."""
    from oracle import mhd_oracle as mo

    g = mo.Grid(n, dtype=np.float32)
    st = mo.Stepper(g, nu, eta, dt, "RK4", literal=True)
    s = np.array(fields_or_state, dtype=np.complex64, copy=True)
    for _ in range(warmup):
        st.stepforward(s)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        st.stepforward(s)
        times.append(time.perf_counter() - t0)
    return times, s


def cpu_baseline(n: int, steps: int = 2):
    """The CPU restatement of the reference path timed on this host's cores, on bounded samples:
    whole RK4 steps of the benchmark workload, and the reference's own CPU case (Taylor-Green
    32^3, nu = eta = 1e-2, dt = 1e-3, 100 RK4 steps) with per-step p50 / p99."""
    from oracle import mhd_oracle as mo

    os.environ.setdefault("MHD_ORACLE_WORKERS", str(os.cpu_count()))
    times, _ = _cpu_steps(n, initial_state(n), NU, ETA, DT, steps, 1)
    el = sum(times) / len(times)
    g32 = mo.Grid(32, dtype=np.float64)
    tg = mo.physical_to_state(g32, mo.taylor_green(g32))
    t32, _ = _cpu_steps(32, tg, 1e-2, 1e-2, 1e-3, 100, 2)
    return {"value": n ** 3 / el, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "ms_per_step": el * 1e3, "p50_ms": 1e3 * float(np.percentile(times, 50)),
            "p99_ms": 1e3 * float(np.percentile(times, 99)),
            "sample": f"{steps} whole RK4 steps (4 right-hand sides each) at {n}^3 after 1 warm-up step; oracle literal "
                      f"restatement of the reference path, scipy.fft float32, workers={os.cpu_count()}",
            "taylor_green_32": {"steps": 100, "ms_per_step": 1e3 * sum(t32) / len(t32),
                                "p50_ms": 1e3 * float(np.percentile(t32, 50)),
                                "p99_ms": 1e3 * float(np.percentile(t32, 99)),
                                "grid_pt_steps_per_s": 32 ** 3 * len(t32) / sum(t32),
                                "reference_readme_s_per_step": 0.049}}


def run_forms(args, pkg, lib, local):
    """The spec forms beside the plain FP32 step, each at 256^3 on the same workload:
    split TF32 (tcgen05) and FP16 / BF16 (mma.sync) tensor-core x rows (ms per step and relative L2 of
    the state after 20 steps against the plain form from the same state) and LSRK4 (ms per step)."""
    chk = pkg._lib.check
    n, K = 256, 20
    s0 = initial_state(n)
    out, states = {}, {}
    for name, prec, scheme in (("plain_fp32", "fp32", "RK4"), ("split_tf32", "split_tf32", "RK4"),
                               ("split_fp16", "split_fp16", "RK4"), ("split_bf16", "split_bf16", "RK4"),
                               ("lsrk4", "fp32", "LSRK4")):
        p = pkg.Problem(pkg.GPU(local), nx=n, Lx=2 * math.pi, nu=NU, eta=ETA, dt=DT, stepper=scheme, precision=prec)
        p.set_sol(s0.T)
        pkg.autotune(p)
        pkg.stepforward(p, K)  # the accuracy run from s0 (also warms up)
        if scheme == "RK4":
            states[name] = p.sol_c()
        arr = (C.c_double * K)()
        chk(lib.mhd_step_timed(p.handle, K, arr))
        ms = list(arr)
        out[name] = {"ms_per_step": sum(ms) / K, "p50_ms": float(np.percentile(ms, 50)),
                     "p99_ms": float(np.percentile(ms, 99)), "grid_pt_steps_per_s": n ** 3 / (sum(ms) / K / 1e3)}
        p.close()
    ref = states["plain_fp32"]
    den = float(np.linalg.norm(ref.ravel()))
    for name in ("split_tf32", "split_fp16", "split_bf16"):
        out[name]["rel_l2_vs_plain_after_20_steps"] = float(np.linalg.norm((states[name] - ref).ravel()) / den)
        out[name]["speedup_vs_plain"] = out["plain_fp32"]["ms_per_step"] / out[name]["ms_per_step"]
    out["lsrk4"]["note"] = "five right-hand sides per step"
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--grid", dest="n", type=int, default=256, help="grid points per axis of the step workload")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "split_tf32", "split_fp16", "split_bf16"],
                    help="x-row transforms in FP32 (plain form) or as split 16-bit tensor-core DFTs")
    ap.add_argument("--scheme", default="RK4", choices=["RK4", "LSRK4"], help="time stepper of the step workload")
    ap.add_argument("--hydro", action="store_true", help="hydrodynamic problem (B_field = false)")
    ap.add_argument("--forcing", action="store_true", help="A99 random forcing on (SetUpFk!)")
    ap.add_argument("--vp", action="store_true", help="volume penalisation on (VP_method, a ball obstacle)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", dest="secondary", action="store_false")
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="skip the split-precision / LSRK4 forms, the ensemble and the serving summary")
    ap.add_argument("--workload", default="step", choices=["step", "ensemble", "serve"])
    ap.add_argument("--serve-count", type=int, default=300)
    ap.add_argument("--serve-scale", type=float, default=0.2, help="scale of the 100..2000 steps range")
    ap.add_argument("--no-native", dest="native", action="store_false",
                    help="serving: skip the run through the C++ scheduler (mhd_server_*)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    config = {"workload": f"MHD {args.scheme} step, {args.n}^3 FP32, nu=eta=1e-3, dt=5e-4, seeded k^4 exp(-2(k/4)^2) u and B",
              "n": args.n, "scheme": args.scheme, "precision": args.precision, "hydro": args.hydro, "forcing": args.forcing, "vp": args.vp,
              "l2": "inputs larger than L2 (step working set > 1 GB)",
              "parallelism": "replicas" if args.gpus > 1 else "single"}

    if args.workload != "step" and args.impl != "reference":
        if rank == 0:
            line = run_ensemble(args) if args.workload == "ensemble" else run_serve(args)
            print(json.dumps(line), flush=True)
        return 0

    if args.impl == "reference":
        if rank != 0:
            return 0
        os.environ.setdefault("MHD_ORACLE_WORKERS", str(os.cpu_count()))
        n = args.n
        times, final = _cpu_steps(n, initial_state(n), NU, ETA, DT, args.steps, args.warmup)
        el = sum(times)
        value = n ** 3 * len(times) / el
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / len(times) * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": config,
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                 "sample": f"{args.steps} whole RK4 steps (4 right-hand sides each) at {n}^3 after "
                                           f"{args.warmup} warm-up steps; oracle literal restatement of the reference "
                                           f"path (30 r2c + 6 c2r per right-hand side), scipy.fft float32, "
                                           f"workers={os.cpu_count()}"},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "p50_ms": 1e3 * float(np.percentile(times, 50)), "p99_ms": 1e3 * float(np.percentile(times, 99)),
                "finite": bool(np.isfinite(final).all())}
        print(json.dumps(line), flush=True)
        return 0

    dist = Dist(world)
    r = run_gpu(args, rank, world, local, dist)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.n)
    if rank == 0:
        pub = args.n ** 3 / PUBLISHED_256_S_PER_STEP if args.n == 256 else None
        # the ncu summary that matches this run's kernels (forcing changes only the epilogue)
        form = "hd" if args.hydro and not args.vp else "vp" if args.vp else "" if args.precision == "fp32" else args.precision
        line = {
            "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": (r["value"] / world / pub) if pub else None,
            "dtype": "f32", "data": "synthetic (seeded random-phase solenoidal spectrum)", "config": config,
            "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"],
            "clocks": {"sm_mhz": r["clocks"]["sm_mhz"], "sm_max_mhz": r["clocks"]["sm_max_mhz"],
                       "reasons": r["clocks"]["reasons"], "samples": r["clocks"]["samples"]},
            "e2e": {"value": r["e2e"], "unit": UNIT, "h2d_bytes_per_step": r["e2e_bytes"],
                    "d2h_bytes_per_step": r["e2e_bytes"], "steps": r["e2e_steps"],
                    "path": "mhd_set_state(pinned host) + mhd_step(1) + mhd_get_state(pinned host)",
                    "pieces": r["e2e_pieces"]},
            "gpu_launches": r["launches"],
            "roofline": {"bound": "hbm", "kernel": r["top"], "achieved": r["achieved"], "peak": r["peak"],
                         "unit": "GB/s", "frac": r["achieved"] / r["peak"], "peak_kind": r["peak_kind"],
                         "traffic": ncu_traffic(r["top"], args.n, form), "algorithmic_bytes_per_launch": r["bytes"],
                         "window": "CUDA events around every launch over K steps right after the timed region",
                         "window_ms_per_step": r["prof_ms"]},
            "kernels": r["kernels"],
            "variants": r["variants"],
            "cpu_baseline": cpu,
            "baseline_note": "vs_baseline = per-GPU value / (256^3 / 0.271 s), the reference README's RTX 3080 MHD RK4 256^3 figure",
        }
        if r["secondary"]:
            line["secondary"] = r["secondary"]
        if r["forms"]:
            line["forms"] = r["forms"]
        if args.extras and world == 1:
            ens_args = argparse.Namespace(steps=200, warmup=3)
            e = run_ensemble(ens_args)
            line["ensemble"] = {k: e[k] for k in ("value", "unit", "steps", "ms_per_ensemble_step", "plain_one_at_a_time",
                                                  "speedup_vs_plain", "boxes", "finite")}
            line["ensemble"]["workload"] = e["config"]["workload"] + ", LSRK4, dt = 0.2 dx / u_rms, 200 steps"
            sv_args = argparse.Namespace(serve_count=120, serve_scale=0.25, native=False)
            sv = run_serve(sv_args)
            line["serving"] = {k: sv[k] for k in ("value", "unit", "p50_latency_s", "p99_latency_s", "makespan_s", "done",
                                                 "failed", "peak_active", "plain_one_at_a_time", "speedup_vs_plain")}
            line["serving"]["workload"] = ("Poisson requests at 20/s, N in {32,48,64,128,256}^3 with p = "
                                           "{.3,.25,.2,.15,.1}, 120 requests, steps U[25, 500] (the configuration's "
                                           "[100, 2000] scaled by 0.25, so that a backlog forms), 150 GB budget")
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
