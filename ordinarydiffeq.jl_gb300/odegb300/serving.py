"""Continuous-batching serving over the C ABI (ode_submit / ode_next_completed).

A `Server` owns one library handle with its own HBM budget and slot count.
Requests (packed ensembles of any registered model, algorithm, size and
tolerance) are submitted without waiting; the library's serving thread
starts each one on a free slot (CUDA stream) as soon as the budget allows, so
requests that arrive while others run overlap on the device.  Completions
come back in completion order with their submit / start / finish times.

`run_open_loop` drives a Server with an open-loop Poisson arrival process and
reports latency percentiles and throughput.
"""
import ctypes as C
import math
import time

import numpy as np

from . import _lib
from .ensemble import MODELS, ALG_BY_NAME, EnsembleGB300, _options
from .saveat import resolve_saveat

# precision="auto": FP32 stages down to a model's reltol floor, FP64 below it
# (FP32 stage arithmetic cannot carry tighter tolerances).  Measured on GB300
# against ground-truth solves, the mixed form stays within 2x (+1 tol) of the
# FP64 form's error at the median and p99 down to 1e-6 for Lorenz/Tsit5 and
# Robertson/Rodas5P and down to 1e-7 for the Brusselator (Rodas5P with one
# refinement sweep per solve); one decade further it does not.
MIXED_MIN_RELTOL = 1e-6
MIXED_MIN_RELTOL_BY_MODEL = {"brusselator_1d": 1e-7}

_NAMES = ("nf", "njacs", "nw", "nsolve", "naccept", "nreject")


def pick_precision(precision, reltol, model=None):
    if precision == "auto":
        floor = MIXED_MIN_RELTOL_BY_MODEL.get(model, MIXED_MIN_RELTOL)
        return "mixed" if reltol >= floor * (1 - 1e-12) else "fp64"
    return precision


class Server:
    """queue_limit > 0: submit() sheds a request (returns None) while that many
    wait, instead of queuing without bound."""

    def __init__(self, device=0, hbm_budget=0, slots=8, queue_limit=0):
        self.L = _lib.load()
        hp = C.c_void_p(0)
        _lib.check(self.L.ode_create(device, int(hbm_budget), C.byref(hp)))
        self.h = hp
        _lib.check(self.L.ode_set_serving_slots(self.h, int(slots)), self.h)
        _lib.check(self.L.ode_set_serving_queue_limit(self.h, int(queue_limit)), self.h)
        self.live = {}

    def close(self):
        if self.h:
            self.L.ode_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, model, alg, u0s, ps, tspans, saveat=None, reltol=1e-3, abstol=1e-6, precision="fp64",
               ir_sweeps=-1, tag=None, tstops=None, save_idxs=None):
        """Queue one packed ensemble; returns its ticket at once (the library
        copies the inputs, tstops included, before this returns), or None when
        the server's queue is full (the request was shed)."""
        name = model if isinstance(model, str) else None
        if isinstance(model, str):
            model = MODELS[model]
        if isinstance(alg, str):
            alg = ALG_BY_NAME[alg]
        u0s = np.ascontiguousarray(u0s, dtype=np.float64)
        ps = np.ascontiguousarray(ps, dtype=np.float64)
        tspans = np.ascontiguousarray(tspans, dtype=np.float64)
        n, N = u0s.shape
        prec = pick_precision(precision, reltol, name)
        ens = EnsembleGB300(precision=prec, ir_sweeps=ir_sweeps if prec == "mixed" else -1)
        sv = saveat if hasattr(saveat, "nsave") else resolve_saveat(saveat, tspans)
        o = _options(reltol, abstol, None, None, None, 1000000, sv, ens, None, None, tstops=tstops, alg=alg,
                     save_idxs=save_idxs)
        d = _lib.ProblemDesc(model, alg.alg_id, n, ps.shape[0], ens.prec_id(), 0)
        cap = sv.cap
        rows = n if save_idxs is None else int(np.size(save_idxs))
        out = {"t": np.empty((cap, N)), "u": np.empty((cap, rows, N)), "nsaved": np.empty(N, dtype=np.int32),
               "retcode": np.empty(N, dtype=np.int32), "stats": np.empty((N, 6), dtype=np.int64)}
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        ticket = C.c_uint64(0)
        st = self.L.ode_submit(self.h, C.byref(d), C.byref(o), N, None, dp(u0s), dp(ps), dp(tspans),
                               dp(sv.values) if sv.nsave else None, dp(out["t"]), dp(out["u"]),
                               ip(out["nsaved"]), ip(out["retcode"]),
                               out["stats"].ctypes.data_as(C.POINTER(_lib.Stats)), C.byref(ticket))
        if st == -5:   # ODE_E_BUSY: queue full
            return None
        _lib.check(st, self.h)
        self.live[ticket.value] = (out, N, tag, prec)
        return ticket.value

    def next_completed(self, timeout=0.0):
        """(ticket, status, times(submit, start, done), outputs, ntraj, tag, precision), or None."""
        t = C.c_uint64(0)
        st = C.c_int32(0)
        times = (C.c_double * 3)()
        _lib.check(self.L.ode_next_completed(self.h, float(timeout), C.byref(t), C.byref(st), times), self.h)
        if t.value == 0:
            return None
        out, N, tag, prec = self.live.pop(t.value)
        out["stats"] = {k: out["stats"][:, i] for i, k in enumerate(_NAMES)}
        return t.value, st.value, tuple(times), out, N, tag, prec

    def stats(self):
        s = _lib.ServingStats()
        _lib.check(self.L.ode_serving_stats_get(self.h, C.byref(s)), self.h)
        return {k: getattr(s, k) for k, _ in s._fields_}


def serving_mix(n_requests, seed=0, max_traj=4096):
    """Request mix of the serving workload: Lorenz (Tsit5), Robertson (Rodas5P)
    or a periodic Brusselator with 8, 16 or 32 cells (Rodas5P); 1 to max_traj
    trajectories (log-uniform); reltol log-uniform in [1e-8, 1e-4]."""
    from . import workloads as W
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n_requests):
        kind = rng.integers(0, 3)
        ntraj = int(min(max_traj, max(1, math.floor(math.exp(rng.uniform(0.0, math.log(max_traj + 1)))))))
        reltol = float(10.0 ** rng.uniform(-8.0, -4.0))
        s = int(rng.integers(0, 2 ** 31))
        if kind == 0:
            wl = W.lorenz(ntraj, seed=s)
            abstol = reltol
        elif kind == 1:
            wl = W.robertson(ntraj, seed=s)
            abstol = reltol * 1e-4
        else:
            wl = W.brusselator(ntraj, seed=s, cells=int(rng.choice([8, 16, 32])))
            abstol = reltol * 1e-3
        sv = resolve_saveat(wl["saveat"], wl["tspan"])
        reqs.append(dict(model=wl["model"], alg=wl["alg"], u0s=np.ascontiguousarray(wl["u0"]),
                         ps=np.ascontiguousarray(wl["p"]), tspans=np.ascontiguousarray(wl["tspan"]), saveat=sv,
                         reltol=reltol, abstol=abstol, ir_sweeps=wl.get("ir_sweeps", -1), ntraj=ntraj))
    return reqs


def run_open_loop(server, requests, rate, duration, seed=1, precision="auto", drain_timeout=120.0):
    """Poisson arrivals at `rate` requests/s for `duration` seconds, cycling
    through `requests`.  Latency = completion (outputs in the caller's
    buffers) minus the scheduled arrival time.  Requests the server sheds
    (queue full) are counted, not retried; `launches` counts the kernel
    launches the server made for this run."""
    rng = np.random.default_rng(seed)
    clock = lambda: time.clock_gettime(time.CLOCK_MONOTONIC)
    launches0 = server.stats()["launches"]
    t0 = clock() + 0.01
    end = t0 + duration
    nxt = t0 + rng.exponential(1.0 / rate)
    arrival = {}
    lat, wait, ntraj_done, failures, shed = [], [], 0, 0, 0
    first_done, last_done = None, None
    i = 0
    submitted = 0

    def collect(timeout):
        nonlocal ntraj_done, failures, first_done, last_done
        got = server.next_completed(timeout)
        while got is not None:
            ticket, status, times, out, N, tag, prec = got
            if status != 0:
                failures += 1
            else:
                lat.append(times[2] - arrival.pop(ticket))
                wait.append(times[1] - times[0])
                ntraj_done += N
                last_done = times[2] if last_done is None else max(last_done, times[2])
                first_done = times[2] if first_done is None else min(first_done, times[2])
            got = server.next_completed(0.0)

    while True:
        now = clock()
        if now >= end:
            break
        while nxt <= now and nxt < end:
            r = requests[i % len(requests)]
            i += 1
            tk = server.submit(r["model"], r["alg"], r["u0s"], r["ps"], r["tspans"], r["saveat"], r["reltol"],
                               r["abstol"], precision=precision, ir_sweeps=r["ir_sweeps"])
            if tk is None:
                shed += 1
            else:
                arrival[tk] = nxt
                submitted += 1
            nxt += rng.exponential(1.0 / rate)
        collect(max(0.0, min(nxt, end) - clock()))
    deadline = clock() + drain_timeout
    while arrival and clock() < deadline:
        collect(0.05)
    lat = np.array(lat)
    wait = np.array(wait)
    span = (last_done - t0) if last_done is not None else float("nan")
    pct = lambda a, q: float(np.percentile(a, q) * 1e3) if len(a) else None
    st = server.stats()
    return {"offered_rate": rate, "duration_s": duration, "submitted": submitted, "completed": int(len(lat)),
            "failed": failures, "unfinished": len(arrival), "shed_queue_full": shed,
            "launches": st["launches"] - launches0,
            "requests_per_s": len(lat) / span if span == span and span > 0 else None,
            "trajectories_per_s": ntraj_done / span if span == span and span > 0 else None,
            "latency_ms": {"p50": pct(lat, 50), "p90": pct(lat, 90), "p99": pct(lat, 99), "max": pct(lat, 100)},
            "queue_wait_ms": {"p50": pct(wait, 50), "p99": pct(wait, 99)}}
