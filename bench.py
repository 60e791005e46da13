#!/usr/bin/env python3
"""Benchmark of the GB300 ensemble ODE integrator (libode_b200.so).

Headline workload (one "step" = one full ensemble solve): 100,000 Robertson
trajectories, Rodas5P with the analytic Jacobian, reltol 1e-6, abstol 1e-10,
tspan (0, 1e5), 20 log-spaced saves; rate constants log-uniform-scaled per
trajectory (seeded synthetic inputs; no dataset exists for this path).

Both GPU forms run: plain FP64 and mixed precision (and, for the headline, the
mixed form with one refinement sweep per W solve).  `value` is the
trajectories/s of the mixed form when it is as accurate as the FP64 form
(its error against a ground-truth solve within 2x the FP64 form's, +1
tolerance unit, at the median and p99; checked on the whole ensemble where the
oracle allows), else of the FP64 form; inputs resident in HBM.  `e2e` is the
same metric through the public host-buffer call.  `configs` holds the same
block for 10k Lorenz/Tsit5, 1M uneven Duffing chains/Vern7 and 65,536
Brusselators/Rodas5P; `serving` the open-loop request stream.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--config robertson|lorenz|duffing|brusselator|robertson_ros23|lorenz_dense|
                              bouncing_ball|van_der_pol|pk_dosing|serving]
                    [--trajectories N] [--no-suite] [--no-serving]
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ordinarydiffeq.jl_gb300"))

CONFIGS = {
    "robertson": ("Robertson kinetics, Rodas5P + analytic J, reltol 1e-6 abstol 1e-10, tspan (0,1e5), "
                  "20 log-spaced saves", 100_000),
    "lorenz": ("Lorenz, Tsit5, reltol=abstol=1e-8, tspan (0,1), saveat 0.1", 10_000),
    "duffing": ("uneven Duffing chains N in {2,4,8,16,32}, Vern7, reltol 1e-6, 16 saves, tf log-uniform [1,100]",
                1_000_000),
    "brusselator": ("Brusselator-1D 32 cells (64 states), Rodas5P, reltol 1e-5 abstol 1e-8, tspan (0,10)",
                    65_536),
    "robertson_ros23": ("Robertson kinetics, Rosenbrock23 + analytic J, reltol 1e-4 abstol 1e-8, tspan (0,1e5), "
                        "20 log-spaced saves", 100_000),
    "lorenz_dense": ("Lorenz, Tsit5, reltol=abstol=1e-8, tspan (0,1), dense output (every step with its "
                     "interpolation vectors), then sol(t) at 101 times for every trajectory", 10_000),
    "van_der_pol": ("van der Pol oscillators, mu log-uniform in [1, 1000], AutoTsit5(Rosenbrock23()) (stiffness "
                    "switching), reltol=abstol=1e-6, tspan (0,6), saveat 0.5", 100_000),
    "bouncing_ball": ("bouncing balls with the model's ContinuousCallback (condition x, affect_neg! v <- -e v, "
                      "half terminate! after t_stop), Tsit5, reltol=abstol=1e-6, tspan (0,10), saveat 0.25",
                      1_000_000),
    "pk_dosing": ("population PK: one-compartment model with first-order absorption, ka/ke log-normal, "
                  "100 mg every 12 h for a week by the model's DiscreteCallback (t in tstops), Tsit5, "
                  "reltol 1e-6 abstol 1e-8, tspan (0,168), hourly saves", 1_000_000),
    "serving": ("open-loop Poisson request stream; each request 1-4096 trajectories (log-uniform) of Lorenz/Tsit5, "
                "Robertson/Rodas5P or Brusselator-1D (8/16/32 cells)/Rodas5P, reltol 10^U(-8,-4)", 0),
}
SERVE_HBM_BUDGET = 8 << 30
SERVE_QUEUE_LIMIT = 2048      # requests waiting before the server sheds new ones
SERVE_RATES = "100,300,1000,3000,10000"
SERVE_SECONDS = 10.0          # arrival window per rate (the workload names 60 s)


def serving_block(args, local, rates, seconds):
    """Continuous-batching serving under open-loop Poisson arrivals (one Server,
    fixed HBM budget, precision chosen per request from its reltol)."""
    from odegb300.serving import MIXED_MIN_RELTOL, MIXED_MIN_RELTOL_BY_MODEL, Server, run_open_loop, serving_mix
    reqs = serving_mix(2000, seed=3)
    out = []
    with Server(device=local, hbm_budget=SERVE_HBM_BUDGET, slots=args.serve_slots,
                queue_limit=SERVE_QUEUE_LIMIT) as srv:
        run_open_loop(srv, reqs[-40:], rate=200.0, duration=0.2, drain_timeout=30.0)   # module load, pools
        for r in rates:
            out.append(run_open_loop(srv, reqs, rate=r, duration=seconds, drain_timeout=max(15.0, 3 * seconds)))
        st = srv.stats()
    return {"workload": CONFIGS["serving"][0], "hbm_budget_bytes": SERVE_HBM_BUDGET, "slots": args.serve_slots,
            "queue_limit": SERVE_QUEUE_LIMIT, "seconds_per_rate": seconds,
            "batching": "queued requests with the same model, method, precision, options and saveat are merged "
                        "into one launch, each trajectory keeping its own request's tolerances",
            "precision": "mixed when reltol >= %g (%s), else fp64" % (
                MIXED_MIN_RELTOL, ", ".join("%s: %g" % kv for kv in MIXED_MIN_RELTOL_BY_MODEL.items())),
            "latency": "completion (outputs in the caller's host buffers) minus scheduled arrival",
            "rates": out, "rejected_total": st["rejected"]}


def run_serving(args, rank, local):
    if rank != 0:
        return
    import torch
    torch.cuda.set_device(local)
    rates = [float(x) for x in (args.serve_rates or SERVE_RATES).split(",")]
    blk = serving_block(args, local, rates, args.serve_seconds or SERVE_SECONDS)
    best = max(blk["rates"], key=lambda m: m["trajectories_per_s"] or 0.0)
    reqs = sum(m["completed"] for m in blk["rates"])
    print(json.dumps({
        "metric": METRIC,
        "value": best["trajectories_per_s"], "unit": "trajectories/s", "n_gpus": 1, "steps": len(rates),
        "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 / f32 stages per request", "data": "synthetic (seeded request mix)",
        "config": {"workload": CONFIGS["serving"][0], "rates_req_per_s": rates,
                   "seconds_per_rate": args.serve_seconds or SERVE_SECONDS},
        "serving": blk,
        "e2e": {"value": best["trajectories_per_s"], "unit": "trajectories/s", "note": "host buffers in and out",
                "h2d_bytes_per_step": None, "d2h_bytes_per_step": None},
        "gpu_launches": None, "requests_completed": reqs}))


# DRAM bytes (read + write) per launch of the integrator kernel, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the same kernel on
# the full 100,000-trajectory Robertson ensemble.  Filled in only for kernels
# captured at the benchmarked size; every other kernel reports null.
NCU_TRAFFIC = {("robertson", "fp64"): 18.22e6, ("robertson", "mixed"): 17.04e6}
METRIC = "trajectories/sec at equal accuracy, mixed vs plain FP64 GPU; p50/p99 latency"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="robertson", choices=sorted(CONFIGS))
    ap.add_argument("--trajectories", type=int, default=0)
    ap.add_argument("--lanes", type=int, default=0, help="lanes per trajectory of the device solves (0: default)")
    ap.add_argument("--scheduler", default="auto", choices=["auto", "static", "persistent"],
                    help="scheduler of the device solves")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="target CPU-baseline sample time")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-small", action="store_true",
                    help="one small FP64+mixed solve pair for ncu captures (no JSON line)")
    ap.add_argument("--serve-rates", default="",
                    help="comma-separated Poisson request rates (req/s) of the serving measurement")
    ap.add_argument("--serve-seconds", type=float, default=0.0, help="arrival window per rate")
    ap.add_argument("--serve-slots", type=int, default=32, help="concurrent device slots of the server")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving measurement")
    ap.add_argument("--no-suite", action="store_true",
                    help="headline configuration only (by default the Lorenz, uneven Duffing and Brusselator "
                         "configurations are measured beside it)")
    return ap.parse_args()


def dist_setup(args, backend=None, timeout_s=300.0):
    """One process per GPU (torchrun environment).  Replicas only: the ranks
    meet at barriers and in one max-reduction of their times; a rank that dies
    makes the others' next collective fail within timeout_s instead of hanging."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import datetime
        import torch.distributed as dist
        if backend is None:
            backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend, timeout=datetime.timedelta(seconds=timeout_s))
    return world, rank, local, dist


def max_over_ranks(x, dist, device="cpu"):
    """The job's time is its slowest replica's: max of x over the ranks."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world, n_per_rank, seconds):
    """Whole-job throughput: every rank integrates n_per_rank trajectories."""
    return world * n_per_rank / seconds


def workload(name, N, seed):
    from odegb300 import workloads as W
    if name == "robertson_ros23":
        return W.robertson(N, seed=seed, alg="rosenbrock23", reltol=1e-4, abstol=1e-8)
    if name == "lorenz_dense":   # no saveat: every step kept (the reference's dense default)
        return dict(W.lorenz(N, seed=seed), saveat=None, everystep=True, max_step_saves=DENSE_MAX_STEPS)
    return {"robertson": W.robertson, "lorenz": W.lorenz, "duffing": W.duffing,
            "brusselator": W.brusselator, "bouncing_ball": W.bouncing_ball,
            "van_der_pol": W.van_der_pol, "pk_dosing": W.pk_dosing}[name](N, seed=seed)


DENSE_MAX_STEPS = 512   # step slots per trajectory of the dense workload (Lorenz at 1e-8 takes < 200)


def oracle_solve(wl, idx, nthreads=0, truth=False):
    """CPU oracle (test infrastructure) on the trajectories `idx` of workload wl; with
    truth=True a ground-truth solve (Vern9 at 1e-14, or Rodas5P at reltol 1e-12 for the
    stiff Rodas5P workloads) that stops exactly at every save."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    from odegb300.saveat import resolve_saveat
    alg = {"tsit5": O.TSIT5, "vern7": O.VERN7, "rodas5p": O.RODAS5P, "rosenbrock23": O.ROSENBROCK23,
           "autotsit5_rosenbrock23": O.AUTOTSIT5_ROSENBROCK23}[wl["alg"]]
    model = {"lorenz": O.LORENZ, "robertson": O.ROBERTSON, "duffing_chain": O.DUFFING,
             "brusselator_1d": O.BRUSSELATOR, "bouncing_ball": O.BOUNCING_BALL, "van_der_pol": O.VANDERPOL,
             "pk_one_compartment": O.PK1}[wl["model"]]
    cb = wl.get("callback")
    cbkw = dict(callback=True, interp_points=cb.interp_points, max_events=cb.max_events) if cb else {}
    if wl.get("tstops") is not None:
        cbkw["tstops"] = wl["tstops"]
    ts = wl["tspan"][:, idx]
    sv = wl["saveat"]
    if isinstance(sv, np.ndarray) and sv.ndim == 2:
        sv = sv[:, idx]
    every = bool(wl.get("everystep")) and not truth
    spec = resolve_saveat(sv, ts, save_everystep=every, max_step_saves=wl.get("max_step_saves", 1024))
    npt = wl.get("n_per_traj")
    rt, at = wl["reltol"], wl["abstol"]
    if truth:
        stiff = wl["alg"] in ("rodas5p", "rosenbrock23", "autotsit5_rosenbrock23")
        alg, rt, at = (O.RODAS5P, 1e-12, 1e-16) if stiff else (O.VERN9, 1e-14, 1e-14)
        if cb and wl["model"] == "bouncing_ball":   # events need a dense interpolant: Tsit5 at 1e-13
            alg, rt, at = O.TSIT5, 1e-13, 1e-13
    return O.solve_ensemble(alg, model, wl["u0"][:, idx], wl["p"][:, idx], ts, spec.values, rt,
                            at, n_per_traj=None if npt is None else npt[idx], saveat_as_tstops=truth,
                            saveat_per_traj=spec.per_traj, save_start=spec.save_start, save_end=spec.save_end,
                            save_end_user=spec.save_end_user, saveat_given=spec.nsave > 0,
                            saveat_scalar=spec.scalar, save_everystep=spec.everystep,
                            max_step_saves=spec.max_step_saves, nthreads=nthreads, **cbkw)


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
                power.append(float(f[3]))
            except ValueError:
                continue
            for k, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(k)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


def compare_err(g_u, o, reltol, abstol):
    """Per-trajectory worst save error in units of the tolerance (reltol*|u| + abstol):
    max, p99 and median over the checked trajectories."""
    ns = int(o["nsaved"].max())
    ou = o["u"][:ns]
    gu = g_u[:ns]
    mask = ~np.isnan(ou)
    r = np.where(mask, np.abs(gu - ou) / (reltol * np.abs(ou) + abstol), 0.0)
    per = r.max(axis=(0, 1))
    return {"max": float(per.max()), "p99": float(np.percentile(per, 99)), "median": float(np.median(per))}


# Configurations measured beside the headline (Robertson/Rodas5P, 100k) in the
# default run: the other single-GPU configurations of the benchmark.
SUITE = ("lorenz", "duffing", "brusselator")
# Trajectories checked against the FP64 oracle and against the ground truth, per
# configuration (None: the whole ensemble).
CHECK = {"robertson": (None, 8192), "lorenz": (None, None), "duffing": (4096, 4096), "brusselator": (4096, 256),
         "robertson_ros23": (None, 4096), "van_der_pol": (4096, 1024), "bouncing_ball": (4096, 4096),
         "pk_dosing": (4096, 4096)}
L2_NOTE = "256 MB buffer written between timed steps"
MIXED_DTYPE = ("f32 stages, W and LU; compensated f32-pair state and stage sums; f32-pair parameters; "
               "double-float stiff right-hand side, error-norm accumulator and refinement residual; "
               "f32 controller powers; f64 t and dt")


def dtype_of(form):
    return "f64" if form == "fp64" else MIXED_DTYPE


def peak_with_clock(ctx, prec):
    """ode_measure_fma_peak (FMA chains on every SM; ~20-35 ms per call) repeated
    for about 1.5 s with the SM clock sampled meanwhile: the roofline denominator
    and the clock it was measured at (once per precision per run)."""
    key = ("peak", prec)
    if key not in ctx:
        L, local = ctx["L"], ctx["local"]
        clk = Clocks(local)
        clk.start()
        vals = []
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 1.5 or len(vals) < 3:
            v = C.c_double(0)
            _check_peak(L.ode_measure_fma_peak(local, prec, C.byref(v)))
            vals.append(v.value)
        c = clk.stop()
        ctx[key] = (float(np.median(vals)), c.get("sm_mhz"))
    return ctx[key]


def _check_peak(status):
    if status != 0:
        raise RuntimeError("ode_measure_fma_peak failed with status %d" % status)


def measure(cfg, args, ctx, steps, warmup, headline=False):
    """One configuration: both GPU forms timed on device-resident inputs, their
    error against the FP64 oracle and the ground truth, the form the equal-
    accuracy rule picks, its roofline, the end-to-end rate through the public
    host-buffer call and the CPU baseline."""
    import torch
    import odegb300
    from odegb300 import _lib, workloads as W
    from odegb300.ensemble import _options, ALG_BY_NAME
    from odegb300.saveat import resolve_saveat

    L, h, dev, work, flush = ctx["L"], ctx["h"], ctx["dev"], ctx["work"], ctx["flush"]
    world, rank, local, dist = ctx["world"], ctx["rank"], ctx["local"], ctx["dist"]
    desc_name, N0 = CONFIGS[cfg]
    N = (args.trajectories or N0) if headline else N0
    wl = workload(cfg, N, seed=42 + rank)
    alg = ALG_BY_NAME[wl["alg"]]
    model = odegb300.ensemble.MODELS[wl["model"]]
    n, _ = wl["u0"].shape
    sv = resolve_saveat(wl["saveat"], wl["tspan"])
    cb = wl.get("callback")
    cap = sv.cap + (2 * cb.max_events if cb else 0)
    npt = wl.get("n_per_traj")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    t_u0, t_p, t_ts = T(wl["u0"]), T(wl["p"]), T(wl["tspan"])
    t_sv = T(sv.values if sv.nsave else np.zeros(1))
    t_npt = T(npt) if npt is not None else None
    tst = wl.get("tstops")
    t_tst = T(np.sort(np.asarray(tst, dtype=np.float64))) if tst is not None else None
    t_out = torch.empty((cap, N), dtype=torch.float64, device=dev)
    u_out = torch.empty((cap, n, N), dtype=torch.float64, device=dev)
    ns_out = torch.empty(N, dtype=torch.int32, device=dev)
    rc_out = torch.empty(N, dtype=torch.int32, device=dev)
    st_out = torch.empty((N, 6), dtype=torch.int64, device=dev)
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    ir_default = wl.get("ir_sweeps", -1)
    fwd_spans = int(bool(np.all(wl["tspan"][1] >= wl["tspan"][0])))

    def solve_device(prec, ir=None, u0=None, p=None):
        ens = odegb300.EnsembleGB300(precision=prec, ir_sweeps=(ir_default if ir is None else ir)
                                     if prec == "mixed" else -1, lanes_per_traj=args.lanes, scheduler=args.scheduler)
        o = _options(wl["reltol"], wl["abstol"], None, None, None, 1000000, sv, ens, None, None, cb)
        # the device entry point cannot see the spans: the caller states that all run forward
        o.forward_only = fwd_spans
        if t_tst is not None:   # the device entry point takes tstops in device memory, sorted
            o.ntstops = int(t_tst.numel())
            o.tstops = C.cast(C.c_void_p(t_tst.data_ptr()), C.POINTER(C.c_double))
        d = _lib.ProblemDesc(model, alg.alg_id, n, wl["p"].shape[0], ens.prec_id(), 0)
        _lib.check(L.ode_solve_ensemble_device(h, C.byref(d), C.byref(o), N, ptr(t_npt),
                                               ptr(t_u0 if u0 is None else u0), ptr(t_p if p is None else p),
                                               ptr(t_ts), ptr(t_sv), ptr(t_out), ptr(u_out), ptr(ns_out),
                                               ptr(rc_out), ptr(st_out), C.c_void_p(work.cuda_stream)), h)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def launches():
        v = C.c_int64(0)
        L.ode_kernel_launches(h, C.byref(v))
        return v.value

    n_or, n_tr = CHECK.get(cfg, (4096, 1024))
    idx_or = np.arange(N if n_or is None else min(N, n_or))
    idx_tr = np.arange(N if n_tr is None else min(N, n_tr))
    idx_u = idx_or if len(idx_or) >= len(idx_tr) else idx_tr
    t_idx = torch.from_numpy(idx_u).to(dev)

    # forms: plain FP64 and mixed; the headline also times the mixed form with one
    # refinement sweep per W solve (its default is none for register-resident W)
    # forms: plain FP64 and mixed; the Rosenbrock workloads also time the mixed
    # form with the other refinement setting (one sweep per W solve for the
    # register-resident W, whose default is none; none for the Brusselator,
    # whose default is one)
    forms = [("fp64", None), ("mixed", None)]
    if cfg in ("robertson", "robertson_ros23") and ir_default <= 0:
        forms.append(("mixed_ir1", 1))
    if cfg == "brusselator" and ir_default >= 1:
        forms.append(("mixed_ir0", 0))
    results = {}
    clocks = Clocks(local)
    clocks.start()
    for name, ir in forms:
        prec = "fp64" if name == "fp64" else "mixed"
        for _ in range(warmup):
            flush.fill_(1.0)
            solve_device(prec, ir)
        barrier()
        l0 = launches()
        times = []
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        t_wall0 = time.perf_counter()
        for _ in range(steps):
            flush.fill_(1.0)
            e0.record(work)
            solve_device(prec, ir)
            e1.record(work)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        barrier()
        wall = time.perf_counter() - t_wall0
        nl = launches() - l0
        ms = max_over_ranks(float(np.mean(times)), dist, dev)
        st = st_out.cpu().numpy()
        rc = rc_out.cpu().numpy()
        results[name] = {"ms": ms, "launches": nl, "attempts": int(st[:, 4].sum() + st[:, 5].sum()),
                         "success": float(((rc == 1) | (rc == 7)).mean()),
                         "u": u_out.index_select(2, t_idx).cpu().numpy(), "naccept_mean": float(st[:, 4].mean()),
                         "wall_s": wall, "steps": steps, "ir_sweeps": ir if ir is not None else
                         (ir_default if prec == "mixed" else None)}
    clk = clocks.stop()

    # conditioning control (uneven Duffing chains): the FP64 kernel on inputs
    # perturbed by one FP32 rounding, against the same FP64 oracle; it shows how
    # far a perturbation of the mixed form's size moves these trajectories
    control = {}
    if cfg == "duffing":
        u0p = t_u0 * (1.0 + 2.0 ** -24)
        solve_device("fp64", u0=u0p)
        control["u0_times_1p2em24"] = u_out.index_select(2, t_idx).cpu().numpy()
        pf = t_p.float().double()
        solve_device("fp64", p=pf)
        control["p_rounded_to_fp32"] = u_out.index_select(2, t_idx).cpu().numpy()
        del u0p, pf
        torch.cuda.synchronize(dev)

    acc, acc_truth = {}, {}
    if rank == 0:
        sel = lambda u, idx: u[:, :, :len(idx)]   # both samples are prefixes of the ensemble
        o = oracle_solve(wl, idx_or, nthreads=os.cpu_count() or 1)
        tr = oracle_solve(wl, idx_tr, nthreads=os.cpu_count() or 1, truth=True)
        for name in results:
            acc[name] = compare_err(sel(results[name]["u"], idx_or), o, wl["reltol"], wl["abstol"])
            acc_truth[name] = compare_err(sel(results[name]["u"], idx_tr), tr, wl["reltol"], wl["abstol"])
        for k, u in control.items():
            control[k] = {"err_vs_fp64_oracle_x_tol": compare_err(sel(u, idx_or), o, wl["reltol"], wl["abstol"])}
    # the fastest mixed form as accurate as the FP64 form, else the FP64 form
    best = "fp64"
    if rank == 0:
        for name in sorted((f for f in results if f != "fp64"), key=lambda f: results[f]["ms"]):
            if all(acc_truth[name][q] <= 2.0 * acc_truth["fp64"][q] + 1.0 for q in ("median", "p99")):
                best = name
                break
    if dist is not None:   # every rank reports the form rank 0 checked
        import torch
        t = torch.tensor([list(results).index(best)], device=dev)
        dist.broadcast(t, 0)
        best = list(results)[int(t.item())]
    R = results[best]
    value = replica_rate(world, N, R["ms"] * 1e-3)

    # roofline of the dominant kernel (the chosen form's integrator kernel)
    prec_id = 0 if best == "fp64" else 1
    peak, peak_mhz = peak_with_clock(ctx, prec_id)
    nmean = float(np.mean(npt)) if npt is not None else n
    fl = W.attempt_flops(wl["alg"], wl["model"], int(round(nmean)))
    nsaves = sv.nsave if sv.nsave else 2
    total_flops = R["attempts"] * fl + N * nsaves * W.save_flops(wl["alg"], wl["model"], int(round(nmean)))
    achieved = total_flops / (R["ms"] * 1e-3)
    traffic = NCU_TRAFFIC.get((cfg, best)) if N == N0 else None

    # end to end through the public host-buffer call (ode_solve_ensemble): inputs in
    # page-locked host memory, outputs back into page-locked host memory, every step
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    h_u0, h_p, h_ts = pin(wl["u0"]), pin(wl["p"]), pin(wl["tspan"])
    h_sv = pin(sv.values if sv.nsave else np.zeros(1))
    h_npt = pin(npt) if npt is not None else None
    h_t = torch.empty((cap, N), dtype=torch.float64).pin_memory()
    h_u = torch.empty((cap, n, N), dtype=torch.float64).pin_memory()
    h_ns = torch.empty(N, dtype=torch.int32).pin_memory()
    h_rc = torch.empty(N, dtype=torch.int32).pin_memory()
    h_st = torch.empty((N, 6), dtype=torch.int64).pin_memory()
    best_prec = "fp64" if best == "fp64" else "mixed"
    ens_e2e = odegb300.EnsembleGB300(precision=best_prec, ir_sweeps=results[best]["ir_sweeps"]
                                     if best_prec == "mixed" else -1, scheduler=args.scheduler)
    o_e2e = _options(wl["reltol"], wl["abstol"], None, None, None, 1000000, sv, ens_e2e, None, None, cb,
                     tstops=wl.get("tstops"))
    d_e2e = _lib.ProblemDesc(model, alg.alg_id, n, wl["p"].shape[0], ens_e2e.prec_id(), 0)
    hp = lambda t, ty=C.c_double: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ty)) if t is not None else None

    def solve_host():
        _lib.check(L.ode_solve_ensemble(h, C.byref(d_e2e), C.byref(o_e2e), N, hp(h_npt, C.c_int32), hp(h_u0),
                                        hp(h_p), hp(h_ts), hp(h_sv) if sv.nsave else None, hp(h_t), hp(h_u),
                                        hp(h_ns, C.c_int32), hp(h_rc, C.c_int32), hp(h_st, _lib.Stats)), h)

    for _ in range(max(1, min(warmup, 2))):
        solve_host()
    e2e_t = []
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        solve_host()
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(float(np.mean(e2e_t)), dist, "cpu" if dist is None else dev)
    h2d = wl["u0"].nbytes + wl["p"].nbytes + wl["tspan"].nbytes + (sv.values.nbytes if sv.nsave else 0) + \
        (npt.nbytes if npt is not None else 0)
    d2h = cap * N * 8 + cap * n * N * 8 + N * 8 + N * 48
    del h_u, h_t, u_out, t_out

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl, N, args.cpu_seconds)
    return {
        "workload": desc_name, "trajectories": N, "value": value, "unit": "trajectories/s", "ms_per_step": R["ms"],
        "steps": steps, "warmup": warmup, "precision_chosen": best, "dtype": dtype_of(best_prec),
        "forms": {p: {"trajectories_per_s": world * N / (results[p]["ms"] * 1e-3), "ms": results[p]["ms"],
                      "ir_sweeps": results[p]["ir_sweeps"], "dtype": dtype_of("fp64" if p == "fp64" else "mixed"),
                      "err_vs_fp64_oracle_x_tol": acc.get(p), "err_vs_ground_truth_x_tol": acc_truth.get(p),
                      "success_frac": results[p]["success"], "mean_accepted_steps": results[p]["naccept_mean"],
                      "gpu_launches": results[p]["launches"]} for p in results},
        "accuracy_checked": {"vs_fp64_oracle": int(len(idx_or)), "vs_ground_truth": int(len(idx_tr)),
                             "ground_truth": "FP64 Rodas5P at reltol 1e-12, abstol 1e-16" if wl["alg"] in (
                                 "rodas5p", "rosenbrock23", "autotsit5_rosenbrock23") else
                             "FP64 Vern9 at reltol = abstol = 1e-14", "saves hit exactly": True,
                             "equal_accuracy_rule": "mixed error vs ground truth <= 2x FP64's + 1 tol unit "
                                                    "at the median and p99"},
        "conditioning_control": control or None,
        "speedup_mixed_vs_fp64": results["fp64"]["ms"] / results[best if best != "fp64" else "mixed"]["ms"],
        "e2e": {"value": world * N / e2e_s, "unit": "trajectories/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "call": "ode_solve_ensemble on page-locked host buffers"},
        "roofline": {"bound": "fp64 pipe" if best == "fp64" else "fp32 pipe", "achieved": achieved / 1e12,
                     "peak": peak / 1e12, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                     "traffic": traffic,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch of this kernel"
                     if traffic else "not captured for this kernel at this size",
                     "flops_per_attempt": fl, "attempted_steps": R["attempts"],
                     "peak_source": "ode_measure_fma_peak (FMA chains on every SM, this GPU; measured in this run)",
                     "peak_sm_mhz": peak_mhz},
        "hbm": {"achieved_gbs": (h2d + d2h) / (R["ms"] * 1e-3) / 1e9, "bytes_per_solve": int(h2d + d2h),
                "note": "algorithmic bytes (inputs read + outputs written) / device time; not the bound"},
        "cpu_baseline": cpu, "clocks": clk, "gpu_launches": R["launches"],
    }


def run_gb300(args, world, rank, local, dist):
    import torch
    from odegb300 import _lib
    from odegb300.ensemble import get_handle

    torch.cuda.set_device(local)
    L = _lib.load()
    h = get_handle(local)
    dev = torch.device("cuda", local)
    # every launch, flush and event goes on one explicit stream (a null stream
    # pointer would make the library fall back to its own stream)
    work = torch.cuda.Stream(dev)
    torch.cuda.set_stream(work)
    ctx = dict(L=L, h=h, dev=dev, work=work, world=world, rank=rank, local=local, dist=dist,
               flush=torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev))   # 256 MB > 129 MB L2

    if args.profile_small:
        run_profile_small(args, ctx)
        return
    head = measure(args.config, args, ctx, args.steps, args.warmup, headline=True)
    suite = {}
    if args.config == "robertson" and not args.no_suite and not args.trajectories:
        for cfg in SUITE:
            suite[cfg] = measure(cfg, args, ctx, min(args.steps, 5), 3)
    serving = None
    if rank == 0 and not args.no_serving:
        rates = [float(x) for x in (args.serve_rates or SERVE_RATES).split(",")]
        serving = serving_block(args, local, rates, args.serve_seconds or SERVE_SECONDS)
    if rank == 0:
        line = {
            "metric": METRIC, "value": head["value"], "unit": "trajectories/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": head["dtype"],
            "data": "synthetic (seeded, config distributions)",
            "config": {"workload": head["workload"], "trajectories": head["trajectories"], "l2": L2_NOTE},
            "precision_chosen": head["precision_chosen"],
        }
        for k in ("forms", "accuracy_checked", "speedup_mixed_vs_fp64", "e2e", "roofline", "hbm", "cpu_baseline",
                  "clocks", "gpu_launches"):
            line[k] = head[k]
        line["configs"] = suite or None
        line["serving"] = serving
        print(json.dumps(line))


def run_profile_small(args, ctx):
    """One small FP64 + mixed solve pair of a configuration for ncu captures (no JSON line)."""
    import torch
    import odegb300
    from odegb300 import _lib
    from odegb300.ensemble import _options, ALG_BY_NAME
    from odegb300.saveat import resolve_saveat
    L, h, dev, work = ctx["L"], ctx["h"], ctx["dev"], ctx["work"]
    N = args.trajectories or CONFIGS[args.config][1]
    wl = workload(args.config, N, seed=42)
    alg = ALG_BY_NAME[wl["alg"]]
    model = odegb300.ensemble.MODELS[wl["model"]]
    n = wl["u0"].shape[0]
    sv = resolve_saveat(wl["saveat"], wl["tspan"])
    cb = wl.get("callback")
    cap = sv.cap + (2 * cb.max_events if cb else 0)
    npt = wl.get("n_per_traj")
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    ins = [T(npt) if npt is not None else None, T(wl["u0"]), T(wl["p"]), T(wl["tspan"]),
           T(sv.values if sv.nsave else np.zeros(1))]
    outs = [torch.empty((cap, N), dtype=torch.float64, device=dev),
            torch.empty((cap, n, N), dtype=torch.float64, device=dev),
            torch.empty(N, dtype=torch.int32, device=dev), torch.empty(N, dtype=torch.int32, device=dev),
            torch.empty((N, 6), dtype=torch.int64, device=dev)]
    tst = wl.get("tstops")
    t_tst = T(np.sort(np.asarray(tst, dtype=np.float64))) if tst is not None else None
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    for prec in ("fp64", "mixed"):
        ens = odegb300.EnsembleGB300(precision=prec, ir_sweeps=wl.get("ir_sweeps", -1) if prec == "mixed" else -1,
                                     scheduler=args.scheduler)
        o = _options(wl["reltol"], wl["abstol"], None, None, None, 1000000, sv, ens, None, None, cb)
        o.forward_only = int(bool(np.all(wl["tspan"][1] >= wl["tspan"][0])))   # the timed solves' kernels
        if t_tst is not None:
            o.ntstops = int(t_tst.numel())
            o.tstops = C.cast(C.c_void_p(t_tst.data_ptr()), C.POINTER(C.c_double))
        d = _lib.ProblemDesc(model, alg.alg_id, n, wl["p"].shape[0], ens.prec_id(), 0)
        _lib.check(L.ode_solve_ensemble_device(h, C.byref(d), C.byref(o), N, *[ptr(x) for x in ins + outs],
                                               C.c_void_p(work.cuda_stream)), h)
    torch.cuda.synchronize(dev)
    print(json.dumps({"profile_small": True, "config": args.config, "trajectories": N}))


def cpu_baseline(wl, N, target_s):
    """CPU restatement of the reference (the oracle), all host threads, bounded sample."""
    ncores = os.cpu_count() or 1
    k = min(N, 2048)
    t0 = time.perf_counter()
    oracle_solve(wl, np.arange(k), nthreads=ncores)
    t1 = time.perf_counter() - t0
    m = int(min(N, max(k, k * target_s / max(t1, 1e-3))))
    if m > k:
        t0 = time.perf_counter()
        oracle_solve(wl, np.arange(m), nthreads=ncores)
        t1 = time.perf_counter() - t0
        k = m
    return {"value": k / t1, "unit": "trajectories/s", "cores": ncores, "kind": "port",
            "sample": "%d of %d trajectories of the same workload, oracle with %d threads (%.1f s)" % (k, N, ncores, t1)}


def run_reference(args, world, rank):
    """The reference's CPU path (its restatement: Julia is not installed) on all
    host threads, over the whole headline ensemble every step, with the GPU arm's
    config; the other configurations as one bounded sample each."""
    if rank != 0:
        return
    if args.config == "serving":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no serving loop (EnsembleThreads "
                                                              "solves one ensemble per call)"}))
        return
    desc_name, N0 = CONFIGS[args.config]
    N = args.trajectories or N0
    wl = workload(args.config, N, seed=42)
    ncores = os.cpu_count() or 1
    idx = np.arange(N)
    for _ in range(args.warmup):
        oracle_solve(wl, idx[:min(N, 4096)], nthreads=ncores)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle_solve(wl, idx, nthreads=ncores)
        ts.append(time.perf_counter() - t0)
    v = N / float(np.mean(ts))
    sample = "all %d trajectories every step, CPU restatement of the reference (Julia is not installed), " \
             "%d threads" % (N, ncores)
    suite = {}
    if args.config == "robertson" and not args.no_suite and not args.trajectories:
        for cfg in SUITE:
            wl_c = workload(cfg, CONFIGS[cfg][1], seed=42)
            suite[cfg] = dict(cpu_baseline(wl_c, CONFIGS[cfg][1], args.cpu_seconds), workload=CONFIGS[cfg][0])
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "trajectories/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.mean(ts)) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded, config distributions)",
        "config": {"workload": desc_name, "trajectories": N, "l2": L2_NOTE},
        "cpu_baseline": {"value": v, "unit": "trajectories/s", "cores": ncores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "trajectories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "configs": suite or None}))


def measured_hbm_gbs():
    """The machine's measured copy bandwidth (MEASURED_PEAKS.json, written by the
    measurement job), or the recorded fallback of 6.8 TB/s."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def run_dense(args, world, rank, local, dist):
    """Dense output through the public calls: ode_solve_ensemble_dense on
    page-locked host buffers (every accepted step kept with its interpolation
    vectors, written in place by the kernels), then sol(t) of every trajectory
    at 101 times in one ode_dense_eval launch.  value: trajectories/s of the
    dense solve on the device (its launch's CUDA-event time); e2e: the same
    through the host call; dense_eval: (trajectory, time) pairs per second."""
    import torch
    import odegb300
    from odegb300 import _lib, workloads as W
    from odegb300.ensemble import ALG_BY_NAME, MODELS, _options, get_handle
    from odegb300.saveat import resolve_saveat

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = _lib.load()
    h = get_handle(local)
    desc_name, N0 = CONFIGS[args.config]
    N = args.trajectories or N0
    wl = workload(args.config, N, seed=42 + rank)
    n = wl["u0"].shape[0]
    alg = ALG_BY_NAME[wl["alg"]]
    sv = resolve_saveat(None, wl["tspan"], save_everystep=True, max_step_saves=wl["max_step_saves"])
    cap = sv.cap
    ens = odegb300.EnsembleGB300(precision="fp64")
    o = _options(wl["reltol"], wl["abstol"], None, None, None, 1000000, sv, ens, None, None)
    d = _lib.ProblemDesc(MODELS[wl["model"]], alg.alg_id, n, wl["p"].shape[0], 0, 0)
    nk = L.ode_dense_nk(alg.alg_id)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    h_u0, h_p, h_ts = pin(wl["u0"]), pin(wl["p"]), pin(wl["tspan"])
    h_t = torch.empty((cap, N), dtype=torch.float64).pin_memory()
    h_u = torch.empty((cap, n, N), dtype=torch.float64).pin_memory()
    h_k = torch.empty((cap, nk, n, N), dtype=torch.float64).pin_memory()
    h_ns = torch.empty(N, dtype=torch.int32).pin_memory()
    h_rc = torch.empty(N, dtype=torch.int32).pin_memory()
    h_st = torch.empty((N, 6), dtype=torch.int64).pin_memory()
    NQ = 101
    tq = np.linspace(0.0, 1.0, NQ)
    h_tq = pin(tq)
    h_out = torch.empty((NQ, n, N), dtype=torch.float64).pin_memory()
    hp = lambda t, ty=C.c_double: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ty))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    x = C.c_double(0)
    cnt = C.c_int64(0)

    def last_ms():
        L.ode_last_kernel_ms(h, C.byref(x))
        return x.value

    def launches():
        L.ode_kernel_launches(h, C.byref(cnt))
        return cnt.value

    def solve():
        _lib.check(L.ode_solve_ensemble_dense(h, C.byref(d), C.byref(o), N, hp(h_u0), hp(h_p), hp(h_ts), hp(h_t),
                                              hp(h_u), hp(h_k), hp(h_ns, C.c_int32), hp(h_rc, C.c_int32),
                                              hp(h_st, _lib.Stats)), h)

    def evaluate():
        _lib.check(L.ode_dense_eval(h, C.byref(d), N, hp(h_p), hp(h_t), hp(h_u), hp(h_k), hp(h_ns, C.c_int32), cap,
                                    NQ, hp(h_tq), 0, hp(h_out)), h)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)
        dms, wall = [], []
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            fn()
            wall.append(time.perf_counter() - t0)
            dms.append(last_ms())
        return max_over_ranks(float(np.mean(dms)), dist, dev), max_over_ranks(float(np.mean(wall)), dist, dev)

    clocks = Clocks(local)
    clocks.start()
    l0 = launches()
    ms, wall_s = timed(solve)
    nl = launches() - l0
    ev_ms, ev_wall = timed(evaluate)   # saves staged on the device, results written in place
    clk = clocks.stop()
    st = h_st.numpy()
    ns = h_ns.numpy().astype(np.int64)
    attempts = int(st[:, 4].sum() + st[:, 5].sum())
    fl = W.attempt_flops(wl["alg"], wl["model"], n)
    peak = C.c_double(0)
    L.ode_measure_fma_peak(local, 0, C.byref(peak))
    achieved = attempts * fl / (ms * 1e-3)
    written = int(ns.sum()) * (1 + n + nk * n) * 8 + N * (8 + 48)
    hbm_peak, hbm_src = measured_hbm_gbs()
    # sol(t): per (trajectory, time) pair the interval search reads ~log2(steps)
    # saved times, then u at both ends and the nk vectors (n each), and writes n values
    pair_bytes = (int(np.ceil(np.log2(max(2.0, ns.mean())))) + 2 * n + nk * n + n) * 8
    ev_gbs = NQ * N * pair_bytes / (ev_ms * 1e-3) / 1e9

    acc, cpu = None, None
    if rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as O
        errs, same = [], 0
        out = h_out.numpy()
        for j in range(0, min(N, 64)):
            r = O.solve(O.TSIT5, O.LORENZ, wl["u0"][:, j], wl["p"][:, j], wl["tspan"][:, j], dense=True,
                        reltol=wl["reltol"], abstol=wl["abstol"], saveat_given=False, save_everystep=True,
                        max_step_saves=wl["max_step_saves"], save_start=True, save_end=True)
            ref = r["dense"](tq)
            errs.append(float(np.max(np.abs(out[:, :, j] - ref) / (wl["reltol"] * np.abs(ref) + wl["abstol"]))))
            same += int(r["dense"].nsteps + 1 == ns[j])
        errs = np.array(errs)
        acc = {"sol_t_err_vs_oracle_x_tol": {"max": float(errs.max()), "p99": float(np.percentile(errs, 99)),
                                             "median": float(np.median(errs))},
               "same_step_count_frac": same / len(errs), "checked": int(len(errs))}
        if not args.no_cpu_baseline:
            cpu = cpu_baseline(wl, N, args.cpu_seconds)
        print(json.dumps({
            "metric": "trajectories/sec, dense output (every step with its interpolation vectors), FP64",
            "value": world * N / (ms * 1e-3), "unit": "trajectories/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, config distributions)",
            "config": {"workload": desc_name, "trajectories": N, "max_step_saves": wl["max_step_saves"],
                       "l2": "256 MB buffer written between timed steps",
                       "buffers": "page-locked host buffers, written in place by the kernels"},
            "e2e": {"value": world * N / wall_s, "unit": "trajectories/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0, "note": "page-locked buffers: the kernels read the inputs and write "
                    "%d bytes of saves and vectors in place over NVLink-C2C" % written},
            "dense_eval": {"queries_per_trajectory": NQ, "ms": ev_ms, "pairs_per_s": NQ * N / (ev_ms * 1e-3),
                           "e2e_pairs_per_s": NQ * N / ev_wall, "algorithmic_gbs": ev_gbs,
                           "hbm_peak_gbs": hbm_peak, "hbm_frac": ev_gbs / hbm_peak, "peak_source": hbm_src,
                           "bytes_per_pair": pair_bytes},
            "accuracy": acc,
            "roofline": {"bound": "fp64 pipe", "achieved": achieved / 1e12, "peak": peak.value / 1e12,
                         "unit": "TFLOP/s", "frac": achieved / peak.value if peak.value else None, "traffic": None,
                         "flops_per_attempt": fl, "attempted_steps": attempts,
                         "peak_source": "ode_measure_fma_peak (FMA-chain kernel, this GPU)"},
            "hbm": {"bytes_written_per_solve": written, "achieved_gbs": written / (ms * 1e-3) / 1e9},
            "mean_accepted_steps": float(st[:, 4].mean()),
            "cpu_baseline": cpu, "clocks": clk, "gpu_launches": nl}))


def main():
    args = parse()
    world, rank, local, dist = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.config == "serving":
        run_serving(args, rank, local)
    elif args.config == "lorenz_dense":
        run_dense(args, world, rank, local, dist)
    else:
        run_gb300(args, world, rank, local, dist)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
