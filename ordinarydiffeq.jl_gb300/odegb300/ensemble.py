"""SciML-shaped host API over libode_b200.so.

Mirrors the reference's ensemble call
    solve(EnsembleProblem(prob; prob_func, output_func, reduction, u_init), alg,
          EnsembleGB300(); trajectories, batch_size, saveat, reltol, abstol, ...)
(SciMLBase semantics as exercised in lib/DiffEqBase/test/downstream/ensemble.jl:7-118
and NEWS.md "Ensemble RNG redesign": prob_func(prob, ctx), output_func(sol, ctx)).
prob_func runs on the host for every trajectory; the packed structure-of-arrays
batch goes to the GPU in one call.  A vectorised form (u0s / ps / tspans
arrays instead of prob_func) skips the per-trajectory Python work.
"""
import ctypes as C
import time
import warnings
from dataclasses import dataclass, field
from enum import IntEnum

import numpy as np

from . import _lib
from .saveat import resolve_saveat


class ReturnCode(IntEnum):
    Default = 0
    Success = 1
    MaxIters = 2
    DtNaN = 3
    DtLessThanMin = 4
    Unstable = 5
    Aborted = 6
    Terminated = 7
    InitialFailure = 8   # a NaN time span


MODELS = {"linear": _lib.MODEL_LINEAR, "lorenz": _lib.MODEL_LORENZ, "robertson": _lib.MODEL_ROBERTSON,
          "duffing_chain": _lib.MODEL_DUFFING_CHAIN, "brusselator_1d": _lib.MODEL_BRUSSELATOR_1D,
          "bouncing_ball": _lib.MODEL_BOUNCING_BALL, "van_der_pol": _lib.MODEL_VANDERPOL,
          "pk_one_compartment": _lib.MODEL_PK_ONE_COMPARTMENT, "forced_duffing": _lib.MODEL_FORCED_DUFFING}
N_PARAMS = {_lib.MODEL_LINEAR: 1, _lib.MODEL_LORENZ: 3, _lib.MODEL_ROBERTSON: 3,
            _lib.MODEL_DUFFING_CHAIN: 3, _lib.MODEL_BRUSSELATOR_1D: 3, _lib.MODEL_BOUNCING_BALL: 3,
            _lib.MODEL_VANDERPOL: 1, _lib.MODEL_PK_ONE_COMPARTMENT: 3, _lib.MODEL_FORCED_DUFFING: 5}


@dataclass
class ContinuousCallback:
    """The model's registered ContinuousCallback (device code cannot call Python or
    Julia closures: the condition and affect are compiled in with the model, e.g.
    "bouncing_ball": condition x, affect_neg! v <- -e v or terminate! once
    t >= t_stop).  interp_points as SciMLBase's ContinuousCallback (default 10);
    max_events sizes the output: each event adds two saves (before and after its
    affect, save_positions = (true, true))."""
    interp_points: int = 10
    max_events: int = 16


@dataclass
class DiscreteCallback:
    """The model's registered DiscreteCallback, e.g. "pk_one_compartment": condition
    t in tstops (the dose times, passed as solve's tstops: the pattern of
    DiffEqCallbacks' PresetTimeCallback), affect! depot += dose.  max_events
    sizes the output: each firing adds two saves (before and after its affect,
    save_positions = (true, true))."""
    max_events: int = 16
    interp_points = 10   # unused by a discrete callback; the options carry one field for both


class _Alg:
    alg_id = -1

    def __repr__(self):
        return type(self).__name__ + "()"


class Tsit5(_Alg):
    """Tsitouras 5(4) (lib/OrdinaryDiffEqTsit5/src/algorithms.jl:16-21)."""
    alg_id = _lib.ODE_TSIT5


class Vern7(_Alg):
    """Verner 7(6), lazy interpolation stages (lib/OrdinaryDiffEqVerner/src/algorithms.jl:44-50)."""
    alg_id = _lib.ODE_VERN7


class Rodas5P(_Alg):
    """Rodas5P Rosenbrock method with the analytic Jacobian of the model
    (lib/OrdinaryDiffEqRosenbrock/src/algorithms.jl:83-87)."""
    alg_id = _lib.ODE_RODAS5P


class Rosenbrock23(_Alg):
    """Rosenbrock23 (Shampine's ode23s W-method pair) with the analytic Jacobian of
    the model (lib/OrdinaryDiffEqRosenbrock/src/algorithms.jl:108-146).  As a
    W-method it may keep J across accepted steps: max_jac_age = 1 (the
    reference's default) takes a fresh J on every attempt; a larger value keeps
    it for up to that many accepted steps while dt*gamma stays within
    jac_reuse_gamma_tol of the J's (_rosenbrock_jac_reuse_decision)."""
    alg_id = _lib.ODE_ROSENBROCK23

    def __init__(self, max_jac_age=1, jac_reuse_gamma_tol=0.03):
        self.max_jac_age = int(max_jac_age)
        self.jac_reuse_gamma_tol = float(jac_reuse_gamma_tol)

    def __repr__(self):
        return "Rosenbrock23(max_jac_age=%d)" % self.max_jac_age if self.max_jac_age != 1 else "Rosenbrock23()"


class AutoTsit5(_Alg):
    """AutoTsit5(stiff_alg): Tsit5 with stiffness detection, switching to the stiff
    method and back (AutoSwitch defaults: maxstiffstep 10, maxnonstiffstep 3,
    tolerances 9/10, dtfac 2; lib/OrdinaryDiffEqTsit5/src/algorithms.jl:27-33,
    lib/OrdinaryDiffEqCore/src/composite_algs.jl).  The stiff method compiled in is
    Rosenbrock23."""

    def __init__(self, stiff_alg=None):
        if stiff_alg is not None and not isinstance(stiff_alg, Rosenbrock23):
            raise ValueError("AutoTsit5 is compiled with Rosenbrock23 as its stiff method")
        self.stiff_alg = stiff_alg or Rosenbrock23()

    alg_id = _lib.ODE_AUTOTSIT5_ROSENBROCK23

    def __repr__(self):
        return "AutoTsit5(Rosenbrock23())"


ALG_BY_NAME = {"tsit5": Tsit5(), "vern7": Vern7(), "rodas5p": Rodas5P(), "rosenbrock23": Rosenbrock23(),
               "autotsit5_rosenbrock23": AutoTsit5(Rosenbrock23())}


@dataclass
class PIController:
    """The reference's PIController knobs (controllers.jl:745-843: beta1, beta2,
    qoldinit and the CommonControllerOptions qmin, qmax, qmax_first_step, gamma,
    qsteady_min, qsteady_max); None keeps the method's default."""
    beta1: float = None
    beta2: float = None
    qoldinit: float = None
    qmin: float = None
    qmax: float = None
    qmax_first_step: float = None
    gamma: float = None
    qsteady_min: float = None
    qsteady_max: float = None


@dataclass
class EnsembleGB300:
    """Ensemble algorithm running every trajectory on one GB300.

    precision: "fp64" (the reference's arithmetic) or "mixed" (FP32 stages and,
    for Rodas5P, FP32 LU with FP64-residual refinement; FP64 t, dt, error norm
    and controller).  scheduler: "auto" | "static" | "persistent".
    """
    precision: str = "fp64"
    lanes_per_traj: int = 0
    scheduler: str = "auto"
    block_size: int = 0
    ir_sweeps: int = -1
    device: int = 0

    def prec_id(self):
        return {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[self.precision]

    def sched_id(self):
        return {"auto": 0, "static": 1, "persistent": 2}[self.scheduler]


@dataclass
class ODEProblem:
    """An ODE over a registered model.  `model` is a name ("lorenz",
    "robertson", "duffing_chain", "brusselator_1d", "linear") or id."""
    model: object
    u0: np.ndarray
    tspan: tuple
    p: np.ndarray = None

    def __post_init__(self):
        if isinstance(self.model, str):
            self.model = MODELS[self.model]
        self.u0 = np.asarray(self.u0, dtype=np.float64).ravel()
        self.p = np.asarray(self.p if self.p is not None else [], dtype=np.float64).ravel()
        self.tspan = (float(self.tspan[0]), float(self.tspan[1]))


def remake(prob, u0=None, p=None, tspan=None):
    return ODEProblem(prob.model, prob.u0 if u0 is None else u0, prob.tspan if tspan is None else tspan,
                      prob.p if p is None else p)


@dataclass
class EnsembleContext:
    sim_id: int
    repeat: int
    rng: np.random.Generator

    @property
    def i(self):
        return self.sim_id


def _default_output(sol, ctx):
    return sol, False


def _default_reduction(u, batch, I):
    return u + list(batch), False


@dataclass
class EnsembleProblem:
    prob: ODEProblem
    prob_func: object = None
    output_func: object = None
    reduction: object = None
    u_init: object = None
    safetycopy: bool = True
    # vectorised inputs (trajectory index last): u0s (n, N), ps (np, N), tspans (2, N)
    u0s: np.ndarray = None
    ps: np.ndarray = None
    tspans: np.ndarray = None
    n_per_traj: np.ndarray = None


class ODESolution:
    """One trajectory's result: t, u (list of state vectors), retcode, stats.
    sol(t) evaluates the solution between saves (see __call__)."""

    def __init__(self, t, u, retcode, stats, prob=None, alg=None, dense=None):
        self.t = t
        self.u = u
        self.retcode = ReturnCode(int(retcode))
        self.stats = stats
        self.prob = prob
        self.alg = alg
        self._dense = dense   # (solve outputs, trajectory index) of a dense solve

    @property
    def dense(self):
        return self._dense is not None

    def __call__(self, t, deriv=0, idxs=None, continuity="left"):
        """sol(t) as ode_interpolation (generic_dense.jl:1094-1190) evaluates it:
        the method's interpolant on the saved steps for a dense solve (on the
        GPU), linear interpolation between saves otherwise.  deriv=1 is
        sol(t, Val{1}) (dense solves); idxs selects components.  A time equal
        to a saved one returns that save; continuity="right" the later of two
        saves at one time.  Scalar t gives one state vector, an array of times
        one row per time."""
        tq = np.atleast_1d(np.asarray(t, dtype=np.float64))
        if self._dense is not None:
            res, j = self._dense
            sub = {"t": res["t"][:, j:j + 1].copy(), "u": res["u"][:, :, j:j + 1].copy(),
                   "k": res["k"][..., j:j + 1].copy(), "nsaved": res["nsaved"][j:j + 1].copy(),
                   "dense": dict(res["dense"], p=res["dense"]["p"][:, j:j + 1].copy())}
            vals = dense_eval(sub, tq, deriv=deriv, continuity=continuity)[:, :, 0]
        elif deriv:
            raise ValueError("derivatives of the interpolant need a dense solve")
        else:
            ts = np.asarray(self.t, dtype=np.float64)
            us = np.asarray(self.u, dtype=np.float64)
            vals = np.empty((tq.size, us.shape[1]))
            for r, tv in enumerate(tq):
                i0 = int(np.searchsorted(ts, tv, side="left"))   # the exact-time rule first
                if i0 < len(ts) and ts[i0] == tv:
                    k = i0 + 1 if continuity == "right" and i0 + 1 < len(ts) and ts[i0 + 1] == tv else i0
                    vals[r] = us[k]
                    continue
                ip = min(len(ts) - 1, 1 + int(np.searchsorted(ts[1:], tv, side="left")))
                im = ip - 1 if ip > 0 else ip
                dt = ts[ip] - ts[im]
                th = 1.0 if dt == 0 else (tv - ts[im]) / dt
                vals[r] = (1 - th) * us[im] + th * us[ip]
        if idxs is not None:
            vals = vals[:, idxs]
        return vals[0] if np.ndim(t) == 0 else vals

    def __repr__(self):
        return "ODESolution(retcode=%s, %d saves%s)" % (self.retcode.name, len(self.t),
                                                      ", dense" if self.dense else "")


class _LazySolutions:
    """List-like view creating ODESolution objects on access (cheap for 1M trajectories)."""

    def __init__(self, res, alg, n_per_traj=None):
        self.r = res
        self.alg = alg
        self.npt = n_per_traj

    def __len__(self):
        return self.r["retcode"].shape[0]

    def __getitem__(self, j):
        if isinstance(j, slice):
            return [self[k] for k in range(*j.indices(len(self)))]
        if j < 0:
            j += len(self)
        r = self.r
        ns = int(r["nsaved"][j])
        # with save_idxs every row (one for a state past a smaller trajectory's size is not written)
        n = r["u"].shape[1] if (self.npt is None or r.get("save_idxs") is not None) else int(self.npt[j])
        t = r["t"][:ns, j].copy()
        u = [r["u"][s, :n, j].copy() for s in range(ns)]
        st = {k: int(r["stats"][k][j]) for k in r["stats"]}
        return ODESolution(t, u, r["retcode"][j], st, alg=self.alg, dense=(r, j) if r.get("dense") else None)

    def __iter__(self):
        for j in range(len(self)):
            yield self[j]


@dataclass
class EnsembleSolution:
    u: object
    elapsedTime: float
    converged: bool = True
    raw: dict = field(default=None, repr=False)


_handles = {}


def get_handle(device=0):
    h = _handles.get(device)
    if h is None:
        L = _lib.load()
        hp = C.c_void_p(0)
        _lib.check(L.ode_create(device, 0, C.byref(hp)))
        h = hp
        _handles[device] = h
    return h


def _options(reltol, abstol, dt, dtmax, dtmin, maxiters, sv, ens, qmax_first_step, qmax, callback=None,
             tstops=None, alg=None, save_idxs=None, adaptive=True, controller=None, force_dtmin=False,
             isoutofdomain=None):
    o = _lib.Options()
    L = _lib.load()
    L.ode_options_default(C.byref(o))
    if isinstance(alg, Rosenbrock23):   # its W-method Jacobian reuse knobs
        o.max_jac_age = alg.max_jac_age
        o.jac_reuse_gamma_tol = alg.jac_reuse_gamma_tol
    # array tolerances: one per state (solve(...; abstol = [...])); the scalar fields
    # then hold their smallest entries (checked, unused)
    keep = []
    for name, tol in (("abstol", abstol), ("reltol", reltol)):
        if np.ndim(tol):
            v = np.ascontiguousarray(tol, dtype=np.float64).ravel()
            keep.append(v)
            setattr(o, name + "_vec", v.ctypes.data_as(C.POINTER(C.c_double)))
            setattr(o, name, float(v.min()))
        else:
            setattr(o, name, float(tol))
    o._keep_tol = keep
    o.dt = abs(dt or 0.0)   # either sign is taken in the span's direction (handle_dt!, solve.jl:968-985)
    o.dtmax = dtmax or 0.0
    o.dtmin = dtmin or 0.0
    o.maxiters = int(maxiters)
    o.save_start, o.save_end, o.save_end_user = int(sv.save_start), int(sv.save_end), sv.save_end_user
    o.saveat_scalar = int(sv.scalar)
    o.nsave = sv.nsave
    o.saveat_per_traj = int(sv.per_traj)
    o.qmax_first_step = qmax_first_step or 0.0
    o.qmax = qmax or 0.0
    if controller is not None:   # solve(...; controller = PIController(...))
        o.controller_given = 1
        for k in ("beta1", "beta2", "qoldinit", "qmin", "gamma", "qsteady_min", "qsteady_max"):
            v = getattr(controller, k)
            setattr(o, k, float("nan") if v is None else float(v))
        if controller.qmax is not None:
            o.qmax = float(controller.qmax)
        if controller.qmax_first_step is not None:
            o.qmax_first_step = float(controller.qmax_first_step)
    o.lanes_per_traj = ens.lanes_per_traj
    o.scheduler = ens.sched_id()
    o.block_size = ens.block_size
    o.ir_sweeps = ens.ir_sweeps
    o.save_everystep = int(sv.everystep)
    o.max_step_saves = int(sv.max_step_saves)
    if callback is not None:
        o.callback = 1
        o.interp_points = int(callback.interp_points)
        o.max_events = int(callback.max_events)
    if tstops is not None and np.size(tstops) > 0:
        ts = np.ascontiguousarray(np.atleast_1d(tstops), dtype=np.float64).ravel()
        if np.isnan(ts).any():
            raise ValueError("tstops contain NaN")
        o.ntstops = ts.size
        o.tstops = ts.ctypes.data_as(C.POINTER(C.c_double))
        o._tstops = ts   # the options hold the array while the call reads it
    o.adaptive = int(bool(adaptive))
    o.force_dtmin = int(bool(force_dtmin))
    # isoutofdomain: the common any(x -> x < 0, u) ("negative" or True), else none
    if isoutofdomain not in (None, False, True, "negative"):
        raise ValueError('isoutofdomain: "negative" (any state < 0) or None')
    o.isoutofdomain = 1 if isoutofdomain in (True, "negative") else 0
    if save_idxs is not None:
        ix = np.ascontiguousarray(np.atleast_1d(save_idxs), dtype=np.int32).ravel()
        o.nsave_idxs = ix.size
        o.save_idxs = ix.ctypes.data_as(C.POINTER(C.c_int32))
        o._save_idxs = ix
    return o


def register_model(source, name, n_states, n_params, jac=False, tgrad=False, nonautonomous=False,
                   continuous_callback=None, vector_callback=0, discrete_callback=False):
    """Register a model given as CUDA C++ source (ode_register_model): the device
    form of the reference's f(du, u, p, t), with its optional jac and tgrad.  For a
    model named `name` the source defines the templates

        template <class T, class P> __device__ void NAME_f(T* du, const T* u, const P* p, double t);
        template <class T, class P> __device__ void NAME_jac(T* J, const T* u, const P* p, double t);   # jac=True
        template <class T, class P> __device__ void NAME_tgrad(T* dT, const T* u, const P* p, double t); # tgrad=True

    (J row-major).  Without NAME_jac the Rosenbrock methods differentiate NAME_f
    by forward-mode AD.  Callbacks registered with the model (enabled per solve
    by passing ContinuousCallback(...) / DiscreteCallback(...) as `callback`):

        continuous_callback="up" | "down" | "both": a ContinuousCallback,
            __device__ double NAME_condition(const double* u, const double* p, double t);
            __device__ int NAME_affect(double* u, const double* p, double t, int upcrossing);
            acting on upcrossings (affect!), downcrossings (affect_neg!) or both;
        vector_callback=len: a VectorContinuousCallback of len conditions,
            __device__ void NAME_vcondition(double* out, const double* u, const double* p, double t);
            __device__ int NAME_vaffect(double* u, const double* p, double t, const int* events);
        discrete_callback=True: a DiscreteCallback,
            __device__ int NAME_dcondition(const double* u, const double* p, double t);
            __device__ int NAME_daffect(double* u, const double* p, double t);

    (an affect returning nonzero calls terminate!).  Returns the model id; the
    name also becomes a model name for ODEProblem and solve_arrays.  The kernels
    are compiled on the first solve of each method and precision."""
    L = _lib.load()
    flags = (_lib.MODEL_HAS_JAC if jac else 0) | (_lib.MODEL_HAS_TGRAD if tgrad else 0) | \
        (_lib.MODEL_NONAUTONOMOUS if nonautonomous else 0)
    if continuous_callback is not None:
        flags |= _lib.MODEL_CONTINUOUS_CALLBACK | {
            "up": _lib.MODEL_CALLBACK_AFFECT, "down": _lib.MODEL_CALLBACK_AFFECT_NEG,
            "both": _lib.MODEL_CALLBACK_AFFECT | _lib.MODEL_CALLBACK_AFFECT_NEG}[continuous_callback]
    if vector_callback:
        flags |= _lib.MODEL_VECTOR_CALLBACK | _lib.model_callback_len(int(vector_callback))
    if discrete_callback:
        flags |= _lib.MODEL_DISCRETE_CALLBACK
    mid = C.c_int32(0)
    _lib.check(L.ode_register_model(source.encode(), name.encode(), int(n_states), int(n_params), flags,
                                    C.byref(mid)))
    MODELS[name] = mid.value
    N_PARAMS[mid.value] = int(n_params)
    return mid.value


def solve_arrays(model, alg, ens, u0s, ps, tspans, saveat=None, reltol=1e-3, abstol=1e-6, dt=None,
                 dtmax=None, dtmin=None, maxiters=1000000, save_start=None, save_end=None, n_per_traj=None,
                 qmax_first_step=None, qmax=None, return_times=False, save_everystep=False, max_step_saves=1024,
                 dense=False, callback=None, tstops=None, save_idxs=None, adaptive=True, controller=None,
                 force_dtmin=False, isoutofdomain=None):
    """Solve a packed ensemble.  u0s (n, N), ps (np, N), tspans (2, N).  Returns the
    raw structure-of-arrays outputs dict (t, u, nsaved, retcode, stats).
    save_everystep keeps every accepted step, up to max_step_saves per
    trajectory (past that the last slot holds the final point and a warning is
    issued), beside the saveat points if any.  dense (with save_everystep) also keeps
    each step's interpolation vectors, k (cap, nk, n, N), for dense_eval.
    callback: the model's ContinuousCallback (ContinuousCallback(...)); a
    trajectory it terminates reports ReturnCode.Terminated.  tstops: times every
    trajectory steps to exactly (those inside its (t0, tf)), as the reference's
    tstops keyword.  save_idxs: the states saved (0-based, in order; the
    reference's save_idxs): u is then (cap, len(save_idxs), N).  adaptive=False:
    fixed steps of dt (the reference's adaptive = false).  controller: a
    PIController with the step-size controller's knobs.  force_dtmin: steps at
    the smallest dt are taken whatever their error (no DtLessThanMin exit).
    isoutofdomain="negative": adaptive steps ending with a negative state are
    rejected (the reference's isoutofdomain = (u, p, t) -> any(x -> x < 0, u))."""
    L = _lib.load()
    if isinstance(model, str):
        model = MODELS[model]
    u0s = np.ascontiguousarray(u0s, dtype=np.float64)
    ps = np.ascontiguousarray(ps, dtype=np.float64)
    tspans = np.ascontiguousarray(tspans, dtype=np.float64)
    n, N = u0s.shape
    sv = resolve_saveat(saveat, tspans, save_start, save_end, save_everystep, max_step_saves)
    o = _options(reltol, abstol, dt, dtmax, dtmin, maxiters, sv, ens, qmax_first_step, qmax, callback, tstops, alg,
                 save_idxs, adaptive, controller, force_dtmin, isoutofdomain)
    d = _lib.ProblemDesc(model, alg.alg_id, n, ps.shape[0], ens.prec_id(), 0)
    rows = n if save_idxs is None else int(np.size(save_idxs))
    cap = sv.cap + (2 * callback.max_events if callback is not None else 0)
    if dense and not sv.everystep:
        raise ValueError("dense output keeps every step: use it without saveat, with save_everystep")
    if dense and n_per_traj is not None:
        raise ValueError("dense output needs trajectories of one size")
    if dense and save_idxs is not None:
        raise ValueError("save_idxs with dense output is not supported")
    t_out = np.full((cap, N), np.nan)
    u_out = np.full((cap, rows, N), np.nan)
    k_out = np.empty((cap, L.ode_dense_nk(alg.alg_id), n, N)) if dense else None
    nsaved = np.zeros(N, dtype=np.int32)
    rc = np.zeros(N, dtype=np.int32)
    stats = np.zeros((N, 6), dtype=np.int64)
    npt = None
    if n_per_traj is not None:
        npt = np.ascontiguousarray(n_per_traj, dtype=np.int32)
    h = get_handle(ens.device)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
    t0 = time.perf_counter()
    if dense:
        status = L.ode_solve_ensemble_dense(h, C.byref(d), C.byref(o), N, dp(u0s), dp(ps), dp(tspans), dp(t_out),
                                            dp(u_out), dp(k_out), ip(nsaved), ip(rc),
                                            stats.ctypes.data_as(C.POINTER(_lib.Stats)))
    else:
        status = L.ode_solve_ensemble(h, C.byref(d), C.byref(o), N, ip(npt) if npt is not None else None,
                                      dp(u0s), dp(ps), dp(tspans), dp(sv.values) if sv.nsave else None,
                                      dp(t_out), dp(u_out), ip(nsaved), ip(rc),
                                      stats.ctypes.data_as(C.POINTER(_lib.Stats)))
    elapsed = time.perf_counter() - t0
    _lib.check(status, h)
    names = ("nf", "njacs", "nw", "nsolve", "naccept", "nreject")
    if callback is not None and np.any(nsaved == cap):
        warnings.warn("some trajectories filled all %d save slots: raise max_events (their latest save is kept "
                      "in the last slot)" % cap)
    elif sv.everystep:
        lost = int(np.sum(stats[:, 4] + int(sv.save_start) + sv.nsave > cap))
        if lost:
            warnings.warn("%d trajectories took more than max_step_saves=%d steps; their middle steps were "
                          "dropped (the final point is kept)" % (lost, sv.max_step_saves))
    out = {"t": t_out, "u": u_out, "nsaved": nsaved, "retcode": rc,
           "stats": {k: stats[:, i] for i, k in enumerate(names)}, "elapsed": elapsed}
    if save_idxs is not None:
        out["save_idxs"] = np.atleast_1d(save_idxs).astype(np.int32)
    if dense:
        out["k"] = k_out
        out["dense"] = {"model": model, "alg": alg.alg_id, "p": ps, "device": ens.device}
    return out


def dense_eval(res, tq, device=None, deriv=0, continuity="left"):
    """sol_j(t) of a dense solve (solve_arrays(..., dense=True)) for every
    trajectory j at the query times tq, shared (nq,) or per trajectory (nq, N),
    evaluated on the GPU in FP64 (ode_dense_eval_deriv).  deriv=1 gives
    sol_j(t, Val{1}), the derivative of the interpolant; deriv=2 and 3
    sol_j(t, Val{2}) and sol_j(t, Val{3}) for Tsit5 and Rodas5P solutions.  A
    query at a saved time returns that save; continuity="right" takes the later
    of two saves at one time (an event's post-affect state).  Returns (nq, n, N)."""
    info = res.get("dense")
    if not info:
        raise ValueError("not a dense solve: pass dense=True")
    L = _lib.load()
    t, u, k, ns = res["t"], res["u"], res["k"], res["nsaved"]
    cap, n, N = u.shape
    ps = np.ascontiguousarray(info["p"], dtype=np.float64)
    tq = np.ascontiguousarray(np.atleast_1d(tq), dtype=np.float64)
    per = tq.ndim == 2
    if per and tq.shape[1] != N:
        raise ValueError("per-trajectory query times must have shape (nq, N)")
    nq = tq.shape[0]
    out = np.empty((nq, n, N))
    d = _lib.ProblemDesc(info["model"], info["alg"], n, ps.shape[0], 0, 0)
    h = get_handle(info["device"] if device is None else device)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    if continuity not in ("left", "right"):
        raise ValueError('continuity: "left" or "right"')
    _lib.check(L.ode_dense_eval_ex(h, C.byref(d), N, dp(ps), dp(t), dp(u), dp(k),
                                   ns.ctypes.data_as(C.POINTER(C.c_int32)), cap, nq, dp(tq), int(per), int(deriv),
                                   int(continuity == "right"), dp(out)), h)
    return out


def autotune(model, alg, ens, u0s, ps, tspans, saveat=None, reltol=1e-3, abstol=1e-6):
    """Time every compiled launch shape (lanes per trajectory, block size,
    scheduler) on this sample and keep the fastest for later solves of the same
    (alg, model, precision, n) on the ensemble's device handle (used when the
    EnsembleGB300 leaves lanes_per_traj, block_size and scheduler at auto)."""
    L = _lib.load()
    if isinstance(model, str):
        model = MODELS[model]
    u0s = np.ascontiguousarray(u0s, dtype=np.float64)
    ps = np.ascontiguousarray(ps, dtype=np.float64)
    tspans = np.ascontiguousarray(tspans, dtype=np.float64)
    n, N = u0s.shape
    sv = resolve_saveat(saveat, tspans)
    o = _options(reltol, abstol, None, None, None, 1000000, sv, ens, None, None)
    d = _lib.ProblemDesc(model, alg.alg_id, n, ps.shape[0], ens.prec_id(), 0)
    h = get_handle(ens.device)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    lanes, block, sched, ms = C.c_int32(0), C.c_int32(0), C.c_int32(0), C.c_double(0)
    _lib.check(L.ode_autotune(h, C.byref(d), C.byref(o), N, dp(u0s), dp(ps), dp(tspans),
                              dp(sv.values) if sv.nsave else None, C.byref(lanes), C.byref(block),
                              C.byref(sched), C.byref(ms)), h)
    return {"lanes_per_traj": lanes.value, "block_size": block.value,
            "scheduler": {1: "static", 2: "persistent"}.get(sched.value, sched.value), "ms": ms.value}


def solve(eprob, alg, ensemblealg=None, trajectories=None, batch_size=None, saveat=None, reltol=1e-3,
          abstol=1e-6, dt=None, dtmax=None, dtmin=None, maxiters=1000000, save_start=None, save_end=None,
          seed=0, qmax_first_step=None, qmax=None, save_everystep=None, max_step_saves=1024, dense=None,
          callback=None, tstops=None, save_idxs=None, adaptive=True, controller=None, force_dtmin=False,
          isoutofdomain=None):
    """solve(EnsembleProblem, alg, EnsembleGB300(); trajectories, saveat, reltol, abstol, ...).
    As in the reference (solve.jl:138-146), save_everystep defaults to "no
    saveat given" (every accepted step is kept, up to max_step_saves per
    trajectory) and dense to save_everystep without saveat (each step's
    interpolant; a callback's saves keep them as well); ensembles of uneven
    sizes are not dense by default.  callback: the model's ContinuousCallback or
    DiscreteCallback.  tstops: times every trajectory steps to exactly.
    save_idxs: the states saved (0-based); no dense output with it."""
    no_saveat = saveat is None or (not np.isscalar(saveat) and np.size(saveat) == 0)
    if save_everystep is None:
        save_everystep = no_saveat
    dense_default = dense is None
    if dense is None:
        dense = bool(save_everystep and no_saveat and save_idxs is None)
    ens = ensemblealg or EnsembleGB300()
    if not isinstance(ens, EnsembleGB300):
        raise TypeError("ensemble algorithm must be EnsembleGB300")
    prob = eprob.prob
    t_start = time.perf_counter()
    if eprob.u0s is not None:
        N = eprob.u0s.shape[1]
        if trajectories is not None and trajectories != N:
            raise ValueError("trajectories does not match the packed inputs")
        u0s = eprob.u0s
        ps = eprob.ps if eprob.ps is not None else np.repeat(prob.p[:, None], N, axis=1)
        tspans = eprob.tspans if eprob.tspans is not None else np.repeat(np.array(prob.tspan)[:, None], N, axis=1)
        res = solve_arrays(prob.model, alg, ens, u0s, ps, tspans, saveat, reltol, abstol, dt, dtmax, dtmin,
                           maxiters, save_start, save_end, eprob.n_per_traj, qmax_first_step, qmax,
                           save_everystep=save_everystep, max_step_saves=max_step_saves,
                           dense=dense and not (dense_default and eprob.n_per_traj is not None), callback=callback,
                           tstops=tstops, save_idxs=save_idxs, adaptive=adaptive, controller=controller,
                           force_dtmin=force_dtmin, isoutofdomain=isoutofdomain)
        sols = _LazySolutions(res, alg, eprob.n_per_traj)
        return EnsembleSolution(sols, time.perf_counter() - t_start, True, res)
    if trajectories is None:
        raise ValueError("trajectories is required")
    batch_size = batch_size or trajectories
    output_func = eprob.output_func or _default_output
    reduction = eprob.reduction or _default_reduction
    u = eprob.u_init if eprob.u_init is not None else []
    converged = False
    root = np.random.SeedSequence(seed)
    done = 0
    while done < trajectories:
        ids = list(range(done, min(trajectories, done + batch_size)))
        outs = _solve_batch(eprob, alg, ens, ids, root, saveat, reltol, abstol, dt, dtmax, dtmin, maxiters,
                            save_start, save_end, output_func, qmax_first_step, qmax, save_everystep, max_step_saves,
                            dense, dense_default, callback, tstops, save_idxs, adaptive, controller, force_dtmin,
                            isoutofdomain)
        u, converged = reduction(u, outs, range(ids[0] + 1, ids[-1] + 2))
        done = ids[-1] + 1
        if converged:
            break
    return EnsembleSolution(u, time.perf_counter() - t_start, converged)


def _solve_batch(eprob, alg, ens, ids, root, saveat, reltol, abstol, dt, dtmax, dtmin, maxiters, save_start,
                 save_end, output_func, qmax_first_step, qmax, save_everystep=False, max_step_saves=1024,
                 dense=False, dense_default=True, callback=None, tstops=None, save_idxs=None, adaptive=True,
                 controller=None, force_dtmin=False, isoutofdomain=None):
    repeat = {i: 1 for i in ids}
    results = {}
    todo = list(ids)
    while todo:
        probs, ctxs = [], []
        for i in todo:
            rng = np.random.default_rng(np.random.SeedSequence([root.entropy, i, repeat[i]]))
            ctx = EnsembleContext(i + 1, repeat[i], rng)
            pi = eprob.prob_func(eprob.prob, ctx) if eprob.prob_func else eprob.prob
            probs.append(pi)
            ctxs.append(ctx)
        n = max(pp.u0.size for pp in probs)
        if any(pp.model != probs[0].model for pp in probs):
            raise ValueError("all trajectories of an ensemble must use the same model")
        N = len(probs)
        u0s = np.zeros((n, N))
        npt = None
        if any(pp.u0.size != n for pp in probs):
            npt = np.array([pp.u0.size for pp in probs], dtype=np.int32)
        for k, pp in enumerate(probs):
            u0s[:pp.u0.size, k] = pp.u0
        ps = np.stack([pp.p for pp in probs], axis=1)
        tspans = np.array([pp.tspan for pp in probs]).T
        res = solve_arrays(probs[0].model, alg, ens, u0s, ps, tspans, saveat, reltol, abstol, dt, dtmax, dtmin,
                           maxiters, save_start, save_end, npt, qmax_first_step, qmax,
                           save_everystep=save_everystep, max_step_saves=max_step_saves,
                           dense=dense and not (dense_default and npt is not None), callback=callback,
                           tstops=tstops, save_idxs=save_idxs, adaptive=adaptive, controller=controller,
                           force_dtmin=force_dtmin, isoutofdomain=isoutofdomain)
        sols = _LazySolutions(res, alg, npt)
        again = []
        for k, i in enumerate(todo):
            s = sols[k]
            s.prob = probs[k]
            out, rerun = output_func(s, ctxs[k])
            if rerun:
                repeat[i] += 1
                again.append(i)
            else:
                results[i] = out
        todo = again
    return [results[i] for i in ids]
