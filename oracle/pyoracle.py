"""TEST INFRASTRUCTURE — ctypes binding of the CPU oracle (liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, as the checker.  The product never imports it.  See oracle.h for what
the oracle restates and how far its parity is pinned.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

TSIT5, VERN7, RODAS5P, VERN9, ROSENBROCK23, AUTOTSIT5_ROSENBROCK23 = 0, 1, 2, 3, 4, 5
LINEAR, LORENZ, ROBERTSON, DUFFING, BRUSSELATOR, BOUNCING_BALL, VANDERPOL, PK1, FORCED_DUFFING = 0, 1, 2, 3, 4, 5, 6, 7, 8
LOTKA_VOLTERRA, OREGONATOR, BALL_BOX, THRESHOLD_DOSE = 9, 10, 11, 12
RC_DEFAULT, RC_SUCCESS, RC_MAXITERS, RC_DTNAN, RC_DTLESSTHANMIN, RC_UNSTABLE = range(6)
RC_TERMINATED = 7


class Stats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("nf", "njacs", "nw", "nsolve", "naccept", "nreject")]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Opts(C.Structure):
    _fields_ = [
        ("reltol", C.c_double), ("abstol", C.c_double), ("dtmax", C.c_double),
        ("dtmin", C.c_double), ("dt", C.c_double), ("adaptive", C.c_int32),
        ("maxiters", C.c_int64), ("save_start", C.c_int32), ("save_end", C.c_int32),
        ("save_end_user", C.c_int32), ("saveat_given", C.c_int32), ("saveat_scalar", C.c_int32),
        ("qmax_first_step", C.c_double), ("qmax", C.c_double), ("saveat_as_tstops", C.c_int32),
        ("save_everystep", C.c_int32), ("max_step_saves", C.c_int32),
        ("callback", C.c_int32), ("interp_points", C.c_int32), ("max_events", C.c_int32), ("ntstops", C.c_int32),
        ("tstops", C.POINTER(C.c_double)), ("max_jac_age", C.c_int32), ("jac_reuse_gamma_tol", C.c_double),
        ("ctrl_given", C.c_int32), ("c_beta1", C.c_double), ("c_beta2", C.c_double), ("c_qoldinit", C.c_double),
        ("c_qmin", C.c_double), ("c_gamma", C.c_double), ("c_qsteady_min", C.c_double),
        ("c_qsteady_max", C.c_double), ("force_dtmin", C.c_int32), ("abstol_vec", C.POINTER(C.c_double)),
        ("reltol_vec", C.POINTER(C.c_double)), ("isoutofdomain", C.c_int32),
    ]


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        L.orc_solve.restype = C.c_int
        L.orc_solve.argtypes = [C.c_int, C.c_int, C.c_int, dp, C.c_double, C.c_double, dp,
                                C.POINTER(Opts), dp, C.c_int, dp, C.c_int, dp, dp, C.c_int,
                                C.POINTER(C.c_int32), C.POINTER(Stats), C.POINTER(C.c_void_p)]
        L.orc_dense_eval.argtypes = [C.c_void_p, dp, C.c_int, dp]
        L.orc_dense_eval_deriv.argtypes = [C.c_void_p, dp, C.c_int, C.c_int, dp]
        L.orc_dense_eval_ex.argtypes = [C.c_void_p, dp, C.c_int, C.c_int, C.c_int, dp]
        L.orc_dense_free.argtypes = [C.c_void_p]
        L.orc_dense_nsteps.argtypes = [C.c_void_p]
        L.orc_dense_step.restype = C.c_int
        L.orc_dense_step.argtypes = [C.c_void_p, C.c_int, dp, dp, dp, dp]
        L.orc_solve_ensemble.restype = C.c_int
        L.orc_solve_ensemble.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32), C.c_int,
                                         C.c_int64, dp, dp, dp, C.POINTER(Opts), dp, C.c_int, C.c_int,
                                         dp, dp, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                         C.POINTER(Stats), C.c_int]
        L.orc_last_alg_choice.restype = C.c_int
        L.orc_last_alg_choice.argtypes = [C.POINTER(C.c_int32), C.c_int]
        L.orc_rhs_calls.restype = C.c_int64
        L.orc_rhs_calls.argtypes = [C.c_int]
        L.orc_initdt.restype = C.c_double
        L.orc_initdt.argtypes = [C.c_int, C.c_int, C.c_int, dp, C.c_double, C.c_double, dp, C.POINTER(Opts), dp,
                                 C.c_int]
        L.orc_record_eval_times.argtypes = [C.c_int]
        L.orc_eval_times.restype = C.c_int
        L.orc_eval_times.argtypes = [dp, C.c_int]
        L.orc_rhs.argtypes = [C.c_int, C.c_int, dp, dp, C.c_double, dp]
        L.orc_jac.argtypes = [C.c_int, C.c_int, dp, dp, C.c_double, dp]
        L.orc_tgrad.restype = C.c_int
        L.orc_tgrad.argtypes = [C.c_int, C.c_int, dp, dp, C.c_double, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_opts(reltol=1e-3, abstol=1e-6, dtmax=0.0, dtmin=0.0, dt=0.0, adaptive=True,
              maxiters=1000000, save_start=False, save_end=True, save_end_user=-1,
              saveat_given=True, saveat_scalar=False, qmax_first_step=0.0, qmax=0.0, saveat_as_tstops=False,
              save_everystep=False, max_step_saves=0, callback=False, interp_points=10, max_events=0,
              tstops=(), max_jac_age=1, jac_reuse_gamma_tol=0.03, controller=None, force_dtmin=False,
              isoutofdomain=0):
    ts = np.ascontiguousarray(tstops, dtype=np.float64).ravel()
    # array tolerances: one per state (the scalars then stand unused)
    av = np.ascontiguousarray(abstol, dtype=np.float64).ravel() if np.ndim(abstol) else None
    rv = np.ascontiguousarray(reltol, dtype=np.float64).ravel() if np.ndim(reltol) else None
    abstol = float(av[0]) if av is not None else abstol
    reltol = float(rv[0]) if rv is not None else reltol
    o = Opts(reltol, abstol, dtmax, dtmin, dt, int(adaptive), maxiters, int(save_start),
             int(save_end), save_end_user, int(saveat_given), int(saveat_scalar),
             qmax_first_step, qmax, int(saveat_as_tstops), int(save_everystep), int(max_step_saves),
             int(callback), int(interp_points), int(max_events), int(ts.size), _dp(ts) if ts.size else None,
             int(max_jac_age), float(jac_reuse_gamma_tol))
    if controller:   # dict of PIController knobs (beta1, beta2, qoldinit, qmin, gamma, qsteady_min, qsteady_max)
        o.ctrl_given = 1
        for k in ("beta1", "beta2", "qoldinit", "qmin", "gamma", "qsteady_min", "qsteady_max"):
            v = controller.get(k)
            setattr(o, "c_" + k, float("nan") if v is None else float(v))
    o.force_dtmin = int(bool(force_dtmin))
    o.isoutofdomain = int(isoutofdomain)
    if av is not None:
        o.abstol_vec = _dp(av)
    if rv is not None:
        o.reltol_vec = _dp(rv)
    o._keep = (ts, av, rv)   # keeps the arrays alive as long as the options
    return o


def solve(alg, model, u0, p, tspan, saveat=(), tstops=(), dense=False, **kw):
    """Solve one trajectory; returns dict(t, u, retcode, stats, dense).  dense
    keeps every step (the reference's dense output saves every step: its
    default save_everystep = isempty(saveat))."""
    L = lib()
    if dense and "save_everystep" not in kw:
        kw["save_everystep"] = True
        kw.setdefault("max_step_saves", 65536)
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    p = np.ascontiguousarray(np.atleast_1d(p), dtype=np.float64)
    n = u0.size
    sv = np.ascontiguousarray(saveat, dtype=np.float64)
    ts = np.ascontiguousarray(tstops, dtype=np.float64)
    cap = sv.size + 2
    if kw.get("saveat_given", True) is False or sv.size == 0:
        cap = 4
    if kw.get("save_everystep"):
        cap = sv.size + kw.get("max_step_saves", 0) + 2
    if kw.get("callback"):
        cap += 2 * max(kw.get("max_events", 0), 64)
    t_out = np.zeros(cap)
    u_out = np.zeros((cap, n))
    rc = C.c_int32(0)
    st = Stats()
    h = C.c_void_p(0)
    o = make_opts(**kw)
    ns = L.orc_solve(alg, model, n, _dp(p), tspan[0], tspan[1], _dp(u0), C.byref(o),
                     _dp(sv) if sv.size else None, sv.size, _dp(ts) if ts.size else None, ts.size,
                     _dp(t_out), _dp(u_out), cap, C.byref(rc), C.byref(st),
                     C.byref(h) if dense else None)
    ns = min(ns, cap)
    out = {"t": t_out[:ns].copy(), "u": u_out[:ns].copy(), "retcode": rc.value, "stats": st.as_dict()}
    if dense:
        out["dense"] = DenseSolution(h, n)
    if alg == AUTOTSIT5_ROSENBROCK23:
        ch = np.zeros(cap, dtype=np.int32)
        m = L.orc_last_alg_choice(ch.ctypes.data_as(C.POINTER(C.c_int32)), cap)
        out["alg_choice"] = ch[:m].copy()
    return out


class DenseSolution:
    def __init__(self, h, n):
        self.h, self.n = h, n

    def __call__(self, ts, deriv=0, continuity="left"):
        ts = np.ascontiguousarray(np.atleast_1d(ts), dtype=np.float64)
        out = np.zeros((ts.size, self.n))
        rc = lib().orc_dense_eval_ex(self.h, _dp(ts), ts.size, int(deriv), int(continuity == "right"), _dp(out))
        if rc != 0:
            raise ValueError("dense evaluation failed (%d): derivative order %d" % (rc, deriv))
        return out

    @property
    def nsteps(self):
        return lib().orc_dense_nsteps(self.h)

    def step(self, s):
        """(tprev, tend, y0, y1, k) of step s; k (nk, n) in the library's dense order."""
        t2, y0, y1 = np.zeros(2), np.zeros(self.n), np.zeros(self.n)
        k = np.zeros((16, self.n))
        nk = lib().orc_dense_step(self.h, s, _dp(t2), _dp(y0), _dp(y1), _dp(k))
        if nk < 0:
            raise IndexError(s)
        return t2[0], t2[1], y0, y1, k[:nk].copy()

    def __del__(self):
        try:
            lib().orc_dense_free(self.h)
        except Exception:
            pass


def solve_ensemble(alg, model, u0, p, tspan, saveat, reltol, abstol, n_per_traj=None,
                   saveat_per_traj=False, nthreads=0, **kw):
    """SoA ensemble solve.  u0: (nmax, N), p: (np, N), tspan: (2, N),
    saveat: (nsave,) or (nsave, N).  Returns dict of SoA outputs."""
    L = lib()
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    tspan = np.ascontiguousarray(tspan, dtype=np.float64)
    sv = np.ascontiguousarray(saveat, dtype=np.float64)
    nmax, N = u0.shape
    nsave = sv.shape[0]
    cap = nsave + (kw.get("max_step_saves", 0) if kw.get("save_everystep") else 0) + 2 + \
        (2 * kw.get("max_events", 0) if kw.get("callback") else 0)
    t_out = np.full((cap, N), np.nan)
    u_out = np.full((cap, nmax, N), np.nan)
    nsaved = np.zeros(N, dtype=np.int32)
    rc = np.zeros(N, dtype=np.int32)
    stats = (Stats * N)()
    npt = None
    if n_per_traj is not None:
        npt = np.ascontiguousarray(n_per_traj, dtype=np.int32)
    o = make_opts(reltol=reltol, abstol=abstol, **kw)
    L.orc_solve_ensemble(alg, model, nmax, npt.ctypes.data_as(C.POINTER(C.c_int32)) if npt is not None else None,
                         p.shape[0], N, _dp(u0), _dp(p), _dp(tspan), C.byref(o), _dp(sv), nsave,
                         int(saveat_per_traj), _dp(t_out), _dp(u_out),
                         nsaved.ctypes.data_as(C.POINTER(C.c_int32)), rc.ctypes.data_as(C.POINTER(C.c_int32)),
                         stats, nthreads)
    st = np.array([[getattr(stats[j], k) for k, _ in Stats._fields_] for j in range(N)], dtype=np.int64)
    return {"t": t_out, "u": u_out, "nsaved": nsaved, "retcode": rc,
            "stats": {k: st[:, i] for i, (k, _) in enumerate(Stats._fields_)}}


def rhs(model, u, p, t=0.0):
    u = np.ascontiguousarray(u, dtype=np.float64)
    p = np.ascontiguousarray(np.atleast_1d(p), dtype=np.float64)
    du = np.zeros_like(u)
    lib().orc_rhs(model, u.size, _dp(u), _dp(p), t, _dp(du))
    return du


def jac(model, u, p, t=0.0):
    u = np.ascontiguousarray(u, dtype=np.float64)
    p = np.ascontiguousarray(np.atleast_1d(p), dtype=np.float64)
    J = np.zeros((u.size, u.size))
    lib().orc_jac(model, u.size, _dp(u), _dp(p), t, _dp(J))
    return J


def tgrad(model, u, p, t=0.0):
    """df/dt of a non-autonomous model, or None for an autonomous one."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    p = np.ascontiguousarray(np.atleast_1d(p), dtype=np.float64)
    dT = np.zeros_like(u)
    return dT if lib().orc_tgrad(model, u.size, _dp(u), _dp(p), t, _dp(dT)) else None


def rhs_calls(reset=False):
    return lib().orc_rhs_calls(int(reset))


def initdt(alg, model, u0, p, tspan, tstops=(), **kw):
    """The signed initial step of a solve (ode_determine_initdt)."""
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    p = np.ascontiguousarray(np.atleast_1d(p), dtype=np.float64)
    ts = np.ascontiguousarray(tstops, dtype=np.float64)
    o = make_opts(**kw)
    return lib().orc_initdt(alg, model, u0.size, _dp(p), tspan[0], tspan[1], _dp(u0), C.byref(o),
                            _dp(ts) if ts.size else None, ts.size)


def record_eval_times(enable=True):
    lib().orc_record_eval_times(int(enable))


def eval_times():
    """The t of every RHS call since record_eval_times() (this thread)."""
    n = lib().orc_eval_times(None, 0)
    out = np.zeros(n)
    lib().orc_eval_times(_dp(out), n)
    return out
