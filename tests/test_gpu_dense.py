"""GPU parity of dense output (the reference's dense = true, its default without
saveat): every accepted step is saved with the method's interpolation vectors
(save_dense_at_t!, lib/OrdinaryDiffEqCore/src/integrators/integrator_utils.jl:455-473)
and sol(t) evaluates the interpolant between saves as ode_interpolation does
(lib/OrdinaryDiffEqCore/src/dense/generic_dense.jl:1094-1190).

Checked against the oracle's dense record and its sol(t), and through
properties that hold at any size: sol(t_i) reproduces the saved u_i, and sol(t)
equals the saveat interpolant of a solve with the same steps.
"""
import numpy as np
import pytest

import pyoracle as O
from gpu_common import ALG, MODEL, brusselator_inputs, duffing_inputs, gpu, lorenz_inputs, robertson_inputs
from odegb300 import dense_eval

pytestmark = pytest.mark.gpu


def inputs(model, N, seed):
    if model == "lorenz":
        return lorenz_inputs(N, seed=seed)
    if model == "robertson":
        return robertson_inputs(N, seed=seed)
    if model == "duffing_chain":
        u0, p, ts, _, _ = duffing_inputs(N, 8, seed=seed, tf_range=(1.0, 10.0))
        return u0, p, ts
    return brusselator_inputs(N, cells=8, seed=seed)


CASES = [("lorenz", "tsit5", 1e-8, 1e-8), ("lorenz", "vern7", 1e-8, 1e-8), ("robertson", "rodas5p", 1e-6, 1e-10),
         ("duffing_chain", "vern7", 1e-6, 1e-6), ("brusselator_1d", "rodas5p", 1e-5, 1e-8)]


@pytest.mark.parametrize("model,alg,rt,at", CASES)
def test_dense_steps_and_sol_t_match_oracle(model, alg, rt, at):
    N = 32
    u0, p, ts = inputs(model, N, 5)
    n = u0.shape[0]
    g = gpu(model, alg, u0, p, ts, None, rt, at, save_everystep=True, max_step_saves=4096, dense=True)
    rng = np.random.default_rng(1)
    tq = ts[0] + (ts[1] - ts[0]) * rng.uniform(0.0, 1.0, (24, N))
    tq[0], tq[1] = ts[0], ts[1]
    ev = dense_eval(g, tq)
    same_steps = 0
    for j in range(N):
        o = O.solve(ALG[alg][1], MODEL[model], u0[:, j], p[:, j], ts[:, j], dense=True, reltol=rt, abstol=at,
                    saveat_given=False, save_everystep=True, max_step_saves=4096, save_start=True, save_end=True)
        D = o["dense"]
        ns = int(g["nsaved"][j])
        # sol(t) at the queries: within 10 (reltol |u| + abstol) of the oracle's sol(t)
        ref = D(tq[:, j])
        assert np.all(np.abs(ev[:, :, j] - ref) <= 10 * (rt * np.abs(ref) + at)), (j, ev[:, :, j], ref)
        if D.nsteps + 1 != ns:
            continue
        # FP64 on both sides, but FMA contraction (and the LU's rounding) differs: the
        # step times drift apart slowly; compare the stored vectors step by step where
        # the two step sequences still coincide to 1e-9
        tends = np.array([D.step(s)[1] for s in range(ns - 1)])
        if np.max(np.abs(g["t"][1:ns, j] - tends) / np.abs(tends).clip(1e-300)) > 1e-9:
            continue
        same_steps += 1
        for s in range(1, ns):
            tprev, tend, y0, y1, ko = D.step(s - 1)
            kg = g["k"][s, :, :, j]
            # relative to the step's largest vector: a cancelling combination (Rodas5P's
            # third dense vector) is small next to the others and carries their rounding
            scale = np.abs(ko).max() + 1e-300
            assert np.all(np.abs(kg - ko) <= 1e-5 * scale), (j, s, kg, ko)
    assert same_steps >= 1
    # the start save carries no step
    assert np.all(g["k"][0] == 0.0)
    # sol(t_i) reproduces the saved u_i (left continuity: theta = 1 on the step ending at t_i)
    for j in range(0, N, 7):
        ns = int(g["nsaved"][j])
        at_saves = dense_eval({**g, "t": g["t"][:, j:j + 1].copy(), "u": g["u"][:, :, j:j + 1].copy(),
                               "k": g["k"][..., j:j + 1].copy(), "nsaved": g["nsaved"][j:j + 1].copy(),
                               "dense": dict(g["dense"], p=g["dense"]["p"][:, j:j + 1].copy())},
                              g["t"][:ns, j])[:, :, 0]
        saved = g["u"][:ns, :n, j]
        assert np.all(np.abs(at_saves - saved) <= 1e-9 * (np.abs(saved) + np.abs(saved).max() + 1e-300))


def test_dense_eval_equals_the_saveat_interpolant():
    # saveat changes no step, so sol(t) of a dense solve and the saveat values of a
    # saveat solve evaluate the same polynomial (up to theta's rounding), except in
    # the final step clipped to tf, where the saveat path interpolates with the
    # unclipped dt that the reference restores before savevalues!
    # (integrator_utils.jl:626-631)
    N = 256
    u0, p, ts = lorenz_inputs(N, seed=9)
    sv = np.arange(1, 20) * 0.05
    a = gpu("lorenz", "tsit5", u0, p, ts, sv, 1e-8, 1e-8)
    b = gpu("lorenz", "tsit5", u0, p, ts, None, 1e-8, 1e-8, save_everystep=True, max_step_saves=4096, dense=True)
    assert np.array_equal(a["stats"]["naccept"], b["stats"]["naccept"])
    ev = dense_eval(b, sv)
    last_start = b["t"][b["nsaved"] - 2, np.arange(N)]
    inner = sv[:, None] <= last_start[None, :]
    got = np.transpose(ev, (0, 2, 1))[inner]
    want = np.transpose(a["u"][:sv.size], (0, 2, 1))[inner]
    assert inner.sum() > 0.8 * inner.size
    assert np.all(np.abs(got - want) <= 1e-12 * (np.abs(want) + 1.0))


def test_mixed_dense_is_within_tolerance_of_fp64():
    N = 256
    u0, p, ts = robertson_inputs(N, seed=11)
    rt, at = 1e-6, 1e-10
    f = gpu("robertson", "rodas5p", u0, p, ts, None, rt, at, save_everystep=True, max_step_saves=4096, dense=True)
    m = gpu("robertson", "rodas5p", u0, p, ts, None, rt, at, precision="mixed", save_everystep=True,
            max_step_saves=4096, dense=True)
    tq = 10.0 ** np.linspace(-4.0, 5.0, 40)
    a, b = dense_eval(f, tq), dense_eval(m, tq)
    assert np.all(np.isfinite(b))
    ratio = np.abs(a - b) / (rt * np.abs(a) + at)
    assert np.percentile(ratio, 99) < 20.0 and ratio.max() < 200.0, (np.percentile(ratio, 99), ratio.max())


def test_dense_overflow_marks_the_last_interval():
    # more steps than slots: the last slot keeps the final point with NaN vectors,
    # so sol(t) in the last (gapped) interval is NaN and elsewhere exact
    N = 64
    u0, p, ts = lorenz_inputs(N, seed=8)
    with pytest.warns(UserWarning, match="max_step_saves"):
        g = gpu("lorenz", "tsit5", u0, p, ts, None, 1e-8, 1e-8, save_everystep=True, max_step_saves=5, dense=True)
    assert (g["nsaved"] == 7).all()
    assert np.isnan(g["k"][6]).all() and np.isfinite(g["k"][1:6]).all()
    full = gpu("lorenz", "tsit5", u0, p, ts, None, 1e-8, 1e-8, save_everystep=True, max_step_saves=4096, dense=True)
    tq = np.vstack([0.5 * (g["t"][2] + g["t"][3]), 0.5 * (g["t"][5] + g["t"][6])])
    ev, ref = dense_eval(g, tq), dense_eval(full, tq)
    assert np.array_equal(ev[0], ref[0])
    assert np.isnan(ev[1]).all()


def test_solution_call_uses_the_dense_interpolant():
    from odegb300 import EnsembleGB300, EnsembleProblem, ODEProblem, Vern7, remake, solve
    prob = ODEProblem("lorenz", [1.0, 0.0, 0.0], (0.0, 1.0), [10.0, 14.0, 8.0 / 3.0])
    ep = EnsembleProblem(prob, prob_func=lambda pr, ctx: remake(pr, p=[10.0, 10.0 + ctx.sim_id, 8.0 / 3.0]))
    sim = solve(ep, Vern7(), EnsembleGB300(), trajectories=6, reltol=1e-8, abstol=1e-8)   # no saveat: dense
    sol = sim.u[3]
    assert sol.dense
    tq = np.array([0.0, 0.123, 0.5, 0.999, 1.0])
    vals = sol(tq)
    assert vals.shape == (5, 3) and np.allclose(sol(0.5), vals[2], rtol=0, atol=0)
    o = O.solve(O.VERN7, O.LORENZ, np.array([1.0, 0.0, 0.0]), np.array([10.0, 14.0, 8.0 / 3.0]), (0.0, 1.0),
                dense=True, reltol=1e-8, abstol=1e-8, saveat_given=False, save_everystep=True,
                max_step_saves=4096, save_start=True, save_end=True)
    ref = o["dense"](tq)
    assert np.all(np.abs(vals - ref) <= 10 * (1e-8 * np.abs(ref) + 1e-8))
    # with saveat the solution is not dense: linear interpolation between saves
    sim2 = solve(ep, Vern7(), EnsembleGB300(), trajectories=2, saveat=0.5, reltol=1e-8, abstol=1e-8)
    s2 = sim2.u[0]
    assert not s2.dense and np.allclose(s2(0.25), 0.5 * (np.asarray(s2.u[0]) + np.asarray(s2.u[1])))


def test_page_locked_dense_eval_output_is_identical():
    import ctypes as C
    import torch
    from odegb300 import _lib
    from odegb300.ensemble import get_handle
    N = 200
    u0, p, ts = lorenz_inputs(N, seed=12)
    g = gpu("lorenz", "tsit5", u0, p, ts, None, 1e-8, 1e-8, save_everystep=True, max_step_saves=512, dense=True)
    tq = np.linspace(0.0, 1.0, 37)
    staged = dense_eval(g, tq)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    h_p, h_t, h_u, h_k, h_ns, h_tq = (pin(g["dense"]["p"]), pin(g["t"]), pin(g["u"]), pin(g["k"]), pin(g["nsaved"]),
                                      pin(tq))
    h_out = torch.empty((tq.size, 3, N), dtype=torch.float64).pin_memory()
    ptr = lambda t, ty=C.c_double: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ty))
    L = _lib.load()
    h = get_handle(0)
    d = _lib.ProblemDesc(g["dense"]["model"], g["dense"]["alg"], 3, 3, 0, 0)
    _lib.check(L.ode_dense_eval(h, C.byref(d), N, ptr(h_p), ptr(h_t), ptr(h_u), ptr(h_k), ptr(h_ns, C.c_int32),
                                g["t"].shape[0], tq.size, ptr(h_tq), 0, ptr(h_out)), h)
    assert np.array_equal(h_out.numpy(), staged)


@pytest.mark.parametrize("model,alg,rt,at", [("lorenz", "tsit5", 1e-8, 1e-8), ("lorenz", "vern7", 1e-8, 1e-8),
                                             ("robertson", "rodas5p", 1e-6, 1e-10),
                                             ("lorenz", "rosenbrock23", 1e-6, 1e-8)])
def test_dense_derivative_matches_oracle(model, alg, rt, at):
    # sol(t, Val{1}) on the device (ode_dense_eval_deriv) against the oracle's, and
    # against the derivative of the device's own interpolant (a polynomial in theta on
    # each step, fitted from its values inside the step)
    N = 32
    u0, p, ts = inputs(model, N, 7)
    n = u0.shape[0]
    g = gpu(model, alg, u0, p, ts, None, rt, at, save_everystep=True, max_step_saves=4096, dense=True)
    rng = np.random.default_rng(3)
    tq = ts[0] + (ts[1] - ts[0]) * rng.uniform(0.0, 1.0, (16, N))
    der = dense_eval(g, tq, deriv=1)
    deg = {"tsit5": 4, "vern7": 7, "rodas5p": 4, "rosenbrock23": 2}[alg]
    for j in range(N):
        o = O.solve(ALG[alg][1], MODEL[model], u0[:, j], p[:, j], ts[:, j], dense=True, reltol=rt, abstol=at,
                    saveat_given=False, save_everystep=True, max_step_saves=4096, save_start=True, save_end=True)
        ref = o["dense"](tq[:, j], deriv=1)
        scale = np.abs(ref).max(axis=0) + 1e-300
        assert np.all(np.abs(der[:, :, j] - ref) <= 1e-4 * scale + 10 * at), j
        ns = int(g["nsaved"][j])
        tj = g["t"][:ns, j]
        for r in range(0, 16, 5):
            ip = max(1, int(np.searchsorted(tj, tq[r, j], side="left")))
            a, b = tj[ip - 1], tj[ip]
            x = a + (b - a) * np.linspace(0.1, 1.0, 3 * deg)
            vals = dense_eval(g, np.tile(x[:, None], (1, N)))[:, :, j]
            th = (tq[r, j] - a) / (b - a)
            for i in range(n):
                c = np.polyfit((x - a) / (b - a), vals[:, i], deg)
                want = np.polyval(np.polyder(c), th) / (b - a)
                assert der[r, i, j] == pytest.approx(want, rel=1e-7, abs=1e-9 * scale[i] + 1e-12), (j, r, i)


def test_dense_derivative_order_checks():
    from odegb300 import _lib
    from odegb300.ensemble import get_handle
    import ctypes as C
    L = _lib.load()
    d = _lib.ProblemDesc(_lib.MODEL_LORENZ, _lib.ODE_TSIT5, 3, 3, _lib.PREC_FP64, 0)
    h = get_handle(0)
    x = np.zeros(8)
    dp = x.ctypes.data_as(C.POINTER(C.c_double))
    ns = np.ones(1, dtype=np.int32)
    ip = ns.ctypes.data_as(C.POINTER(C.c_int32))
    assert L.ode_dense_eval_deriv(h, C.byref(d), 1, dp, dp, dp, dp, ip, 1, 1, dp, 0, 4, dp) == -4
    assert L.ode_dense_eval_deriv(h, C.byref(d), 1, dp, dp, dp, dp, ip, 1, 1, dp, 0, -1, dp) == -1
    # Val{2} exists for Tsit5 and Rodas5P only, as in the reference's interpolants
    for alg in (_lib.ODE_VERN7, _lib.ODE_ROSENBROCK23):
        d2 = _lib.ProblemDesc(_lib.MODEL_LORENZ, alg, 3, 3, _lib.PREC_FP64, 0)
        assert L.ode_dense_eval_deriv(h, C.byref(d2), 1, dp, dp, dp, dp, ip, 1, 1, dp, 0, 2, dp) == -4


@pytest.mark.parametrize("model,alg,rt", [("lorenz", "tsit5", 1e-8), ("duffing_chain", "tsit5", 1e-6),
                                          ("lorenz", "rodas5p", 1e-6), ("brusselator_1d", "rodas5p", 1e-5)])
def test_dense_second_derivative_matches_oracle(model, alg, rt):
    # sol(t, Val{2}) on the device against the oracle's (the same arithmetic on the same
    # step data: equal to rounding), and against central differences of sol(t, Val{1})
    N = 32
    u0, p, ts = inputs(model, N, 8)
    g = gpu(model, alg, u0, p, ts, None, rt, rt, save_everystep=True, max_step_saves=4096, dense=True)
    rng = np.random.default_rng(4)
    tq = ts[0] + (ts[1] - ts[0]) * rng.uniform(0.05, 0.95, (12, N))
    d2 = dense_eval(g, tq, deriv=2)
    d3 = dense_eval(g, tq, deriv=3)
    for j in range(N):
        o = O.solve(ALG[alg][1], MODEL[model], u0[:, j], p[:, j], ts[:, j], dense=True, reltol=rt, abstol=rt,
                    saveat_given=False, save_everystep=True, max_step_saves=4096, save_start=True, save_end=True)
        for dv, ref in ((d2, o["dense"](tq[:, j], deriv=2)), (d3, o["dense"](tq[:, j], deriv=3))):
            scale = np.abs(ref).max(axis=0) + 1e-300
            assert np.all(np.abs(dv[:, :, j] - ref) <= 1e-4 * scale + 10 * rt), j
    h = 1e-7 * np.abs(ts[1] - ts[0]).max()
    fd = (dense_eval(g, tq + h, deriv=1) - dense_eval(g, tq - h, deriv=1)) / (2 * h)
    sc = np.abs(d2).max(axis=0, keepdims=True) + 1e-300
    # a query within h of a step boundary straddles two interpolants: most agree closely
    assert (np.abs(d2 - fd) <= 1e-3 * sc).mean() > 0.95
