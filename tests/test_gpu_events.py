"""GPU parity of the model's ContinuousCallback (events) against the CPU oracle:
event detection and the left root to adjacent floats (lib/DiffEqBase/src/
callbacks.jl:364-458, 480-492), apply_callback!'s saves before and after the
affect and terminate! (:557-643), and the reference's own event tests on the
falling ball (test/Integrators_I/ode_event_tests.jl:153-171, 283-360).
"""
import numpy as np
import pytest

import pyoracle as O
from gpu_common import ALG, gpu, oracle
from odegb300 import ContinuousCallback

pytestmark = pytest.mark.gpu


def balls(N, seed, t_stop=None):
    from odegb300 import workloads as W
    wl = W.bouncing_ball(N, seed=seed)
    if t_stop is not None:
        wl["p"][2] = t_stop
    return wl


@pytest.mark.parametrize("alg", ["tsit5", "vern7", "rodas5p", "rosenbrock23"])
def test_events_match_oracle_fp64(alg):
    N = 256
    wl = balls(N, seed=3)
    rt = at = 1e-8
    cb = ContinuousCallback(interp_points=10, max_events=8)
    g = gpu("bouncing_ball", alg, wl["u0"], wl["p"], wl["tspan"], 0.25, rt, at, callback=cb)
    o = oracle("bouncing_ball", alg, wl["u0"], wl["p"], wl["tspan"], 0.25, rt, at, callback=True, interp_points=10,
               max_events=8)
    assert np.array_equal(g["retcode"], o["retcode"])
    assert set(np.unique(g["retcode"])) == {1, 7}   # some terminated, the rest reached tf
    assert np.array_equal(g["nsaved"], o["nsaved"])
    ns = int(g["nsaved"].max())
    gt, ot = g["t"][:ns], o["t"][:ns]
    m = ~np.isnan(ot)
    # event times (saved twice) agree to a few ulps of the root; saveat times exactly
    assert np.all(np.abs(gt[m] - ot[m]) <= 1e-12 * np.abs(ot[m]) + 1e-14)
    gu, ou = g["u"][:ns], o["u"][:ns]
    mu = ~np.isnan(ou)
    assert np.all(np.abs(gu[mu] - ou[mu]) <= 10 * (rt * np.abs(ou[mu]) + at))
    # counters: the FSAL re-evaluation after an event is counted on both sides
    for k in ("nf", "naccept", "nreject", "njacs"):
        assert np.abs(g["stats"][k] - o["stats"][k]).max() <= 16, k


def test_events_mixed_match_fp64():
    N = 512
    wl = balls(N, seed=4)
    cb = ContinuousCallback(max_events=8)
    f = gpu("bouncing_ball", "tsit5", wl["u0"], wl["p"], wl["tspan"], 0.25, 1e-8, 1e-8, callback=cb)
    m = gpu("bouncing_ball", "tsit5", wl["u0"], wl["p"], wl["tspan"], 0.25, 1e-8, 1e-8, callback=cb,
            precision="mixed")
    assert np.array_equal(f["retcode"], m["retcode"]) and np.array_equal(f["nsaved"], m["nsaved"])
    ns = int(f["nsaved"].max())
    a, b = f["t"][:ns], m["t"][:ns]
    k = ~np.isnan(a)
    assert np.all(np.abs(a[k] - b[k]) <= 1e-6 * np.abs(a[k]) + 1e-9)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_terminate_at_ground_contact(precision):
    # ode_event_tests.jl:283-315: Terminated at t = sqrt(50*2/9.81), height < 3e-12
    N = 64
    u0 = np.tile([[50.0], [0.0]], (1, N))
    p = np.tile([[9.81], [1.0], [0.0]], (1, N))
    ts = np.tile([[0.0], [100.0]], (1, N))
    g = gpu("bouncing_ball", "tsit5", u0, p, ts, None, 1e-3, 1e-6, save_everystep=True, max_step_saves=64,
            callback=ContinuousCallback(interp_points=10, max_events=2), precision=precision)
    assert (g["retcode"] == 7).all()
    last = g["nsaved"] - 1
    t_end = g["t"][last, np.arange(N)]
    x_end = g["u"][last, 0, np.arange(N)]
    if precision == "fp64":
        assert np.allclose(t_end, np.sqrt(50 * 2 / 9.81), rtol=1e-12, atol=0)
        assert (np.abs(x_end) < 3e-12).all()
    else:
        assert np.allclose(t_end, np.sqrt(50 * 2 / 9.81), rtol=1e-6, atol=0)


def test_reference_bounce_then_terminate_and_both_sides_saved():
    # ode_event_tests.jl:332-360: reflect until t >= 3.5, then terminate! at
    # 3 sqrt(50*2/9.81) with the height below 1.3e-10; and :153-171: each event
    # time is saved twice, v < 0 before and v > 0 after the reflection
    N = 32
    u0 = np.tile([[50.0], [0.0]], (1, N))
    p = np.tile([[9.81], [1.0], [3.5]], (1, N))
    ts = np.tile([[0.0], [100.0]], (1, N))
    g = gpu("bouncing_ball", "tsit5", u0, p, ts, None, 1e-3, 1e-6, save_everystep=True, max_step_saves=128,
            callback=ContinuousCallback(interp_points=100, max_events=4))
    assert (g["retcode"] == 7).all()
    j = np.arange(N)
    last = g["nsaved"] - 1
    assert np.allclose(g["t"][last, j], 3 * np.sqrt(50 * 2 / 9.81), rtol=1e-12, atol=0)
    assert (np.abs(g["u"][last, 0, j]) < 1.3e-10).all()
    t0 = g["t"][:g["nsaved"][0], 0]
    te = np.sqrt(50 * 2 / 9.81)
    hit = np.nonzero(np.abs(t0 - te) < 1e-9)[0]
    assert len(hit) == 2
    assert g["u"][hit[0], 1, 0] < 0 < g["u"][hit[1], 1, 0]
    r = O.solve(O.TSIT5, O.BOUNCING_BALL, u0[:, 0], p[:, 0], ts[:, 0], saveat=[], saveat_given=False,
                callback=True, interp_points=100, save_everystep=True, max_step_saves=128, save_start=True,
                reltol=1e-3, abstol=1e-6)
    assert len(r["t"]) == g["nsaved"][0]
    assert np.allclose(r["t"], t0, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("alg", ["tsit5", "vern7", "rodas5p", "rosenbrock23"])
def test_events_with_dense_output_match_oracle(alg):
    # dense output with events: the event's step is recomputed shortened to the event
    # (reeval_internals_due_to_modification!), every save keeps the step's vectors, and
    # sol(t) on both sides of each contact matches the oracle's
    from odegb300 import dense_eval
    N = 64
    wl = balls(N, seed=5)
    rt = at = 1e-8 if alg != "rosenbrock23" else 1e-6
    cb = ContinuousCallback(interp_points=10, max_events=16)
    g = gpu("bouncing_ball", alg, wl["u0"], wl["p"], wl["tspan"], None, rt, at, callback=cb, save_everystep=True,
            max_step_saves=4096, dense=True)
    ts = wl["tspan"]
    rng = np.random.default_rng(4)
    tq = ts[0] + (ts[1] - ts[0]) * np.sort(rng.uniform(0.0, 1.0, (64, N)), axis=0)
    ev = dense_eval(g, tq)
    for j in range(N):
        o = O.solve(ALG[alg][1], O.BOUNCING_BALL, wl["u0"][:, j], wl["p"][:, j], ts[:, j], dense=True, reltol=rt,
                    abstol=at, saveat_given=False, save_everystep=True, max_step_saves=4096, save_start=True,
                    callback=True, interp_points=10, max_events=16)
        assert g["retcode"][j] == o["retcode"]
        ns = int(g["nsaved"][j])
        assert ns == len(o["t"])
        assert np.all(np.abs(g["t"][:ns, j] - o["t"]) <= 1e-12 * np.abs(o["t"]) + 1e-14), j
        ref = o["dense"](tq[:, j])
        assert np.all(np.abs(ev[:, :, j] - ref) <= 10 * (rt * np.abs(ref) + at)), j


@pytest.mark.parametrize("alg", ["tsit5", "rodas5p"])
def test_dense_output_at_event_times_takes_the_saves(alg):
    # ode_interpolation's exact-time rule: sol(t) at a saved time is that save; at a
    # contact (saved twice) the pre-affect state, and with continuity = :right the
    # post-affect one (ode_event_tests.jl:170-172: sol(t, continuity = :right)[2] > 0)
    from odegb300 import dense_eval
    N = 32
    wl = balls(N, seed=6)
    rt = at = 1e-8
    cb = ContinuousCallback(interp_points=10, max_events=16)
    g = gpu("bouncing_ball", alg, wl["u0"], wl["p"], wl["tspan"], None, rt, at, callback=cb, save_everystep=True,
            max_step_saves=4096, dense=True)
    ns = g["nsaved"]
    k = int(ns.min())
    tq = g["t"][:k]                       # (k, N): every trajectory's own first k saved times
    left = dense_eval(g, tq)
    right = dense_eval(g, tq, continuity="right")
    dup = np.zeros((k, N), dtype=bool)          # save r is followed by a save at the same time
    dup[:-1] = g["t"][:k - 1] == g["t"][1:k]
    second = np.zeros((k, N), dtype=bool)       # save r repeats the time of save r - 1
    second[1:] = dup[:-1]
    assert dup.any()
    m = ~second
    assert np.array_equal(left.transpose(1, 0, 2)[:, m], g["u"][:k].transpose(1, 0, 2)[:, m])
    r, j = np.nonzero(dup)
    assert np.array_equal(left[r + 1, :, j], g["u"][r, :, j])      # either query time: the first save
    assert np.array_equal(right[r, :, j], g["u"][r + 1, :, j])     # :right, the second
    assert np.array_equal(right[r + 1, :, j], g["u"][r + 1, :, j])
    # falling into the floor before, rising after (a ball that terminate!s at its
    # contact keeps its velocity in the post-affect save)
    live = g["retcode"][j] == 1
    assert live.any() and (left[r, 1, j] <= 0).all() and (right[r[live], 1, j[live]] >= 0).all()
