"""GPU parity of fixed steps (the reference's adaptive = false: no error estimate is
judged, every step is accepted, and a step is cut short only to land on a tstop or
tf -- modify_dt_for_tstops!, integrator_utils.jl:268-324; the non-adaptive footer,
integrator_utils.jl loopfooter!).  The time grids are the reference's own test
pins (test/InterfaceI/ode_tstops_tests.jl, ode_backwards_test.jl); the solutions
are checked against the oracle on the same grid, and an event with fixed steps
(test/Integrators_I/ode_event_tests.jl:121) against the oracle's event times.
"""
import numpy as np
import pytest

from gpu_common import compare, gpu, lorenz_inputs, oracle
from odegb300 import ContinuousCallback

pytestmark = pytest.mark.gpu

ALGS = ["tsit5", "vern7", "rodas5p", "rosenbrock23", "autotsit5_rosenbrock23"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


def grid(alg, tspan, dt=None, tstops=None, N=4):
    u0 = np.tile([[0.5]], (1, N))
    p = np.full((1, N), 1.01)
    ts = np.tile(np.asarray(tspan, float)[:, None], (1, N))
    g = gpu("linear", alg, u0, p, ts, None, 1e-6, 1e-6, adaptive=False, dt=dt, tstops=tstops,
            save_everystep=True, max_step_saves=256, save_start=True)
    assert (g["retcode"] == 1).all() and (g["nsaved"] == g["nsaved"][0]).all()
    t = g["t"][:int(g["nsaved"][0])]
    assert (t == t[:, :1]).all()
    assert (g["stats"]["nreject"] == 0).all()
    return list(t[:, 0])


@pytest.mark.parametrize("alg", ALGS)
def test_fixed_step_time_grids_are_the_references(alg):
    # ode_tstops_tests.jl:14-15, :29-30, :32-36, :38-42
    assert grid(alg, (0.0, 1.0), dt=1 / 3, tstops=[0.5]) == [0.0, 1 / 3, 1 / 2, 1 / 3 + 1 / 2, 1.0]
    ts = [1 / 5, 1 / 4, 1 / 3, 1 / 2, 3 / 4]
    assert grid(alg, (0.0, 1.0), tstops=ts) == [0.0] + ts + [1.0]
    assert grid(alg, (0.0, 1.0), tstops=[0.0] + ts + [1.0]) == [0.0] + ts + [1.0]
    assert grid(alg, (0.0, 1.0), tstops=np.arange(17) / 16) == list(np.arange(17) / 16)
    # ode_backwards_test.jl:11-15: a positive dt is taken in the direction of (1, 0)
    assert grid(alg, (1.0, 0.0), dt=0.25) == [1.0, 0.75, 0.5, 0.25, 0.0]
    assert grid(alg, (1.0, 0.0), dt=-0.25) == [1.0, 0.75, 0.5, 0.25, 0.0]
    t = grid(alg, (1.0, 0.0), dt=0.25, tstops=[0.5, 0.33])
    assert np.allclose(t, [1.0, 0.75, 0.5, 0.33, 0.08, 0.0], rtol=0, atol=1e-15) and 0.33 in t


@pytest.mark.parametrize("alg", ALGS)
def test_fixed_steps_match_oracle(alg):
    # the same grid, so the saves, step counts and RHS counts match the oracle's
    N = 256
    u0, p, ts = lorenz_inputs(N, seed=9)
    dt = 1e-3 if alg in ("tsit5", "vern7") else 2e-3
    g = gpu("lorenz", alg, u0, p, ts, 0.1, 1e-6, 1e-6, adaptive=False, dt=dt)
    o = oracle("lorenz", alg, u0, p, ts, 0.1, 1e-6, 1e-6, adaptive=False, dt=dt)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, 1e-11, 1e-11, step_slack=0)
    assert c["ok"] and c["steps_ok"], c
    for k in ("naccept", "nreject", "nf", "njacs", "nsolve"):
        assert np.array_equal(g["stats"][k], o["stats"][k]), k
    assert (g["stats"]["nreject"] == 0).all()


def test_composite_switches_with_fixed_steps():
    # AutoTsit5(Rosenbrock23()) on van der Pol, mu log-uniform in [1, 1000], dt = 1e-3:
    # the stiffness test still runs on every step and moves the stiff oscillators to
    # Rosenbrock23 (J evaluations); the grid is fixed, so only a switch decision that a
    # rounding moves can differ from the oracle
    from odegb300 import workloads as W
    wl = W.van_der_pol(128, seed=13)
    kw = dict(adaptive=False, dt=1e-3)
    g = gpu("van_der_pol", "autotsit5_rosenbrock23", wl["u0"], wl["p"], wl["tspan"], 0.5, 1e-6, 1e-6, **kw)
    o = oracle("van_der_pol", "autotsit5_rosenbrock23", wl["u0"], wl["p"], wl["tspan"], 0.5, 1e-6, 1e-6, **kw)
    assert np.array_equal(g["retcode"], o["retcode"])
    assert np.array_equal(g["stats"]["naccept"], o["stats"]["naccept"])
    same = g["stats"]["njacs"] == o["stats"]["njacs"]
    assert same.mean() > 0.8, same.mean()
    ok = (g["retcode"] == 1) & same
    c = compare({k: (v[..., ok] if k != "stats" else {n: a[ok] for n, a in v.items()}) for k, v in g.items()
                 if k in ("t", "u", "nsaved", "retcode", "stats")},
                {k: (v[..., ok] if k != "stats" else {n: a[ok] for n, a in v.items()}) for k, v in o.items()},
                1e-9, 1e-9, step_slack=0)
    assert c["ok"], c
    assert (g["stats"]["njacs"][wl["p"][0] > 300.0] > 0).any()


@pytest.mark.parametrize("alg", ["tsit5", "rodas5p"])
def test_mixed_fixed_steps_stay_on_the_oracle(alg):
    # FP32 stages with compensated updates: the same grid, saves within 1e-5 relative
    # (500 steps of FP32 stage rounding; the truncation error at dt = 2e-3 is far below)
    N = 256
    u0, p, ts = lorenz_inputs(N, seed=10)
    g = gpu("lorenz", alg, u0, p, ts, 0.1, 1e-6, 1e-6, precision="mixed", adaptive=False, dt=2e-3)
    o = oracle("lorenz", alg, u0, p, ts, 0.1, 1e-6, 1e-6, adaptive=False, dt=2e-3)
    c = compare(g, o, 1e-6, 1e-6, step_slack=0)
    assert c["ok"] and c["steps_ok"], c


def test_fixed_step_events_match_oracle():
    # ode_event_tests.jl:121: the bouncing ball with Tsit5, adaptive = false, dt = 1/4;
    # the event shortens the step it falls in and the grid resumes from the event
    N = 128
    rng = np.random.default_rng(12)
    u0 = np.vstack([rng.uniform(5.0, 50.0, N), rng.uniform(-5.0, 5.0, N)])
    p = np.vstack([np.full(N, 9.81), rng.uniform(0.6, 1.0, N), np.full(N, 1e9)])
    ts = np.vstack([np.zeros(N), np.full(N, 15.0)])
    cb = ContinuousCallback(interp_points=100, max_events=64)
    kw = dict(adaptive=False, dt=0.25, save_everystep=True, max_step_saves=512)
    g = gpu("bouncing_ball", "tsit5", u0, p, ts, None, 1e-6, 1e-6, callback=cb, **kw)
    o = oracle("bouncing_ball", "tsit5", u0, p, ts, None, 1e-6, 1e-6, callback=True, interp_points=100,
               max_events=64, **kw)
    assert np.array_equal(g["retcode"], o["retcode"]) and np.array_equal(g["nsaved"], o["nsaved"])
    ns = int(g["nsaved"].max())
    gt, ot = g["t"][:ns], o["t"][:ns]
    m = ~np.isnan(ot)
    assert np.all(np.abs(gt[m] - ot[m]) <= 1e-11 * np.abs(ot[m]) + 1e-13)
    gu, ou = g["u"][:ns], o["u"][:ns]
    mu = ~np.isnan(ou)
    assert np.all(np.abs(gu[mu] - ou[mu]) <= 1e-9 * np.abs(ou[mu]) + 1e-9)
    assert (g["nsaved"] > 15 * 4 + 1).all()   # every ball bounced at least once


@pytest.mark.parametrize("alg", ["tsit5", "rodas5p"])
def test_fixed_steps_with_dense_output(alg):
    # the dense vectors of each fixed step: sol(t) between the steps matches the oracle's
    from gpu_common import ALG, MODEL
    import pyoracle as O
    from odegb300 import dense_eval
    N = 16
    u0, p, ts = lorenz_inputs(N, seed=14)
    g = gpu("lorenz", alg, u0, p, ts, None, 1e-6, 1e-6, adaptive=False, dt=1e-2, save_everystep=True,
            max_step_saves=256, dense=True)
    tq = np.linspace(0.0, 1.0, 37)[:, None] * np.ones((1, N))
    ev = dense_eval(g, tq)
    for j in range(N):
        o = O.solve(ALG[alg][1], MODEL["lorenz"], u0[:, j], p[:, j], ts[:, j], dense=True, adaptive=False, dt=1e-2,
                    reltol=1e-6, abstol=1e-6, saveat_given=False, save_everystep=True, max_step_saves=256,
                    save_start=True, save_end=True)
        ref = o["dense"](tq[:, j])
        assert np.all(np.abs(ev[:, :, j] - ref) <= 1e-10 * (np.abs(ref) + 1.0)), j
