"""GPU parity of backward integration (tf < t0, the reference's tdir = -1:
lib/OrdinaryDiffEqCore/src/solve.jl:273 and every tdir in initdt.jl,
integrator_utils.jl and callbacks.jl).  The kernels run the loop on s = -t and
hand the model and the method the reference's own t and signed dt, so a
backward solve takes the oracle's steps just as a forward one does: checked
against the oracle (which follows the reference's tdir arithmetic directly)
at the parity bar, with the fraction of bit-identical trajectories no lower
than forward on the same problem; ensembles mixing both directions; saveat
numbers and tstops; dense output; an event; a DiscreteCallback; the mixed form.
"""
import numpy as np
import pytest

import pyoracle as O
from gpu_common import ALG, MODEL, assert_mixed_accuracy, compare, gpu, lorenz_inputs, oracle
from odegb300 import ContinuousCallback, DiscreteCallback, dense_eval

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


def forced(N, seed=0, t0=10.0, tf=0.0, damping=(0.1, 0.5)):
    rng = np.random.default_rng(seed)
    p = np.vstack([rng.uniform(*damping, N), rng.uniform(1.0, 4.0, N), rng.uniform(0.0, 1.0, N),
                   rng.uniform(0.5, 2.0, N), rng.uniform(0.5, 3.0, N)])
    u0 = rng.uniform(-1.0, 1.0, (2, N))
    ts = np.vstack([np.full(N, t0), np.full(N, tf)])
    return u0, p, ts


ALGS = ["tsit5", "vern7", "rodas5p", "rosenbrock23", "autotsit5_rosenbrock23"]
TOL = {"tsit5": 1e-8, "vern7": 1e-8, "rodas5p": 1e-6, "rosenbrock23": 1e-4, "autotsit5_rosenbrock23": 1e-6}


@pytest.mark.parametrize("alg", ALGS)
def test_backward_forced_oscillator_matches_oracle(alg):
    # t in every stage and, for the Rosenbrock methods, dT with dtd_s dT in the stages.
    # Backward the damped oscillator grows (e^{delta t / 2}, stiffening with the cubic
    # term): over 10 time units a 1e-14 change of u0 moves no save measurably (checked
    # on the oracle); over 20, Rosenbrock23 at 1e-4 amplifies it to ~400x the parity bar
    N = 256
    u0, p, ts = forced(N)
    rt = TOL[alg]
    sv = np.linspace(0.0, 9.0, 10)
    g = gpu("forced_duffing", alg, u0, p, ts, sv, rt, rt)
    o = oracle("forced_duffing", alg, u0, p, ts, sv, rt, rt)
    assert (g["retcode"] == 1).all()
    # saves in the integration direction: 9, 8, ..., 0
    assert np.array_equal(g["t"][:10], np.repeat(sv[::-1, None], N, axis=1))
    c = compare(g, o, rt, rt)
    assert c["ok"] and c["steps_ok"], c
    # the reflection is exact: as many trajectories bit-identical to the oracle as forward
    uf, pf, tf_ = forced(N, t0=0.0, tf=10.0)
    svf = np.linspace(1.0, 10.0, 10)
    cf = compare(gpu("forced_duffing", alg, u0, p, tf_, svf, rt, rt), oracle("forced_duffing", alg, u0, p, tf_, svf,
                                                                             rt, rt), rt, rt)
    assert c["frac_bit_identical"] >= 0.5 * cf["frac_bit_identical"], (c, cf)


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
def test_lorenz_both_directions_in_one_ensemble(alg):
    # every other trajectory runs from 1 back to 0; a saveat number gives each its own
    # (t0 + tdir d):(tdir d):tf row; a shared tstop at 0.55 is hit in both directions
    N = 512
    u0, p, ts = lorenz_inputs(N, seed=3)
    ts[:, 1::2] = ts[::-1, 1::2].copy()
    rt = 1e-8
    g = gpu("lorenz", alg, u0, p, ts, 0.1, rt, rt, tstops=[0.55])
    o = oracle("lorenz", alg, u0, p, ts, 0.1, rt, rt, tstops=[0.55])
    assert (g["retcode"] == 1).all()
    c = compare(g, o, rt, rt)
    assert c["ok"] and c["steps_ok"], c
    tb = g["t"][:11, 1]
    assert np.array_equal(tb, [1.0, 0.9, 0.8, 0.7, 0.6, 0.5, 0.4, 0.3, 0.2, 0.1, 0.0])
    assert np.array_equal(g["t"][:11, 0], tb[::-1])


@pytest.mark.parametrize("model,alg", [("forced_duffing", "tsit5"), ("forced_duffing", "rodas5p"),
                                       ("lorenz", "vern7")])
def test_backward_dense_output_matches_oracle(model, alg):
    # sol(t) searches the saved times in the integration direction
    N = 32
    if model == "lorenz":
        u0, p, _ = lorenz_inputs(N, seed=4)
        ts = np.vstack([np.full(N, 0.5), np.zeros(N)])
    else:
        u0, p, ts = forced(N, seed=4, t0=10.0, tf=0.0)
    rt = 1e-8 if alg != "rodas5p" else 1e-6
    g = gpu(model, alg, u0, p, ts, None, rt, rt, save_everystep=True, max_step_saves=4096, dense=True)
    rng = np.random.default_rng(2)
    tq = rng.uniform(0.0, 1.0, (24, N)) * ts[0]
    tq[0], tq[1] = ts[0], 0.0
    ev = dense_eval(g, tq)
    for j in range(N):
        o = O.solve(ALG[alg][1], MODEL[model], u0[:, j], p[:, j], ts[:, j], dense=True, reltol=rt,
                    abstol=rt, saveat_given=False, save_everystep=True, max_step_saves=4096, save_start=True,
                    save_end=True)
        ref = o["dense"](tq[:, j])
        assert np.all(np.abs(ev[:, :, j] - ref) <= 10 * (rt * np.abs(ref) + rt)), j
        ns = int(g["nsaved"][j])
        assert np.all(np.diff(g["t"][:ns, j]) < 0)


@pytest.mark.parametrize("alg", ["tsit5", "vern7", "rodas5p"])
def test_backward_bouncing_ball_events_match_oracle(alg):
    N = 128
    rng = np.random.default_rng(6)
    u0 = np.vstack([rng.uniform(5.0, 50.0, N), rng.uniform(-5.0, 15.0, N)])
    p = np.vstack([np.full(N, 9.81), rng.uniform(0.6, 1.0, N), np.full(N, 1e9)])
    ts = np.vstack([np.full(N, 10.0), np.zeros(N)])
    rt = 1e-8 if alg != "rodas5p" else 1e-6
    cb = ContinuousCallback(interp_points=10, max_events=32)
    g = gpu("bouncing_ball", alg, u0, p, ts, 0.25, rt, rt, callback=cb)
    o = oracle("bouncing_ball", alg, u0, p, ts, 0.25, rt, rt, callback=True, interp_points=10, max_events=32)
    assert np.array_equal(g["retcode"], o["retcode"]) and np.array_equal(g["nsaved"], o["nsaved"])
    ns = int(g["nsaved"].max())
    gt, ot = g["t"][:ns], o["t"][:ns]
    m = ~np.isnan(ot)
    # event times (saved twice) agree to a few ulps of the root; saveat times exactly
    assert np.all(np.abs(gt[m] - ot[m]) <= 1e-12 * np.abs(ot[m]) + 1e-14)
    gu, ou = g["u"][:ns], o["u"][:ns]
    mu = ~np.isnan(ou)
    assert np.all(np.abs(gu[mu] - ou[mu]) <= 10 * (rt * np.abs(ou[mu]) + rt))
    # every ball meets the floor at least once going back 10 s: two saves more than the saveat
    assert (g["nsaved"] >= 41 + 2).all()


def test_backward_dosing_callback_matches_oracle():
    # the doses at the tstops apply in the integration order (backward: 8, 4, then 2)
    N = 64
    rng = np.random.default_rng(8)
    p = np.vstack([rng.uniform(0.5, 2.0, N), rng.uniform(0.05, 0.3, N), rng.uniform(50.0, 150.0, N)])
    u0 = np.vstack([np.full(N, 10.0), np.full(N, 5.0)])
    ts = np.vstack([np.full(N, 12.0), np.zeros(N)])
    sv = np.arange(0.0, 12.0)
    rt = 1e-8
    doses = np.array([2.0, 4.0, 8.0])
    g = gpu("pk_one_compartment", "tsit5", u0, p, ts, sv, rt, rt, tstops=doses,
            callback=DiscreteCallback(max_events=16))
    o = oracle("pk_one_compartment", "tsit5", u0, p, ts, sv, rt, rt, tstops=doses, callback=True, max_events=16)
    c = compare(g, o, rt, rt)
    assert c["ok"] and c["steps_ok"], c


@pytest.mark.parametrize("alg", ["tsit5", "rodas5p"])
def test_backward_mixed_form(alg):
    # light damping: backward the oscillator's growth e^{delta t / 2} stays below 1.7, so
    # the FP32 stages' per-step rounding is not amplified past what forward sees
    N = 256
    u0, p, ts = forced(N, seed=9, damping=(0.02, 0.1))
    sv = np.linspace(0.0, 9.0, 10)
    rt = 1e-6
    g = gpu("forced_duffing", alg, u0, p, ts, sv, rt, rt, precision="mixed")
    assert (g["retcode"] == 1).all()
    assert_mixed_accuracy("forced_duffing", alg, g, u0, p, ts, sv, rt, rt)


def test_round_trip_returns_to_the_start():
    # forward 0 -> 5 and back 5 -> 0 from the end state: u0 again within the tolerance's reach
    N = 256
    u0, p, ts = forced(N, seed=10, t0=0.0, tf=5.0)
    rt = 1e-10
    fwd = gpu("forced_duffing", "vern7", u0, p, ts, None, rt, rt)
    end = np.stack([fwd["u"][int(fwd["nsaved"][j]) - 1, :, j] for j in range(N)], axis=1)
    back = gpu("forced_duffing", "vern7", end, p, ts[::-1].copy(), None, rt, rt)
    start = np.stack([back["u"][int(back["nsaved"][j]) - 1, :, j] for j in range(N)], axis=1)
    assert np.abs(start - u0).max() < 1e-6
