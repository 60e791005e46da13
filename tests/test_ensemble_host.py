"""Host-side EnsembleProblem semantics (no GPU): prob_func contexts, output_func
reruns, batched reductions with early convergence, u_init, packed inputs.

Follows the reference's ensemble tests (lib/DiffEqBase/test/downstream/ensemble.jl:
prob_func(prob, ctx) with 1-based sim_id, output_func returning (out, rerun),
reduction(u, batch, I) returning (u, converged), batch_size).  The GPU solve is
replaced by the exact solution of u' = p0 u so only the orchestration is tested.
"""
import numpy as np
import pytest

import odegb300.ensemble as E
from odegb300 import EnsembleGB300, EnsembleProblem, ODEProblem, Tsit5, remake, solve
from odegb300.saveat import resolve_saveat

pytestmark = pytest.mark.filterwarnings("ignore::RuntimeWarning")


@pytest.fixture
def exact_linear(monkeypatch):
    calls = []

    def fake(model, alg, ens, u0s, ps, tspans, saveat=None, reltol=1e-3, abstol=1e-6, dt=None, dtmax=None,
             dtmin=None, maxiters=1000000, save_start=None, save_end=None, n_per_traj=None, qmax_first_step=None,
             qmax=None, return_times=False, save_everystep=False, max_step_saves=1024, dense=False, callback=None,
             tstops=None, save_idxs=None, adaptive=True, controller=None, force_dtmin=False,
             isoutofdomain=None):
        u0s, ps, tspans = np.asarray(u0s, float), np.asarray(ps, float), np.asarray(tspans, float)
        n, N = u0s.shape
        sv = resolve_saveat(saveat, tspans, save_start, save_end, save_everystep, max_step_saves)
        cap = sv.cap
        t = np.full((cap, N), np.nan)
        u = np.full((cap, n, N), np.nan)
        ns = np.zeros(N, dtype=np.int32)
        for j in range(N):
            pts = ([tspans[0, j]] if sv.save_start else []) + list(sv.values if not sv.per_traj else sv.values[:, j])
            if sv.save_end and (not pts or pts[-1] != tspans[1, j]):
                pts.append(tspans[1, j])
            for s, tt in enumerate(pts):
                t[s, j] = tt
                u[s, :, j] = u0s[:, j] * np.exp(ps[0, j] * (tt - tspans[0, j]))
            ns[j] = len(pts)
        calls.append(N)
        fake.last = {"save_everystep": save_everystep, "max_step_saves": max_step_saves, "dense": dense}
        names = ("nf", "njacs", "nw", "nsolve", "naccept", "nreject")
        return {"t": t, "u": u, "nsaved": ns, "retcode": np.ones(N, dtype=np.int32),
                "stats": {k: np.zeros(N, dtype=np.int64) for k in names}, "elapsed": 0.0}

    monkeypatch.setattr(E, "solve_arrays", fake)
    return calls


PROB = ODEProblem("linear", [1.0], (0.0, 1.0), [0.5])


def test_prob_func_sees_one_based_sim_ids_and_deterministic_rngs(exact_linear):
    seen = []

    def prob_func(prob, ctx):
        seen.append((ctx.sim_id, ctx.repeat))
        return remake(prob, u0=[float(ctx.sim_id)], p=[ctx.rng.uniform(0.0, 1.0)])

    ep = EnsembleProblem(PROB, prob_func=prob_func)
    a = solve(ep, Tsit5(), EnsembleGB300(), trajectories=5, saveat=0.5, seed=7)
    assert sorted(seen) == [(i, 1) for i in range(1, 6)]
    b = solve(ep, Tsit5(), EnsembleGB300(), trajectories=5, saveat=0.5, seed=7)
    assert [s.u[0][0] for s in a.u] == [1.0, 2.0, 3.0, 4.0, 5.0]
    assert all(np.array_equal(x.u[-1], y.u[-1]) for x, y in zip(a.u, b.u))   # same seed, same draws
    assert list(a.u[0].t) == [0.0, 0.5, 1.0]


def test_output_func_rerun_increments_repeat(exact_linear):
    repeats = {}

    def prob_func(prob, ctx):
        repeats.setdefault(ctx.sim_id, []).append(ctx.repeat)
        return prob

    def output_func(sol, ctx):
        return sol.u[-1][0], ctx.sim_id == 2 and ctx.repeat < 3   # trajectory 2 is redone twice

    ep = EnsembleProblem(PROB, prob_func=prob_func, output_func=output_func)
    sim = solve(ep, Tsit5(), EnsembleGB300(), trajectories=3, saveat=[1.0])
    assert repeats[2] == [1, 2, 3] and repeats[1] == [1] and repeats[3] == [1]
    assert np.allclose(sim.u, np.exp(0.5))


def test_batched_reduction_stops_when_converged(exact_linear):
    batches = []

    def reduction(u, batch, I):
        batches.append(list(I))
        u = u + [b.u[-1][0] for b in batch]
        return u, len(u) >= 4

    ep = EnsembleProblem(PROB, reduction=reduction, u_init=[])
    sim = solve(ep, Tsit5(), EnsembleGB300(), trajectories=10, batch_size=2, saveat=[1.0])
    assert batches == [[1, 2], [3, 4]]
    assert sim.converged and len(sim.u) == 4
    assert exact_linear == [2, 2]   # two solves of two trajectories


def test_packed_inputs_and_uneven_sizes(exact_linear):
    N = 6
    npt = np.array([4, 8, 4, 8, 4, 8], dtype=np.int32)
    u0s = np.ones((8, N))
    ep = EnsembleProblem(ODEProblem("duffing_chain", np.ones(8), (0.0, 2.0), [0.5, 0.1, 0.0]),
                         u0s=u0s, ps=np.full((3, N), 0.5), tspans=np.tile([[0.0], [2.0]], (1, N)), n_per_traj=npt)
    sim = solve(ep, Tsit5(), EnsembleGB300(), saveat=[1.0, 2.0])
    assert len(sim.u) == N
    assert [len(s.u[0]) for s in sim.u] == list(npt)
    assert sim.u[1].retcode.name == "Success" and list(sim.u[1].t) == [1.0, 2.0]


def test_no_saveat_defaults_to_every_step(exact_linear):
    # the reference's defaults (solve.jl:138-146): save_everystep = isempty(saveat),
    # dense = save_everystep && isempty(saveat)
    solve(EnsembleProblem(PROB), Tsit5(), EnsembleGB300(), trajectories=2)
    assert E.solve_arrays.last["save_everystep"] is True and E.solve_arrays.last["dense"] is True
    solve(EnsembleProblem(PROB), Tsit5(), EnsembleGB300(), trajectories=2, saveat=0.5)
    assert E.solve_arrays.last["save_everystep"] is False and E.solve_arrays.last["dense"] is False
    solve(EnsembleProblem(PROB), Tsit5(), EnsembleGB300(), trajectories=2, dense=False)
    assert E.solve_arrays.last["save_everystep"] is True and E.solve_arrays.last["dense"] is False


def test_uneven_ensembles_are_not_dense_by_default(exact_linear):
    npt = np.array([4, 8], dtype=np.int32)
    ep = EnsembleProblem(ODEProblem("duffing_chain", np.ones(8), (0.0, 1.0), [0.5, 0.1, 0.0]),
                         u0s=np.ones((8, 2)), ps=np.full((3, 2), 0.5), tspans=np.tile([[0.0], [1.0]], (1, 2)),
                         n_per_traj=npt)
    solve(ep, Tsit5(), EnsembleGB300())
    assert E.solve_arrays.last["save_everystep"] is True and E.solve_arrays.last["dense"] is False


def test_linear_interpolation_between_saves_without_dense():
    # ode_interpolation's non-dense branch (generic_dense.jl:1121-1122, linear_interpolant :2119-2127)
    from odegb300.ensemble import ODESolution
    s = ODESolution(np.array([0.0, 1.0, 3.0]), [np.array([0.0, 10.0]), np.array([1.0, 20.0]),
                                                 np.array([5.0, 0.0])], 1, {})
    assert np.allclose(s(0.5), [0.5, 15.0]) and np.allclose(s(2.0), [3.0, 10.0])
    assert np.allclose(s([0.0, 1.0, 3.0]), [[0.0, 10.0], [1.0, 20.0], [5.0, 0.0]])
    # left continuity: t == ts[i] takes the interval ending at ts[i]; outside the
    # range the first or last interval's line continues
    assert np.allclose(s(4.0), [7.0, -10.0]) and np.allclose(s(-1.0), [-1.0, 0.0])
    # a time saved twice (an event): the first save, or with continuity = :right the second
    e = ODESolution(np.array([0.0, 1.0, 1.0, 2.0]), [np.array([0.0]), np.array([1.0]), np.array([-1.0]),
                                                     np.array([0.0])], 1, {})
    assert e(1.0)[0] == 1.0 and e(1.0, continuity="right")[0] == -1.0 and e(0.5)[0] == 0.5
