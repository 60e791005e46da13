"""odegb300 — host side of the GB300 ensemble ODE integrator (libode_b200.so).

    from odegb300 import ODEProblem, EnsembleProblem, solve, Tsit5, Vern7, Rodas5P, EnsembleGB300
    prob = ODEProblem("lorenz", [1.0, 0.0, 0.0], (0.0, 1.0), [10.0, 28.0, 8 / 3])
    eprob = EnsembleProblem(prob, prob_func=lambda prob, ctx: remake(prob, p=[10.0, ctx.rng.uniform(0, 21), 8 / 3]))
    sim = solve(eprob, Tsit5(), EnsembleGB300(), trajectories=10_000, saveat=0.1, reltol=1e-8, abstol=1e-8)
    sim.u[0].t, sim.u[0].u, sim.u[0].retcode, sim.u[0].stats
"""
from .ensemble import (AutoTsit5, ContinuousCallback, DiscreteCallback, EnsembleContext, EnsembleGB300,
                       EnsembleProblem, EnsembleSolution, ODEProblem, ODESolution, PIController, ReturnCode, Rodas5P,
                       Rosenbrock23,
                       Tsit5, Vern7, autotune, dense_eval, get_handle, register_model, remake, solve, solve_arrays)
from .saveat import julia_float_range, resolve_saveat
from .serving import Server, run_open_loop
from . import _lib, build

__all__ = ["AutoTsit5", "ContinuousCallback", "DiscreteCallback", "EnsembleContext", "EnsembleGB300", "EnsembleProblem",
           "EnsembleSolution", "ODEProblem", "ODESolution", "PIController", "ReturnCode", "Rodas5P", "Rosenbrock23", "Tsit5", "Vern7",
           "autotune", "dense_eval", "get_handle", "register_model", "remake", "solve", "solve_arrays", "julia_float_range",
           "resolve_saveat", "Server", "run_open_loop"]
