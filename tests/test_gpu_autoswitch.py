"""GPU parity of AutoTsit5(Rosenbrock23()) (stiffness detection and switching,
lib/OrdinaryDiffEqCore/src/composite_algs.jl, perform_step/composite_perform_step.jl)
against the CPU oracle, and the properties that pin the composite: on a non-stiff
problem it never switches and is Tsit5 step for step; on stiff ones it uses the
stiff method (its Jacobian count is non-zero) and stays within the tolerance.
"""
import numpy as np
import pytest

from gpu_common import compare, gpu, lorenz_inputs, oracle, robertson_inputs, ROBER_SAVEAT

pytestmark = pytest.mark.gpu


def vdp(N, seed, lo=0.0, hi=3.0):
    rng = np.random.default_rng(seed)
    u0 = np.tile(np.array([[2.0], [0.0]]), (1, N))
    p = (10.0 ** rng.uniform(lo, hi, N))[None, :]
    ts = np.vstack([np.zeros(N), np.full(N, 6.0)])
    return u0, p, ts


def test_autotsit5_matches_oracle_on_van_der_pol():
    N = 256
    u0, p, ts = vdp(N, seed=3)
    rt = at = 1e-6
    g = gpu("van_der_pol", "autotsit5_rosenbrock23", u0, p, ts, 0.5, rt, at)
    o = oracle("van_der_pol", "autotsit5_rosenbrock23", u0, p, ts, 0.5, rt, at)
    assert (g["retcode"] == 1).all() and (o["retcode"] == 1).all()
    # a switch decision is discrete: a rounding difference can move one, after which
    # the two step sequences differ while both stay accurate
    c = compare(g, o, rt, at, factor=50.0, step_slack=10 ** 9)
    assert c["ok"], c
    same = g["stats"]["naccept"] == o["stats"]["naccept"]
    assert same.mean() > 0.8, same.mean()
    # the stiff ones used Rosenbrock23 (J evaluations), the mild ones never did
    stiff = p[0] > 300.0
    assert (g["stats"]["njacs"][stiff] > 0).all() and (g["stats"]["njacs"][p[0] < 2.0] == 0).all()


def test_autotsit5_on_a_nonstiff_problem_is_tsit5_bitwise():
    N = 512
    u0, p, ts = lorenz_inputs(N, seed=6)
    a = gpu("lorenz", "autotsit5_rosenbrock23", u0, p, ts, 0.1, 1e-8, 1e-8)
    b = gpu("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8)
    assert (a["stats"]["njacs"] == 0).all()
    assert np.array_equal(a["u"], b["u"], equal_nan=True) and np.array_equal(a["stats"]["naccept"],
                                                                              b["stats"]["naccept"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotsit5_on_robertson(precision):
    N = 256
    u0, p, ts = robertson_inputs(N, seed=9)
    rt, at = 1e-6, 1e-10
    g = gpu("robertson", "autotsit5_rosenbrock23", u0, p, ts, ROBER_SAVEAT, rt, at, precision=precision)
    o = oracle("robertson", "autotsit5_rosenbrock23", u0, p, ts, ROBER_SAVEAT, rt, at)
    assert (g["retcode"] == 1).all()
    assert (g["stats"]["njacs"] > 0).all()   # stiff: switched to Rosenbrock23
    c = compare(g, o, rt, at, factor=50.0, step_slack=10 ** 9)
    assert c["ok"], c
