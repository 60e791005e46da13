"""GPU parity on a non-autonomous problem: the forced Duffing oscillator
x'' + delta x' + alpha x + beta x^3 = g cos(w t), whose right-hand side reads
t at every stage (t + c dt) and whose Rosenbrock steps take the analytic time
derivative dT (derivative_utils.jl:181-227; Rodas5P adds dtd_s dT to every
stage, rosenbrock_perform_step.jl:729-800; Rosenbrock23 to its first and error
stages, :34-146).  Against the FP64 oracle at the parity bar (10x tolerance,
accepted steps within 1), and with beta = 0 against the closed form."""
import numpy as np
import pytest

from gpu_common import assert_mixed_accuracy, compare, gpu, oracle

pytestmark = pytest.mark.gpu

ALGS = ["tsit5", "vern7", "rodas5p", "rosenbrock23"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


def forced_inputs(N, seed=0, beta=(0.0, 1.0)):
    rng = np.random.default_rng(seed)
    p = np.vstack([rng.uniform(0.1, 0.5, N), rng.uniform(1.0, 4.0, N), rng.uniform(*beta, N),
                   rng.uniform(0.5, 2.0, N), rng.uniform(0.5, 3.0, N)])
    u0 = rng.uniform(-1.0, 1.0, (2, N))
    ts = np.vstack([np.zeros(N), np.full(N, 20.0)])
    return u0, p, ts


SAVEAT = np.linspace(1.0, 20.0, 20)
TOL = {"tsit5": 1e-8, "vern7": 1e-8, "rodas5p": 1e-6, "rosenbrock23": 1e-4}


@pytest.mark.parametrize("alg", ALGS)
def test_forced_oscillator_fp64_matches_oracle(alg):
    N = 256
    u0, p, ts = forced_inputs(N)
    rt = TOL[alg]
    g = gpu("forced_duffing", alg, u0, p, ts, SAVEAT, rt, rt)
    o = oracle("forced_duffing", alg, u0, p, ts, SAVEAT, rt, rt)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, rt, rt)
    assert c["ok"] and c["steps_ok"], c
    # the analytic tgrad is not an f call: Rosenbrock f counts equal the oracle's
    if alg in ("rodas5p", "rosenbrock23"):
        assert np.abs(g["stats"]["nf"] - o["stats"]["nf"]).max() <= 16


@pytest.mark.parametrize("alg", ALGS)
def test_forced_linear_oscillator_matches_the_closed_form(alg):
    from test_oracle import forced_exact
    N = 64
    u0, p, ts = forced_inputs(N, seed=3, beta=(0.0, 0.0))
    rt = TOL[alg]
    g = gpu("forced_duffing", alg, u0, p, ts, SAVEAT, rt, rt)
    ex = forced_exact(SAVEAT[:, None], u0[0], u0[1], p[0], p[1], p[3], p[4])   # (nsave, N, 2)
    got = np.moveaxis(g["u"][:20], 1, 2)
    err = np.abs(got - ex) / (rt * np.abs(ex) + rt)
    # global error of the method at this tolerance (Rosenbrock23 is second order)
    assert err.max() < (500.0 if alg == "rosenbrock23" else 50.0), err.max()


@pytest.mark.parametrize("alg", ["tsit5", "vern7", "rodas5p"])
def test_forced_oscillator_mixed_matches_oracle(alg):
    # the forcing g cos(w t) is evaluated in FP64 from the FP64 t in both forms
    N = 256
    u0, p, ts = forced_inputs(N, seed=5)
    rt = 1e-6
    g = gpu("forced_duffing", alg, u0, p, ts, SAVEAT, rt, rt, precision="mixed")
    assert (g["retcode"] == 1).all()
    assert_mixed_accuracy("forced_duffing", alg, g, u0, p, ts, SAVEAT, rt, rt)
