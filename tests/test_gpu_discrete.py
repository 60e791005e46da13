"""GPU parity for the model-registered DiscreteCallback: the one-compartment
dosing model, doses given as the solve's tstops with condition t in tstops
(apply_discrete_callback!, lib/DiffEqBase/src/callbacks.jl:645-682;
handle_callbacks!, lib/OrdinaryDiffEqCore/src/integrators/integrator_utils.jl:
1081-1132).  A population of 512 patients (ka, ke log-normal) dosed every 12 h
for a week: FP64 saves within 10x the tolerance of the oracle with accepted
steps within 1, two saves at every dose (before and after it), and the closed
form within the tolerance; the mixed form as accurate as FP64 against it at
reltol 1e-6.
"""
import numpy as np
import pytest

from gpu_common import compare, gpu, oracle

pytestmark = pytest.mark.gpu

DOSES = np.array([12.0 * k for k in range(1, 14)])
SAVEAT = np.arange(0.5, 168.0, 1.0)
TOL = {"tsit5": (1e-8, 1e-8), "vern7": (1e-8, 1e-8), "rodas5p": (1e-7, 1e-8), "rosenbrock23": (1e-5, 1e-7),
       "autotsit5_rosenbrock23": (1e-7, 1e-8)}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


def population(N, seed=3):
    rng = np.random.default_rng(seed)
    ka = 1.2 * np.exp(0.3 * rng.standard_normal(N))
    ke = 0.15 * np.exp(0.3 * rng.standard_normal(N))
    dose = np.full(N, 100.0)
    u0 = np.vstack([dose, np.zeros(N)])
    return u0, np.vstack([ka, ke, dose]), np.vstack([np.zeros(N), np.full(N, 168.0)])


def closed_form(t, ka, ke, dose):
    taus = np.concatenate([[0.0], DOSES[DOSES <= t]])
    x1 = np.sum(dose * np.exp(-ka * (t - taus)))
    x2 = np.sum(dose * ka / (ka - ke) * (np.exp(-ke * (t - taus)) - np.exp(-ka * (t - taus))))
    return np.array([x1, x2])


def solve_pair(alg, precision="fp64", N=512, tol=None):
    from odegb300 import DiscreteCallback
    rt, at = tol or TOL[alg]
    u0, p, ts = population(N)
    g = gpu("pk_one_compartment", alg, u0, p, ts, SAVEAT, rt, at, precision=precision, tstops=DOSES,
            callback=DiscreteCallback(max_events=16))
    o = oracle("pk_one_compartment", alg, u0, p, ts, SAVEAT, rt, at, tstops=DOSES, callback=True, max_events=16)
    return g, o, p, rt, at


@pytest.mark.parametrize("alg", list(TOL))
def test_dosing_fp64_matches_oracle(alg):
    g, o, p, rt, at = solve_pair(alg)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, rt, at)
    assert c["ok"] and c["steps_ok"], c
    assert np.abs(g["stats"]["nf"] - o["stats"]["nf"]).max() <= 16
    # every trajectory saved each dose twice: before and after the affect
    ns = int(g["nsaved"][0])
    assert (g["nsaved"] == len(SAVEAT) + 2 * len(DOSES)).all()   # saveat without tf: no end save
    for tau in DOSES:
        at_tau = np.flatnonzero(g["t"][:ns, 0] == tau)
        assert len(at_tau) == 2
        jump = g["u"][at_tau[1], 0, :] - g["u"][at_tau[0], 0, :]
        assert np.allclose(jump, 100.0, rtol=1e-12)
    for j in range(0, 512, 64):
        for s in np.flatnonzero(np.isin(g["t"][:ns, j], SAVEAT)):
            ex = closed_form(g["t"][s, j], p[0, j], p[1, j], p[2, j])
            assert np.allclose(g["u"][s, :, j], ex, rtol=200 * rt, atol=200 * at), (alg, j, s)


@pytest.mark.parametrize("alg", ["tsit5", "rodas5p"])
def test_dosing_mixed_is_as_accurate_as_fp64(alg):
    # at reltol 1e-6: the mixed form keeps the parameters in FP32 (ka, ke to
    # ~3e-8 relative), so its bar is a tolerance well above that
    g, o, p, rt, at = solve_pair(alg, precision="mixed", tol=(1e-6, 1e-8))
    g64 = solve_pair(alg, tol=(1e-6, 1e-8))[0]
    assert (g["retcode"] == 1).all()
    assert np.array_equal(g["nsaved"], o["nsaved"])
    ns = int(g["nsaved"][0])
    err = {}
    for name, r in (("mixed", g), ("fp64", g64)):
        e = []
        for j in range(0, 512, 8):
            for s in np.flatnonzero(np.isin(r["t"][:ns, j], SAVEAT)):
                ex = closed_form(r["t"][s, j], p[0, j], p[1, j], p[2, j])
                e.append(np.max(np.abs(r["u"][s, :, j] - ex) / (rt * np.abs(ex) + at)))
        err[name] = np.array(e)
    for q in (50, 90):
        assert np.percentile(err["mixed"], q) <= 2.0 * np.percentile(err["fp64"], q) + 1.0, (q, err)
