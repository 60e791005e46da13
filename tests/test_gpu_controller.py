"""The PI controller's knobs (solve(...; controller = PIController(beta1, beta2;
qoldinit, qmin, qmax, gamma, qsteady_min, qsteady_max)), controllers.jl:745-843)
on the GPU: for every method the saves and step counts match the oracle's with
the same knobs, in FP64 and in the mixed form, and the steady band pinned in
the oracle (dt constant after the first step) holds on the device."""
import numpy as np
import pytest

from gpu_common import compare, gpu, lorenz_inputs, oracle
from odegb300 import PIController

pytestmark = pytest.mark.gpu

ALGS = ["tsit5", "vern7", "rodas5p", "rosenbrock23", "autotsit5_rosenbrock23"]
KNOBS = dict(beta1=0.12, beta2=0.05, qoldinit=1e-3, qmin=0.3, qmax=5.0, gamma=0.8, qsteady_min=0.95,
             qsteady_max=1.3)


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


@pytest.mark.parametrize("alg", ALGS)
def test_controller_knobs_match_oracle(alg):
    N = 256
    u0, p, ts = lorenz_inputs(N, seed=51)
    rt = 1e-8 if alg in ("tsit5", "vern7") else 1e-6
    ctl = PIController(**KNOBS)
    g = gpu("lorenz", alg, u0, p, ts, 0.1, rt, rt, controller=ctl)
    knobs = {k: v for k, v in KNOBS.items() if k != "qmax"}
    o = oracle("lorenz", alg, u0, p, ts, 0.1, rt, rt, controller=knobs, qmax=KNOBS["qmax"])
    assert (g["retcode"] == 1).all()
    c = compare(g, o, rt, rt)
    assert c["ok"] and c["steps_ok"], c
    base = gpu("lorenz", alg, u0, p, ts, 0.1, rt, rt)
    assert not np.array_equal(base["stats"]["naccept"], g["stats"]["naccept"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_steady_band_keeps_dt(precision):
    N = 64
    u0 = np.full((1, N), 0.5)
    p = np.full((1, N), 1.01)
    ts = np.tile([[0.0], [1.0]], (1, N))
    g = gpu("linear", "tsit5", u0, p, ts, None, 1e-6, 1e-6, precision=precision, save_everystep=True,
            max_step_saves=512, controller=PIController(qsteady_min=0.0, qsteady_max=1e9))
    t = g["t"][:int(g["nsaved"][0]), 0]
    d = np.diff(t)
    assert (g["stats"]["nreject"] == 0).all() and len(d) > 5
    assert np.allclose(d[:-1], d[0], rtol=1e-12, atol=0) and d[-1] <= d[0]


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
def test_force_dtmin_matches_oracle(alg):
    # a tolerance that needs steps below dtmin: DtLessThanMin, or with force_dtmin
    # every step at dtmin, as in the oracle
    N = 128
    u0, p, ts = lorenz_inputs(N, seed=52)
    kw = dict(dtmin=2e-3 if alg == "tsit5" else 3e-2)   # above the steps each method takes at 1e-12
    g0 = gpu("lorenz", alg, u0, p, ts, 0.1, 1e-12, 1e-12, **kw)
    o0 = oracle("lorenz", alg, u0, p, ts, 0.1, 1e-12, 1e-12, **kw)
    assert np.array_equal(g0["retcode"], o0["retcode"]) and (g0["retcode"] == 4).any()
    g = gpu("lorenz", alg, u0, p, ts, 0.1, 1e-12, 1e-12, force_dtmin=True, **kw)
    o = oracle("lorenz", alg, u0, p, ts, 0.1, 1e-12, 1e-12, force_dtmin=True, **kw)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, 1e-9, 1e-9, step_slack=0)
    assert c["ok"] and c["steps_ok"], c


@pytest.mark.parametrize("alg,precision", [("vern7", "fp64"), ("tsit5", "fp64"), ("rodas5p", "fp64"),
                                           ("vern7", "mixed")])
def test_isoutofdomain_negative_matches_oracle(alg, precision):
    # u' = p u with p ~ -U(20, 80) at loose tolerance overshoots below zero; with
    # isoutofdomain = "negative" such steps are rejected and retried at dt * qmin
    N = 256
    rng = np.random.default_rng(53)
    u0 = rng.uniform(0.5, 2.0, (1, N))
    p = -rng.uniform(20.0, 80.0, (1, N))
    ts = np.tile([[0.0], [2.0]], (1, N))
    kw = dict(save_everystep=True, max_step_saves=2048)
    g = gpu("linear", alg, u0, p, ts, None, 1e-2, 1e-2, precision=precision, isoutofdomain="negative", **kw)
    o = oracle("linear", alg, u0, p, ts, None, 1e-2, 1e-2, isoutofdomain=1, **kw)
    assert (g["retcode"] == 1).all()
    k = int(g["nsaved"].max())
    m = np.arange(k)[:, None] < g["nsaved"][None, :]
    assert g["u"][:k, 0][m].min() >= 0.0
    if precision == "fp64":
        c = compare(g, o, 1e-2, 1e-2, step_slack=0)
        assert c["ok"] and c["steps_ok"], c
        assert np.array_equal(g["stats"]["nreject"], o["stats"]["nreject"])
