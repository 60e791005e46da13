"""save_everystep together with saveat (_savevalues!, integrator_utils.jl:340-414:
the saveat points up to t by the step's interpolant, then the step itself unless
a saveat point landed on it; ode_saveat_tests.jl:44-124): on the GPU the saves
match the oracle's, the time set is the every-step set plus the saveat points,
for every method, both directions, fixed steps and the mixed form."""
import numpy as np
import pytest

from gpu_common import compare, gpu, oracle

pytestmark = pytest.mark.gpu

ALGS = ["tsit5", "vern7", "rodas5p", "rosenbrock23", "autotsit5_rosenbrock23"]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


@pytest.mark.parametrize("alg", ALGS)
def test_every_step_saves_with_saveat_match_oracle(alg):
    # u' = p u (p ~ U(-3, 3)), half of the spans backward (1, 0): every direction
    # and method takes a few dozen steps
    N = 256
    rng = np.random.default_rng(41)
    u0 = rng.uniform(0.5, 2.0, (1, N))
    p = rng.uniform(-3.0, 3.0, (1, N))
    ts = np.tile([[0.0], [1.0]], (1, N))
    ts[:, 1::2] = ts[::-1, 1::2].copy()
    rt = 1e-8 if alg in ("tsit5", "vern7") else 1e-6
    pts = [0.125, 0.6, 0.61, 0.8]
    kw = dict(save_everystep=True, max_step_saves=4096)
    g = gpu("linear", alg, u0, p, ts, pts, rt, rt, **kw)
    o = oracle("linear", alg, u0, p, ts, pts, rt, rt, **kw)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, rt, rt)
    assert c["ok"] and c["steps_ok"], c
    # the time set: every step, the start, and the four points
    ns = g["nsaved"]
    assert np.array_equal(ns, g["stats"]["naccept"] + 1 + len(pts))
    for j in (0, 1):
        t = g["t"][:ns[j], j]
        assert set(pts) <= set(t.tolist())
        assert np.all(np.diff(t) > 0) if j == 0 else np.all(np.diff(t) < 0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fixed_steps_every_step_and_saveat(precision):
    # ode_saveat_tests.jl:44-50 (RK4, dt = 1/4, adaptive = false): the step times
    # 0, 1/4, ..., 1 and the four points
    N = 64
    u0 = np.full((1, N), 0.5)
    p = np.full((1, N), 1.01)
    ts = np.tile([[0.0], [1.0]], (1, N))
    pts = [0.125, 0.6, 0.61, 0.8]
    g = gpu("linear", "tsit5", u0, p, ts, pts, 1e-6, 1e-6, precision=precision, adaptive=False, dt=0.25,
            save_everystep=True, max_step_saves=64)
    assert (g["nsaved"] == 9).all()
    assert np.array_equal(g["t"][:9, 0], [0.0, 0.125, 0.25, 0.5, 0.6, 0.61, 0.75, 0.8, 1.0])
    ex = 0.5 * np.exp(1.01 * g["t"][:9, 0])
    assert np.abs(g["u"][:9, 0, 0] - ex).max() < 1e-4
