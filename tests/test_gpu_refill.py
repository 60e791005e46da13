"""A lane group whose trajectory ends takes the next one inside the same step
loop (the persistent scheduler's refill).  Every trajectory's arithmetic is the
same whichever lane and slot runs it, so the persistent scheduler's results are
bitwise those of one group per trajectory (the static scheduler) -- for
trajectories whose step counts differ a hundredfold, for events and every-step
saves, for dense output, and for ensembles mixing both directions."""
import numpy as np
import pytest

from gpu_common import gpu, lorenz_inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


def same(a, b):
    assert np.array_equal(a["nsaved"], b["nsaved"]) and np.array_equal(a["retcode"], b["retcode"])
    for k in a["stats"]:
        assert np.array_equal(a["stats"][k], b["stats"][k]), k
    k = int(a["nsaved"].max())
    m = np.arange(k)[:, None] < a["nsaved"][None, :]
    assert np.array_equal(a["t"][:k][m], b["t"][:k][m])
    assert np.array_equal(a["u"][:k].transpose(1, 0, 2)[:, m], b["u"][:k].transpose(1, 0, 2)[:, m])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_van_der_pol_refill_is_bitwise_static(precision):
    # mu from 1 to 1000: AutoTsit5(Rosenbrock23()) takes from ~100 to ~6000 steps
    from odegb300 import workloads as W
    wl = W.van_der_pol(4096, seed=21)
    args = (wl["u0"], wl["p"], wl["tspan"], wl["saveat"], wl["reltol"], wl["abstol"])
    a = gpu("van_der_pol", "autotsit5_rosenbrock23", *args, precision=precision, scheduler="static")
    b = gpu("van_der_pol", "autotsit5_rosenbrock23", *args, precision=precision, scheduler="persistent")
    steps = a["stats"]["naccept"]
    assert steps.max() > 10 * steps.min()
    same(a, b)


@pytest.mark.parametrize("alg", ["tsit5", "rodas5p"])
def test_events_and_every_step_saves_refill_is_bitwise_static(alg):
    from odegb300 import ContinuousCallback
    from odegb300 import workloads as W
    wl = W.bouncing_ball(2048, seed=22)
    cb = ContinuousCallback(interp_points=10, max_events=16)
    kw = dict(callback=cb, save_everystep=True, max_step_saves=512)
    args = (wl["u0"], wl["p"], wl["tspan"], None, 1e-7, 1e-7)
    same(gpu("bouncing_ball", alg, *args, scheduler="static", **kw),
         gpu("bouncing_ball", alg, *args, scheduler="persistent", **kw))


def test_dense_and_both_directions_refill_is_bitwise_static():
    N = 2048
    u0, p, ts = lorenz_inputs(N, seed=23)
    ts[:, 1::3] = ts[::-1, 1::3].copy()        # every third trajectory runs backward
    ts[1, ::5] *= 10.0                          # spans of 1 and 10 (or -1 and -10)
    kw = dict(save_everystep=True, max_step_saves=4096, dense=True)
    a = gpu("lorenz", "vern7", u0, p, ts, None, 1e-8, 1e-8, scheduler="static", **kw)
    b = gpu("lorenz", "vern7", u0, p, ts, None, 1e-8, 1e-8, scheduler="persistent", **kw)
    same(a, b)
    k = int(a["nsaved"].max())
    m = np.arange(k)[:, None] < a["nsaved"][None, :]
    ka, kb = (r["k"][:k].transpose(1, 2, 0, 3)[:, :, m] for r in (a, b))
    assert np.array_equal(ka, kb, equal_nan=True)
