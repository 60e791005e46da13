"""Kernel forms that must agree bit for bit.  (1) A lane group whose trajectory
ends takes the next one inside the same step loop (the persistent scheduler's
refill).  Every trajectory's arithmetic is the same whichever lane and slot
runs it, so the persistent scheduler's results are bitwise those of one group
per trajectory (the static scheduler) -- for trajectories whose step counts
differ a hundredfold, for events and every-step saves, for dense output, and
for ensembles mixing both directions.  (2) The forward-only kernels (no
integration direction in the step loop) give the general kernels' results."""
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


def device_solve(wl, precision, forward_only, ir=None, sv_tspan=None):
    """ode_solve_ensemble_device with the caller's forward_only statement (the save
    rules resolved on sv_tspan when given)."""
    import ctypes as C
    import torch
    from gpu_common import ALG
    from odegb300 import EnsembleGB300, _lib
    from odegb300.ensemble import MODELS, _options, get_handle
    from odegb300.saveat import resolve_saveat
    L = _lib.load()
    h = get_handle(0)
    n, N = wl["u0"].shape
    sv = resolve_saveat(wl["saveat"], wl["tspan"] if sv_tspan is None else sv_tspan)
    ir = wl.get("ir_sweeps", -1) if ir is None else ir
    ens = EnsembleGB300(precision=precision, ir_sweeps=ir if precision == "mixed" else -1)
    o = _options(wl["reltol"], wl["abstol"], None, None, None, 10 ** 6, sv, ens, None, None)
    o.forward_only = forward_only
    d = _lib.ProblemDesc(MODELS[wl["model"]], ALG[wl["alg"]][0].alg_id, n, wl["p"].shape[0], ens.prec_id(), 0)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    cap = sv.cap
    outs = [torch.empty((cap, N), dtype=torch.float64, device=dev),
            torch.empty((cap, n, N), dtype=torch.float64, device=dev),
            torch.empty(N, dtype=torch.int32, device=dev), torch.empty(N, dtype=torch.int32, device=dev),
            torch.empty((N, 6), dtype=torch.int64, device=dev)]
    ins = [t(wl["u0"]), t(wl["p"]), t(wl["tspan"]), t(sv.values if sv.nsave else np.zeros(1))]
    npt = t(wl["n_per_traj"]) if wl.get("n_per_traj") is not None else None
    vp = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)   # the inputs' copies are done before the solve's stream reads them
    _lib.check(L.ode_solve_ensemble_device(h, C.byref(d), C.byref(o), N, vp(npt), *[vp(x) for x in ins + outs],
                                           C.c_void_p(stream.cuda_stream)), h)
    stream.synchronize()
    names = ("nf", "njacs", "nw", "nsolve", "naccept", "nreject")
    st = outs[4].cpu().numpy()
    return {"t": outs[0].cpu().numpy(), "u": outs[1].cpu().numpy(), "nsaved": outs[2].cpu().numpy(),
            "retcode": outs[3].cpu().numpy(), "stats": {k: st[:, i] for i, k in enumerate(names)}}


@pytest.mark.parametrize("name,precision", [("robertson", "mixed"), ("robertson", "fp64"), ("lorenz", "fp64"),
                                            ("duffing", "mixed"), ("brusselator", "mixed")])
def test_forward_only_form_is_bitwise_the_general_one(name, precision):
    # the forward-only kernels (no direction in the step loop) of the benchmarked
    # workloads give the general kernels' results bit for bit
    from odegb300 import workloads as W
    wl = {"robertson": lambda: W.robertson(4096, seed=31), "lorenz": lambda: W.lorenz(2048, seed=31),
          "duffing": lambda: W.duffing(8192, seed=31), "brusselator": lambda: W.brusselator(256, seed=31)}[name]()
    ir = 0 if name == "brusselator" else None
    same(device_solve(wl, precision, 0, ir), device_solve(wl, precision, 1, ir))


def test_forward_only_statement_with_a_backward_span():
    # a caller that states forward spans but passes a backward one gets InitialFailure
    # for it (the forward-only loop has no direction), the rest unchanged
    from odegb300 import workloads as W
    wl = W.robertson(1024, seed=32)
    fwd = wl["tspan"].copy()
    wl["tspan"][:, 5] = wl["tspan"][::-1, 5].copy()
    a, b = device_solve(wl, "mixed", 0, sv_tspan=fwd), device_solve(wl, "mixed", 1, sv_tspan=fwd)
    assert a["retcode"][5] == 1 and b["retcode"][5] != 1
    keep = np.arange(1024) != 5
    sub = lambda r: {k: (v[..., keep] if k != "stats" else {n: x[keep] for n, x in v.items()}) for k, v in r.items()}
    same(sub(a), sub(b))
