"""The reference's save_idxs (solve keyword; copyat_or_push!(sol.u, ..., u[save_idxs])
in savevalues!, lib/OrdinaryDiffEqCore/src/integrators/integrator_utils.jl): only
the chosen states are saved, one output row each, in the given order.  Every
entry point gives rows bit-identical to the same rows of a full solve."""
import ctypes as C

import numpy as np
import pytest

from gpu_common import duffing_inputs, gpu, lorenz_inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


def rows_equal(sub, full, idx, npt=None):
    assert np.array_equal(sub["nsaved"], full["nsaved"]) and np.array_equal(sub["retcode"], full["retcode"])
    k = int(full["nsaved"].max())
    m = np.arange(k)[:, None] < full["nsaved"][None, :]
    assert np.array_equal(sub["t"][:k][m], full["t"][:k][m])
    for r, i in enumerate(idx):
        valid = m if npt is None else m & (i < np.asarray(npt))[None, :]
        assert np.array_equal(sub["u"][:k, r][valid], full["u"][:k, i][valid]), (r, i)


@pytest.mark.parametrize("alg,precision", [("tsit5", "fp64"), ("vern7", "mixed"), ("rodas5p", "fp64")])
def test_host_solve_saves_the_chosen_states(alg, precision):
    N = 512
    u0, p, ts = lorenz_inputs(N, seed=2)
    full = gpu("lorenz", alg, u0, p, ts, 0.1, 1e-8, 1e-8, precision=precision)
    idx = [2, 0, 2]
    sub = gpu("lorenz", alg, u0, p, ts, 0.1, 1e-8, 1e-8, precision=precision, save_idxs=idx)
    assert sub["u"].shape[1] == 3
    rows_equal(sub, full, idx)


def test_pipelined_uneven_solve_with_save_idxs():
    # 40,000 uneven chains take the sliced copy/compute pipeline; a state past a
    # smaller chain's size leaves its row unwritten
    N = 40000
    u0, p, ts, sv, npt = duffing_inputs(N, [2, 4, 8, 16, 32], tf_range=(1.0, 3.0), seed=5)
    idx = [0, 5, 31]
    kw = dict(precision="mixed", n_per_traj=npt)
    full = gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, **kw)
    sub = gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, save_idxs=idx, **kw)
    rows_equal(sub, full, idx, npt)


def test_events_with_save_idxs():
    from odegb300 import ContinuousCallback
    from odegb300 import workloads as W
    wl = W.bouncing_ball(256, seed=4)
    cb = ContinuousCallback(interp_points=10, max_events=8)
    full = gpu("bouncing_ball", "tsit5", wl["u0"], wl["p"], wl["tspan"], 0.25, 1e-8, 1e-8, callback=cb)
    sub = gpu("bouncing_ball", "tsit5", wl["u0"], wl["p"], wl["tspan"], 0.25, 1e-8, 1e-8, callback=cb, save_idxs=[1])
    rows_equal(sub, full, [1])


def test_device_entry_and_serving_with_save_idxs():
    import torch
    from gpu_common import ALG
    from odegb300 import EnsembleGB300, _lib
    from odegb300.ensemble import MODELS, _options, get_handle
    from odegb300.saveat import resolve_saveat
    from odegb300.serving import Server
    N = 300
    u0, p, ts = lorenz_inputs(N, seed=7)
    idx = [1, 2]
    full = gpu("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8)
    # ode_solve_ensemble_device: save_idxs in device memory
    L = _lib.load()
    h = get_handle(0)
    sv = resolve_saveat(0.1, ts)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    didx = t(np.array(idx, dtype=np.int32))
    o = _options(1e-8, 1e-8, None, None, None, 10 ** 6, sv, EnsembleGB300(), None, None)
    o.nsave_idxs = len(idx)
    o.save_idxs = C.cast(C.c_void_p(didx.data_ptr()), C.POINTER(C.c_int32))
    d = _lib.ProblemDesc(MODELS["lorenz"], ALG["tsit5"][0].alg_id, 3, 3, 0, 0)
    cap = sv.cap
    bufs = [t(u0), t(p), t(ts), t(sv.values), torch.empty((cap, N), dtype=torch.float64, device=dev),
            torch.full((cap, len(idx), N), float("nan"), dtype=torch.float64, device=dev),
            torch.empty(N, dtype=torch.int32, device=dev), torch.empty(N, dtype=torch.int32, device=dev),
            torch.empty((N, 6), dtype=torch.int64, device=dev)]
    vp = lambda x: C.c_void_p(x.data_ptr())
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)   # the inputs' copies are done before the solve's stream reads them
    _lib.check(L.ode_solve_ensemble_device(h, C.byref(d), C.byref(o), N, None, *[vp(b) for b in bufs],
                                           C.c_void_p(stream.cuda_stream)), h)
    stream.synchronize()
    dsub = {"t": bufs[4].cpu().numpy(), "u": bufs[5].cpu().numpy(), "nsaved": bufs[6].cpu().numpy(),
            "retcode": bufs[7].cpu().numpy()}
    rows_equal(dsub, full, idx)
    # the serving loop copies the save_idxs with the request
    with Server(device=0) as srv:
        tk = srv.submit("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8, precision="fp64", save_idxs=idx)
        got = None
        for _ in range(600):
            r = srv.next_completed(timeout=0.1)
            if r is not None and r[0] == tk:
                got = r
                break
        assert got is not None and got[1] == 0
    rows_equal(got[3], full, idx)


def test_front_door_and_checks():
    from odegb300 import EnsembleGB300, EnsembleProblem, ODEProblem, Tsit5, solve, _lib
    prob = ODEProblem("lorenz", [1.0, 0.0, 0.0], (0.0, 1.0), [10.0, 28.0, 8 / 3])
    sim = solve(EnsembleProblem(prob), Tsit5(), EnsembleGB300(), trajectories=4, saveat=0.25, reltol=1e-8,
                abstol=1e-8, save_idxs=[2])
    full = solve(EnsembleProblem(prob), Tsit5(), EnsembleGB300(), trajectories=4, saveat=0.25, reltol=1e-8,
                 abstol=1e-8)
    assert len(sim.u[0].u[0]) == 1
    assert [v[0] for v in sim.u[0].u] == [v[2] for v in full.u[0].u]
    # a host index outside the states is rejected before any device work
    u0, p, ts = lorenz_inputs(8)
    with pytest.raises(_lib.OdeError):
        gpu("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8, save_idxs=[3])
    with pytest.raises(ValueError):
        gpu("lorenz", "tsit5", u0, p, ts, None, 1e-8, 1e-8, save_everystep=True, dense=True, save_idxs=[0])
