"""The four single-GPU workloads at their full sizes, checked through properties
that hold at any size (the oracle's per-trajectory comparison runs on samples
elsewhere; here every trajectory is checked):

* 100,000 Robertson trajectories (Rodas5P): y1 + y2 + y3 = 1 at every save (f
  sums to zero, so every Rosenbrock stage preserves the sum: a linear invariant);
* 10,000 Lorenz trajectories (Tsit5): every trajectory against the FP64 oracle;
* 1,000,000 uneven Duffing chains (Vern7, mixed, one launch): the damped chain's
  energy never grows between saves (dE/dt = -delta sum v^2);
* 65,536 Brusselators (Rodas5P, mixed): every trajectory succeeds and stays
  positive;

and every solve is bitwise repeatable (the kernels are deterministic).
"""
import ctypes as C

import numpy as np
import pytest

from gpu_common import ALG, compare, oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


def device_solve(wl, precision, ir=None):
    """Solve a workload through ode_solve_ensemble_device; outputs stay on the device."""
    import torch
    from odegb300 import EnsembleGB300, _lib
    from odegb300.ensemble import MODELS, _options, get_handle
    from odegb300.saveat import resolve_saveat
    L = _lib.load()
    h = get_handle(0)
    n, N = wl["u0"].shape
    sv = resolve_saveat(wl["saveat"], wl["tspan"])
    ir = wl.get("ir_sweeps", -1) if ir is None else ir
    ens = EnsembleGB300(precision=precision, ir_sweeps=ir if precision == "mixed" else -1)
    o = _options(wl["reltol"], wl["abstol"], None, None, None, 10 ** 6, sv, ens, None, None)
    d = _lib.ProblemDesc(MODELS[wl["model"]], ALG[wl["alg"]][0].alg_id, n, wl["p"].shape[0], ens.prec_id(), 0)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    cap = sv.cap
    out = {"t": torch.empty((cap, N), dtype=torch.float64, device=dev),
           "u": torch.empty((cap, n, N), dtype=torch.float64, device=dev),
           "nsaved": torch.empty(N, dtype=torch.int32, device=dev),
           "retcode": torch.empty(N, dtype=torch.int32, device=dev),
           "stats": torch.empty((N, 6), dtype=torch.int64, device=dev)}
    ins = [t(wl["u0"]), t(wl["p"]), t(wl["tspan"]), t(sv.values if sv.nsave else np.zeros(1))]
    npt = t(wl["n_per_traj"]) if wl.get("n_per_traj") is not None else None
    vp = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)   # the inputs' copies are done before the solve's stream reads them
    _lib.check(L.ode_solve_ensemble_device(h, C.byref(d), C.byref(o), N, vp(npt), *[vp(x) for x in ins],
                                           vp(out["t"]), vp(out["u"]), vp(out["nsaved"]), vp(out["retcode"]),
                                           vp(out["stats"]), C.c_void_p(stream.cuda_stream)), h)
    stream.synchronize()
    return out


def same(a, b, npt=None):
    """Bitwise equal saves (slots up to each trajectory's nsaved, states up to its size)."""
    import torch
    assert torch.equal(a["nsaved"], b["nsaved"]) and torch.equal(a["retcode"], b["retcode"])
    cap, n = a["u"].shape[0], a["u"].shape[1]
    dev = a["t"].device
    m = torch.arange(cap, device=dev)[:, None] < a["nsaved"][None, :].long()
    assert torch.equal(a["t"][m], b["t"][m])
    mu = m[:, None, :].expand_as(a["u"])
    if npt is not None:
        rows = torch.arange(n, device=dev)[:, None] < torch.from_numpy(npt).to(dev)[None, :].long()
        mu = mu & rows[None]
    assert torch.equal(a["u"][mu], b["u"][mu])


@pytest.mark.parametrize("precision,bound", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_robertson_100k_conserves_mass(precision, bound):
    from odegb300 import workloads as W
    wl = W.robertson(100_000, seed=11)
    g = device_solve(wl, precision)
    assert bool((g["retcode"] == 1).all()) and bool((g["nsaved"] == 20).all())
    s = g["u"][:20].sum(dim=1)
    assert float((s - 1.0).abs().max()) < bound
    same(g, device_solve(wl, precision))


def test_lorenz_10k_every_trajectory_against_the_oracle():
    from odegb300 import workloads as W
    wl = W.lorenz(10_000, seed=11)
    g = device_solve(wl, "fp64")
    host = {k: (v.cpu().numpy() if k != "stats" else
                {n: v[:, i].cpu().numpy() for i, n in enumerate(("nf", "njacs", "nw", "nsolve", "naccept",
                                                                  "nreject"))})
            for k, v in g.items()}
    o = oracle("lorenz", "tsit5", wl["u0"], wl["p"], wl["tspan"], wl["saveat"], wl["reltol"], wl["abstol"])
    c = compare(host, o, wl["reltol"], wl["abstol"])
    assert c["ok"] and c["steps_ok"], c
    same(g, device_solve(wl, "fp64"))


def test_duffing_1m_energy_never_grows():
    import torch
    from odegb300 import workloads as W
    wl = W.duffing(1_000_000, seed=11)
    g = device_solve(wl, "mixed")
    assert bool((g["retcode"] == 1).all()) and bool((g["nsaved"] == 16).all())
    dev = g["u"].device
    npt = torch.from_numpy(wl["n_per_traj"]).to(dev)
    u = g["u"][:16]
    nmax = u.shape[1]
    mask = (torch.arange(nmax, device=dev)[:, None] < npt[None, :]).to(u.dtype)
    u = u * mask[None]                         # rows past a chain's states are not written
    x, v = u[:, 0::2, :], u[:, 1::2, :]
    k, beta = [torch.from_numpy(wl["p"][i]).to(dev) for i in (0, 2)]
    zero = torch.zeros_like(x[:, :1, :])
    dx = torch.diff(torch.cat([zero, x, zero], dim=1), dim=1)   # fixed ends x_0 = x_{N+1} = 0
    E = 0.5 * (v * v).sum(1) + 0.5 * k * (dx * dx).sum(1) + 0.25 * beta * (x ** 4).sum(1)   # (16, N)
    growth = (E[1:] - E[:-1]) / E[0]
    assert float(growth.max()) < 1e-4, float(growth.max())
    del u, x, v, dx, E
    same(g, device_solve(wl, "mixed"), wl["n_per_traj"])


def test_brusselator_65536_succeeds_and_stays_positive():
    from odegb300 import workloads as W
    wl = W.brusselator(65_536, seed=11)
    g = device_solve(wl, "mixed", ir=0)
    assert bool((g["retcode"] == 1).all())
    assert bool((g["nsaved"] == 9).all())   # t0 and 1.25:1.25:10
    u = g["u"][1:9]   # after the start (a perturbed u0 may dip below zero; the source A > 0 lifts it)
    assert float(u.min()) > 0.0 and float(u.max()) < 100.0
    same(g, device_solve(wl, "mixed", ir=0))
