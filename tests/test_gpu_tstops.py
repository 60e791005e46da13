"""GPU parity for the solve's tstops: the reference's `tstops` keyword
(test/InterfaceI/ode_tstops_tests.jl), built as initialize_tstops
(lib/OrdinaryDiffEqCore/src/solve.jl:1021-1040) and stepped to by
modify_dt_for_tstops! / handle_tstop! (integrator_utils.jl:268-324, 1290-1313).

One tstops list is shared by the ensemble, unsorted, with duplicates and
entries outside some trajectories' spans: every trajectory must land exactly on
each tstop inside its own (t0, tf) and otherwise meet the FP64 parity bar
against the oracle (saves within 10x the tolerance, accepted steps within 1).
"""
import ctypes as C

import numpy as np
import pytest

from gpu_common import ROBER_SAVEAT, compare, gpu, lorenz_inputs, oracle, robertson_inputs

pytestmark = pytest.mark.gpu

TSTOPS = np.array([0.7, 0.05, 0.5, 0.5, 1.5, -1.0, 1.0 / 3.0, 0.95, 0.0, 1.0])
TOL = {"tsit5": (1e-8, 1e-8), "vern7": (1e-8, 1e-8), "rodas5p": (1e-7, 1e-9), "rosenbrock23": (1e-5, 1e-7),
       "autotsit5_rosenbrock23": (1e-7, 1e-9)}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


@pytest.mark.parametrize("alg", list(TOL))
def test_tstops_saveat_parity_fp64(alg):
    N = 256
    rt, at = TOL[alg]
    u0, p, ts = lorenz_inputs(N)
    g = gpu("lorenz", alg, u0, p, ts, 0.1, rt, at, tstops=TSTOPS)
    o = oracle("lorenz", alg, u0, p, ts, 0.1, rt, at, tstops=TSTOPS)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, rt, at)
    assert c["ok"] and c["steps_ok"], c
    for k in ("nf", "naccept", "nreject"):
        assert np.abs(g["stats"][k] - o["stats"][k]).max() <= 16, k
    # the tstops changed the step sequence
    o0 = oracle("lorenz", alg, u0, p, ts, 0.1, rt, at)
    assert (o["stats"]["naccept"] != o0["stats"]["naccept"]).any()


@pytest.mark.parametrize("alg", ["tsit5", "rodas5p", "rosenbrock23"])
def test_tstops_are_in_every_trajectorys_steps(alg):
    # ode_tstops_tests.jl:8-9, 43-61: each tstop inside the span is a step time
    N = 128
    rt, at = TOL[alg]
    rng = np.random.default_rng(11)
    u0, p, _ = lorenz_inputs(N)
    ts = np.vstack([rng.uniform(0.0, 0.2, N), rng.uniform(0.6, 1.0, N)])
    g = gpu("lorenz", alg, u0, p, ts, None, rt, at, save_everystep=True, max_step_saves=4096, tstops=TSTOPS)
    o = oracle("lorenz", alg, u0, p, ts, None, rt, at, save_everystep=True, max_step_saves=4096, tstops=TSTOPS)
    assert (g["retcode"] == 1).all()
    same_grid = 0
    for j in range(N):
        ns = int(g["nsaved"][j])
        tj = g["t"][:ns, j]
        assert np.all(np.diff(tj) > 0), j
        for t in TSTOPS:
            if ts[0, j] < t < ts[1, j]:
                assert t in tj, (j, t)
        assert not np.any((tj < ts[0, j]) | (tj > ts[1, j]))
        if ns == int(o["nsaved"][j]) and np.array_equal(tj, o["t"][:ns, j]):
            same_grid += 1
    assert same_grid >= 0.9 * N, same_grid
    assert np.abs(g["stats"]["naccept"] - o["stats"]["naccept"]).max() <= 1


def test_tstops_mixed_rodas5p_robertson():
    N = 512
    u0, p, ts = robertson_inputs(N)
    tst = np.array([1e3, 1e-3, 1.0, 50.0])
    g = gpu("robertson", "rodas5p", u0, p, ts, ROBER_SAVEAT, 1e-6, 1e-10, precision="mixed", tstops=tst)
    o = oracle("robertson", "rodas5p", u0, p, ts, ROBER_SAVEAT, 1e-6, 1e-10, tstops=tst)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, 1e-6, 1e-10, step_slack=10 ** 9)
    assert c["ok"], c
    ge = gpu("robertson", "rodas5p", u0[:, :64], p[:, :64], ts[:, :64], None, 1e-6, 1e-10, precision="mixed",
             save_everystep=True, max_step_saves=1024, tstops=tst)
    for j in range(64):
        tj = ge["t"][:int(ge["nsaved"][j]), j]
        for t in tst:
            assert t in tj, (j, t)


def test_tstops_device_entry_and_serving_match_host():
    import torch
    from gpu_common import ALG
    from odegb300 import EnsembleGB300, _lib
    from odegb300.ensemble import MODELS, _options, get_handle
    from odegb300.saveat import resolve_saveat
    from odegb300.serving import Server
    N = 200
    u0, p, ts = lorenz_inputs(N)
    rt, at = 1e-8, 1e-8
    host = gpu("lorenz", "tsit5", u0, p, ts, 0.1, rt, at, tstops=TSTOPS)
    # ode_solve_ensemble_device: tstops in device memory, sorted
    L = _lib.load()
    h = get_handle(0)
    sv = resolve_saveat(0.1, ts)
    ens = EnsembleGB300(precision="fp64")
    o = _options(rt, at, None, None, None, 10 ** 6, sv, ens, None, None)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    dts = t(np.sort(TSTOPS))
    o.ntstops = int(dts.numel())
    o.tstops = C.cast(C.c_void_p(dts.data_ptr()), C.POINTER(C.c_double))
    d = _lib.ProblemDesc(MODELS["lorenz"], ALG["tsit5"][0].alg_id, 3, 3, ens.prec_id(), 0)
    cap = sv.cap
    bufs = [t(u0), t(p), t(ts), t(sv.values), torch.empty((cap, N), dtype=torch.float64, device=dev),
            torch.empty((cap, 3, N), dtype=torch.float64, device=dev), torch.empty(N, dtype=torch.int32, device=dev),
            torch.empty(N, dtype=torch.int32, device=dev), torch.empty((N, 6), dtype=torch.int64, device=dev)]
    vp = lambda x: C.c_void_p(x.data_ptr())
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)   # the inputs' copies are done before the solve's stream reads them
    _lib.check(L.ode_solve_ensemble_device(h, C.byref(d), C.byref(o), N, None, *[vp(b) for b in bufs],
                                           C.c_void_p(stream.cuda_stream)), h)
    stream.synchronize()
    ns = bufs[6].cpu().numpy()
    assert np.array_equal(ns, host["nsaved"])
    k = int(ns.max())
    assert np.array_equal(bufs[5].cpu().numpy()[:k], host["u"][:k])
    assert np.array_equal(bufs[8].cpu().numpy()[:, 4], host["stats"]["naccept"])
    # the serving loop (ode_submit) copies the tstops with the request
    with Server(device=0) as srv:
        tk = srv.submit("lorenz", "tsit5", u0, p, ts, 0.1, rt, at, precision="fp64", tstops=TSTOPS)
        got = None
        for _ in range(600):
            r = srv.next_completed(timeout=0.1)
            if r is not None and r[0] == tk:
                got = r
                break
        assert got is not None and got[1] == 0
        out = got[3]
    assert np.array_equal(out["nsaved"], host["nsaved"])
    assert np.array_equal(out["u"][:k], host["u"][:k])


def test_nan_span_reports_initial_failure():
    # a trajectory with a NaN span is not stepped and reports ReturnCode.InitialFailure;
    # one running backward (tf < t0) beside the others is stepped; the rest are unaffected
    N = 64
    u0, p, ts = lorenz_inputs(N)
    ts = ts.copy()
    ts[:, 3] = [1.0, 0.5]
    ts[0, 7] = np.nan
    kw = dict(save_start=False, save_end=True)   # the spans differ, so the save flags are given
    g = gpu("lorenz", "tsit5", u0, p, ts, [0.5, 1.0], 1e-8, 1e-8, **kw)
    assert g["retcode"][7] == 8 and g["stats"]["naccept"][7] == 0
    assert g["retcode"][3] == 1 and g["stats"]["naccept"][3] > 0
    ok = np.setdiff1d(np.arange(N), [3, 7])
    assert (g["retcode"][ok] == 1).all()
    ref = gpu("lorenz", "tsit5", u0[:, ok], p[:, ok], ts[:, ok], [0.5, 1.0], 1e-8, 1e-8, **kw)
    assert np.array_equal(g["nsaved"][ok], ref["nsaved"])
    k = int(ref["nsaved"].max())   # slots past nsaved are not written
    assert np.array_equal(g["u"][:k, :, ok], ref["u"][:k])
