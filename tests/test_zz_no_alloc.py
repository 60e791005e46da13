"""The allocation-free entry point (ode_solve_ensemble_noalloc) against the
regular device entry point.

Callers that cannot allocate device memory (a framework's caching allocator
owns the GPU, or a fixed memory budget) use ode_solve_ensemble_noalloc: its
scratch is a fixed array inside the library.  This checks, through the C ABI,
that two calls in a row give the same saves, counters and retcodes as
ode_solve_ensemble_device, both for the size-bucketed path (which uses the
array's index list) and for the uniform-size path (counters only).  The file
name sorts last so a stop-at-first-failure run has already run every other
test.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_common import compare, duffing_inputs, lorenz_inputs

pytestmark = pytest.mark.gpu


def _device_solve(entry, model, alg_id, prec, u0, p, ts, saveat, reltol, abstol, npt=None):
    import torch
    from odegb300 import _lib
    from odegb300.ensemble import EnsembleGB300, _options, get_handle
    from odegb300.saveat import resolve_saveat

    L = _lib.load()
    dev = torch.device("cuda", 0)
    n, N = u0.shape
    sv = resolve_saveat(saveat, ts)
    cap = sv.cap
    ens = EnsembleGB300(precision=prec)
    o = _options(reltol, abstol, None, None, None, 1000000, sv, ens, None, None)
    d = _lib.ProblemDesc(model, alg_id, n, p.shape[0], ens.prec_id(), 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    b_u0, b_p, b_ts, b_sv = t(u0), t(p), t(ts), t(sv.values)
    b_npt = t(npt) if npt is not None else None
    t_out = torch.full((cap, N), float("nan"), dtype=torch.float64, device=dev)
    u_out = torch.full((cap, n, N), float("nan"), dtype=torch.float64, device=dev)
    ns = torch.zeros(N, dtype=torch.int32, device=dev)
    rc = torch.zeros(N, dtype=torch.int32, device=dev)
    st = torch.zeros((N, 6), dtype=torch.int64, device=dev)
    ptr = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None
    torch.cuda.synchronize(dev)   # the inputs' copies are done before the solve's stream reads them
    stream = torch.cuda.Stream(dev)
    args = (C.byref(d), C.byref(o), N, ptr(b_npt), ptr(b_u0), ptr(b_p), ptr(b_ts), ptr(b_sv), ptr(t_out),
            ptr(u_out), ptr(ns), ptr(rc), ptr(st), C.c_void_p(stream.cuda_stream))
    if entry == "device":
        h = get_handle(0)
        status = L.ode_solve_ensemble_device(h, *args)
        _lib.check(status, h)
    else:
        status = L.ode_solve_ensemble_noalloc(*args)
        _lib.check(status, None)
    stream.synchronize()
    names = ("nf", "njacs", "nw", "nsolve", "naccept", "nreject")
    s = st.cpu().numpy()
    return {"t": t_out.cpu().numpy(), "u": u_out.cpu().numpy(), "nsaved": ns.cpu().numpy(),
            "retcode": rc.cpu().numpy(), "stats": {k: s[:, i] for i, k in enumerate(names)}}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_noalloc_bucketed_matches_device_entry(prec):
    from odegb300 import _lib
    N = 700
    u0, p, ts, sv, npt = duffing_inputs(N, [2, 4, 8, 16, 32], seed=11, tf_range=(1.0, 10.0))
    ref = _device_solve("device", _lib.MODEL_DUFFING_CHAIN, _lib.ODE_VERN7, prec, u0, p, ts, sv, 1e-6, 1e-6, npt)
    for _ in range(2):  # the shared scratch keeps the last call's contents; both calls must match
        got = _device_solve("noalloc", _lib.MODEL_DUFFING_CHAIN, _lib.ODE_VERN7, prec, u0, p, ts, sv, 1e-6, 1e-6,
                            npt)
        c = compare(got, ref, 1e-6, 1e-6, step_slack=0)
        assert c["ok"] and c["steps_ok"], c
        assert np.array_equal(got["stats"]["naccept"], ref["stats"]["naccept"])
        assert (got["retcode"] == 1).all()


def test_noalloc_uniform_matches_device_entry():
    from odegb300 import _lib
    N = 3000
    u0, p, ts = lorenz_inputs(N, seed=5)
    ref = _device_solve("device", _lib.MODEL_LORENZ, _lib.ODE_TSIT5, "fp64", u0, p, ts, 0.1, 1e-8, 1e-8)
    for _ in range(2):
        got = _device_solve("noalloc", _lib.MODEL_LORENZ, _lib.ODE_TSIT5, "fp64", u0, p, ts, 0.1, 1e-8, 1e-8)
        c = compare(got, ref, 1e-8, 1e-8, step_slack=0)
        assert c["ok"] and c["steps_ok"], c
        assert np.array_equal(got["u"], ref["u"], equal_nan=True)


@pytest.mark.parametrize("alg", ["rodas5p", "rosenbrock23"])
def test_noalloc_per_class_kernels_match_device_entry(alg):
    # methods without a one-launch class kernel run one kernel per size class,
    # from per-class queues inside the fixed array
    from odegb300 import _lib
    alg_id = {"rodas5p": _lib.ODE_RODAS5P, "rosenbrock23": _lib.ODE_ROSENBROCK23}[alg]
    N = 500
    u0, p, ts, sv, npt = duffing_inputs(N, 2, seed=13, tf_range=(1.0, 10.0))
    ref = _device_solve("device", _lib.MODEL_DUFFING_CHAIN, alg_id, "fp64", u0, p, ts, sv, 1e-6, 1e-6, npt)
    for _ in range(2):
        got = _device_solve("noalloc", _lib.MODEL_DUFFING_CHAIN, alg_id, "fp64", u0, p, ts, sv, 1e-6, 1e-6, npt)
        assert np.array_equal(got["u"], ref["u"], equal_nan=True)
        assert np.array_equal(got["nsaved"], ref["nsaved"]) and (got["retcode"] == 1).all()
        assert np.array_equal(got["stats"]["naccept"], ref["stats"]["naccept"])


def test_noalloc_size_class_without_kernel_is_rejected_before_outputs_are_written():
    # Rodas5P is compiled for 4-state Duffing chains only: an ensemble with
    # 8-state chains fails with ODE_E_UNSUPPORTED (-4), and the outputs keep the
    # caller's contents (nothing was scattered or integrated)
    import torch
    from odegb300 import _lib
    from odegb300.ensemble import EnsembleGB300, _options
    from odegb300.saveat import resolve_saveat
    L = _lib.load()
    dev = torch.device("cuda", 0)
    N = 64
    u0, p, ts, sv, npt = duffing_inputs(N, [2, 4], seed=3, tf_range=(1.0, 2.0))
    s = resolve_saveat(sv, ts)
    o = _options(1e-6, 1e-6, None, None, None, 1000000, s, EnsembleGB300(), None, None)
    d = _lib.ProblemDesc(_lib.MODEL_DUFFING_CHAIN, _lib.ODE_RODAS5P, u0.shape[0], 3, 0, 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    b_u0, b_p, b_ts, b_sv, b_npt = t(u0), t(p), t(ts), t(s.values), t(npt)
    u_out = torch.full((s.cap, u0.shape[0], N), 7.0, dtype=torch.float64, device=dev)
    ns = torch.full((N,), -5, dtype=torch.int32, device=dev)
    rc = torch.full((N,), -5, dtype=torch.int32, device=dev)
    ptr = lambda x: C.c_void_p(x.data_ptr())
    status = L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), N, ptr(b_npt), ptr(b_u0), ptr(b_p), ptr(b_ts),
                                          ptr(b_sv), None, ptr(u_out), ptr(ns), ptr(rc), None, None)
    torch.cuda.synchronize()
    assert status == -4, status
    assert b"8-state" in L.ode_last_error(None)
    assert (ns.cpu().numpy() == -5).all() and (rc.cpu().numpy() == -5).all()
    assert (u_out.cpu().numpy() == 7.0).all()


def test_noalloc_rejects_oversized_bucketed_request():
    from odegb300 import _lib
    L = _lib.load()
    o = _lib.Options()
    L.ode_options_default(C.byref(o))
    d = _lib.ProblemDesc(_lib.MODEL_DUFFING_CHAIN, _lib.ODE_VERN7, 64, 3, 0, 0)
    fake = C.c_void_p(16)  # never dereferenced: the size check comes first
    status = L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), (1 << 20) + 1, fake, fake, fake, fake, None,
                                          fake, fake, fake, fake, fake, None)
    assert status == -1
    assert b"maximum" in L.ode_last_error(None)
