"""Array tolerances (solve(...; abstol = [...], reltol = [...]): calculate_residuals
broadcast over the per-state tolerances, calculate_residuals.jl:117-125, and the
initial step's scale) on the GPU: saves and step counts match the oracle's for
ROBER's classic per-species abstol (Rodas5P and Rosenbrock23, FP64 and mixed)
and for Lorenz with Tsit5 and Vern7; equal entries give the scalar solve bit for
bit; the device entry point takes the arrays in device memory; the host checks
them."""
import ctypes as C

import numpy as np
import pytest

from gpu_common import ROBER_SAVEAT, compare, gpu, lorenz_inputs, oracle, robertson_inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


@pytest.mark.parametrize("alg,precision", [("rodas5p", "fp64"), ("rodas5p", "mixed"), ("rosenbrock23", "fp64")])
def test_robertson_per_species_abstol_matches_oracle(alg, precision):
    N = 512
    u0, p, ts = robertson_inputs(N, seed=61)
    at = np.array([1e-8, 1e-14, 1e-6])
    rt = 1e-4 if alg == "rosenbrock23" else 1e-6
    g = gpu("robertson", alg, u0, p, ts, ROBER_SAVEAT, rt, at, precision=precision)
    o = oracle("robertson", alg, u0, p, ts, ROBER_SAVEAT, rt, at)
    assert (g["retcode"] == 1).all()
    if precision == "fp64":
        c = compare(g, o, rt, 1e-14)
        assert c["ok"] and c["steps_ok"], c
    else:   # the mixed form within 10x of the tightest tolerance against the FP64 oracle
        ns = int(o["nsaved"].max())
        err = np.abs(g["u"][:ns] - o["u"][:ns]) / (rt * np.abs(o["u"][:ns]) + at[None, :, None])
        assert np.nanmax(err) < 10.0
    sc = gpu("robertson", alg, u0, p, ts, ROBER_SAVEAT, rt, 1e-8, precision=precision)
    assert (g["stats"]["naccept"] > sc["stats"]["naccept"]).mean() > 0.5   # the 1e-14 species takes more steps


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
def test_lorenz_array_tolerances(alg):
    N = 256
    u0, p, ts = lorenz_inputs(N, seed=62)
    at, rt = np.array([1e-8, 1e-10, 1e-9]), np.array([1e-8, 1e-9, 1e-10])
    g = gpu("lorenz", alg, u0, p, ts, 0.1, rt, at)
    o = oracle("lorenz", alg, u0, p, ts, 0.1, rt, at)
    c = compare(g, o, 1e-8, 1e-8)
    assert c["ok"] and c["steps_ok"], c
    # equal entries: the scalar solve, bit for bit
    a = gpu("lorenz", alg, u0, p, ts, 0.1, np.full(3, 1e-8), np.full(3, 1e-9))
    b = gpu("lorenz", alg, u0, p, ts, 0.1, 1e-8, 1e-9)
    assert np.array_equal(a["nsaved"], b["nsaved"]) and np.array_equal(a["stats"]["nf"], b["stats"]["nf"])
    k = int(a["nsaved"].max())
    assert np.array_equal(a["u"][:k], b["u"][:k], equal_nan=True)


def test_device_arrays_and_host_checks():
    import torch
    from gpu_common import ALG
    from odegb300 import EnsembleGB300, _lib
    from odegb300.ensemble import MODELS, _options, get_handle
    from odegb300.saveat import resolve_saveat
    N = 128
    u0, p, ts = robertson_inputs(N, seed=63)
    at = np.array([1e-8, 1e-14, 1e-6])
    host = gpu("robertson", "rodas5p", u0, p, ts, ROBER_SAVEAT, 1e-6, at)
    L = _lib.load()
    h = get_handle(0)
    sv = resolve_saveat(ROBER_SAVEAT, ts)
    dev = torch.device("cuda", 0)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(dev)
    o = _options(1e-6, 1e-8, None, None, None, 10 ** 6, sv, EnsembleGB300(), None, None)
    datol = t(at)
    o.abstol_vec = C.cast(C.c_void_p(datol.data_ptr()), C.POINTER(C.c_double))
    d = _lib.ProblemDesc(MODELS["robertson"], ALG["rodas5p"][0].alg_id, 3, 3, 0, 0)
    cap = sv.cap
    outs = [torch.empty((cap, N), dtype=torch.float64, device=dev),
            torch.empty((cap, 3, N), dtype=torch.float64, device=dev),
            torch.empty(N, dtype=torch.int32, device=dev), torch.empty(N, dtype=torch.int32, device=dev),
            torch.empty((N, 6), dtype=torch.int64, device=dev)]
    vp = lambda x: C.c_void_p(x.data_ptr())
    ins = [t(u0), t(p), t(ts), t(sv.values)]
    torch.cuda.synchronize(dev)   # the inputs' copies (current stream) are done before the solve's stream reads them
    stream = torch.cuda.Stream(dev)
    _lib.check(L.ode_solve_ensemble_device(h, C.byref(d), C.byref(o), N, None, *[vp(x) for x in ins + outs],
                                           C.c_void_p(stream.cuda_stream)), h)
    stream.synchronize()
    k = int(host["nsaved"].max())
    assert np.array_equal(outs[2].cpu().numpy(), host["nsaved"])
    assert np.array_equal(outs[1].cpu().numpy()[:k], host["u"][:k])
    with pytest.raises(_lib.OdeError):
        gpu("robertson", "rodas5p", u0, p, ts, ROBER_SAVEAT, 1e-6, np.array([1e-8, -1.0, 1e-6]))


def test_uneven_chains_with_array_tolerances():
    # the one-launch class kernel: each chain takes the first n entries of the arrays
    from gpu_common import duffing_inputs
    N = 4096
    u0, p, ts, sv, npt = duffing_inputs(N, [2, 4, 8], tf_range=(1.0, 3.0), seed=64)
    nmax = u0.shape[0]
    at = np.where(np.arange(nmax) % 2 == 0, 1e-9, 1e-7)   # positions tighter than velocities
    rt = np.full(nmax, 1e-8)
    g = gpu("duffing_chain", "vern7", u0, p, ts, sv, rt, at, n_per_traj=npt)
    o = oracle("duffing_chain", "vern7", u0, p, ts, sv, rt, at, n_per_traj=npt)
    c = compare(g, o, 1e-8, 1e-8)
    assert c["ok"] and c["steps_ok"], c
