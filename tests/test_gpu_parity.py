"""GPU parity: the CUDA kernels (through the C ABI) against the CPU oracle.

Bar: per-trajectory saveat values within 10x the tolerance (10*(reltol*|u| + abstol))
and accepted-step counts within 1 for the FP64 path.  The mixed path must be as
accurate as the FP64 path against a ground-truth solve (Vern9 at 1e-14, or
Rodas5P at 1e-12 for stiff models), and agree with the FP64 oracle within 10x
the tolerance (all trajectories of the well-conditioned Robertson ensemble,
95% of the Duffing chains, some of which amplify perturbations ~10^4-fold).
"""
import numpy as np
import pytest

from gpu_common import (ROBER_SAVEAT, brusselator_inputs, compare, duffing_inputs, err_vs, gpu, lorenz_inputs,
                        oracle, robertson_inputs, truth)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
def test_lorenz_fp64(alg):
    N = 512
    u0, p, ts = lorenz_inputs(N)
    g = gpu("lorenz", alg, u0, p, ts, 0.1, 1e-8, 1e-8)
    o = oracle("lorenz", alg, u0, p, ts, 0.1, 1e-8, 1e-8)
    assert g["nsaved"].min() == 11
    c = compare(g, o, 1e-8, 1e-8)
    assert c["ok"] and c["steps_ok"], c
    # same operation order on both sides: most trajectories are bit-identical
    assert c["frac_bit_identical"] > 0.9, c


def test_robertson_rodas5p_fp64():
    N = 512
    u0, p, ts = robertson_inputs(N)
    g = gpu("robertson", "rodas5p", u0, p, ts, ROBER_SAVEAT, 1e-6, 1e-10)
    o = oracle("robertson", "rodas5p", u0, p, ts, ROBER_SAVEAT, 1e-6, 1e-10)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, 1e-6, 1e-10)
    assert c["ok"] and c["steps_ok"], c
    for k in ("nf", "njacs", "nw", "nsolve", "naccept", "nreject"):
        assert np.abs(g["stats"][k] - o["stats"][k]).max() <= 16, k


def assert_equal_accuracy(gmx, g64, tr, reltol, abstol):
    """The mixed form is as accurate as the FP64 form: its error against the ground
    truth stays within 2x the FP64 form's (plus one tolerance unit), at the median
    and at the 90th percentile of trajectories."""
    emx, e64 = err_vs(gmx, tr, reltol, abstol), err_vs(g64, tr, reltol, abstol)
    for q in (50, 90):
        a, b = np.percentile(emx, q), np.percentile(e64, q)
        assert a <= 2.0 * b + 1.0, (q, a, b)
    return emx, e64


@pytest.mark.parametrize("ir", [0, 1])
def test_robertson_rodas5p_mixed(ir):
    N = 512
    u0, p, ts = robertson_inputs(N)
    g = gpu("robertson", "rodas5p", u0, p, ts, ROBER_SAVEAT, 1e-6, 1e-10, precision="mixed", ir_sweeps=ir)
    o = oracle("robertson", "rodas5p", u0, p, ts, ROBER_SAVEAT, 1e-6, 1e-10)
    assert (g["retcode"] == 1).all()
    # well conditioned: every trajectory within 10x the tolerance of the FP64 oracle
    c = compare(g, o, 1e-6, 1e-10, step_slack=10 ** 9)
    assert c["ok"], c
    g64 = gpu("robertson", "rodas5p", u0, p, ts, ROBER_SAVEAT, 1e-6, 1e-10)
    tr = truth("robertson", u0, p, ts, ROBER_SAVEAT, stiff=True)
    assert_equal_accuracy(g, g64, tr, 1e-6, 1e-10)


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
@pytest.mark.parametrize("n_osc", [2, 4, 8, 16, 32])
def test_duffing_fp64_lane_groups(alg, n_osc):
    N = 256
    u0, p, ts, sv, _ = duffing_inputs(N, n_osc, tf_range=(1.0, 10.0))
    g = gpu("duffing_chain", alg, u0, p, ts, sv, 1e-6, 1e-6)
    o = oracle("duffing_chain", alg, u0, p, ts, sv, 1e-6, 1e-6)
    c = compare(g, o, 1e-6, 1e-6)
    assert c["ok"] and c["steps_ok"], c


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
@pytest.mark.parametrize("n_osc", [2, 4, 16])
def test_duffing_mixed(alg, n_osc):
    # Some chains amplify a 1e-10 relative change of u0 to ~0.5x the tolerance by
    # t = 10, so FP32 stage arithmetic cannot track the FP64 path on every
    # trajectory; the bar is accuracy against the ground truth (as good as FP64)
    # and 10x-tolerance agreement with FP64 on at least 95% of trajectories.
    N = 256
    u0, p, ts, sv, _ = duffing_inputs(N, n_osc, tf_range=(1.0, 10.0))
    g = gpu("duffing_chain", alg, u0, p, ts, sv, 1e-6, 1e-6, precision="mixed")
    o = oracle("duffing_chain", alg, u0, p, ts, sv, 1e-6, 1e-6)
    d = err_vs(g, o, 1e-6, 1e-6)
    assert np.mean(d <= 10.0) >= 0.95, np.sort(d)[-10:]
    g64 = gpu("duffing_chain", alg, u0, p, ts, sv, 1e-6, 1e-6)
    tr = truth("duffing_chain", u0, p, ts, sv)
    assert_equal_accuracy(g, g64, tr, 1e-6, 1e-6)


def assert_within_conditioning(g, u0, p, ts, sv, reltol, abstol, npt=None, alg="vern7"):
    """The mixed form against the FP64 oracle, next to a conditioning control: the
    FP64 kernel on u0 perturbed by one FP32 rounding (1 + 2^-24) against the same
    oracle.  The mixed form's spread may not exceed the control's by more than 2x
    (+1 tolerance unit) at the median, p90 and p99, and 90% of its trajectories
    stay within 10x the tolerance."""
    o = oracle("duffing_chain", alg, u0, p, ts, sv, reltol, abstol, n_per_traj=npt)
    kw = {"n_per_traj": npt} if npt is not None else {}
    ctl = gpu("duffing_chain", alg, u0 * (1.0 + 2.0 ** -24), p, ts, sv, reltol, abstol, **kw)
    d, dc = err_vs(g, o, reltol, abstol), err_vs(ctl, o, reltol, abstol)
    for q in (50, 90, 99):
        a, b = np.percentile(d, q), np.percentile(dc, q)
        assert a <= 2.0 * b + 1.0, (q, a, b)
    assert np.mean(d <= 10.0) >= 0.9, np.sort(d)[-10:]
    return d, dc


@pytest.mark.parametrize("n_osc", [8, 32])
def test_duffing_mixed_vern7_long_spans(n_osc):
    # the C3 distribution's long half: tf log-uniform in [1, 100] (step counts vary ~50x)
    N = 512
    u0, p, ts, sv, _ = duffing_inputs(N, n_osc, seed=21, tf_range=(1.0, 100.0))
    g = gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, precision="mixed")
    assert (g["retcode"] == 1).all()
    assert_within_conditioning(g, u0, p, ts, sv, 1e-6, 1e-6)
    g64 = gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6)
    tr = truth("duffing_chain", u0, p, ts, sv)
    assert_equal_accuracy(g, g64, tr, 1e-6, 1e-6)


def test_duffing_uneven_mixed_one_launch_against_oracle():
    # the one-launch mixed kernel over every size class, tf up to 100, against the FP64 oracle
    N = 2048
    u0, p, ts, sv, npt = duffing_inputs(N, [2, 4, 8, 16, 32], seed=31, tf_range=(1.0, 100.0))
    g = gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, precision="mixed", n_per_traj=npt)
    assert (g["retcode"] == 1).all()
    assert_within_conditioning(g, u0, p, ts, sv, 1e-6, 1e-6, npt=npt)
    g64 = gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, n_per_traj=npt)
    tr = truth("duffing_chain", u0, p, ts, sv, n_per_traj=npt)
    assert_equal_accuracy(g, g64, tr, 1e-6, 1e-6)


@pytest.mark.parametrize("cells", [8, 16, 32])
def test_brusselator_rodas5p_fp64_shared_memory_lu(cells):
    # 16 to 64 states: one lane group per trajectory, W and its LU in shared memory
    N = 128
    u0, p, ts = brusselator_inputs(N, cells=cells)
    g = gpu("brusselator_1d", "rodas5p", u0, p, ts, 1.25, 1e-5, 1e-8)
    o = oracle("brusselator_1d", "rodas5p", u0, p, ts, 1.25, 1e-5, 1e-8)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, 1e-5, 1e-8)
    assert c["ok"] and c["steps_ok"], c
    assert (g["stats"]["njacs"] == o["stats"]["njacs"]).mean() > 0.9


def test_brusselator_lane_layouts_agree():
    # 64 states on 32 lanes x 2 rows and on 16 lanes x 4 rows: same factorisation
    N = 128
    u0, p, ts = brusselator_inputs(N, cells=32, seed=3)
    a = gpu("brusselator_1d", "rodas5p", u0, p, ts, 1.25, 1e-5, 1e-8, lanes=32)
    b = gpu("brusselator_1d", "rodas5p", u0, p, ts, 1.25, 1e-5, 1e-8, lanes=16)
    c = compare(a, b, 1e-5, 1e-8, factor=1.0)
    assert c["ok"] and c["steps_ok"], c


@pytest.mark.parametrize("ir", [0, 1])
def test_brusselator_rodas5p_mixed(ir):
    # FP32 W and LU; with ir = 1 each solve takes one refinement sweep whose
    # residual is formed in double-float
    N = 128
    u0, p, ts = brusselator_inputs(N, cells=32)
    g = gpu("brusselator_1d", "rodas5p", u0, p, ts, 1.25, 1e-5, 1e-8, precision="mixed", ir_sweeps=ir)
    o = oracle("brusselator_1d", "rodas5p", u0, p, ts, 1.25, 1e-5, 1e-8)
    assert (g["retcode"] == 1).all()
    c = compare(g, o, 1e-5, 1e-8, step_slack=10 ** 9)
    assert c["ok"], c
    g64 = gpu("brusselator_1d", "rodas5p", u0, p, ts, 1.25, 1e-5, 1e-8)
    tr = truth("brusselator_1d", u0, p, ts, 1.25, stiff=True)
    assert_equal_accuracy(g, g64, tr, 1e-5, 1e-8)


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
def test_duffing_uneven_sizes_one_launch(alg):
    # every size class in one persistent launch (device bucketing, no host round trip)
    N = 600
    u0, p, ts, sv, npt = duffing_inputs(N, [2, 4, 8, 16, 32], tf_range=(1.0, 10.0))
    g = gpu("duffing_chain", alg, u0, p, ts, sv, 1e-6, 1e-6, n_per_traj=npt)
    o = oracle("duffing_chain", alg, u0, p, ts, sv, 1e-6, 1e-6, n_per_traj=npt)
    c = compare(g, o, 1e-6, 1e-6)
    assert c["ok"] and c["steps_ok"], c


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_uneven_one_launch_equals_one_kernel_per_class(precision):
    # lanes_per_traj > 0 selects the one-kernel-per-class form (same lane
    # layout per class): results must be bit-identical to the single launch
    N = 400
    u0, p, ts, sv, npt = duffing_inputs(N, [2, 4, 8, 16, 32], tf_range=(1.0, 10.0), seed=11)
    a = gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, precision=precision, n_per_traj=npt)
    b = gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, precision=precision, n_per_traj=npt, lanes=4)
    assert np.array_equal(a["u"], b["u"], equal_nan=True)
    assert np.array_equal(a["stats"]["naccept"], b["stats"]["naccept"])


def test_uneven_sizes_must_be_size_classes():
    from odegb300 import _lib
    N = 8
    u0, p, ts, sv, npt = duffing_inputs(N, 2)
    npt = npt.copy()
    npt[3] = 6
    with pytest.raises(_lib.OdeError, match="sizes must be"):
        gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, n_per_traj=npt)


def test_static_and_persistent_schedulers_agree():
    N = 1000
    u0, p, ts = lorenz_inputs(N, seed=7)
    a = gpu("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8, scheduler="static")
    b = gpu("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8, scheduler="persistent")
    assert np.array_equal(a["u"], b["u"], equal_nan=True)
    assert np.array_equal(a["stats"]["naccept"], b["stats"]["naccept"])


def test_retcodes_match_oracle():
    N = 64
    u0, p, ts = lorenz_inputs(N)
    p[0, :8] = np.nan
    g = gpu("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8)
    o = oracle("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8)
    assert np.array_equal(g["retcode"], o["retcode"])
    assert (g["retcode"][:8] != 1).all() and (g["retcode"][8:] == 1).all()
    g = gpu("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8, maxiters=5)
    o = oracle("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8, maxiters=5)
    assert np.array_equal(g["retcode"], o["retcode"])
    assert (g["retcode"][8:] == 2).all()
    assert np.array_equal(g["nsaved"], o["nsaved"])


def test_empty_ensemble():
    u0, p, ts = lorenz_inputs(0)
    g = gpu("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8)
    assert g["retcode"].shape == (0,)


def test_graph_replay_with_new_data_in_same_buffers():
    # repeated solves of the same shape replay one captured CUDA graph; the
    # inputs are copied into the same device buffers, so a replay must see them
    N = 256
    u0, p1, ts = lorenz_inputs(N, seed=1)
    _, p2, _ = lorenz_inputs(N, seed=2)
    r1 = gpu("lorenz", "tsit5", u0, p1, ts, 0.1, 1e-8, 1e-8)
    r2 = gpu("lorenz", "tsit5", u0, p2, ts, 0.1, 1e-8, 1e-8)
    r3 = gpu("lorenz", "tsit5", u0, p1, ts, 0.1, 1e-8, 1e-8)
    assert np.array_equal(r1["u"], r3["u"], equal_nan=True)
    assert not np.array_equal(r1["u"], r2["u"], equal_nan=True)
    o2 = oracle("lorenz", "tsit5", u0, p2, ts, 0.1, 1e-8, 1e-8)
    c = compare(r2, o2, 1e-8, 1e-8)
    assert c["ok"] and c["steps_ok"], c


def test_autotune_picks_a_compiled_shape():
    import ctypes as C
    from odegb300 import EnsembleGB300, Rodas5P, _lib, autotune
    N = 512
    u0, p, ts = brusselator_inputs(N, cells=32, seed=4)
    ens = EnsembleGB300(precision="mixed", ir_sweeps=1)
    t = autotune("brusselator_1d", Rodas5P(), ens, u0, p, ts, 1.25, 1e-5, 1e-8)
    lanes = (C.c_int32 * 8)()
    k = _lib.load().ode_query_variants(2, _lib.MODEL_BRUSSELATOR_1D, _lib.PREC_MIXED, 64, lanes, 8)
    assert t["lanes_per_traj"] in list(lanes[:k]) and t["ms"] > 0, t
    g = gpu("brusselator_1d", "rodas5p", u0, p, ts, 1.25, 1e-5, 1e-8, precision="mixed", ir_sweeps=1)
    o = oracle("brusselator_1d", "rodas5p", u0, p, ts, 1.25, 1e-5, 1e-8)
    assert (g["retcode"] == 1).all()
    assert compare(g, o, 1e-5, 1e-8, step_slack=10 ** 9)["ok"]


def test_abort_stops_running_kernels():
    # ode_abort sets a host-mapped flag that the kernels poll every 64 steps;
    # a solve that would run for seconds ends early with ODE_RC_ABORTED
    import ctypes as C
    import time
    import torch
    from odegb300 import EnsembleGB300, Tsit5, _lib
    from odegb300.ensemble import MODELS, _options, get_handle
    from odegb300.saveat import resolve_saveat
    L = _lib.load()
    h = get_handle(0)
    N = 2048
    u0, p, ts = lorenz_inputs(N, seed=9)
    p[1, :] = 28.0 + 0.01 * np.arange(N) / N   # chaotic: steps stay small for the whole span
    ts[1, :] = 1.0e5   # about 1e7 steps per trajectory: many seconds unaborted
    sv = resolve_saveat(None, ts)
    ens = EnsembleGB300()
    o = _options(1e-8, 1e-8, None, None, None, 10 ** 8, sv, ens, None, None)
    d = _lib.ProblemDesc(MODELS["lorenz"], Tsit5().alg_id, 3, 3, ens.prec_id(), 0)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    du0, dp, dts = t(u0), t(p), t(ts)
    cap = sv.cap
    tout = torch.empty((cap, N), dtype=torch.float64, device=dev)
    uout = torch.empty((cap, 3, N), dtype=torch.float64, device=dev)
    ns = torch.empty(N, dtype=torch.int32, device=dev)
    rc = torch.empty(N, dtype=torch.int32, device=dev)
    st = torch.empty((N, 6), dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream(dev)
    vp = lambda x: C.c_void_p(x.data_ptr())
    t0 = time.perf_counter()
    torch.cuda.synchronize(dev)   # the inputs' copies are done before the solve's stream reads them
    _lib.check(L.ode_solve_ensemble_device(h, C.byref(d), C.byref(o), N, None, vp(du0), vp(dp), vp(dts), None,
                                           vp(tout), vp(uout), vp(ns), vp(rc), vp(st),
                                           C.c_void_p(stream.cuda_stream)), h)
    time.sleep(0.05)
    _lib.check(L.ode_abort(h), h)
    stream.synchronize()
    elapsed = time.perf_counter() - t0
    r = rc.cpu().numpy()
    assert (r == 6).all(), np.unique(r, return_counts=True)
    assert elapsed < 5.0, elapsed
    naccept = st.cpu().numpy()[:, 4]
    assert (naccept > 0).all() and (naccept < 10 ** 7).all()


def _device_solve(model, alg, u0, p, ts, saveat, reltol, abstol, precision="fp64", npt=None):
    """The same solve through ode_solve_ensemble_device on torch buffers."""
    import ctypes as C
    import torch
    from gpu_common import ALG
    from odegb300 import EnsembleGB300, _lib
    from odegb300.ensemble import MODELS, _options, get_handle
    from odegb300.saveat import resolve_saveat
    L = _lib.load()
    h = get_handle(0)
    n, N = u0.shape
    sv = resolve_saveat(saveat, ts)
    ens = EnsembleGB300(precision=precision)
    o = _options(reltol, abstol, None, None, None, 10 ** 6, sv, ens, None, None)
    d = _lib.ProblemDesc(MODELS[model], ALG[alg][0].alg_id, n, p.shape[0], ens.prec_id(), 0)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    cap = sv.cap
    bufs = [t(u0), t(p), t(ts), t(sv.values if sv.nsave else np.zeros(1)),
            torch.empty((cap, N), dtype=torch.float64, device=dev),
            torch.empty((cap, n, N), dtype=torch.float64, device=dev),
            torch.empty(N, dtype=torch.int32, device=dev), torch.empty(N, dtype=torch.int32, device=dev),
            torch.empty((N, 6), dtype=torch.int64, device=dev)]
    dn = t(npt) if npt is not None else None
    vp = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None
    stream = torch.cuda.Stream(dev)
    torch.cuda.synchronize(dev)   # the inputs' copies are done before the solve's stream reads them
    _lib.check(L.ode_solve_ensemble_device(h, C.byref(d), C.byref(o), N, vp(dn), *[vp(b) for b in bufs],
                                           C.c_void_p(stream.cuda_stream)), h)
    stream.synchronize()
    names = ("nf", "njacs", "nw", "nsolve", "naccept", "nreject")
    st = bufs[8].cpu().numpy()
    return {"t": bufs[4].cpu().numpy(), "u": bufs[5].cpu().numpy(), "nsaved": bufs[6].cpu().numpy(),
            "retcode": bufs[7].cpu().numpy(), "stats": {k: st[:, i] for i, k in enumerate(names)}}


def _same_saved(a, b, npt=None):
    """Equal saves; only the slots each trajectory wrote are compared (rows past
    nsaved and, for uneven sizes, components past the trajectory's size are
    unspecified)."""
    ns = a["nsaved"]
    assert np.array_equal(ns, b["nsaved"]) and np.array_equal(a["retcode"], b["retcode"])
    m = np.arange(a["t"].shape[0])[:, None] < ns[None, :]
    assert np.array_equal(a["t"][m], b["t"][m])
    mu = np.broadcast_to(m[:, None, :], a["u"].shape)
    if npt is not None:
        mu = mu & (np.arange(a["u"].shape[1])[None, :, None] < np.asarray(npt)[None, None, :])
    assert np.array_equal(a["u"][mu], b["u"][mu])
    assert np.array_equal(a["stats"]["naccept"], b["stats"]["naccept"])


def test_host_solve_equals_device_solve():
    # the host-buffer entry point (copies + graph replay) and the device-buffer
    # entry point give the same trajectories
    N = 40000
    u0, p, ts = lorenz_inputs(N, seed=21)
    _same_saved(gpu("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8),
                _device_solve("lorenz", "tsit5", u0, p, ts, 0.1, 1e-8, 1e-8))


def test_pipelined_uneven_host_solve_equals_device_solve():
    # 32768+ trajectories with many output bytes each (64-state class slots,
    # 18 saves) run as a 4-slice copy/compute pipeline; every trajectory must
    # come out as in one device-buffer solve
    N = 40000
    u0, p, ts, sv, npt = duffing_inputs(N, [2, 4, 8, 16, 32], tf_range=(1.0, 3.0), seed=5)
    _same_saved(gpu("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, precision="mixed", n_per_traj=npt),
                _device_solve("duffing_chain", "vern7", u0, p, ts, sv, 1e-6, 1e-6, precision="mixed", npt=npt), npt)


@pytest.mark.parametrize("model,alg,rt,at", [("lorenz", "tsit5", 1e-8, 1e-8), ("lorenz", "vern7", 1e-8, 1e-8),
                                             ("robertson", "rodas5p", 1e-6, 1e-10)])
def test_save_everystep_matches_oracle(model, alg, rt, at):
    # no saveat: every accepted step is saved (the reference's default)
    N = 128
    u0, p, ts = lorenz_inputs(N, seed=4) if model == "lorenz" else robertson_inputs(N, seed=4)
    g = gpu(model, alg, u0, p, ts, None, rt, at, save_everystep=True, max_step_saves=4096)
    o = oracle(model, alg, u0, p, ts, None, rt, at, save_everystep=True, max_step_saves=4096)
    c = compare(g, o, rt, at)
    assert c["ok"] and c["steps_ok"], c
    # start + every accepted step (tf included)
    assert np.array_equal(g["nsaved"], g["stats"]["naccept"] + 1)
    last = g["t"][g["nsaved"] - 1, np.arange(N)]
    assert np.array_equal(last, ts[1])


def test_save_everystep_overflow_keeps_the_final_point():
    N = 64
    u0, p, ts = lorenz_inputs(N, seed=8)
    g = gpu("lorenz", "tsit5", u0, p, ts, None, 1e-8, 1e-8, save_everystep=True, max_step_saves=5)
    assert (g["nsaved"] == 7).all()
    assert np.array_equal(g["t"][6], ts[1])   # the last slot holds tf
    o = oracle("lorenz", "tsit5", u0, p, ts, None, 1e-8, 1e-8, save_everystep=True, max_step_saves=5)
    assert np.allclose(g["u"][6], o["u"][6], rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("uneven", [False, True])
def test_page_locked_host_buffers_solve_in_place(uneven):
    # page-locked host buffers are read and written by the kernels directly
    # (no staging copies); results must equal the staged path's
    import ctypes as C
    import torch
    from gpu_common import ALG
    from odegb300 import EnsembleGB300, _lib
    from odegb300.ensemble import MODELS, _options, get_handle
    from odegb300.saveat import resolve_saveat
    if uneven:
        u0, p, ts, sv, npt = duffing_inputs(3000, [2, 4, 8, 16, 32], tf_range=(1.0, 5.0), seed=13)
        model, alg, rt, at, prec = "duffing_chain", "vern7", 1e-6, 1e-6, "mixed"
    else:
        u0, p, ts = robertson_inputs(3000, seed=13)
        sv, npt = ROBER_SAVEAT, None
        model, alg, rt, at, prec = "robertson", "rodas5p", 1e-6, 1e-10, "mixed"
    ref = gpu(model, alg, u0, p, ts, sv, rt, at, precision=prec, n_per_traj=npt)
    spec = resolve_saveat(sv, ts)
    ens = EnsembleGB300(precision=prec)
    o = _options(rt, at, None, None, None, 10 ** 6, spec, ens, None, None)
    n, N = u0.shape
    d = _lib.ProblemDesc(MODELS[model], ALG[alg][0].alg_id, n, p.shape[0], ens.prec_id(), 0)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    h_u0, h_p, h_ts, h_sv = pin(u0), pin(p), pin(ts), pin(spec.values)
    h_npt = pin(npt) if npt is not None else None
    cap = spec.cap
    h_t = torch.empty((cap, N), dtype=torch.float64).pin_memory()
    h_u = torch.empty((cap, n, N), dtype=torch.float64).pin_memory()
    h_ns = torch.empty(N, dtype=torch.int32).pin_memory()
    h_rc = torch.empty(N, dtype=torch.int32).pin_memory()
    h_st = torch.empty((N, 6), dtype=torch.int64).pin_memory()
    ptr = lambda t, ty=C.c_double: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(ty)) if t is not None else None
    L = _lib.load()
    h = get_handle(0)
    _lib.check(L.ode_solve_ensemble(h, C.byref(d), C.byref(o), N, ptr(h_npt, C.c_int32), ptr(h_u0), ptr(h_p),
                                    ptr(h_ts), ptr(h_sv), ptr(h_t), ptr(h_u), ptr(h_ns, C.c_int32),
                                    ptr(h_rc, C.c_int32), ptr(h_st, _lib.Stats)), h)
    names = ("nf", "njacs", "nw", "nsolve", "naccept", "nreject")
    st = h_st.numpy()
    got = {"t": h_t.numpy(), "u": h_u.numpy(), "nsaved": h_ns.numpy(), "retcode": h_rc.numpy(),
           "stats": {k: st[:, i] for i, k in enumerate(names)}}
    _same_saved(got, ref, npt)
