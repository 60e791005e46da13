"""Serving: requests of different models, sizes and tolerances submitted at once
run overlapped on the device, and each result is bit-identical to the same
request solved alone (the kernels are deterministic: a trajectory's arithmetic
does not depend on what else runs)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build
    build.build()


def _same(a, b):
    ns = a["nsaved"]
    assert np.array_equal(ns, b["nsaved"])
    assert np.array_equal(a["retcode"], b["retcode"])
    cap = a["t"].shape[0]
    m = np.arange(cap)[:, None] < ns[None, :]
    assert np.array_equal(a["t"][m], b["t"][m])
    mu = np.broadcast_to(m[:, None, :], a["u"].shape)
    assert np.array_equal(a["u"][mu], b["u"][mu])
    for k in ("naccept", "nreject", "nf"):
        assert np.array_equal(a["stats"][k], b["stats"][k])


def test_serving_results_same_alone_and_in_mix():
    from odegb300 import EnsembleGB300, solve_arrays
    from odegb300.ensemble import ALG_BY_NAME
    from odegb300.serving import Server, serving_mix
    reqs = serving_mix(24, seed=5, max_traj=256)
    res = {}
    with Server(hbm_budget=1 << 30, slots=8) as srv:
        for i, r in enumerate(reqs):
            srv.submit(r["model"], r["alg"], r["u0s"], r["ps"], r["tspans"], r["saveat"], r["reltol"], r["abstol"],
                       precision="auto", ir_sweeps=r["ir_sweeps"], tag=i)
        while len(res) < len(reqs):
            got = srv.next_completed(30.0)
            assert got is not None, "serving loop stalled"
            ticket, status, times, out, N, tag, prec = got
            assert status == 0
            res[tag] = (out, prec, times)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["queued"] == 0 and st["running"] == 0
    spans = sorted((v[2][1], v[2][2]) for v in res.values())
    overlapped = any(spans[k + 1][0] < spans[k][1] for k in range(len(spans) - 1))
    assert overlapped, "no two requests ran at the same time"
    for i, r in enumerate(reqs):
        out, prec, _ = res[i]
        ens = EnsembleGB300(precision=prec, ir_sweeps=r["ir_sweeps"] if prec == "mixed" else -1)
        alone = solve_arrays(r["model"], ALG_BY_NAME[r["alg"]], ens, r["u0s"], r["ps"], r["tspans"], r["saveat"],
                             r["reltol"], r["abstol"])
        _same(out, alone)


def test_serving_rejects_request_above_budget():
    from odegb300.serving import Server, serving_mix
    r = serving_mix(1, seed=1)[0]
    with Server(hbm_budget=4096, slots=2) as srv:
        srv.submit(r["model"], r["alg"], r["u0s"], r["ps"], r["tspans"], r["saveat"], r["reltol"], r["abstol"])
        got = srv.next_completed(10.0)
        assert got is not None and got[1] == -3   # ODE_E_NOMEM
        assert srv.stats()["rejected"] == 1


def test_open_loop_reports_latency():
    from odegb300.serving import Server, run_open_loop, serving_mix
    reqs = serving_mix(64, seed=2, max_traj=512)
    with Server(hbm_budget=2 << 30, slots=8) as srv:
        m = run_open_loop(srv, reqs, rate=200.0, duration=1.0)
    assert m["completed"] == m["submitted"] > 0 and m["failed"] == 0 and m["unfinished"] == 0
    assert m["latency_ms"]["p50"] > 0 and m["latency_ms"]["p99"] >= m["latency_ms"]["p50"]


def test_compatible_requests_merge_into_one_launch_with_their_own_tolerances():
    # one slot: while the first request runs the others queue; those that differ
    # only in trajectories and tolerances then share one launch, and each
    # result is still bit-identical to the request solved alone
    from odegb300 import EnsembleGB300, solve_arrays
    from odegb300.ensemble import ALG_BY_NAME
    from odegb300.serving import Server
    from odegb300 import workloads as W
    rng = np.random.default_rng(9)
    reqs = []
    for i in range(12):
        wl = W.lorenz(int(rng.integers(1, 200)), seed=100 + i)
        rt = float(10.0 ** rng.uniform(-8.0, -6.0))
        reqs.append((wl, rt))
    res = {}
    with Server(hbm_budget=1 << 30, slots=1) as srv:
        for i, (wl, rt) in enumerate(reqs):
            srv.submit(wl["model"], wl["alg"], wl["u0"], wl["p"], wl["tspan"], wl["saveat"], rt, rt,
                       precision="fp64", tag=i)
        while len(res) < len(reqs):
            got = srv.next_completed(30.0)
            assert got is not None, "serving loop stalled"
            assert got[1] == 0
            res[got[5]] = got[3]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["launches"] < len(reqs), st
    for i, (wl, rt) in enumerate(reqs):
        alone = solve_arrays(wl["model"], ALG_BY_NAME[wl["alg"]], EnsembleGB300(precision="fp64"), wl["u0"], wl["p"],
                             wl["tspan"], wl["saveat"], rt, rt)
        _same(res[i], alone)


def test_full_queue_sheds_requests():
    from odegb300.serving import Server, serving_mix
    from odegb300 import workloads as W
    from odegb300.saveat import resolve_saveat
    # a first request that keeps the one slot busy (~0.1 s), then a burst
    wl = W.brusselator(2048, seed=1, cells=32)
    heavy = dict(model=wl["model"], alg=wl["alg"], u0s=wl["u0"], ps=wl["p"], tspans=wl["tspan"],
                 saveat=resolve_saveat(wl["saveat"], wl["tspan"]), reltol=1e-8, abstol=1e-11, ir_sweeps=-1)
    reqs = [heavy] + serving_mix(40, seed=4, max_traj=64)
    with Server(hbm_budget=4 << 30, slots=1, queue_limit=4) as srv:
        tickets = [srv.submit(r["model"], r["alg"], r["u0s"], r["ps"], r["tspans"], r["saveat"], r["reltol"],
                              r["abstol"], precision="auto", ir_sweeps=r["ir_sweeps"]) for r in reqs]
        accepted = [t for t in tickets if t is not None]
        assert len(accepted) < len(reqs)   # some were shed while 4 waited
        done = 0
        while done < len(accepted):
            got = srv.next_completed(30.0)
            assert got is not None and got[1] == 0
            done += 1
