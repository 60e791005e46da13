"""Models registered at run time (ode_register_model): CUDA C++ source for the
right-hand side (and optionally its Jacobian and time derivative), compiled by
the library with NVRTC against the integrator templates.  None of these models
is compiled into the library; each is checked against the FP64 oracle, which
restates them natively: Lotka-Volterra (the reference's own benchmark problem,
benchmark/benchmarks.jl:13-26) with the Jacobian left to forward-mode AD, the
stiff Oregonator with an analytic Jacobian, and the forced oscillator with its
tgrad, which must equal the compiled-in forced model bit for bit."""
import numpy as np
import pytest

import pyoracle as O
from gpu_common import MODEL, assert_mixed_accuracy, compare, gpu, oracle

pytestmark = pytest.mark.gpu

LV = r'''
template <class T, class P> __device__ void lv_f(T* du, const T* u, const P* p, double t) {
    du[0] = p[0] * u[0] - p[1] * u[0] * u[1];
    du[1] = p[3] * u[0] * u[1] - p[2] * u[1];
}
'''
OREGO = r'''
template <class T, class P> __device__ void orego_f(T* du, const T* u, const P* p, double t) {
    du[0] = p[0] * (u[1] + u[0] * (1.0 - p[2] * u[0] - u[1]));
    du[1] = (u[2] - (1.0 + u[0]) * u[1]) / p[0];
    du[2] = p[1] * (u[0] - u[2]);
}
template <class T, class P> __device__ void orego_jac(T* J, const T* u, const P* p, double t) {
    J[0] = p[0] * (1.0 - 2.0 * p[2] * u[0] - u[1]); J[1] = p[0] * (1.0 - u[0]); J[2] = 0.0;
    J[3] = -u[1] / p[0]; J[4] = -(1.0 + u[0]) / p[0]; J[5] = 1.0 / p[0];
    J[6] = p[1]; J[7] = 0.0; J[8] = -p[1];
}
'''
# the compiled-in forced Duffing oscillator's arithmetic, operation for operation
FORCED = r'''
template <class T, class P> __device__ void forced_f(T* du, const T* u, const P* p, double t) {
    const T fo = odegb::from_double<T>(odegb::pdouble(p[3]) * cos(odegb::pdouble(p[4]) * t));
    du[0] = u[1];
    du[1] = ((fo - p[0] * u[1]) - p[1] * u[0]) - p[2] * (u[0] * u[0] * u[0]);
}
template <class T, class P> __device__ void forced_jac(T* J, const T* u, const P* p, double t) {
    J[0] = T(0); J[1] = T(1);
    J[2] = -p[1] - p[2] * (T(3) * (u[0] * u[0])); J[3] = -p[0];
}
template <class T, class P> __device__ void forced_tgrad(T* dT, const T* u, const P* p, double t) {
    const double w = odegb::pdouble(p[4]);
    dT[0] = T(0);
    dT[1] = odegb::from_double<T>(-(odegb::pdouble(p[3]) * w) * sin(w * t));
}
'''


@pytest.fixture(scope="module", autouse=True)
def registered():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from odegb300 import build, register_model
    build.build()
    return {"lv": register_model(LV, "lv", 2, 4),
            "orego": register_model(OREGO, "orego", 3, 3, jac=True),
            "forced": register_model(FORCED, "forced", 2, 5, jac=True, tgrad=True, nonautonomous=True)}


def lv_inputs(N, seed=0):
    rng = np.random.default_rng(seed)
    p = np.array([1.5, 1.0, 3.0, 1.0])[:, None] * rng.uniform(0.8, 1.2, (4, N))
    u0 = rng.uniform(0.5, 1.5, (2, N))
    return u0, p, np.vstack([np.zeros(N), np.full(N, 10.0)])


def orego_inputs(N, seed=0):
    rng = np.random.default_rng(seed)
    p = np.array([77.27, 0.161, 8.375e-6])[:, None] * rng.uniform(0.9, 1.1, (3, N))
    u0 = np.array([1.0, 2.0, 3.0])[:, None] * rng.uniform(0.9, 1.1, (3, N))
    return u0, p, np.vstack([np.zeros(N), np.full(N, 50.0)])


# the oracle's native restatements of the registered models
MODEL.setdefault("lv", O.LOTKA_VOLTERRA)
MODEL.setdefault("orego", O.OREGONATOR)
MODEL.setdefault("forced", O.FORCED_DUFFING)


def oracle_of(name, alg, u0, p, ts, saveat, rt, at):
    return oracle(name, alg, u0, p, ts, saveat, rt, at)


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
def test_registered_lotka_volterra_fp64(alg):
    N = 256
    u0, p, ts = lv_inputs(N)
    g = gpu("lv", alg, u0, p, ts, 0.5, 1e-6, 1e-8)
    o = oracle_of("lv", alg, u0, p, ts, 0.5, 1e-6, 1e-8)
    c = compare(g, o, 1e-6, 1e-8)
    assert c["ok"] and c["steps_ok"], c
    # the adapter adds no arithmetic: most trajectories match the oracle bit for bit
    assert c["frac_bit_identical"] > 0.5, c


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
def test_registered_lotka_volterra_mixed(alg):
    N = 256
    u0, p, ts = lv_inputs(N, seed=1)
    g = gpu("lv", alg, u0, p, ts, 0.5, 1e-6, 1e-8, precision="mixed")
    assert (g["retcode"] == 1).all()
    assert_mixed_accuracy("lv", alg, g, u0, p, ts, 0.5, 1e-6, 1e-8)


def test_registered_lotka_volterra_rodas5p_with_ad_jacobian():
    # no NAME_jac: J by forward-mode AD of lv_f (one counted f call per Jacobian,
    # as the reference counts a ForwardDiff chunk); the oracle uses the analytic J
    N = 256
    u0, p, ts = lv_inputs(N, seed=2)
    g = gpu("lv", "rodas5p", u0, p, ts, 0.5, 1e-6, 1e-8)
    o = oracle_of("lv", "rodas5p", u0, p, ts, 0.5, 1e-6, 1e-8)
    c = compare(g, o, 1e-6, 1e-8)
    assert c["ok"] and c["steps_ok"], c
    same = g["stats"]["naccept"] == o["stats"]["naccept"]
    assert np.array_equal((g["stats"]["nf"] - g["stats"]["njacs"])[same], o["stats"]["nf"][same])


@pytest.mark.parametrize("alg", ["rodas5p", "rosenbrock23"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_registered_oregonator(alg, precision):
    N = 128
    u0, p, ts = orego_inputs(N)
    rt, at = (1e-6, 1e-8) if alg == "rodas5p" else (1e-4, 1e-6)
    g = gpu("orego", alg, u0, p, ts, 5.0, rt, at, precision=precision)
    o = oracle_of("orego", alg, u0, p, ts, 5.0, rt, at)
    assert (g["retcode"] == 1).all()
    if precision == "fp64":
        c = compare(g, o, rt, at)
        assert c["ok"] and c["steps_ok"], c
    else:
        assert_mixed_accuracy("orego", alg, g, u0, p, ts, 5.0, rt, at, stiff=True)


@pytest.mark.parametrize("alg", ["tsit5", "rodas5p", "rosenbrock23"])
def test_registered_forced_oscillator_equals_the_compiled_in_model(alg):
    from test_gpu_nonautonomous import SAVEAT, forced_inputs
    N = 128
    u0, p, ts = forced_inputs(N, seed=7)
    a = gpu("forced", alg, u0, p, ts, SAVEAT, 1e-6, 1e-6)
    b = gpu("forced_duffing", alg, u0, p, ts, SAVEAT, 1e-6, 1e-6)
    assert np.array_equal(a["u"], b["u"], equal_nan=True)
    for k in ("nf", "njacs", "naccept", "nreject"):
        assert np.array_equal(a["stats"][k], b["stats"][k]), k


def test_compile_errors_are_reported():
    from odegb300 import _lib, register_model
    bad = register_model("template <class T, class P> __device__ void broken_f(T* du, const T* u, const P* p, "
                         "double t) { du[0] = undefined_symbol; }", "broken", 1, 1)
    u0, p, ts = np.ones((1, 4)), np.ones((1, 4)), np.vstack([np.zeros(4), np.ones(4)])
    with pytest.raises(_lib.OdeError) as e:
        gpu(bad, "tsit5", u0, p, ts, 0.5, 1e-6, 1e-6)
    assert e.value.status == -4 and "undefined_symbol" in str(e.value)


# ---------------------------------------------------------------- callbacks registered with a model
BALL = r'''
template <class T, class P> __device__ void rball_f(T* du, const T* u, const P* p, double t) {
    du[0] = u[1];
    du[1] = -p[0];
}
__device__ double rball_condition(const double* u, const double* p, double t) { return u[0]; }
__device__ int rball_affect(double* u, const double* p, double t, int upcrossing) {
    if (t >= p[2]) return 1;   // terminate!
    u[1] = -p[1] * u[1];
    return 0;
}
'''
BOX = r'''
template <class T, class P> __device__ void box_f(T* du, const T* u, const P* p, double t) {
    du[0] = u[2]; du[1] = u[3]; du[2] = T(0); du[3] = -p[0];
}
__device__ void box_vcondition(double* out, const double* u, const double* p, double t) {
    out[0] = u[1]; out[1] = u[0]; out[2] = p[2] - u[0];
}
__device__ int box_vaffect(double* u, const double* p, double t, const int* events) {
    if (events[0] != 0) u[3] = -p[1] * u[3];
    if (events[1] != 0 || events[2] != 0) u[2] = -u[2];
    return 0;
}
'''
THRESHOLD = r'''
template <class T, class P> __device__ void thr_f(T* du, const T* u, const P* p, double t) { du[0] = -p[0] * u[0]; }
__device__ int thr_dcondition(const double* u, const double* p, double t) { return u[0] < p[1]; }
__device__ int thr_daffect(double* u, const double* p, double t) { u[0] += p[2]; return 0; }
'''


@pytest.fixture(scope="module")
def with_callbacks():
    from odegb300 import register_model
    MODEL.setdefault("rball", O.BOUNCING_BALL)
    MODEL.setdefault("box", O.BALL_BOX)
    MODEL.setdefault("thr", O.THRESHOLD_DOSE)
    return {"rball": register_model(BALL, "rball", 2, 3, continuous_callback="down"),
            "box": register_model(BOX, "box", 4, 3, vector_callback=3),
            "thr": register_model(THRESHOLD, "thr", 1, 3, discrete_callback=True)}


def test_registered_continuous_callback_equals_the_compiled_in_ball(with_callbacks):
    from odegb300 import workloads as W
    from odegb300.saveat import resolve_saveat
    wl = W.bouncing_ball(256, seed=4)
    kw = dict(callback=wl["callback"])
    a = gpu("rball", "tsit5", wl["u0"], wl["p"], wl["tspan"], wl["saveat"], 1e-6, 1e-6, **kw)
    b = gpu("bouncing_ball", "tsit5", wl["u0"], wl["p"], wl["tspan"], wl["saveat"], 1e-6, 1e-6, **kw)
    assert np.array_equal(a["u"], b["u"], equal_nan=True) and np.array_equal(a["retcode"], b["retcode"])
    assert (a["retcode"] == 7).any()   # terminate! from the registered affect


def box_inputs(N, seed=0):
    rng = np.random.default_rng(seed)
    W = rng.uniform(3.0, 6.0, N)
    u0 = np.vstack([rng.uniform(0.5, 2.5, N), rng.uniform(3.0, 9.0, N), rng.uniform(-4.0, 4.0, N),
                    rng.uniform(-2.0, 2.0, N)])
    p = np.vstack([np.full(N, 9.81), rng.uniform(0.8, 1.0, N), W])
    return u0, p, np.vstack([np.zeros(N), np.full(N, 6.0)])


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
def test_registered_vector_callback_matches_oracle(with_callbacks, alg):
    from odegb300 import ContinuousCallback
    N = 128
    u0, p, ts = box_inputs(N)
    cb = ContinuousCallback(interp_points=10, max_events=64)
    g = gpu("box", alg, u0, p, ts, 0.25, 1e-8, 1e-8, callback=cb)
    o = oracle_of_cb("box", alg, u0, p, ts, 0.25, 1e-8, 1e-8, cb)
    c = compare(g, o, 1e-8, 1e-8)
    assert c["ok"] and c["steps_ok"], c
    assert (g["nsaved"] > 25).all()   # every trajectory hit a wall or the floor (two saves per event)


def test_registered_discrete_callback_matches_oracle(with_callbacks):
    from odegb300 import DiscreteCallback
    N = 256
    rng = np.random.default_rng(3)
    p = np.vstack([rng.uniform(0.3, 1.0, N), rng.uniform(0.2, 0.5, N), np.ones(N)])
    u0 = rng.uniform(0.8, 1.5, (1, N))
    ts = np.vstack([np.zeros(N), np.full(N, 20.0)])
    cb = DiscreteCallback(max_events=64)
    g = gpu("thr", "tsit5", u0, p, ts, 0.5, 1e-8, 1e-10, callback=cb)
    o = oracle_of_cb("thr", "tsit5", u0, p, ts, 0.5, 1e-8, 1e-10, cb)
    c = compare(g, o, 1e-8, 1e-10)
    assert c["ok"] and c["steps_ok"], c
    assert (g["nsaved"] > 41).all()   # doses happened (two extra saves each)


def oracle_of_cb(name, alg, u0, p, ts, saveat, rt, at, cb):
    return oracle(name, alg, u0, p, ts, saveat, rt, at, callback=True, interp_points=cb.interp_points,
                  max_events=cb.max_events)
