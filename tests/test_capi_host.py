"""CPU-side checks: the C-ABI library builds, loads and exports every declared
entry point; host-side saveat/save_start/save_end resolution follows the
reference's rules; error paths that need no GPU."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from odegb300 import _lib, build
from odegb300.saveat import julia_float_range, julia_rat, resolve_saveat

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(ode_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    path = build.build()
    L = C.CDLL(path)
    names = declared_functions()
    assert "ode_solve_ensemble" in names and "ode_submit" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the Python binding declares a signature for every exported entry point
    assert names <= set(_lib.SIGNATURES), names - set(_lib.SIGNATURES)


def test_struct_layouts_match_the_bindings():
    L = _lib.load()
    assert L.ode_options_size() == C.sizeof(_lib.Options)
    assert L.ode_problem_desc_size() == C.sizeof(_lib.ProblemDesc)


def _julia_struct(name):
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "ordinarydiffeq.jl_gb300",
                            "julia", "EnsembleGB300.jl")).read()
    body = re.search(r"(?:mutable )?struct %s\n(.*?)\nend" % name, src, re.S).group(1)
    out = []
    for part in re.split(r"[;\n]", body):
        if part.strip():
            n, t = part.split("::")
            out.append((n.strip(), t.strip()))
    return out


def test_julia_binding_mirrors_the_c_structs():
    # the Julia ccall glue passes ode_options and ode_problem_desc by reference: its
    # structs must hold the same fields, in order, with the same widths
    width = {"Float64": C.c_double, "Int64": C.c_int64, "Int32": C.c_int32}
    for jname, ctype in (("Options", _lib.Options), ("ProblemDesc", _lib.ProblemDesc)):
        jl = _julia_struct(jname)
        assert [n for n, _ in jl] == [n for n, _ in ctype._fields_], jname
        for (n, jt), (_, ct) in zip(jl, ctype._fields_):
            if jt.startswith("Ptr{"):
                assert C.sizeof(ct) == C.sizeof(C.c_void_p), n
            else:
                assert C.sizeof(width[jt]) == C.sizeof(ct), n


def test_abi_version_and_defaults_without_gpu():
    L = _lib.load()
    assert L.ode_abi_version() == 10
    # dense vectors per step (Tsit5 k1..k7, Vern7 k1 and k4..k9, Rodas5P dense k1..k3)
    assert [L.ode_dense_nk(a) for a in (0, 1, 2)] == [7, 7, 3] and L.ode_dense_nk(9) == -1
    o = _lib.Options()
    L.ode_options_default(C.byref(o))
    assert o.reltol == 1e-3 and o.abstol == 1e-6 and o.maxiters == 1000000
    assert o.save_start == 1 and o.save_end == 1 and o.save_end_user == -1
    assert o.ntstops == 0 and not o.tstops and o.interp_points == 10
    assert o.max_jac_age == 1 and o.jac_reuse_gamma_tol == 0.03   # Rosenbrock23's defaults
    assert L.ode_status_string(-4).decode().startswith("unsupported")


def test_tstops_count_without_array_is_rejected_before_any_device_work():
    # ode_solve_ensemble_noalloc validates its arguments on the host first
    L = _lib.load()
    o = _lib.Options()
    L.ode_options_default(C.byref(o))
    o.ntstops = 2   # and tstops left null
    d = _lib.ProblemDesc(_lib.MODEL_LORENZ, _lib.ODE_TSIT5, 3, 3, _lib.PREC_FP64, 0)
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    o.ntstops = -1
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1


def test_noalloc_applies_the_shared_problem_checks():
    # ode_solve_ensemble_noalloc and the handle entry points run the same checks, so
    # both reject the same input with the same status (ODE_E_INVALID = -1) on the host
    L = _lib.load()
    o = _lib.Options()
    L.ode_options_default(C.byref(o))
    d = _lib.ProblemDesc(_lib.MODEL_BOUNCING_BALL, _lib.ODE_TSIT5, 2, 3, _lib.PREC_FP64, 0)
    o.callback = 1
    o.max_events = -1   # would size the save slots negatively
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    assert b"max_events" in L.ode_last_error(None)
    o.max_events = 4
    o.interp_points = -2
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    L.ode_options_default(C.byref(o))
    d = _lib.ProblemDesc(_lib.MODEL_LORENZ, _lib.ODE_TSIT5, 4, 3, _lib.PREC_FP64, 0)   # Lorenz has 3 states
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    assert b"3 states" in L.ode_last_error(None)


def test_jacobian_reuse_options_are_checked_on_the_host():
    L = _lib.load()
    o = _lib.Options()
    L.ode_options_default(C.byref(o))
    d = _lib.ProblemDesc(_lib.MODEL_LORENZ, _lib.ODE_ROSENBROCK23, 3, 3, _lib.PREC_FP64, 0)
    o.max_jac_age = -1
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    o.max_jac_age = 20
    o.jac_reuse_gamma_tol = float("nan")
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    # the kept J lives in registers beside W: not for the shared-memory LU (16-64 states)
    o.jac_reuse_gamma_tol = 0.03
    d = _lib.ProblemDesc(_lib.MODEL_BRUSSELATOR_1D, _lib.ODE_ROSENBROCK23, 16, 3, _lib.PREC_FP64, 0)
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -4
    assert b"max_jac_age" in L.ode_last_error(None)


def test_save_idxs_are_checked_on_the_host():
    L = _lib.load()
    o = _lib.Options()
    L.ode_options_default(C.byref(o))
    assert o.nsave_idxs == 0 and not o.save_idxs
    d = _lib.ProblemDesc(_lib.MODEL_LORENZ, _lib.ODE_TSIT5, 3, 3, _lib.PREC_FP64, 0)
    o.nsave_idxs = -1
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    o.nsave_idxs = 2   # and save_idxs left null
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    assert b"save_idxs" in L.ode_last_error(None)


def test_fixed_steps_are_checked_on_the_host():
    # adaptive = false needs a dt or tstops (solve.jl:277-280); a NaN or infinite dt is rejected
    L = _lib.load()
    o = _lib.Options()
    L.ode_options_default(C.byref(o))
    assert o.adaptive == 1
    d = _lib.ProblemDesc(_lib.MODEL_LORENZ, _lib.ODE_TSIT5, 3, 3, _lib.PREC_FP64, 0)
    o.adaptive = 0
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    assert b"fixed steps" in L.ode_last_error(None)
    o.dt = float("inf")
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1


def test_controller_knobs_are_checked_on_the_host():
    L = _lib.load()
    o = _lib.Options()
    L.ode_options_default(C.byref(o))
    assert o.controller_given == 0 and np.isnan(o.beta1) and np.isnan(o.qsteady_max)
    d = _lib.ProblemDesc(_lib.MODEL_LORENZ, _lib.ODE_TSIT5, 3, 3, _lib.PREC_FP64, 0)
    o.controller_given = 1
    o.qmin = 0.0
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    assert b"qmin" in L.ode_last_error(None)
    o.qmin = float("nan")
    o.beta1 = float("inf")
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1


def test_variant_registry_covers_the_workloads():
    L = _lib.load()
    buf = (C.c_int32 * 8)()
    for alg, model, n in [(0, 1, 3), (1, 1, 3), (2, 2, 3), (1, 3, 4), (1, 3, 8), (1, 3, 16), (1, 3, 32),
                          (1, 3, 64)]:
        for prec in (0, 1):
            assert L.ode_query_variants(alg, model, prec, n, buf, 8) >= 1, (alg, model, n, prec)


def test_julia_range_semantics():
    # 0.1:0.1:1.0 gives correctly rounded tenths (0.3 == 3/10, not 0.1 + 0.2)
    r = julia_float_range(0.1, 0.1, 1.0)
    assert len(r) == 10 and r[2] == 0.3 and r[-1] == 1.0
    assert julia_float_range(4.0, 4.0, 15.0).tolist() == [4.0, 8.0, 12.0]
    assert julia_rat(0.1) == (1, 10)
    assert julia_float_range(0.0, 0.25, 1.0).tolist() == [0.0, 0.25, 0.5, 0.75, 1.0]


def test_save_flags_follow_reference_defaults():
    ts = np.array([[0.0], [0.4]])
    # test/InterfaceI/ode_saveat_tests.jl:240-268
    s = resolve_saveat(0.1, ts)
    assert s.scalar and s.save_start and s.save_end and s.values.tolist() == [0.1, 0.2, 0.3, 0.4]
    s = resolve_saveat([0.2], ts)
    assert not s.save_start and not s.save_end and s.save_end_user == -1
    s = resolve_saveat([0.2], ts, save_start=True, save_end=True)
    assert s.save_start and s.save_end and s.save_end_user == 1
    s = resolve_saveat(np.arange(0, 0.5, 0.1), ts)
    assert s.save_start  # t0 in saveat
    s = resolve_saveat(None, ts)
    assert s.nsave == 0 and s.save_start and s.save_end


def test_per_trajectory_saveat_for_uneven_spans():
    tf = np.array([1.0, 2.0, 4.0])
    ts = np.vstack([np.zeros(3), tf])
    sv = np.outer(np.arange(1, 17) / 16.0, tf)
    s = resolve_saveat(sv, ts)
    assert s.per_traj and s.nsave == 16 and not s.save_start and s.save_end
    s = resolve_saveat(0.5, ts)
    assert s.per_traj and s.values.shape == (8, 3) and np.isinf(s.values[2:, 0]).all()


def test_invalid_arguments_are_rejected_without_gpu():
    L = _lib.load()
    rc = L.ode_solve_ensemble(None, None, None, 0, None, None, None, None, None, None, None, None, None, None)
    assert rc == -1


def test_model_registration_checks_on_the_host():
    # ode_register_model validates its arguments and stores the source; the
    # kernels are compiled (NVRTC) on the first solve, which needs a GPU
    L = _lib.load()
    src = b"template <class T, class P> __device__ void m_f(T* du, const T* u, const P* p, double t) { du[0] = -u[0]; }"
    mid = C.c_int32(0)
    assert L.ode_register_model(src, b"m", 1, 0, 0, C.byref(mid)) == 0
    assert mid.value >= _lib.MODEL_USER_BASE
    mid2 = C.c_int32(0)
    assert L.ode_register_model(src, b"m", 1, 0, 0, C.byref(mid2)) == 0 and mid2.value == mid.value + 1
    assert L.ode_register_model(src, b"1m", 1, 0, 0, C.byref(mid)) == -1         # not an identifier
    assert L.ode_register_model(src, b"m", 0, 0, 0, C.byref(mid)) == -1          # no states
    assert L.ode_register_model(src, b"m", 33, 0, 0, C.byref(mid)) == -1         # too many for registers
    assert L.ode_register_model(src, b"m", 1, 0, 64, C.byref(mid)) == -1         # unknown flag
    assert L.ode_register_model(None, b"m", 1, 0, 0, C.byref(mid)) == -1
    # a registered id is checked like a compiled-in model: state and parameter counts
    o = _lib.Options()
    L.ode_options_default(C.byref(o))
    d = _lib.ProblemDesc(mid2.value, _lib.ODE_TSIT5, 2, 0, _lib.PREC_FP64, 0)
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    assert b"registered model" in L.ode_last_error(None)
    d = _lib.ProblemDesc(mid2.value, _lib.ODE_TSIT5, 1, 3, _lib.PREC_FP64, 0)
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    d = _lib.ProblemDesc(_lib.MODEL_USER_BASE + 100000, _lib.ODE_TSIT5, 1, 0, _lib.PREC_FP64, 0)
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == -1
    d = _lib.ProblemDesc(mid2.value, _lib.ODE_TSIT5, 1, 0, _lib.PREC_FP64, 0)
    assert L.ode_solve_ensemble_noalloc(C.byref(d), C.byref(o), 0, *([None] * 11)) == 0   # valid, nothing to do
