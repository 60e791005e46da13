"""ctypes binding of libode_b200.so (include/ode_gb300.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared object is missing or was built without a GPU
target.
"""
import ctypes as C
import os

from . import build as _build

ODE_TSIT5, ODE_VERN7, ODE_RODAS5P, ODE_ROSENBROCK23, ODE_AUTOTSIT5_ROSENBROCK23 = 0, 1, 2, 3, 4
MODEL_LINEAR, MODEL_LORENZ, MODEL_ROBERTSON, MODEL_DUFFING_CHAIN, MODEL_BRUSSELATOR_1D = 0, 1, 2, 3, 4
MODEL_BOUNCING_BALL, MODEL_VANDERPOL, MODEL_PK_ONE_COMPARTMENT, MODEL_FORCED_DUFFING = 5, 6, 7, 8
MODEL_USER_BASE = 1000   # ids of models registered at run time start here
MODEL_HAS_JAC, MODEL_HAS_TGRAD, MODEL_NONAUTONOMOUS = 1, 2, 4
MODEL_CONTINUOUS_CALLBACK, MODEL_CALLBACK_AFFECT, MODEL_CALLBACK_AFFECT_NEG = 8, 16, 32
MODEL_VECTOR_CALLBACK, MODEL_DISCRETE_CALLBACK = 64, 128


def model_callback_len(n):
    return n << 16
PREC_FP64, PREC_MIXED = 0, 1
STATUS = {0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "out of device memory",
          -4: "unsupported", -5: "busy", -6: "timeout", -7: "unknown ticket"}


class ProblemDesc(C.Structure):
    _fields_ = [("model_id", C.c_int32), ("alg_id", C.c_int32), ("n_states", C.c_int32),
                ("n_params", C.c_int32), ("precision", C.c_int32), ("reserved", C.c_int32)]


class Options(C.Structure):
    _fields_ = [("reltol", C.c_double), ("abstol", C.c_double), ("dtmax", C.c_double),
                ("dtmin", C.c_double), ("dt", C.c_double), ("maxiters", C.c_int64),
                ("save_start", C.c_int32), ("save_end", C.c_int32), ("save_end_user", C.c_int32),
                ("saveat_scalar", C.c_int32), ("nsave", C.c_int32), ("saveat_per_traj", C.c_int32),
                ("qmax_first_step", C.c_double), ("qmax", C.c_double), ("lanes_per_traj", C.c_int32),
                ("scheduler", C.c_int32), ("block_size", C.c_int32), ("ir_sweeps", C.c_int32),
                ("save_everystep", C.c_int32), ("max_step_saves", C.c_int32),
                ("callback", C.c_int32), ("interp_points", C.c_int32), ("max_events", C.c_int32),
                ("ntstops", C.c_int32), ("tstops", C.POINTER(C.c_double)),
                ("max_jac_age", C.c_int32), ("isoutofdomain", C.c_int32), ("jac_reuse_gamma_tol", C.c_double),
                ("nsave_idxs", C.c_int32), ("reserved3", C.c_int32), ("save_idxs", C.POINTER(C.c_int32)),
                ("adaptive", C.c_int32), ("forward_only", C.c_int32),
                ("controller_given", C.c_int32), ("force_dtmin", C.c_int32), ("beta1", C.c_double),
                ("beta2", C.c_double), ("qoldinit", C.c_double), ("qmin", C.c_double), ("gamma", C.c_double),
                ("qsteady_min", C.c_double), ("qsteady_max", C.c_double),
                ("abstol_vec", C.POINTER(C.c_double)), ("reltol_vec", C.POINTER(C.c_double))]


class Stats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("nf", "njacs", "nw", "nsolve", "naccept", "nreject")]


class ServingStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("submitted", "admitted", "completed", "rejected", "queued",
                                         "running", "hbm_in_use", "hbm_budget")] + \
               [("slots", C.c_int32), ("launches", C.c_int32)]


# Every exported entry point of the C ABI with its ctypes signature.
_VP = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int32)
SIGNATURES = {
    "ode_abi_version": (C.c_int, []),
    "ode_options_default": (None, [C.POINTER(Options)]),
    "ode_options_size": (C.c_size_t, []),
    "ode_problem_desc_size": (C.c_size_t, []),
    "ode_create": (C.c_int, [C.c_int, C.c_size_t, C.POINTER(_VP)]),
    "ode_destroy": (None, [_VP]),
    "ode_last_error": (C.c_char_p, [_VP]),
    "ode_status_string": (C.c_char_p, [C.c_int]),
    "ode_solve_ensemble": (C.c_int, [_VP, C.POINTER(ProblemDesc), C.POINTER(Options), C.c_int64, _IP,
                                     _DP, _DP, _DP, _DP, _DP, _DP, _IP, _IP, C.POINTER(Stats)]),
    "ode_solve_ensemble_device": (C.c_int, [_VP, C.POINTER(ProblemDesc), C.POINTER(Options), C.c_int64,
                                            _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
    "ode_dense_nk": (C.c_int, [C.c_int]),
    "ode_solve_ensemble_dense": (C.c_int, [_VP, C.POINTER(ProblemDesc), C.POINTER(Options), C.c_int64, _DP, _DP,
                                           _DP, _DP, _DP, _DP, _IP, _IP, C.POINTER(Stats)]),
    "ode_dense_eval": (C.c_int, [_VP, C.POINTER(ProblemDesc), C.c_int64, _DP, _DP, _DP, _DP, _IP, C.c_int32,
                                 C.c_int32, _DP, C.c_int32, _DP]),
    "ode_dense_eval_deriv": (C.c_int, [_VP, C.POINTER(ProblemDesc), C.c_int64, _DP, _DP, _DP, _DP, _IP, C.c_int32,
                                       C.c_int32, _DP, C.c_int32, C.c_int32, _DP]),
    "ode_dense_eval_ex": (C.c_int, [_VP, C.POINTER(ProblemDesc), C.c_int64, _DP, _DP, _DP, _DP, _IP, C.c_int32,
                                    C.c_int32, _DP, C.c_int32, C.c_int32, C.c_int32, _DP]),
    "ode_submit": (C.c_int, [_VP, C.POINTER(ProblemDesc), C.POINTER(Options), C.c_int64, _IP, _DP, _DP,
                             _DP, _DP, _DP, _DP, _IP, _IP, C.POINTER(Stats), C.POINTER(C.c_uint64)]),
    "ode_poll": (C.c_int, [_VP, C.c_uint64, _IP]),
    "ode_wait": (C.c_int, [_VP, C.c_uint64, C.c_double]),
    "ode_autotune": (C.c_int, [_VP, C.POINTER(ProblemDesc), C.POINTER(Options), C.c_int64, _DP, _DP, _DP, _DP,
                               _IP, _IP, _IP, _DP]),
    "ode_next_completed": (C.c_int, [_VP, C.c_double, C.POINTER(C.c_uint64), _IP, C.POINTER(C.c_double)]),
    "ode_serving_stats_get": (C.c_int, [_VP, C.POINTER(ServingStats)]),
    "ode_set_serving_slots": (C.c_int, [_VP, C.c_int32]),
    "ode_set_serving_queue_limit": (C.c_int, [_VP, C.c_int64]),
    "ode_abort": (C.c_int, [_VP]),
    "ode_kernel_launches": (C.c_int, [_VP, C.POINTER(C.c_int64)]),
    "ode_last_kernel_ms": (C.c_int, [_VP, _DP]),
    "ode_query_variants": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, _IP, C.c_int32]),
    "ode_register_model": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.c_int32, C.c_int32, _IP]),
    "ode_measure_fma_peak": (C.c_int, [C.c_int, C.c_int, _DP]),
    "ode_solve_ensemble_noalloc": (C.c_int, [C.POINTER(ProblemDesc), C.POINTER(Options), C.c_int64, _VP, _VP,
                                             _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP]),
}

_lib = None


def lib_path():
    return _build.LIB_PATH


def load(build_if_missing=True):
    """Load libode_b200.so, building it first if it is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if build_if_missing and (not os.path.exists(path) or not _build.up_to_date()):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libode_b200.so is not built (" + path + "); run odegb300.build.build()")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    # the ctypes mirrors must match the library's struct layouts
    if L.ode_options_size() != C.sizeof(Options) or L.ode_problem_desc_size() != C.sizeof(ProblemDesc):
        raise RuntimeError("odegb300: Options/ProblemDesc do not match the library's ode_options/ode_problem_desc "
                           "(%d/%d vs %d/%d bytes)" % (C.sizeof(Options), C.sizeof(ProblemDesc),
                                                       L.ode_options_size(), L.ode_problem_desc_size()))
    _lib = L
    return L


class OdeError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(status, "error"), status, msg))
        self.status = status


def check(status, handle=None):
    if status != 0:
        L = load()
        msg = L.ode_last_error(handle)
        raise OdeError(status, msg.decode() if msg else "")
    return status
