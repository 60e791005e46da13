/* libode_b200.so — C ABI of the GB300 ensemble ODE integrator.
 *
 * The drop-in point is the reference's many-trajectory solve
 *   solve(EnsembleProblem(prob; prob_func), alg, ensemblealg; trajectories, saveat,
 *         reltol, abstol)
 * where ensemblealg is a SciMLBase.EnsembleAlgorithm (SciMLBase is not
 * vendored; the call shape is exercised in lib/DiffEqBase/test/downstream/
 * ensemble.jl:15-42).  A Julia `EnsembleGB300 <: EnsembleAlgorithm` evaluates
 * prob_func on the host, packs the per-trajectory u0/p/tspan structure-of-
 * arrays, and calls ode_solve_ensemble through ccall; it then builds one
 * ODESolution per trajectory from t_out/u_out/retcode/stats.
 *
 * Everything the per-trajectory `solve(prob_i, alg; kwargs...)` does
 * (lib/OrdinaryDiffEqCore/src/solve.jl:1-12, 128-946) runs on the GPU:
 * initdt, the step loop with the PI controller, saveat interpolation and the
 * retcode checks, for Tsit5, Vern7 and Rodas5P.
 *
 * Conventions: plain C types, caller-owned host buffers, 0 = success and a
 * negative ode_status on error (never aborts the process).  Layouts are
 * structure-of-arrays with the trajectory index fastest:
 *   u0[i*N + j]          state i of trajectory j            (n_states x N)
 *   p[k*N + j]           parameter k of trajectory j        (n_params x N)
 *   tspan[j], tspan[N+j] t0 and tf of trajectory j          (2 x N; tf < t0 integrates backward)
 *   saveat[s] shared, or saveat[s*N + j] per trajectory     (nsave or nsave x N; ascending in s
 *                                                           whatever the direction)
 *   t_out[s*N + j], u_out[(s*n_states + i)*N + j]         (cap x N, cap x n_states x N; with save_idxs
 *                                                           nsave_idxs rows replace the n_states)
 * with cap = nsave + 2 save slots per trajectory (start and end saves), or
 * max_step_saves + 2 with save_everystep, plus 2 * max_events with a callback.
 */
#ifndef ODE_GB300_H
#define ODE_GB300_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define ODE_ABI_VERSION 10

typedef struct ode_handle ode_handle;

/* Algorithms: Tsit5 (lib/OrdinaryDiffEqTsit5/src/algorithms.jl:16-21),
 * Vern7 (lib/OrdinaryDiffEqVerner/src/algorithms.jl:44-50, lazy = true),
 * Rodas5P (lib/OrdinaryDiffEqRosenbrock/src/algorithms.jl:83-87),
 * Rosenbrock23 (lib/OrdinaryDiffEqRosenbrock/src/algorithms.jl:1-16,108-146, the
 * default max_jac_age = 1: a fresh J and W on every step attempt). */
enum ode_alg {
    ODE_TSIT5 = 0, ODE_VERN7 = 1, ODE_RODAS5P = 2, ODE_ROSENBROCK23 = 3,
    ODE_AUTOTSIT5_ROSENBROCK23 = 4  /* AutoTsit5(Rosenbrock23()): Tsit5 with stiffness detection switching
                                       to Rosenbrock23 (lib/OrdinaryDiffEqTsit5/src/algorithms.jl:27-33,
                                       lib/OrdinaryDiffEqCore/src/composite_algs.jl; default AutoSwitch) */
};

/* Registered right-hand sides (with analytic Jacobians).  The reference takes
 * an arbitrary f(du,u,p,t); device code cannot call Julia closures, so models
 * are compiled in and chosen by id. */
enum ode_model {
    ODE_MODEL_LINEAR = 0,         /* u' = p0 u, any n                                 */
    ODE_MODEL_LORENZ = 1,         /* n = 3, p = (sigma, rho, beta)                     */
    ODE_MODEL_ROBERTSON = 2,      /* n = 3, p = (k1, k2, k3)                           */
    ODE_MODEL_DUFFING_CHAIN = 3,  /* n = 2N, interleaved (x_i, v_i), p = (k, delta, beta) */
    ODE_MODEL_BRUSSELATOR_1D = 4, /* n = 2*cells, interleaved (u_i, v_i), p = (A, B, alpha) */
    ODE_MODEL_VANDERPOL = 6,      /* n = 2 (x, y): x' = y, y' = mu ((1 - x^2) y - x); p = (mu)
                                     (test/InterfaceI/stiffness_detection_test.jl:10-16) */
    ODE_MODEL_PK_ONE_COMPARTMENT = 7, /* n = 2 (depot, central): depot' = -ka depot,
                                     central' = ka depot - ke central; p = (ka, ke, dose).  Its
                                     DiscreteCallback (ode_options.callback): condition t in tstops
                                     (the dose times, passed as the solve's tstops), affect!:
                                     depot += dose; save_positions = (true, true) */
    ODE_MODEL_BOUNCING_BALL = 5,  /* n = 2 (x, v): x' = v, v' = -g; p = (g, e, t_stop).  Its
                                     ContinuousCallback (ode_options.callback): condition x,
                                     affect! = nothing, affect_neg!: terminate! once t >= t_stop,
                                     else v <- -e v (test/Integrators_I/ode_event_tests.jl:100-113,283-360) */
    ODE_MODEL_FORCED_DUFFING = 8  /* n = 2 (x, v), non-autonomous: x' = v,
                                     v' = ((g cos(w t) - delta v) - alpha x) - beta x^3;
                                     p = (delta, alpha, beta, g, w); analytic J and tgrad (df/dt, which
                                     the Rosenbrock methods use: derivative_utils.jl:181-227) */
};

/* Models registered at run time (ode_register_model) take ids from
 * ODE_MODEL_USER_BASE up, in registration order. */
#define ODE_MODEL_USER_BASE 1000

/* Flags of ode_register_model. */
enum ode_model_flags {
    ODE_MODEL_HAS_JAC = 1,        /* the source defines NAME_jac (else the Rosenbrock methods take J by
                                     forward-mode AD of NAME_f, one counted f call per Jacobian) */
    ODE_MODEL_HAS_TGRAD = 2,      /* the source defines NAME_tgrad, df/dt */
    ODE_MODEL_NONAUTONOMOUS = 4,  /* NAME_f reads t (the Rosenbrock methods then need NAME_tgrad) */
    /* Callbacks registered with the model (active when ode_options.callback = 1), each a plain
     * FP64 device function of the state u (n), the parameters p and t:
     *   ContinuousCallback:  double NAME_condition(const double* u, const double* p, double t);
     *                        int NAME_affect(double* u, const double* p, double t, int upcrossing);
     *   VectorContinuousCallback (len conditions):
     *                        void NAME_vcondition(double* out, const double* u, const double* p, double t);
     *                        int NAME_vaffect(double* u, const double* p, double t, const int* events);
     *                        (events[k]: +1 upcrossing, -1 downcrossing, 0 not fired)
     *   DiscreteCallback:    int NAME_dcondition(const double* u, const double* p, double t);
     *                        int NAME_daffect(double* u, const double* p, double t);
     * An affect that returns nonzero calls terminate! (ReturnCode.Terminated).  SciMLBase's
     * defaults: save_positions = (true, true); continuous: interp_points (ode_options),
     * LeftRootFind, abstol = 10eps(), repeat_nudge = 1//100. */
    ODE_MODEL_CONTINUOUS_CALLBACK = 8,
    ODE_MODEL_CALLBACK_AFFECT = 16,      /* the ContinuousCallback acts on upcrossings (affect!) */
    ODE_MODEL_CALLBACK_AFFECT_NEG = 32,  /* ... and/or on downcrossings (affect_neg!) */
    ODE_MODEL_VECTOR_CALLBACK = 64,      /* with ODE_MODEL_CALLBACK_LEN(len), 1 <= len <= 32 */
    ODE_MODEL_DISCRETE_CALLBACK = 128
};
#define ODE_MODEL_CALLBACK_LEN(len) ((len) << 16)

/* FP64: every operation in double (the reference's arithmetic).
 * MIXED: state and stage arithmetic in FP32 (and, for Rodas5P, the W
 * factorisation in FP32 with FP64-residual iterative refinement); t, dt, the
 * error-norm accumulator and the step-size controller stay FP64. */
enum ode_precision { ODE_PREC_FP64 = 0, ODE_PREC_MIXED = 1 };

/* Per-trajectory return codes, SciMLBase.ReturnCode meanings
 * (lib/DiffEqBase/src/check_error.jl:70-118). */
enum ode_retcode {
    ODE_RC_DEFAULT = 0, ODE_RC_SUCCESS = 1, ODE_RC_MAXITERS = 2, ODE_RC_DTNAN = 3,
    ODE_RC_DTLESSTHANMIN = 4, ODE_RC_UNSTABLE = 5,
    ODE_RC_ABORTED = 6, /* stopped by ode_abort(); no reference counterpart */
    ODE_RC_TERMINATED = 7, /* a callback called terminate! (ReturnCode.Terminated) */
    ODE_RC_INITIALFAILURE = 8 /* a NaN time span: the trajectory is not stepped (ReturnCode.InitialFailure) */
};

enum ode_status {
    ODE_OK = 0, ODE_E_INVALID = -1, ODE_E_CUDA = -2, ODE_E_NOMEM = -3,
    ODE_E_UNSUPPORTED = -4, ODE_E_BUSY = -5, ODE_E_TIMEOUT = -6, ODE_E_NOTFOUND = -7
};

/* Per-trajectory counters; mirrors DiffEqBase.Stats (lib/DiffEqBase/src/stats.jl:30-44). */
typedef struct {
    int64_t nf, njacs, nw, nsolve, naccept, nreject;
} ode_stats;

typedef struct {
    int32_t model_id;    /* ode_model */
    int32_t alg_id;      /* ode_alg */
    int32_t n_states;    /* state stride (the largest state count when n_per_traj is given) */
    int32_t n_params;    /* parameters per trajectory */
    int32_t precision;   /* ode_precision */
    int32_t reserved;
} ode_problem_desc;

/* Solver keyword arguments (lib/OrdinaryDiffEqCore/src/solve.jl:128-202).
 * The save_* flags arrive already resolved by the caller with the reference's
 * defaults (solve.jl:141-143, 596-599). */
typedef struct {
    double reltol, abstol;      /* reference defaults 1e-3, 1e-6 when not given */
    double dtmax;               /* <= 0: tf - t0 */
    double dtmin;               /* 0: eps(t) */
    double dt;                  /* > 0: initial dt, skips the initial-step heuristic */
    int64_t maxiters;           /* <= 0: 1e6 */
    int32_t save_start, save_end;
    int32_t save_end_user;      /* -1 not given, else 0/1 (endpoint rule, integrator_utils.jl:540-588) */
    int32_t saveat_scalar;      /* saveat was a number ((t0 + tdir|d|):(tdir|d|):tf) */
    int32_t nsave;              /* saveat entries (0 = no saveat) */
    int32_t saveat_per_traj;    /* 0: saveat[nsave] shared; 1: saveat[nsave*N] */
    double qmax_first_step;     /* <= 0: 10000 */
    double qmax;                /* <= 0: 10 */
    int32_t lanes_per_traj;     /* 0: tuned choice; else 1,2,4,8,16,32 where compiled */
    int32_t scheduler;          /* 0 auto, 1 static (one lane group per trajectory), 2 persistent queue */
    int32_t block_size;         /* 0: tuned */
    int32_t ir_sweeps;          /* MIXED Rodas5P refinement sweeps (< 0: none) */
    int32_t save_everystep;     /* 1: save every accepted step, the reference's default without saveat
                                   (integrator_utils.jl:397-404); with saveat points, both sets (each
                                   step after the saveat points up to it, unless one landed on it) */
    int32_t max_step_saves;     /* save_everystep: step saves kept per trajectory; t_out/u_out hold
                                   nsave + max_step_saves + 2 slots, and past that the last slot keeps the
                                   latest step */
    int32_t callback;           /* 1: the model's registered ContinuousCallback (models with an event;
                                   SciMLBase defaults: rootfind = LeftRootFind, save_positions = (true, true),
                                   abstol = 10eps(), repeat_nudge = 1//100, dtrelax = 1).  An event moves t
                                   back into the step and recomputes the step's interpolation data for the
                                   shortened step (reeval_internals_due_to_modification!), as the reference */
    int32_t interp_points;      /* the callback's interp_points (default 10) */
    int32_t max_events;         /* save slots for events: 2 per event (before and after its affect) are added to
                                   the output, and past the total the last slot keeps the latest save */
    int32_t ntstops;            /* the solve's tstops, shared by every trajectory (solve.jl:1021-1040): */
    const double* tstops;       /* a trajectory stops exactly at each ts with t0 < ts < tf, as at tf
                                   (modify_dt_for_tstops!, handle_tstop!); duplicates allowed.  Host
                                   memory in any order (NaN rejected) for ode_solve_ensemble,
                                   ode_solve_ensemble_dense, ode_submit and ode_autotune; device
                                   memory sorted ascending for ode_solve_ensemble_device and
                                   ode_solve_ensemble_noalloc (entries out of order or NaN are skipped) */
    int32_t max_jac_age;        /* Rosenbrock23 (a W-method) keeps J across accepted steps for at most this
                                   many (Rosenbrock23(max_jac_age = ...), _rosenbrock_jac_reuse_decision,
                                   OrdinaryDiffEqDifferentiation/src/derivative_utils.jl:46-170): 0 or 1, the
                                   reference's default for Rosenbrock23, evaluates J on every attempt.
                                   W = J - I/(dt gamma) and its LU are formed on every attempt either way */
    int32_t isoutofdomain;      /* solve(...; isoutofdomain): 0 (default) none; 1 the common
                                   (u, p, t) -> any(x -> x < 0, u): an adaptive step whose end state has a
                                   negative component is rejected and retried with dt * qmin
                                   (integrator_utils.jl:135-137, 612-623) */
    double jac_reuse_gamma_tol; /* reuse only while |dtgamma / dtgamma_J - 1| <= this (reference default
                                   0.03; < 0 means the default) */
    int32_t nsave_idxs;         /* > 0: the reference's save_idxs: only these states are saved, u_out holds */
    int32_t reserved3;          /* nsave_idxs rows per save (u_out[(s*nsave_idxs + r)*N + j] = state   */
    const int32_t* save_idxs;   /* save_idxs[r] of trajectory j), in the given order, repeats allowed.
                                   0-based.  Host memory for the host entry points (checked against
                                   n_states), device memory for ode_solve_ensemble_device and
                                   ode_solve_ensemble_noalloc (an index outside the trajectory's states
                                   leaves its row unwritten).  Not with dense output */
    int32_t adaptive;           /* 1 (default): error-controlled steps; 0: fixed steps of |dt|, clipped to
                                   land on the tstops and tf; with dt = 0 (then tstops are required)
                                   every step runs to the next tstop (the reference's adaptive = false:
                                   no error estimate is judged, every step is accepted) */
    int32_t forward_only;       /* 1: the caller guarantees tf >= t0 for every trajectory, so the kernels'
                                   plain forms (no integration direction, force_dtmin or isoutofdomain in
                                   their step loops) may run when neither of those two is set; a backward
                                   span then reports ODE_RC_INITIALFAILURE.  0 (default):
                                   either direction.  The host entry points (ode_solve_ensemble, _dense,
                                   ode_submit) find it out themselves from the host spans */
    /* The PI step-size controller's knobs (solve(...; controller = PIController(beta1, beta2;
       qoldinit, qmin, gamma, qsteady_min, qsteady_max)), controllers.jl:745-843; qmax and
       qmax_first_step above).  controller_given = 0: every knob at the method's default
       (alg_utils.jl); 1: each field below that is not NaN replaces the default (for both
       methods of a composite) */
    int32_t controller_given;
    int32_t force_dtmin;        /* 1: the reference's force_dtmin = true: a step at or below max(eps(t), dtmin)
                                   is accepted whatever its error, and no DtLessThanMin or Unstable exit is
                                   taken on dt (check_error.jl:91-106, integrator_utils.jl:613-623) */
    double beta1, beta2, qoldinit, qmin, gamma, qsteady_min, qsteady_max;
    /* Per-state tolerances (solve(...; abstol = [...], reltol = [...]): calculate_residuals with
       array tolerances, calculate_residuals.jl:9-14,117-125, and the initial-step scale): n_states
       entries each (abstol >= 0, reltol > 0), or NULL for the scalar above.  Host memory for the
       host entry points, device memory for ode_solve_ensemble_device and ode_solve_ensemble_noalloc;
       not with ode_submit */
    const double* abstol_vec;
    const double* reltol_vec;
} ode_options;

/* Fill o with the reference's defaults. */
void ode_options_default(ode_options* o);
/* sizeof(ode_options) and sizeof(ode_problem_desc) as compiled: bindings that
 * mirror the structs (Julia, Python) check their layout against these. */
size_t ode_options_size(void);
size_t ode_problem_desc_size(void);

/* Register a right-hand side given as CUDA C++ source, the device form of the
 * reference's f(du, u, p, t) with its optional jac and tgrad (ODEFunction; the
 * solve entry lib/DiffEqBase/src/solve.jl:155-192 takes any user function).
 * For a model named NAME (a C identifier) the source defines
 *   template <class T, class P> __device__ void NAME_f(T* du, const T* u, const P* p, double t);
 *   template <class T, class P> __device__ void NAME_jac(T* J, const T* u, const P* p, double t);   (optional,
 *                                                                        row-major J[i*n + j] = df_i/du_j)
 *   template <class T, class P> __device__ void NAME_tgrad(T* dT, const T* u, const P* p, double t); (optional)
 * written for any arithmetic T and parameter type P (FP64 solves use double;
 * mixed solves a float, a double-float pair or a dual number) with +, -, *, /
 * and exp, log, sqrt, sin, cos, tanh, pow, fabs.  n_states: 1..32 (at most 8 for
 * Rodas5P, Rosenbrock23 and AutoTsit5(Rosenbrock23())); n_params: 0..32.
 * Returns the new model id (>= ODE_MODEL_USER_BASE) for ode_problem_desc.
 * Kernels are compiled with NVRTC on the first solve of each (method,
 * precision) and kept until the process exits; a compile error fails that solve
 * with ODE_E_UNSUPPORTED and the compiler log in ode_last_error.  Uniform sizes
 * only (no n_per_traj), no callback. */
int ode_register_model(const char* source, const char* name, int32_t n_states, int32_t n_params, int32_t flags,
                       int32_t* model_id);

/* Open device `device`; hbm_budget bytes caps device memory the handle may
 * hold (0: 90% of free memory).  One CUDA stream per handle. */
int ode_create(int device, size_t hbm_budget, ode_handle** out);
void ode_destroy(ode_handle* h);
const char* ode_last_error(const ode_handle* h);
const char* ode_status_string(int status);
int ode_abi_version(void);

/* Synchronous ensemble solve on caller-owned HOST buffers (layouts above).
 * n_per_traj (may be NULL) gives each trajectory's state count (DUFFING_CHAIN
 * only; each one of 4, 8, 16, 32, 64 and <= n_states): trajectories are
 * bucketed by size on the device and every size class is integrated in one
 * persistent launch.  On the device-buffer entry points a trajectory of any
 * other size is not integrated (nsaved 0, retcode ODE_RC_DEFAULT); the host
 * entry point rejects it.  Outputs are written before return.  stats and
 * t_out may be NULL. */
int ode_solve_ensemble(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t ntraj,
                       const int32_t* n_per_traj, const double* u0, const double* p, const double* tspan,
                       const double* saveat, double* t_out, double* u_out, int32_t* nsaved,
                       int32_t* retcode, ode_stats* stats);

/* Same solve on DEVICE buffers already resident in HBM, enqueued on
 * `cuda_stream` (NULL: the handle's stream); returns once enqueued.  Device
 * scratch (work queues, size-class buckets) is owned by the handle. */
int ode_solve_ensemble_device(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t ntraj,
                              const int32_t* n_per_traj_dev, const double* u0, const double* p,
                              const double* tspan, const double* saveat, double* t_out, double* u_out,
                              int32_t* nsaved, int32_t* retcode, ode_stats* stats, void* cuda_stream);

/* Dense output: the reference's dense = true, its default when no saveat is
 * given (lib/OrdinaryDiffEqCore/src/solve.jl:145-146; sol.k filled by
 * save_dense_at_t!, integrator_utils.jl:455-473).  ode_dense_nk: vectors
 * stored per saved step, the method's interpolation data (integrator.k):
 * Tsit5 7 (k1..k7), Vern7 7 (k1, k4..k9: its interpolant and lazy extra
 * stages read no others), Rodas5P 3 (the dense k1..k3), Rosenbrock23 2 (k1,
 * k2); 0 for AutoTsit5(Rosenbrock23()) (no dense output).  ODE_E_INVALID for an
 * unknown alg. */
int ode_dense_nk(int alg);

/* Synchronous dense solve on HOST buffers: every accepted step is saved
 * (o->save_everystep = 1, o->nsave = 0) and its vectors go to
 * k_out[((s*nk + q)*n_states + i)*N + j], cap = max_step_saves + 2 slots.
 * The start save's vectors are 0.  A trajectory with more steps than slots
 * keeps its final point in the last slot with NaN vectors: its last interval
 * cannot be interpolated.  With a callback, its saves (before and after the
 * affect, at the same t) store the step's vectors too; an event step's are
 * those of the step shortened to the event.  Uniform sizes only (no
 * n_per_traj).  Page-locked buffers are used in place, as in
 * ode_solve_ensemble. */
int ode_solve_ensemble_dense(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t ntraj,
                             const double* u0, const double* p, const double* tspan, double* t_out,
                             double* u_out, double* k_out, int32_t* nsaved, int32_t* retcode, ode_stats* stats);

/* sol_j(t) of a dense solve for every trajectory j at nq query times (tq[r]
 * shared, or tq[r*N + j] per trajectory), evaluated on the device in FP64 from
 * the solve's HOST outputs (t_saved, u_saved, k_saved with cap slots, layouts
 * as above; p as given to the solve, read by Vern7's extra stages):
 * out[(r*n_states + i)*N + j].  Follows ode_interpolation
 * (lib/OrdinaryDiffEqCore/src/dense/generic_dense.jl:1094-1190): the left-
 * continuous interval ts[i-] < t <= ts[i+], theta = (t - ts[i-]) /
 * (ts[i+] - ts[i-]) and the method's interpolant with the vectors of the step
 * ending at ts[i+] (Vern7 first forms its extra stages from them).  Times
 * outside the saved range use the first or last step's polynomial, as
 * ode_interpolation does; a trajectory with nsaved 0 gets NaN.  The saves are
 * staged on the device; a page-locked `out` is written in place. */
int ode_dense_eval(ode_handle* h, const ode_problem_desc* d, int64_t ntraj, const double* p,
                   const double* t_saved, const double* u_saved, const double* k_saved, const int32_t* nsaved,
                   int32_t cap, int32_t nq, const double* tq, int32_t tq_per_traj, double* out);
/* The same with the derivative order: deriv 0 is sol(t) (ode_dense_eval), 1 is
 * sol(t, Val{1}), the time derivative of the method's interpolant on the same
 * interval (Tsit5 interpolants.jl:143-178, Vern7 :305-334, Rodas5P
 * rosenbrock_interpolants.jl:444-470, Rosenbrock23 :111-127), 2 and 3 are
 * sol(t, Val{2}) and sol(t, Val{3}) for the methods whose interpolant has those
 * forms in the reference (Tsit5: interpolants.jl tsit5pre2, tsit5pre3; Rodas5P:
 * rosenbrock_interpolants.jl:544-560, 644-653).  Other orders and methods:
 * ODE_E_UNSUPPORTED. */
int ode_dense_eval_deriv(ode_handle* h, const ode_problem_desc* d, int64_t ntraj, const double* p,
                         const double* t_saved, const double* u_saved, const double* k_saved, const int32_t* nsaved,
                         int32_t cap, int32_t nq, const double* tq, int32_t tq_per_traj, int32_t deriv, double* out);
/* The same with the continuity of sol(t, continuity): a query equal to a saved
 * time returns that save (ode_interpolation's exact-time rule), the first one at
 * that time, or with continuity_right = 1 (continuity = :right) the next save
 * when it is at the same time (an event's post-affect save).  deriv > 0 always
 * interpolates, as the reference does. */
int ode_dense_eval_ex(ode_handle* h, const ode_problem_desc* d, int64_t ntraj, const double* p,
                      const double* t_saved, const double* u_saved, const double* k_saved, const int32_t* nsaved,
                      int32_t cap, int32_t nq, const double* tq, int32_t tq_per_traj, int32_t deriv,
                      int32_t continuity_right, double* out);

/* Continuous-batching serving API.  ode_submit copies the request's inputs
 * into handle-owned pinned/device memory and returns a ticket at once; the
 * request starts on the device as soon as a slot and enough of the HBM
 * budget are free, overlapping with requests already running.  Queued
 * requests that differ only in their trajectories and tolerances (same model,
 * method, precision, sizes, options, saveat and tstops) are merged into one
 * launch, each trajectory with its own request's tolerances; a request that
 * does not fit the budget lets smaller ones behind it start, unless it has
 * waited 0.25 s.  Outputs land in the caller's buffers (which must stay
 * valid) when ode_poll/ode_wait report completion. */
int ode_submit(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t ntraj,
               const int32_t* n_per_traj, const double* u0, const double* p, const double* tspan,
               const double* saveat, double* t_out, double* u_out, int32_t* nsaved, int32_t* retcode,
               ode_stats* stats, uint64_t* ticket);
/* done = 1 when the request's outputs are in place. */
int ode_poll(ode_handle* h, uint64_t ticket, int32_t* done);
/* Wait at most timeout_s seconds (< 0: forever). */
int ode_wait(ode_handle* h, uint64_t ticket, double timeout_s);
/* The next finished request in completion order, waiting at most timeout_s
 * seconds (< 0: forever, 0: do not wait).  *ticket = 0 when none finished in
 * time.  status: the request's result code; times[0..2]: submit, start on
 * the device and completion (outputs in place), CLOCK_MONOTONIC seconds.
 * Releases the ticket like a completed ode_poll.  No reference counterpart
 * (serving). */
int ode_next_completed(ode_handle* h, double timeout_s, uint64_t* ticket, int32_t* status, double* times);

typedef struct {
    int64_t submitted, admitted, completed, rejected, queued, running;  /* requests (running: launches) */
    int64_t hbm_in_use, hbm_budget;
    int32_t slots;
    int32_t launches;    /* launches so far; requests merged into one launch count once */
} ode_serving_stats;
int ode_serving_stats_get(ode_handle* h, ode_serving_stats* s);
/* Number of concurrent device slots (streams) used by the serving loop (default 8). */
int ode_set_serving_slots(ode_handle* h, int32_t slots);
/* ode_submit answers ODE_E_BUSY, without queuing, while max_queued requests wait
 * (0, the default: no limit): a server sheds load instead of queuing without
 * bound.  No reference counterpart (serving). */
int ode_set_serving_queue_limit(ode_handle* h, int64_t max_queued);

/* Ask running kernels of this handle to stop; affected trajectories report
 * ODE_RC_ABORTED.  Cleared by the next solve. */
int ode_abort(ode_handle* h);

/* Kernel launches made by this handle so far, and the device time of the
 * last ensemble launch measured with CUDA events on its stream. */
int ode_kernel_launches(const ode_handle* h, int64_t* launches);
int ode_last_kernel_ms(const ode_handle* h, double* ms);

/* Autotuner (no reference counterpart): times every compiled kernel variant
 * (lanes per trajectory), block size (32, 64, 128) and scheduler (static,
 * persistent) on the given HOST sample of a uniform-size problem and keeps
 * the fastest for this handle; later solves of the same (alg, model,
 * precision, n_states) with lanes_per_traj, block_size and scheduler left at
 * 0 use it.  Outputs: the chosen shape and its time per solve of the sample. */
int ode_autotune(ode_handle* h, const ode_problem_desc* d, const ode_options* o, int64_t ntraj, const double* u0,
                 const double* p, const double* tspan, const double* saveat, int32_t* lanes, int32_t* block_size,
                 int32_t* scheduler, double* ms);

/* Compiled kernel variants for (alg, model, precision, n): lanes per
 * trajectory, for tuning and diagnostics.  Returns the count written. */
int ode_query_variants(int alg, int model, int precision, int n, int32_t* lanes, int32_t cap);

/* Allocation-free ensemble solve on DEVICE buffers, enqueued on cuda_stream
 * (NULL: the legacy default stream).  No counterpart in the reference: it is
 * for callers that cannot call cudaMalloc (a framework's caching allocator
 * owns the device, or the caller runs under a fixed memory budget), so it
 * needs no handle and allocates nothing.  The work counters and the
 * size-class index list of the persistent kernels live in one fixed device
 * array inside the library (8 MiB + 512 B, held by every GPU that loads the
 * library until exit), so n_per_traj_dev calls take at most 2^20
 * trajectories (larger requests fail with ODE_E_INVALID); uniform-size calls
 * have no limit.  The first call on a device resolves the array's address
 * with that device current; make that first call before any stream capture.
 * Every call shares the array: calls whose work overlaps on the GPU (two
 * streams, or two host threads) race on it and must be serialised by the
 * caller.  Same layouts and results as ode_solve_ensemble_device; returns
 * once the work is enqueued (uneven-size calls of a method without a
 * one-launch class kernel synchronise the stream once to size the buckets). */
int ode_solve_ensemble_noalloc(const ode_problem_desc* d, const ode_options* o, int64_t ntraj,
                               const int32_t* n_per_traj_dev, const double* u0, const double* p,
                               const double* tspan, const double* saveat, double* t_out, double* u_out,
                               int32_t* nsaved, int32_t* retcode, ode_stats* stats, void* cuda_stream);

/* Measured FMA throughput (FLOP/s, 2 per FMA) of the FP64 (precision =
 * ODE_PREC_FP64) or FP32 (ODE_PREC_MIXED) pipe of `device`: the roofline
 * denominator for the integrator kernels, which are bound by that pipe. */
int ode_measure_fma_peak(int device, int precision, double* flops_per_s);

#ifdef __cplusplus
}
#endif
#endif
