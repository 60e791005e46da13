/* TEST INFRASTRUCTURE — not part of the product.
 *
 * CPU restatement (FP64) of the reference's many-trajectory solve path, used
 * only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
 * the checker.  Nothing in the product links or calls it.
 *
 * Parity status: the reference is pure Julia and cannot be run in this
 * environment, and its test-suite holds no stored trajectory values for this
 * path.  The oracle is therefore pinned at the solution level only, against
 * the reference's own tolerance tests (convergence orders, dense-output error
 * bounds, nf accounting, saveat endpoint rules, qmax_first_step); see
 * tests/test_oracle.py.  Bit-level agreement with Julia (LLVM's FMA
 * contraction choices, LinearSolve's LU, FastPower's pow) is not pinned.
 */
#ifndef ODE_ORACLE_H
#define ODE_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_TSIT5 = 0, ORC_VERN7 = 1, ORC_RODAS5P = 2, ORC_VERN9 = 3, ORC_ROSENBROCK23 = 4,
       ORC_AUTOTSIT5_ROSENBROCK23 = 5 /* AutoTsit5(Rosenbrock23()) */ };
enum { ORC_LINEAR = 0, ORC_LORENZ = 1, ORC_ROBERTSON = 2, ORC_DUFFING = 3, ORC_BRUSSELATOR = 4, ORC_BOUNCING_BALL = 5,
       ORC_VANDERPOL = 6, ORC_PK1 = 7, ORC_FORCED_DUFFING = 8,
       ORC_LOTKA_VOLTERRA = 9, ORC_OREGONATOR = 10, ORC_BALL_BOX = 11, ORC_THRESHOLD_DOSE = 12 };
/* SciMLBase ReturnCode subset used by this path (numbering of the C ABI). */
enum { ORC_RC_DEFAULT = 0, ORC_RC_SUCCESS = 1, ORC_RC_MAXITERS = 2, ORC_RC_DTNAN = 3,
       ORC_RC_DTLESSTHANMIN = 4, ORC_RC_UNSTABLE = 5, ORC_RC_TERMINATED = 7 };

typedef struct {
    int64_t nf, njacs, nw, nsolve, naccept, nreject;
} orc_stats;

typedef struct {
    double reltol, abstol;
    double dtmax;      /* <= 0: tf - t0 (reference default) */
    double dtmin;      /* 0: reference default */
    double dt;         /* > 0: user initial dt (skips initdt) */
    int32_t adaptive;  /* 1 default */
    int64_t maxiters;  /* reference default 1e6 */
    int32_t save_start;     /* resolved by the caller: 0/1 */
    int32_t save_end;       /* resolved by the caller: 0/1 */
    int32_t save_end_user;  /* -1 not given, 0/1 given */
    int32_t saveat_given;   /* 0: no saveat (then the caller must request dense) */
    int32_t saveat_scalar;  /* saveat was a Number (affects the endpoint rule) */
    double qmax_first_step; /* <= 0: 10000 */
    double qmax;            /* <= 0: 10 */
    int32_t saveat_as_tstops; /* ensemble only: stop exactly at every save (ground-truth solves) */
    int32_t save_everystep;   /* save every accepted step (integrator_utils.jl:397-404) */
    int32_t max_step_saves;   /* ensemble: slots are max_step_saves + 2; past them the last slot
                                 keeps the latest step (the library's behaviour) */
    int32_t callback;         /* 1: the model's ContinuousCallback (ORC_BOUNCING_BALL) */
    int32_t interp_points;    /* ContinuousCallback interp_points (SciMLBase default 10) */
    int32_t max_events;       /* ensemble: 2 more save slots per event */
    int32_t ntstops;          /* ensemble: user tstops shared by every trajectory, */
    const double* tstops;     /* kept where t0 < ts < tf (initialize_tstops) */
    int32_t max_jac_age;      /* Rosenbrock23: J kept for at most this many accepted steps (1: never) */
    double jac_reuse_gamma_tol; /* ... while |dtgamma / dtgamma_J - 1| <= this (0.03) */
    int32_t ctrl_given;       /* 1: the PIController knobs below replace the defaults where not NaN */
    double c_beta1, c_beta2, c_qoldinit, c_qmin, c_gamma, c_qsteady_min, c_qsteady_max;
    int32_t force_dtmin;       /* accept steps at max(eps(t), dtmin); no dt exits (check_error.jl:91) */
    const double* abstol_vec;  /* per-state tolerances (n entries), or NULL for the scalars */
    const double* reltol_vec;
    int32_t isoutofdomain;     /* 1: reject adaptive steps ending with a negative state (any(x -> x < 0, u)) */
} orc_opts;

/* Solve one trajectory.  saveat: nsave_in times in (t0, tf] sorted ascending.
 * tstops: extra stop times (may be NULL).  Outputs at most cap saves:
 * t_out[cap], u_out[cap*n] (row-major per save).  Returns number saved.
 * dense_* (optional, may be NULL): every accepted step is recorded so that
 * orc_dense_eval can evaluate the method's interpolant afterwards. */
int orc_solve(int alg, int model, int n, const double* p, double t0, double tf,
              const double* u0, const orc_opts* o, const double* saveat, int nsave_in,
              const double* tstops, int ntstops, double* t_out, double* u_out, int cap,
              int32_t* retcode, orc_stats* st, void** dense_handle);

/* The initial step the solve would take (ode_determine_initdt with tdir, its
 * dtmax bounded by the first tstop), signed; counts its two f calls. */
double orc_initdt(int alg, int model, int n, const double* p, double t0, double tf, const double* u0,
                  const orc_opts* o, const double* tstops, int ntstops);

/* Evaluate the stored dense solution at nq times (out: nq*n), as the
 * reference's sol(t) does (ode_interpolation on the every-step saves). */
int orc_dense_eval(void* dense_handle, const double* tq, int nq, double* out);
/* The same with the derivative order (0 the value, 1 sol(t, Val{1})). */
int orc_dense_eval_deriv(void* dense_handle, const double* tq, int nq, int deriv, double* out);
int orc_dense_eval_ex(void* dense_handle, const double* tq, int nq, int deriv, int right, double* out);
/* Step s: t2 = (tprev, tend), y0, y1 (n each), k (returned count x n): the
 * interpolation vectors in the library's dense order. */
int orc_dense_step(void* dense_handle, int s, double* t2, double* y0, double* y1, double* k);
void orc_dense_free(void* dense_handle);
int orc_dense_nsteps(void* dense_handle);

/* Ensemble over N trajectories with nthreads host threads.  Inputs SoA:
 * u0[i*N + j], p[i*N + j], tspan[0*N + j]/tspan[1*N + j], saveat per
 * trajectory saveat[s*N + j] when saveat_per_traj else shared saveat[s];
 * n_per_traj (may be NULL) gives each trajectory's state count (<= nmax).
 * Outputs SoA: t_out[s*N + j], u_out[(s*nmax + i)*N + j], nsaved[j]. */
int orc_solve_ensemble(int alg, int model, int nmax, const int32_t* n_per_traj, int np,
                       int64_t N, const double* u0, const double* p, const double* tspan,
                       const orc_opts* o, const double* saveat, int nsave, int saveat_per_traj,
                       double* t_out, double* u_out, int32_t* nsaved, int32_t* retcode,
                       orc_stats* stats, int nthreads);

/* Method chosen for each saved point of the last orc_solve of this thread
 * (sol.alg_choice: 1 = Tsit5, 2 = Rosenbrock23 for AutoTsit5(Rosenbrock23())).
 * Returns the count written (at most cap). */
int orc_last_alg_choice(int32_t* out, int cap);

/* Number of RHS calls made by this thread's solves (the reference's counting
 * wrapper, test/InterfaceIII/stats_tests.jl:5-13); reset when asked. */
int64_t orc_rhs_calls(int reset);

/* Record the t of every RHS call this thread makes (enable 1; also clears the
 * record), and read it back: returns the number recorded, writes at most cap. */
int orc_record_eval_times(int enable);
int orc_eval_times(double* out, int cap);

/* Model right-hand side and Jacobian (for tests of the models themselves). */
void orc_rhs(int model, int n, const double* u, const double* p, double t, double* du);
void orc_jac(int model, int n, const double* u, const double* p, double t, double* J);
/* df/dt of a non-autonomous model (its tgrad); returns 0 for the autonomous ones */
int orc_tgrad(int model, int n, const double* u, const double* p, double t, double* dT);

#ifdef __cplusplus
}
#endif
#endif
