// The parameter block of one ensemble launch, shared by the kernels, the host
// runtime and the runtime-compiled kernels of registered models (plain types
// only, so the header also compiles under NVRTC, which has no standard headers).
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

namespace odegb {

struct OdeStatsDev {
    long long nf, njacs, nw, nsolve, naccept, nreject;
};

// PI-controller values of EnsembleArgs::kd / kf: beta1, beta2, 1/qmin, gamma,
// qsteady_min, qsteady_max, qoldinit, 1/qmax, 1/qmax_first_step, qmin.
enum { KB1 = 0, KB2, KQMININV, KGAM, KQSMIN, KQSMAX, KQOLD, KIQMAX, KIQMAXF, KQMIN, KNCTRL };

// Everything one ensemble launch needs.  Device pointers; SoA layouts:
//   u0[i*N + j], p[i*N + j], tspan[j] / tspan[N + j],
//   saveat[s] (shared) or saveat[s*N + j] (per trajectory),
//   t_out[s*N + j], u_out[(s*nmax + i)*N + j].
struct EnsembleArgs {
    long long N;            // trajectories in the arrays
    long long count;        // trajectories this launch integrates (entries of order, or N)
    const long long* order; // optional trajectory indices (size-class buckets); nullptr = identity
    int nmax;               // state stride
    const double* u0;
    const double* p;
    const double* tspan;
    const double* saveat;
    int nsave;
    int saveat_per_traj;
    int nsave_cap;          // save slots per trajectory in t_out/u_out
    double* t_out;
    double* u_out;          // u_out[(s*nmax + i)*N + j], or [(s*nsave_rows + r)*N + j] with save_idxs
    const int32_t* save_idxs;  // the states saved, one row each (nullptr: every state)
    int nsave_rows;
    int32_t* nsaved;
    int32_t* retcode;
    OdeStatsDev* stats;
    // options
    double reltol, abstol, dtmax, dtmin, dt;
    const double* reltol_traj;   // per-trajectory tolerances (nullptr: reltol/abstol for all)
    const double* abstol_traj;
    long long maxiters;
    int save_start, save_end, save_end_user, saveat_given, saveat_scalar;
    int save_everystep;     // save every accepted step (saveat empty); nsave_cap bounds the slots
    int callback;           // 1: the model's ContinuousCallback (models with HAS_EVENT)
    int interp_points;      // its interp_points
    const double* tstops;   // the solve's tstops, ascending, shared by every trajectory
    int ntstops;
    double* k_out;          // dense output (nullptr: none): k_out[((s*NDENSE + q)*nmax + i)*N + j], the
                            // method's NDENSE interpolation vectors of the step ending at save s
    double qmax_first_step, qmax;
    int ir_sweeps;          // mixed Rosenbrock: refinement sweeps per solve
    int adaptive;           // 0: fixed steps of dt, every step accepted
    int forward_only;       // the kernel's plain form may run: every span runs forward, and neither
                            // force_dtmin nor isoutofdomain is asked for
    int force_dtmin;        // accept steps at max(eps(t), dtmin) whatever their error
    int isoutofdomain;      // 1: reject adaptive steps ending with a negative state
    // The PI controller of each method (slot 1: a composite's stiff method), its
    // defaults and the caller's knobs resolved on the host, in both precisions
    // (kernel parameters: read where used, held in no register)
    double kd[2][KNCTRL];
    float kf[2][KNCTRL];
    const double* abstol_vec;   // per-state tolerances (device, n entries), or null
    const double* reltol_vec;
    int max_jac_age;        // Rosenbrock23: J kept for at most this many accepted steps (<= 1: never kept)
    double jac_reuse_gamma_tol;  // ... while |dtgamma / dtgamma_J - 1| <= this
    // scheduling
    int persistent;
    int refill_lanes;       // idle lanes of a warp that take new trajectories together (32: the whole warp)
    unsigned long long* queue;     // persistent work counter (zeroed before launch)
    const volatile int* abort_flag;  // host-settable early stop (nullptr: none)
    // size classes of an uneven ensemble (one launch over all classes):
    // class k holds class_count[k] trajectories at order[class_offset[k] ...]
    const unsigned long long* class_count;
    const unsigned long long* class_offset;
    unsigned long long* class_next;  // per-class work counters (zeroed before launch)
};

}  // namespace odegb
