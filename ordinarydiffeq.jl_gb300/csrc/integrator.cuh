// The per-trajectory integrator loop, run by one lane group on the device.
//
// This is the device form of OrdinaryDiffEqCore's solve!/loopheader!/
// loopfooter! with the PI controller, tstop clipping, saveat interpolation,
// initial-step heuristic and retcode checks.  Reference (paths relative to the
// OrdinaryDiffEq.jl checkout):
//   solve!                     lib/OrdinaryDiffEqCore/src/solve.jl:904-946
//   loopheader!/apply_step!    lib/OrdinaryDiffEqCore/src/integrators/integrator_utils.jl:84-203
//   modify_dt_for_tstops!      integrator_utils.jl:268-324
//   _loopfooter!               integrator_utils.jl:597-677
//   _savevalues!               integrator_utils.jl:340-414
//   endpoint save              integrator_utils.jl:540-588
//   fix_dt_at_bounds!, calc_dt_propose!  integrator_utils.jl:1199-1256
//   PI controller              lib/OrdinaryDiffEqCore/src/integrators/controllers.jl:805-843
//   controller defaults        lib/OrdinaryDiffEqCore/src/alg_utils.jl:407-879
//   initdt                     lib/OrdinaryDiffEqCore/src/initdt.jl:17-298
//   residual + norm            lib/DiffEqBase/src/calculate_residuals.jl:9-14, common_defaults.jl:69-75
//   de_check_error             lib/DiffEqBase/src/check_error.jl:70-118
//
// Precision: t, dt, the error norm accumulator and the controller are always
// FP64; the state and stage arithmetic use R (double, or float in the mixed
// mode).  The only tstop is tf.
#pragma once
#include "common.cuh"
#include "ode_kernels.h"

namespace odegb {

enum RetCode { RC_DEFAULT = 0, RC_SUCCESS = 1, RC_MAXITERS = 2, RC_DTNAN = 3, RC_DTLESSTHANMIN = 4,
               RC_UNSTABLE = 5, RC_ABORTED = 6 };

struct StepStats {
    long long nf, njacs, nw, nsolve, naccept, nreject;
};

// Controller constants for one method (alg_utils.jl defaults).
struct Ctrl {
    double beta1, beta2, qmin_inv, qmax, qmax_first, gamma, qsteady_max, qoldinit;
};

template <int ORDER, bool IMPLICIT>
__device__ __forceinline__ Ctrl make_ctrl(const EnsembleArgs& a) {
    Ctrl c;
    c.beta2 = 2.0 / (5.0 * ORDER);
    c.beta1 = 7.0 / (10.0 * ORDER);
    c.qmin_inv = 1.0 / 0.2;
    c.qmax = a.qmax > 0 ? a.qmax : 10.0;
    c.qmax_first = a.qmax_first_step > 0 ? a.qmax_first_step : 10000.0;
    c.gamma = 0.9;
    c.qsteady_max = IMPLICIT ? 1.2 : 1.0;
    c.qoldinit = 1e-4;
    return c;
}

// Residual norm sqrt(sum_i (ut_i / (abstol + max(|u0_i|,|u1_i|) reltol))^2 / n)
// accumulated in FP64 (sequentially within a lane, then across the group).
template <class R, int L, int C>
__device__ __forceinline__ double error_norm(const R* ut, const R* u0, const R* u1, R abstol, R reltol,
                                             const Group<L>& g) {
    double acc = 0.0;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        R sc = FMA(tmax(ABS(u0[c]), ABS(u1[c])), reltol, abstol);
        double e = (double)(ut[c] / sc);
        acc = fma(e, e, acc);
    }
    acc = g.sum(acc);
    return sqrt(acc / (double)(L * C));
}

// Hairer's initial step (initdt.jl:17-298).  f0 is returned for FSAL methods.
template <class Model, class R, int L, int C, int ORDER>
__device__ double initdt(const R* u0, const R* p, double t, double dtmax, double dtmin_user, R abstol, R reltol,
                         R* f0, const Group<L>& g) {
    double dtmin = nextafter(jmax(dtmin_user, jeps(t)), __longlong_as_double(0x7ff0000000000000LL));
    double smalldt = jmax(dtmin, 1e-6);
    R sk[C], f1[C], u1[C];
#pragma unroll
    for (int c = 0; c < C; ++c) sk[c] = FMA(ABS(u0[c]), reltol, abstol);
    Model::template rhs<R, L, C>(f0, u0, p, t, g);
    double a0 = 0.0, a1 = 0.0;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        double x0 = (double)(u0[c] / sk[c]);
        a0 = fma(x0, x0, a0);
        double x1 = (double)(f0[c] / sk[c]);
        a1 = fma(x1, x1, a1);
    }
    double d0 = sqrt(g.sum(a0) / (double)(L * C));
    double d1 = sqrt(g.sum(a1) / (double)(L * C));
    if (d1 != d1) return dtmin;
    double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? smalldt : (d0 / d1) / 100.0;
    dt0 = jmin(dt0, dtmax);
    if (dt0 < 10.0 * 2.220446049250313e-16) return jmax(smalldt, dtmin);
    R dt0r = (R)dt0;
#pragma unroll
    for (int c = 0; c < C; ++c) u1[c] = FMA(dt0r, f0[c], u0[c]);
    Model::template rhs<R, L, C>(f1, u1, p, t + dt0, g);
    bool diff = false;
#pragma unroll
    for (int c = 0; c < C; ++c) diff = diff || (f0[c] != f1[c]);
    if (!g.any(diff)) return jmax(dtmin, 100.0 * dt0);
    double a2 = 0.0;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        double x = (double)((f1[c] - f0[c]) / sk[c]);
        a2 = fma(x, x, a2);
    }
    double d2 = sqrt(g.sum(a2) / (double)(L * C)) / dt0;
    double mx = jmax(d1, d2);
    double dt1;
    if (mx <= 1e-15) {
        dt1 = jmax(1e-6, dt0 * 1e-3);
    } else {
        const double LN10 = 2.302585092994046;
        dt1 = series_exp(-(2.0 * LN10 + series_ln(mx)) / (double)ORDER);
    }
    return jmax(dtmin, jmin(jmin(100.0 * dt0, dt1), dtmax));
}

// One trajectory, start to finish, on lane group g.  Alg provides the cache,
// the step, the interpolant and the FSAL hooks.
template <class Alg, class Model, class R, int L, int C>
__device__ void solve_trajectory(const EnsembleArgs& a, long long j, const Group<L>& g) {
    constexpr int NP = Model::NP;
    const long long N = a.N;
    R u[C], uprev[C];
    R p[NP];
#pragma unroll
    for (int c = 0; c < C; ++c) u[c] = (R)a.u0[(size_t)(g.lane * C + c) * N + j];
#pragma unroll
    for (int i = 0; i < NP; ++i) p[i] = (R)a.p[(size_t)i * N + j];
    const double t0 = a.tspan[j], tf = a.tspan[N + j];
    const double dtmax = a.dtmax > 0 ? a.dtmax : tf - t0;
    const R abstol = (R)a.abstol, reltol = (R)a.reltol;
    const Ctrl K = make_ctrl<Alg::ORDER, Alg::IMPLICIT>(a);

    typename Alg::template Cache<R, C> cache;
    StepStats st = {0, 0, 0, 0, 0, 0};
    int nsaved = 0;
    int isave = 0;
    double last_saved_t = __longlong_as_double(0x7ff8000000000000LL);

    auto save_point = [&](double ts, const R* v) {
        if (nsaved < a.nsave_cap) {
            if (g.lane == 0) a.t_out[(size_t)nsaved * N + j] = ts;
#pragma unroll
            for (int c = 0; c < C; ++c)
                a.u_out[((size_t)nsaved * a.nmax + g.lane * C + c) * N + j] = (double)v[c];
        }
        nsaved++;
        last_saved_t = ts;
    };
    auto saveat_at = [&](int s) -> double {
        return a.saveat_per_traj ? a.saveat[(size_t)s * N + j] : a.saveat[s];
    };

    // saveat entries outside (t0, tf] are skipped (initialize_saveat, solve.jl:1103-1124)
    while (isave < a.nsave && !(saveat_at(isave) > t0)) isave++;

#pragma unroll
    for (int c = 0; c < C; ++c) uprev[c] = u[c];
    if (a.save_start) save_point(t0, u);

    double t = t0, tprev = t0;
    Alg::template initialize<Model, R, L, C>(cache, u, p, t, g, st, a);
    double dt;
    if (a.dt > 0) {
        dt = a.dt;
    } else {
        dt = initdt<Model, R, L, C, Alg::ORDER>(u, p, t, dtmax, a.dtmin, abstol, reltol,
                                                 Alg::template fsal_slot<R, C>(cache), g);
        st.nf += 2;
    }
    double dtpropose = dt;
    double EEst = 1.0, q11 = 1.0, errold = K.qoldinit;
    long long iter = 0, success_iter = 0;
    bool accept = false, next_tstop = false;
    int rc = RC_DEFAULT;

    while (t < tf) {
        // ---- loopheader!
        if (iter > 0) {
            if (accept) {
                success_iter++;
#pragma unroll
                for (int c = 0; c < C; ++c) uprev[c] = u[c];
                dt = dtpropose;
                Alg::template on_accept<R, C>(cache);
                // modify_dt_for_tstops! (inside apply_step!)
                double dist = fabs(tf - t);
                double tol = 100.0 * jeps(jmax(fabs(t), fabs(tf)));
                double orig = fabs(dt);
                dtpropose = orig;
                next_tstop = !(orig + tol < dist);
                dt = jmin(orig, dist);
            } else {
                dt = dt / jmin(K.qmin_inv, q11 / K.gamma);
            }
        }
        iter++;
        // fix_dt_at_bounds!
        dt = jmin(dtmax, dt);
        dt = jmax(dt, fabs(jmax(jeps(t), a.dtmin)));
        {   // modify_dt_for_tstops!
            double dist = fabs(tf - t);
            double tol = 100.0 * jeps(jmax(fabs(t), fabs(tf)));
            double orig = fabs(dt);
            dtpropose = orig;
            next_tstop = !(orig + tol < dist);
            dt = jmin(orig, dist);
        }
        // ---- check_error (de_check_error)
        {
            int e = RC_SUCCESS;
            if (dt != dt) e = RC_DTNAN;
            else if (iter > a.maxiters) e = RC_MAXITERS;
            else if (fabs(dt) <= fabs(a.dtmin) && (!accept || t + dt < tf)) e = RC_DTLESSTHANMIN;
            else if (!accept && fabs(dt) <= fabs(jeps(t))) e = RC_UNSTABLE;
            else if (accept) {
                bool bad = false;
#pragma unroll
                for (int c = 0; c < C; ++c) bad = bad || !isfinite((double)u[c]);
                if (g.any(bad)) e = RC_UNSTABLE;
            }
            if (e == RC_SUCCESS && a.abort_flag != nullptr && (iter & 63) == 0 && *a.abort_flag != 0)
                e = RC_ABORTED;
            if (e != RC_SUCCESS) { rc = e; break; }
        }
        // ---- perform_step! (skipped for a step below eps(t) onto the tstop)
        if (!(next_tstop && fabs(dt) < jeps(fabs(t)))) {
            EEst = Alg::template step<Model, R, L, C>(cache, u, uprev, p, t, dt, abstol, reltol, iter, EEst, g, st);
        }
        // ---- loopfooter!
        double ttmp = t + dt;
        double qmaxc = success_iter == 0 ? K.qmax_first : K.qmax;
        double q;
        if (EEst == 0.0) {
            q = 1.0 / qmaxc;
        } else {
            double qq = ctrl_pow(EEst, K.beta1);
            q = qq / ctrl_pow(errold, K.beta2);
            q11 = qq;
            double x = q / K.gamma, lo = 1.0 / qmaxc, hi = K.qmin_inv;
            q = x > hi ? hi : (x < lo ? lo : x);
        }
        accept = EEst <= 1.0;
        if (accept) {
            st.naccept++;
            tprev = t;
            if (next_tstop) {
                dt = dtpropose;
                next_tstop = false;
                t = tf;
            } else {
                t = ttmp;
            }
            if (1.0 <= q && q <= K.qsteady_max) q = 1.0;
            errold = jmax(EEst, K.qoldinit);
            double dtnew = dt / q;
            double dtp = jmin(fabs(dtmax), fabs(dtnew));
            dtpropose = jmax(fabs(dtp), fabs(jmax(jeps(t), a.dtmin)));
            // ---- savevalues!
            while (isave < a.nsave) {
                double curt = saveat_at(isave);
                if (!(curt <= t)) break;
                isave++;
                if (curt != t) {
                    double th = (curt - tprev) / dt;
                    R out[C];
                    Alg::template interpolate<Model, R, L, C>(cache, out, th, dt, tprev, uprev, u, p, g);
                    save_point(curt, out);
                } else {
                    if (curt == tf && !a.save_end) continue;
                    save_point(t, u);
                }
            }
            Alg::template after_save<R, C>(cache);
        } else {
            st.nreject++;
        }
    }
    if (rc == RC_DEFAULT) rc = RC_SUCCESS;
    // ---- endpoint save (solution_endpoint_match_cur_integrator!)
    if (a.save_end) {
        bool need;
        if (nsaved == 0) {
            need = true;
        } else {
            bool in_saveat = false;
            if (a.saveat_given && !a.saveat_scalar)
                for (int s = 0; s < a.nsave; ++s) in_saveat = in_saveat || (saveat_at(s) == t);
            need = last_saved_t != t && (a.save_end_user == 1 || in_saveat || t == tf || !a.saveat_given);
        }
        if (need) save_point(t, u);
    }
    if (g.lane == 0) {
        a.nsaved[j] = nsaved < a.nsave_cap ? nsaved : a.nsave_cap;
        a.retcode[j] = rc;
        OdeStatsDev* s = a.stats + j;
        s->nf = st.nf; s->njacs = st.njacs; s->nw = st.nw; s->nsolve = st.nsolve;
        s->naccept = st.naccept; s->nreject = st.nreject;
    }
}

// Ensemble kernel: static (one trajectory per group, the plain one-kernel-per-
// ensemble form) or persistent (groups pop trajectory indices from a device
// counter until the ensemble is exhausted).
template <class Alg, class Model, class R, int L, int C>
__global__ void __launch_bounds__(128) ensemble_kernel(EnsembleArgs a) {
    Group<L> g;
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / L;
    if (!a.persistent) {
        if (gid >= a.count) return;
        long long j = a.order ? a.order[gid] : gid;
        solve_trajectory<Alg, Model, R, L, C>(a, j, g);
        return;
    }
    for (;;) {
        unsigned long long idx = 0;
        if (g.lane == 0) idx = atomicAdd(a.queue, 1ull);
        idx = g.bcast(idx, 0);
        if (idx >= (unsigned long long)a.count) break;
        long long j = a.order ? a.order[idx] : (long long)idx;
        solve_trajectory<Alg, Model, R, L, C>(a, j, g);
    }
}

}  // namespace odegb
