// Rosenbrock23 (Shampine's ode23s pair), with the linear algebra as a policy
// (RegLA: registers, n <= 8; SmemLA: shared memory, 16-64 states).
//
//  perform_step!(::Rosenbrock23Cache)  lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_perform_step.jl:34-146
//  initialize! (FSAL, k = [k1, k2])   rosenbrock_perform_step.jl:1-14
//  tableau                             rosenbrock_tableaus.jl:6-10 (c32 = 6 + sqrt(2), d = 1/(2 + sqrt(2)))
//  interpolant                         rosenbrock_interpolants.jl:39-74
//  J reuse (a W-method)                _rosenbrock_jac_reuse_decision
//                                      (OrdinaryDiffEqDifferentiation/src/derivative_utils.jl:46-170)
//                                      with calc_rosenbrock_differentiation! (:1011-1041): the
//                                      default max_jac_age = 1 (algorithms.jl:108-115) takes a fresh
//                                      J on every attempt, rejected or not; a larger one keeps J
//                                      (and dT) across accepted steps; W and its LU every attempt
//  controller                          alg_order 2 (alg_utils.jl:1), qsteady_max 6/5 (AdaptiveImplicit)
//
// With W = J - I/(dt d) (the form the Rodas5P kernels factor), a solve x = W \ b
// gives the stage k = -x/(dt d), the reference's `vecu * neginvdtγ`.
// Multiply-adds follow @muladd: a - b*c -> muladd(-b, c, a).
//
// Mixed precision (R = float): J, W, the LU, the solves and the stages are FP32;
// the right-hand side runs in double-float on the compensated state (rhs_stage),
// the solution is a compensated pair, and the interpolation weights are FP64
// split into float pairs.
#pragma once
#include "erk.cuh"
#include "rodas.cuh"

namespace odegb {

template <class LA>
struct Rosenbrock23T {
    static constexpr int ORDER = 2;
    static constexpr bool IMPLICIT = true;
    // parameters kept in double-float (mixed mode); only the model's NP are
    // touched, so the unused entries take no registers
    static constexpr int MAXP = 32;
    template <class R, int C> struct Cache {
        typename LA::template Store<R, C> la;
        R k[3][C];       // k1, k2 (the dense vectors), k3 (error estimate)
        R f1[C];         // f at the half step
        R fsal[C];       // f(uprev): FSAL from the last accepted step
        R fsallast[C];   // f(u)
        R scratch[C];
        R dT[C];         // df/dt at (uprev, t), non-autonomous models
        ff pff[MAXP];
        int ir;
        // Jacobian reuse (JacReuseState): dtgamma of the last fresh J once an accepted
        // step has passed, the one pending, and naccept at the last age reset
        int max_age;
        bool adaptive;
        double gamma_tol, last_dtg, pending_dtg;
        long long last_naccept, last_step_iter;
    };
    template <class R, int L, int C> __host__ __device__ static constexpr int smem_bytes() {
        return LA::template smem_bytes<R, L, C>();
    }
    template <class R, int C> __device__ static R* fsal_slot(Cache<R, C>& c) { return c.scratch; }

    // linear-algebra storage and the parameters in double-float, without f
    template <class Model, class R, int L, int C>
    __device__ static void prepare(Cache<R, C>& c, const Group<L>& g, const EnsembleArgs& a, long long j) {
        LA::template init<R, L, C>(c.la, g);
        c.ir = a.ir_sweeps;
        c.max_age = a.max_jac_age;
        c.adaptive = a.adaptive != 0;
        c.gamma_tol = a.jac_reuse_gamma_tol;
        c.last_dtg = c.pending_dtg = 0.0;
        c.last_naccept = c.last_step_iter = 0;
        if (sizeof(R) == 4) {
#pragma unroll
            for (int i = 0; i < Model::NP; ++i) c.pff[i] = ff(a.p[(size_t)i * a.N + j]);
            static_assert(Model::NP <= MAXP, "too many parameters for the double-float copy");
        }
    }
    template <class Model, class R, int L, int C>
    __device__ static void initialize(Cache<R, C>& c, const R* u, const PR<R>* p, double t, const Group<L>& g,
                                      StepStats& st, const EnsembleArgs& a, long long j) {
        prepare<Model, R, L, C>(c, g, a, j);
        R zero[C];
#pragma unroll
        for (int i = 0; i < C; ++i) zero[i] = R(0);
        // the start state is exact in the hi part (Acc::split of an FP64 u0 keeps
        // the remainder in lo); f(u0) from the pair, as every later f
        R ulo0[C];
#pragma unroll
        for (int i = 0; i < C; ++i) {
            R hi;
            Acc<R>::split(a.u0[(size_t)(g.lane * C + i) * a.N + j], hi, ulo0[i]);
        }
        rhs_stage<Model, R, L, C, Model::NP>(c.fsal, u, sizeof(R) == 4 ? ulo0 : zero, p, c.pff, t, g);
        st.nf += 1;
    }
    template <class R, int C> __device__ static void on_accept(Cache<R, C>& c) {
#pragma unroll
        for (int i = 0; i < C; ++i) c.fsal[i] = c.fsallast[i];
    }
    template <class R, int C> __device__ static void after_save(Cache<R, C>&) {}

    // Dense output: integrator.k = [k1, k2].
    static constexpr int NDENSE = 2;
    template <class R, int C> __device__ static void prepare_dense(Cache<R, C>&) {}
    template <class R, int C> __device__ static R* dense_slot(Cache<R, C>& c, int q) { return c.k[q]; }

    // A callback moved or modified u: f(u) again (reset_fsal!, one counted call);
    // fsallast becomes the next step's FSAL value when it starts.
    template <class Model, class R, int L, int C>
    __device__ static void reset_fsal(Cache<R, C>& c, const R* u, const R* ulo, const PR<R>* p, double t,
                                      const Group<L>& g, StepStats& st) {
        rhs_stage<Model, R, L, C, Model::NP>(c.fsallast, u, ulo, p, c.pff, t, g);
        st.nf += 1;
    }

    // _rosenbrock_jac_reuse_decision for this W-method (no mass matrix, adaptive, not
    // inside a composite): a fresh J on the first attempt, after a rejected one, when
    // no J has been committed yet, when an attempt was skipped since the last (a
    // step below eps(t) onto a tstop), when dtgamma moved more than gamma_tol from
    // the J's, and every max_age accepted steps (the age reset); else the J (and dT)
    // kept.  iter < 0: an event's recomputation of the shortened step, which keeps
    // the step's J (the in-place addsteps reuses it) and touches no reuse state.
    template <class R, int C>
    __device__ static bool fresh_jacobian(Cache<R, C>& c, double dt, long long iter, bool errorfail,
                                          long long naccept) {
        if (iter < 0) return false;
        if (c.max_age <= 1) return true;   // the age check fires on every attempt
        if (!c.adaptive) return true;      // non-adaptive solves always recompute
        const double dtg = dt * tab::ROS23_D;
        bool fresh = true;
        if (iter > 1) {
            if (naccept > c.last_naccept) c.last_dtg = c.pending_dtg;
            const bool skipped = c.last_step_iter != 0 && iter > c.last_step_iter + 1;
            if (c.last_dtg != 0.0 && !skipped && !errorfail && !(fabs(dtg / c.last_dtg - 1.0) > c.gamma_tol)) {
                if (naccept - c.last_naccept >= c.max_age) c.last_naccept = naccept;
                else fresh = false;
            }
        }
        c.last_step_iter = iter;
        if (fresh) c.pending_dtg = dtg;
        return fresh;
    }

    template <class Model, class R, int L, int C>
    __device__ static typename Ctl<R>::T step(Cache<R, C>& c, R* u, R* ulo, const R* up, const R* uplo,
                                             const PR<R>* p, double t, double dt, const Tol<R>& tol, long long iter,
                                             bool errorfail, const Group<L>& g, StepStats& st) {
        constexpr int NP = Model::NP;
        R dr, idg, ninv, dto2, dto6, c32;
        if constexpr (sizeof(R) == 8) {
            const double dtgamma = dt * tab::ROS23_D;
            idg = 1.0 / dtgamma;
            ninv = -idg;
            dr = dt;
            dto2 = dt / 2.0;
            dto6 = dt / 6.0;
            c32 = tab::ROS23_C32;
        } else {   // dt-derived factors in FP32 (they scale FP32 stage terms)
            dr = (R)dt;
            idg = R(1) / (dr * tab::ROS23_D_HI);
            ninv = -idg;
            dto2 = dr * R(0.5);
            dto6 = dr / R(6);
            c32 = tab::ROS23_C32_HI;
        }
        static_assert(Model::AUTONOMOUS || has_tgrad<Model>::value, "a non-autonomous model needs its tgrad");
        static_assert(Model::AUTONOMOUS || L == 1, "time derivatives are formed on one lane");
        const bool new_jac = fresh_jacobian(c, dt, iter, errorfail, st.naccept);
        LA::template jacobian<Model, R, L, C>(c.la, up, p, t, new_jac, g);
        if (new_jac) {
            st.njacs += 1;
            st.nf += jac_f_calls<Model>::value;
            // the time derivative (calc_tderivative!, derivative_utils.jl:181-227), with a
            // fresh J only: the model's analytic tgrad (not an f call); else dT = 0 for an
            // autonomous model, whose AD evaluation in the reference counts as one f call
            if constexpr (has_tgrad<Model>::value) Model::template tgrad<R, C>(c.dT, up, p, t);
            else st.nf += 1;
        }
        LA::template factor<R, L, C>(c.la, idg, g);
        st.nw += 1;
        R* k1 = c.k[0];
        R* k2 = c.k[1];
        R* k3 = c.k[2];
        R r[C];
#pragma unroll
        for (int i = 0; i < C; ++i) r[i] = c.fsal[i];   // fsalfirst + dtd1 dT (dT = 0: autonomous)
        if constexpr (!Model::AUTONOMOUS) {
            const R dtg = (R)(dt * tab::ROS23_D);
#pragma unroll
            for (int i = 0; i < C; ++i) r[i] = c.fsal[i] + dtg * c.dT[i];
        }
        LA::template wsolve<Model, R, L, C>(c.la, r, dt, idg, c.ir, up, uplo, c.pff, g);
#pragma unroll
        for (int i = 0; i < C; ++i) k1[i] = r[i] * ninv;
        st.nsolve += 1;
        R stlo[C];
#pragma unroll
        for (int i = 0; i < C; ++i) Acc<R>::update(u[i], stlo[i], dto2, k1[i], up[i], uplo[i]);
        rhs_stage<Model, R, L, C, NP>(c.f1, u, stlo, p, c.pff, stage_time<Model>(0.5, dt, t), g);
        st.nf += 1;
#pragma unroll
        for (int i = 0; i < C; ++i) r[i] = c.f1[i] - k1[i];
        LA::template wsolve<Model, R, L, C>(c.la, r, dt, idg, c.ir, up, uplo, c.pff, g);
#pragma unroll
        for (int i = 0; i < C; ++i) k2[i] = FMA(r[i], ninv, k1[i]);
        st.nsolve += 1;
        const R dl = Acc<R>::dt_lo(dt, dr);
#pragma unroll
        for (int i = 0; i < C; ++i) Acc<R>::update2(u[i], ulo[i], dr, dl, k2[i], up[i], uplo[i]);
        rhs_stage<Model, R, L, C, NP>(c.fsallast, u, ulo, p, c.pff, stage_time<Model>(1.0, dt, t), g);
        st.nf += 1;
        if (!c.adaptive) return R(0);   // fixed steps: no k3, no error estimate
#pragma unroll
        for (int i = 0; i < C; ++i) {
            R acc = FMA(-c32, k2[i] - c.f1[i], c.fsallast[i]);
            r[i] = FMA(R(-2), k1[i] - c.fsal[i], acc);
            if constexpr (!Model::AUTONOMOUS) r[i] = FMA(dr, c.dT[i], r[i]);   // + dt dT
        }
        LA::template wsolve<Model, R, L, C>(c.la, r, dt, idg, c.ir, up, uplo, c.pff, g);
#pragma unroll
        for (int i = 0; i < C; ++i) k3[i] = r[i] * ninv;
        st.nsolve += 1;
        R tmp[C];
#pragma unroll
        for (int i = 0; i < C; ++i) tmp[i] = dto6 * (FMA(R(-2), k2[i], k1[i]) + k3[i]);
        return error_norm<R, L, C>(tmp, up, u, tol, g);
    }

    // y0 + dt (c1 k1 + c2 k2), c1 = th (1 - th) / (1 - 2d), c2 = th (th - 2d) / (1 - 2d)
    template <class Model, class R, int L, int C>
    __device__ static void interpolate(Cache<R, C>& c, R* out, R* outlo, double th, double dt, double,
                                       const R* y0, const R* y0lo, const R*, const R*, const PR<R>*,
                                       const Group<L>&) {
        const double thd = th;
        const double d = tab::ROS23_D;
        const double c1 = thd * (1.0 - thd) / (1.0 - 2.0 * d);
        const double c2 = thd * (thd - 2.0 * d) / (1.0 - 2.0 * d);
        if constexpr (sizeof(R) == 8) {
#pragma unroll
            for (int i = 0; i < C; ++i)
                Acc<R>::update(out[i], outlo[i], dt, fma(c1, c.k[0][i], c2 * c.k[1][i]), y0[i], y0lo[i]);
        } else {
            const ff w1 = split_weight(c1), w2 = split_weight(c2);
            const R dh = (R)dt, dl = Acc<R>::dt_lo(dt, dh);
#pragma unroll
            for (int i = 0; i < C; ++i) {
                CSum cs;
                cs.add_pair(w1.hi, w1.lo, (float)c.k[0][i]);
                cs.add_pair(w2.hi, w2.lo, (float)c.k[1][i]);
                Acc<R>::update2(out[i], outlo[i], dh, dl, (R)cs.value(), y0[i], y0lo[i]);
            }
        }
    }
};

using Rosenbrock23Alg = Rosenbrock23T<RegLA>;
using Rosenbrock23GroupAlg = Rosenbrock23T<SmemLA>;

}  // namespace odegb
