// AutoTsit5(Rosenbrock23()): a CompositeAlgorithm of a non-stiff and a stiff
// method with the AutoSwitch choice function.
//
//  AutoTsit5(stiff_alg) = AutoAlgSwitch(Tsit5(), stiff_alg)   lib/OrdinaryDiffEqTsit5/src/algorithms.jl:27-33
//  AutoSwitch defaults, is_stiff, the choice function         lib/OrdinaryDiffEqCore/src/composite_algs.jl:1-94
//    maxstiffstep 10, maxnonstiffstep 3, nonstifftol = stifftol = 9//10, dtfac 2,
//    stiffalgfirst false, switch_max 5
//  choose_algorithm! at each loop header                     integrators/integrator_utils.jl:120-121,
//    (initialize! of the method switched to)                 perform_step/composite_perform_step.jl:181-221
//  stiffness estimate                                         Tsit5Alg::step<..., EIG = true>
//  alg_stability_size(::Tsit5) = 3.5068                       lib/OrdinaryDiffEqTsit5/src/alg_utils.jl:3
//  one PI controller per method                               CompositeController, controllers.jl:1263-1345
//    (the integrator loop banks the state of the method left and resumes the other's)
//
// Both methods' caches live in registers (one lane per trajectory); the step,
// the interpolant and the FSAL hooks dispatch on the current method.
#pragma once
#include "erk.cuh"
#include "ros23.cuh"

namespace odegb {

template <class NS, class S>
struct AutoSwitchAlg {
    using NonStiff = NS;
    using Stiff = S;
    static constexpr bool COMPOSITE = true;
    static constexpr int ORDER = NS::ORDER;   // the start method's (initdt)
    static constexpr bool IMPLICIT = false;
    static constexpr int NDENSE = 0;          // no dense output for the composite
    template <class R, int C> struct Cache {
        typename NS::template Cache<R, C> ns;
        typename S::template Cache<R, C> s;
        int current;          // 0 the non-stiff method, 1 the stiff one
        int count;            // successive stiffness verdicts: > 0 stiff, < 0 not
        int successive;       // successive non-stiff verdicts (successive_switches)
        bool is_stiffalg;
        double eigen_est;     // from the non-stiff method's steps; solve.jl:697 starts it at 1
    };
    template <class R, int C> __device__ static R* fsal_slot(Cache<R, C>& c) { return NS::fsal_slot(c.ns); }

    template <class Model, class R, int L, int C>
    __device__ static void initialize(Cache<R, C>& c, const R* u, const PR<R>* p, double t, const Group<L>& g,
                                      StepStats& st, const EnsembleArgs& a, long long j) {
        c.current = 0;   // stiffalgfirst = false
        c.count = 0;
        c.successive = 0;
        c.is_stiffalg = false;
        c.eigen_est = 1.0;
        NS::template initialize<Model, R, L, C>(c.ns, u, p, t, g, st, a, j);   // the current method's FSAL
        S::template prepare<Model, R, L, C>(c.s, g, a, j);
        c.s.max_age = 1;   // a CompositeAlgorithm always takes a fresh J (derivative_utils.jl:104-108)
    }
    template <class R, int C> __device__ static void on_accept(Cache<R, C>& c) {
        if (c.current == 0) NS::on_accept(c.ns);
        else S::on_accept(c.s);
    }
    template <class R, int C> __device__ static void after_save(Cache<R, C>& c) {
        if (c.current == 0) NS::after_save(c.ns);
        else S::after_save(c.s);
    }
    template <class R, int C> __device__ static void prepare_dense(Cache<R, C>&) {}
    template <class R, int C> __device__ static R* dense_slot(Cache<R, C>& c, int q) { return NS::dense_slot(c.ns, q); }

    // The choice function (composite_algs.jl:55-94) with is_stiff (:17-45).  May
    // scale dt by dtfac on a switch.  Returns true when the method changed; sets
    // do_error_check as is_stiff does.
    __device__ static bool choose(int& current, int& count, int& successive, bool& is_stiffalg, double eigen_est,
                                  double& dt, bool& do_error_check) {
        // |eigen_est dt / 3.5068| <= 9//10 (exact comparison with the rational: < 0.9 in double)
        const double stiffness = fabs(eigen_est * dt / 3.5068);
        const bool stiff = !(stiffness < 0.9);
        successive = stiff ? 0 : successive + 1;
        do_error_check = (successive > 5 || !stiff) || is_stiffalg;
        count = stiff ? (count < 0 ? 1 : count + 1) : (count > 0 ? -1 : count - 1);
        if (!is_stiffalg && count > 10) {
            dt = dt * 2.0;
            is_stiffalg = true;
        } else if (is_stiffalg && count < -3) {
            dt = dt / 2.0;
            is_stiffalg = false;
        }
        const int next = is_stiffalg ? 1 : 0;
        const bool switched = next != current;
        current = next;
        return switched;
    }
    template <class R, int C>
    __device__ static bool choose(Cache<R, C>& c, double& dt, bool& do_error_check) {
        return choose(c.current, c.count, c.successive, c.is_stiffalg, c.eigen_est, dt, do_error_check);
    }

    // initialize! of the method switched to: its FSAL value f(uprev, t) (one counted call)
    template <class Model, class R, int L, int C>
    __device__ static void enter(Cache<R, C>& c, const R* up, const R* uplo, const PR<R>* p, double t, const Group<L>& g,
                                 StepStats& st) {
        if (c.current == 0) {
            Model::template rhs<R, L, C>(c.ns.k[0], up, p, t, g);
        } else {
            rhs_stage<Model, R, L, C, Model::NP>(c.s.fsal, up, uplo, p, c.s.pff, t, g);
        }
        st.nf += 1;
    }

    template <class Model, class R, int L, int C>
    __device__ static typename Ctl<R>::T step(Cache<R, C>& c, R* u, R* ulo, const R* up, const R* uplo,
                                             const PR<R>* p, double t, double dt, const Tol<R>& tol, long long iter,
                                             bool errorfail, const Group<L>& g, StepStats& st) {
        if (c.current == 0) {
            const typename Ctl<R>::T e = NS::template step<Model, R, L, C, true>(c.ns, u, ulo, up, uplo, p, t, dt,
                                                                                tol, iter, errorfail, g, st);
            c.eigen_est = c.ns.eig;
            return e;
        }
        return S::template step<Model, R, L, C>(c.s, u, ulo, up, uplo, p, t, dt, tol, iter, errorfail, g,
                                                st);
    }

    template <class Model, class R, int L, int C>
    __device__ static void interpolate(Cache<R, C>& c, R* out, R* outlo, double th, double dt, double tprev,
                                       const R* y0, const R* y0lo, const R* y1, const R* y1lo, const PR<R>* p,
                                       const Group<L>& g) {
        if (c.current == 0)
            NS::template interpolate<Model, R, L, C>(c.ns, out, outlo, th, dt, tprev, y0, y0lo, y1, y1lo, p, g);
        else
            S::template interpolate<Model, R, L, C>(c.s, out, outlo, th, dt, tprev, y0, y0lo, y1, y1lo, p, g);
    }

    template <class Model, class R, int L, int C>
    __device__ static void reset_fsal(Cache<R, C>& c, const R* u, const R* ulo, const PR<R>* p, double t,
                                      const Group<L>& g, StepStats& st) {
        if (c.current == 0) NS::template reset_fsal<Model, R, L, C>(c.ns, u, ulo, p, t, g, st);
        else S::template reset_fsal<Model, R, L, C>(c.s, u, ulo, p, t, g, st);
    }
};

using AutoTsit5Rosenbrock23Alg = AutoSwitchAlg<Tsit5Alg, Rosenbrock23Alg>;

}  // namespace odegb
