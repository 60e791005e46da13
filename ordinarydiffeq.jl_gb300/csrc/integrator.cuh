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
// Precision policy.  t and dt are FP64 in both modes, and so is the error-
// norm accumulator.  FP64 mode (R = double) evaluates the controller in FP64
// like the reference.  Mixed mode (R = float) computes the controller's
// powers and factors in FP32 and applies them to the FP64 dt with one
// multiply: on GB300 an FP64 instruction occupies the FP64 pipe ~64x longer
// than an FP32 one, so the per-step FP64 work is kept to t/dt updates and the
// error accumulation.  min/max/eps of the (non-negative) time quantities run
// on the integer pipe in both modes; they return exactly what Julia's
// min/max/eps return, NaN propagation included.
#pragma once
#include "common.cuh"
#include "ensemble_args.h"

namespace odegb {

enum RetCode { RC_DEFAULT = 0, RC_SUCCESS = 1, RC_MAXITERS = 2, RC_DTNAN = 3, RC_DTLESSTHANMIN = 4,
               RC_UNSTABLE = 5, RC_ABORTED = 6, RC_TERMINATED = 7,
               RC_INITIALFAILURE = 8 };

// Composite methods (AutoSwitchAlg) declare COMPOSITE; the loop then runs their
// choice function and keeps one controller state per method.
template <class A, class = void> struct is_composite_alg : bool_constant<false> {};
template <class A> struct is_composite_alg<A, void_t<decltype(A::COMPOSITE)>> : bool_constant<true> {};
// models with a registered DiscreteCallback declare HAS_DISCRETE
template <class M, class = void> struct has_discrete_callback : bool_constant<false> {};
template <class M>
struct has_discrete_callback<M, void_t<decltype(M::HAS_DISCRETE)>> : bool_constant<M::HAS_DISCRETE> {};

// Continuous callbacks: a model with HAS_EVENT declares one ContinuousCallback
// (EVENT_LEN = 1, the default) or one VectorContinuousCallback of EVENT_LEN
// conditions.  A model's DiscreteCallback fires at the solve's tstops unless
// the model declares DISCRETE_AT_TSTOPS = false and its own condition.
template <class M, class = void> struct event_len { static constexpr int value = 1; };
template <class M> struct event_len<M, void_t<decltype(M::EVENT_LEN)>> { static constexpr int value = M::EVENT_LEN; };
template <class M, class = void> struct discrete_at_tstops : bool_constant<true> {};
template <class M>
struct discrete_at_tstops<M, void_t<decltype(M::DISCRETE_AT_TSTOPS)>> : bool_constant<M::DISCRETE_AT_TSTOPS> {};

// models with an analytic time derivative (ODEFunction's tgrad) declare HAS_TGRAD
template <class M, class = void> struct has_tgrad : bool_constant<false> {};
template <class M>
struct has_tgrad<M, void_t<decltype(M::HAS_TGRAD)>> : bool_constant<M::HAS_TGRAD> {};

// f calls a Jacobian evaluation is counted as (JAC_F_CALLS: 1 for a Jacobian
// by forward-mode AD of f, as the reference counts its ForwardDiff chunk; 0 for
// an analytic one)
template <class M, class = void> struct jac_f_calls { static constexpr int value = 0; };
template <class M> struct jac_f_calls<M, void_t<decltype(M::JAC_F_CALLS)>> {
    static constexpr int value = M::JAC_F_CALLS;
};

// The left end of a sign change of f in [lo, hi] narrowed to adjacent floats
// (LeftRootFind: the reference solves IntervalNonlinearProblem with ModAB,
// BracketingNonlinearSolve, at abstol = reltol = 0 and returns the left
// bracket; any bracketing method run to adjacent floats ends at the same pair
// where the sign change is unique).  Anderson-Bjorck false position: the
// secant point of the bracket; when the same end is replaced twice in a row
// the retained end's value is scaled by 1 - f_new/f_replaced (by 1/2 when that
// is not positive); a bisection whenever the bracket has not halved over two
// steps, or when the secant point is not strictly inside the bracket.  flo and fhi are
// f(lo) and f(hi), of opposite signs and nonzero.  The oracle runs the same
// iteration.
template <class F>
__device__ __forceinline__ double bracket_left_root(F&& f, double lo, double hi, double flo, double fhi) {
    int side = 0;
    double w_prev = hi - lo, w_prev2 = 2.0 * (hi - lo);
    for (int it = 0; it < 2200; ++it) {
        const double w = hi - lo;
        double m = (w > 0.5 * w_prev2) ? lo + w * 0.5 : lo + w * (flo / (flo - fhi));
        if (!(m > lo && m < hi)) m = lo + w * 0.5;
        if (!(m > lo && m < hi)) break;   // adjacent floats
        const double fm = f(m);
        if (fm == 0.0) return m;
        w_prev2 = w_prev;
        w_prev = w;
        if ((fm > 0.0) == (flo > 0.0)) {
            if (side == -1) {
                const double g = 1.0 - fm / flo;
                fhi *= g > 0.0 ? g : 0.5;
            }
            lo = m;
            flo = fm;
            side = -1;
        } else {
            if (side == +1) {
                const double g = 1.0 - fm / fhi;
                flo *= g > 0.0 ? g : 0.5;
            }
            hi = m;
            fhi = fm;
            side = +1;
        }
    }
    return lo;
}

// sign() with Julia's NaN behaviour
__device__ __forceinline__ double dsign(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : (x == 0.0 ? 0.0 : x)); }
// ContinuousCallback defaults (SciMLBase): abstol = 10eps(), repeat_nudge = 1//100
constexpr double kCbAbstol = 10.0 * 2.220446049250313e-16;
constexpr double kCbRepeatNudge = 0.01;

struct StepStats {
    long long nf, njacs, nw, nsolve, naccept, nreject;
};

// ---------------------------------------------------------------- time helpers (integer pipe)
__device__ __forceinline__ bool bits_nan(long long b) { return abs_bits_i(b) > 0x7ff0000000000000LL; }
__device__ __forceinline__ double dnan() { return __longlong_as_double(0x7ff8000000000000LL); }
// Julia min/max for non-negative doubles (NaN propagates).
__device__ __forceinline__ double pmin(double a, double b) {
    long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    if (bits_nan(x) || bits_nan(y)) return dnan();
    return x < y ? a : b;
}
__device__ __forceinline__ double pmax(double a, double b) {
    long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    if (bits_nan(x) || bits_nan(y)) return dnan();
    return x > y ? a : b;
}
__device__ __forceinline__ double pabs(double a) {
    return __longlong_as_double(abs_bits(a));
}
// Julia eps(x): the spacing of doubles at |x|, built from the exponent bits.
__device__ __forceinline__ double peps(double x) {
    long long b = abs_bits(x);
    if (b >= 0x7ff0000000000000LL) return dnan();
    int e = (int)(b >> 52);
    if (e > 52) return __longlong_as_double((long long)(e - 52) << 52);
    return __longlong_as_double(1LL << (e > 0 ? e - 1 : 0));
}
// a <= b and a < b for non-negative doubles (false when either is NaN, as in IEEE).
__device__ __forceinline__ bool ple(double a, double b) {
    long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return !bits_nan(x) && !bits_nan(y) && x <= y;
}
__device__ __forceinline__ bool plt(double a, double b) {
    long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return !bits_nan(x) && !bits_nan(y) && x < y;
}
// Order-preserving integer key of a double of either sign (-0 and +0 equal).
__device__ __forceinline__ long long okey(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : -abs_bits_i(b);
}
// a <= b and a == b for doubles of either sign, false when either is NaN (IEEE).
__device__ __forceinline__ bool dle(double a, double b) {
    return !bits_nan(__double_as_longlong(a)) && !bits_nan(__double_as_longlong(b)) && okey(a) <= okey(b);
}
__device__ __forceinline__ bool deq(double a, double b) {
    return !bits_nan(__double_as_longlong(a)) && !bits_nan(__double_as_longlong(b)) && okey(a) == okey(b);
}
// 100 * eps(x), exactly: eps is a power of two 2^k and 100 * 2^k = 1.5625 * 2^(k+6).
__device__ __forceinline__ double ptol100(double x) {
    const double e = peps(x);
    const int ex = (int)(__double_as_longlong(e) >> 52);
    if (ex >= 1 && ex + 6 < 2047) return __longlong_as_double(((long long)(ex + 6) << 52) | 0x9000000000000LL);
    return 100.0 * e;
}

// Time argument of a stage's right-hand side, t + c dt (the reference's
// muladd(c, dt, t)).  For an autonomous model (f does not read t) the sum is not
// formed: it would be one FP64 instruction per stage for a value nobody reads.
template <class Model>
__device__ __forceinline__ double stage_time(double c, double dt, double t) {
    if constexpr (Model::AUTONOMOUS) return t;
    else return fma(c, dt, t);
}

// ---------------------------------------------------------------- controller policy
template <class R> struct Ctl;
template <> struct Ctl<double> {   // FP64: the reference's arithmetic
    using T = double;
    static __device__ __forceinline__ double pw(double x, double y) { return ctrl_pow(x, y); }
    static __device__ __forceinline__ double scale_dt(double dt, double q) { return dt / q; }
    // interpolation abscissa theta = (t_save - tprev) / dt
    static __device__ __forceinline__ double theta(double num, double dt) { return num / dt; }
};
template <> struct Ctl<float> {    // mixed: FP32 factors, FP64 dt
    using T = float;
    static __device__ __forceinline__ float pw(float x, float y) { return exp2f(y * log2f(x)); }
    static __device__ __forceinline__ double scale_dt(double dt, float q) { return dt * (double)(1.0f / q); }
    // theta in FP32: a relative error of 6e-8 in theta moves a save by 6e-8 of
    // one step's change, far below the tolerance
    static __device__ __forceinline__ float theta(double num, double dt) { return (float)num / (float)dt; }
};

// A PI-controller value of method slot s (ensemble_args.h: KB1 ... KIQMAXF), in
// the controller's precision.
template <class CT> __device__ __forceinline__ CT kval(const EnsembleArgs& a, int s, int k) {
    if constexpr (sizeof(CT) == 8) return a.kd[s][k];
    else return a.kf[s][k];
}

// A step's tolerances: the trajectory's scalars, or per state when the solve
// gives vectors (abstol[i], reltol[i] of state i = lane*C + c, read from the
// launch's device arrays where used, so no register holds them).
template <class R> struct Tol {
    R abstol, reltol;
    const double* av;   // per-state abstol, or null
    const double* rv;   // per-state reltol, or null
    template <int C> __device__ __forceinline__ R a(int lane, int c) const {
        return av ? (R)av[lane * C + c] : abstol;
    }
    template <int C> __device__ __forceinline__ R r(int lane, int c) const {
        return rv ? (R)rv[lane * C + c] : reltol;
    }
};

// Residual norm sqrt(sum_i (ut_i / (abstol_i + max(|u0_i|,|u1_i|) reltol_i))^2 / n).
// FP64 mode: the sum in FP64 (sequentially within a lane, then across the
// group).  Mixed mode: the same sum carried in double-float (an exact square
// by fma, a two-sum per term; FP64-class precision on the FP32 pipe), since
// on GB300 each FP64 add/fma or float<->double conversion per component would
// cost the FP64 pipe more time than the whole FP32 stage work of a small system.
template <class R, int L, int C>
__device__ __forceinline__ typename Ctl<R>::T error_norm(const R* ut, const R* u0, const R* u1, const Tol<R>& tol,
                                                         const Group<L>& g) {
    if (sizeof(R) == 8) {
        double acc = 0.0;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            R sc = FMA(tmax(ABS(u0[c]), ABS(u1[c])), tol.template r<C>(g.lane, c), tol.template a<C>(g.lane, c));
            double e = (double)(ut[c] / sc);
            acc = fma(e, e, acc);
        }
        acc = g.sum(acc);
        return (typename Ctl<R>::T)sqrt(acc / (double)(L * C));
    }
    float hi = 0.0f, lo = 0.0f;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const float sc = fmaf(tmax(fabsf((float)u0[c]), fabsf((float)u1[c])), (float)tol.template r<C>(g.lane, c),
                              (float)tol.template a<C>(g.lane, c));
        const float e = (float)ut[c] / sc;
        const float p = e * e;
        const float pe = fmaf(e, e, -p);
        const float s = hi + p;
        const float bb = s - hi;
        lo += ((hi - (s - bb)) + (p - bb)) + pe;
        hi = s;
    }
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1) {
        const float oh = __shfl_xor_sync(g.mask, hi, off, L), ol = __shfl_xor_sync(g.mask, lo, off, L);
        const float s = hi + oh;
        const float bb = s - hi;
        lo = lo + ol + ((hi - (s - bb)) + (oh - bb));
        hi = s;
    }
    return (typename Ctl<R>::T)sqrtf((hi + lo) * (1.0f / (float)(L * C)));
}

// Hairer's initial step (initdt.jl:17-298).  f0 is returned for FSAL methods.
// t is the model's time; bwd: the integration runs towards smaller t, so the
// trial step goes to t - dt0 (dt0_tdir), and the magnitude is returned.
template <class Model, class R, int L, int C, int ORDER>
__device__ double initdt(const R* u0, const PR<R>* p, double t, bool bwd, double dtmax, double dtmin_user,
                         const Tol<R>& tol, R* f0, const Group<L>& g) {
    double dtmin = nextafter(jmax(dtmin_user, jeps(t)), __longlong_as_double(0x7ff0000000000000LL));
    double smalldt = jmax(dtmin, 1e-6);
    R sk[C], f1[C], u1[C];
#pragma unroll
    for (int c = 0; c < C; ++c) sk[c] = FMA(ABS(u0[c]), tol.template r<C>(g.lane, c), tol.template a<C>(g.lane, c));
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
    const double dt0_tdir = bwd ? -dt0 : dt0;
    R dt0r = (R)dt0_tdir;
#pragma unroll
    for (int c = 0; c < C; ++c) u1[c] = FMA(dt0r, f0[c], u0[c]);
    Model::template rhs<R, L, C>(f1, u1, p, t + dt0_tdir, g);
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
        // 10^(-(2 + log10 mx)/order) = exp(-(2 ln10 + ln mx)/order)
        const double LN10 = 2.302585092994046;
        dt1 = series_exp(-(2.0 * LN10 + series_ln(mx)) / (double)ORDER);
    }
    return jmax(dtmin, jmin(jmin(100.0 * dt0, dt1), dtmax));
}

// Trajectories one after another on lane group g, as `next` hands them out
// (a negative index: none left).  A group whose trajectory ends takes the next
// one inside the same step loop, so its lanes step again with the rest of the
// warp at the next iteration instead of idling until the warp's longest
// trajectory ends (the trajectories of a warp differ in step counts by up to
// the ratio of their spans or stiffness).  Every trajectory's arithmetic is
// the same whichever group and slot runs it.  Alg provides the cache, the
// step, the interpolant and the FSAL hooks.  FWD, the plain form: the caller
// guarantees forward spans (tf >= t0) and uses neither force_dtmin nor
// isoutofdomain, and the loop carries none of them (a backward span then
// reports InitialFailure, as a NaN span does).
template <class Alg, class Model, class R, int L, int C, bool FWD, class Next>
__device__ void solve_trajectories(const EnsembleArgs& a, const Group<L>& g, Next next) {
    using CT = typename Ctl<R>::T;
    constexpr int NP = Model::NP;
    const long long N = a.N;
    long long j = -1;   // the trajectory in hand
    R u[C], uprev[C], ulo[C], uprevlo[C];   // solution as (hi, lo) pairs, see Acc
    PR<R> p[NP > 0 ? NP : 1];   // FP64, or float pairs in the mixed form (fpair)
    // Backward integration (tf < t0) runs the loop on s = -t: its times, steps,
    // tstops and saveat points are those of the reference negated (the
    // reference's own heaps hold tdir * t), every comparison on them is the
    // reference's with tdir taken out, and the model and the method see the
    // model's time TM(s) = -s and signed step DT(h) = -h, so each stage and each
    // interpolation is the reference's arithmetic exactly (negation is exact).
    // The direction is data, held in the step loop as one mask (bm = -1
    // backward, 0 forward) from which everything direction-dependent is integer
    // arithmetic: TM flips the sign bit, the reversed saveat and tstops indices
    // are (s ^ bm) + (bm & n), and the forward-only dtmin bound is masked to zero
    // (a runtime flag used through branches and selects on doubles cost the
    // mixed Robertson kernel 30%).
    bool bwd = false;
    int bm = 0;
    auto TM = [&bm](double x) -> double {
        return __hiloint2double(__double2hiint(x) ^ (bm & (int)0x80000000u), __double2loint(x));
    };
    double t0 = 0.0, tf = 0.0, dtmax = 0.0;
    // the ensemble's tolerances, or per trajectory (requests merged into one
    // launch by the serving loop keep their own)
    R abstol = R(0), reltol = R(0);
    auto tol = [&]() { return Tol<R>{abstol, reltol, a.abstol_vec, a.reltol_vec}; };

    typename Alg::template Cache<R, C> cache;
    // the PI controller's values: the method's own (a composite's current one)
    auto KV = [&](int k) -> CT {
        if constexpr (is_composite_alg<Alg>::value) return kval<CT>(a, cache.current, k);
        else return kval<CT>(a, 0, k);
    };
    StepStats st = {0, 0, 0, 0, 0, 0};
    int nsaved = 0;
    int isave = 0;
    double last_saved_t = dnan();

    auto save_point = [&](double ts, const R* v, const R* vlo) {
        // past the capacity, step saves keep the latest point in the last slot
        const int slot = nsaved < a.nsave_cap ? nsaved : ((a.save_everystep || a.callback) ? a.nsave_cap - 1 : -1);
        if (slot >= 0) {
            if (g.lane == 0 && a.t_out) a.t_out[(size_t)slot * N + j] = TM(ts);
            if (a.save_idxs) {   // save_idxs: row r holds state save_idxs[r], written by its lane
#pragma unroll 1
                for (int r = 0; r < a.nsave_rows; ++r) {
                    const int si = a.save_idxs[r];
#pragma unroll
                    for (int c = 0; c < C; ++c)
                        if (si == g.lane * C + c)
                            a.u_out[((size_t)slot * a.nsave_rows + r) * N + j] = Acc<R>::join(v[c], vlo[c]);
                }
            } else {
#pragma unroll
                for (int c = 0; c < C; ++c)
                    a.u_out[((size_t)slot * a.nmax + g.lane * C + c) * N + j] = Acc<R>::join(v[c], vlo[c]);
            }
        }
        nsaved++;
        last_saved_t = ts;
    };
    // Dense output: the interpolation vectors of the step ending at the save about
    // to be made (save_dense_at_t!, integrator_utils.jl:455-473), in the slot that
    // save_point will use.  The start save has no step (zeros); a step save past the
    // capacity overwrites the last slot, whose step no longer starts at the slot
    // before it, so its vectors are NaN.
    auto save_dense = [&](bool step) {
        const bool over = nsaved >= a.nsave_cap;
        const int slot = over ? a.nsave_cap - 1 : nsaved;
        if (step) Alg::template prepare_dense<R, C>(cache);
#pragma unroll
        for (int q = 0; q < Alg::NDENSE; ++q) {
            const R* kv = Alg::template dense_slot<R, C>(cache, q);
#pragma unroll
            for (int c = 0; c < C; ++c)
                a.k_out[(((size_t)slot * Alg::NDENSE + q) * a.nmax + g.lane * C + c) * N + j] =
                    !step ? 0.0 : over ? dnan() : (double)kv[c];
        }
    };
    // the saveat points ascend; backward they are read from the end, negated
    auto saveat_at = [&](int s) -> double {
        const int k = (s ^ bm) + (bm & a.nsave);
        return TM(a.saveat_per_traj ? a.saveat[(size_t)k * N + j] : a.saveat[k]);
    };
    auto tstop_at = [&](int k) -> double { return TM(a.tstops[(k ^ bm) + (bm & a.ntstops)]); };

    double t = 0.0, tprev = 0.0, dt = 0.0, dtpropose = 0.0;
    CT EEst = CT(1), q11 = CT(1), errold = CT(1);
    CT bank_errold = CT(1), bank_q11 = CT(1);   // composite: the other method's controller state
    // FP64 form: ln(errold) kept from the step that set errold, so errold^beta2 is one
    // exp series instead of a ctrl_pow (the same value: ctrl_pow(x, y) is
    // series_exp(y * series_ln(x)) for finite positive x); NaN when not kept
    double ln_qoldinit = 0.0, ln_errold = 0.0, bank_ln_errold = 0.0;
    if constexpr (sizeof(CT) == 8) ln_qoldinit = series_ln((double)kval<CT>(a, 0, KQOLD));
    bool do_error_check = true;
    long long iter = 0, success_iter = 0;
    bool accept = false, next_tstop = false;
    bool isout = false;   // the last attempt ended out of the domain (isoutofdomain)
    int rc = RC_DEFAULT;

    // _savevalues! (integrator_utils.jl:340-414) after an accepted step: saveat
    // points up to t by the step's interpolant, then the every-step save; true
    // when a save landed exactly on t (its `savedexactly`)
    // y1/y1lo: the accepted step's end state, which the stiff-aware Rosenbrock
    // interpolant reads (u itself, unless an event has moved u off the step's end)
    auto savevalues = [&](const R* y1, const R* y1lo) -> bool {
        bool exact = false;
        while (isave < a.nsave) {
            double curt = saveat_at(isave);
            if (!dle(curt, t)) break;
            isave++;
            if (!deq(curt, t)) {
                const double th = (double)Ctl<R>::theta(curt - tprev, dt);
                R out[C], outlo[C];
                Alg::template interpolate<Model, R, L, C>(cache, out, outlo, th, TM(dt), TM(tprev), uprev, uprevlo, y1,
                                                          y1lo, p, g);
                save_point(curt, out, outlo);
            } else {
                if (deq(curt, tf) && !a.save_end) continue;
                save_point(t, u, ulo);
                exact = true;
            }
        }
        // save_everystep (integrator_utils.jl:397-404): the accepted step, unless it
        // repeats the last save or is tf with save_end off
        if (a.save_everystep &&
            (nsaved == 0 || ((!deq(t, last_saved_t) || abs_bits(dt) == 0) && (a.save_end || !deq(t, tf))))) {
            if (a.k_out) save_dense(true);
            save_point(t, u, ulo);
            exact = true;
        }
        return exact;
    };

    // After an event moved t back into the step (change_t_via_interpolation!,
    // integrator_interface.jl:5-40): dt = t - tprev and the step's interpolation
    // data recomputed for the shortened step from (tprev, uprev)
    // (reeval_internals_due_to_modification! -> ode_addsteps! with
    // always_calc_begin, :54-79), so the saveat points before the event and a
    // dense save at it use the shortened step's interpolant, as the reference's
    // do.  The reference does not count these evaluations; the state stays the
    // interpolated one and a composite's stiffness estimate is kept.
    auto recompute_step = [&]() {
        if constexpr (Model::HAS_EVENT) {   // only event models move t
            dt = t - tprev;
            R ut[C], utlo[C];
            StepStats uncounted = {0, 0, 0, 0, 0, 0};
            double eig = 0.0;
            if constexpr (is_composite_alg<Alg>::value) eig = cache.eigen_est;
            // iter -1: the recomputation (a W-method keeps the step's J, as the in-place
            // addsteps does, and its reuse state)
            Alg::template step<Model, R, L, C>(cache, ut, utlo, uprev, uprevlo, p, TM(tprev), TM(dt), tol(),
                                               -1, false, g, uncounted);
            if constexpr (is_composite_alg<Alg>::value) cache.eigen_est = eig;
        }
    };
    // A save made by a callback (before or after its affect): with dense output it
    // stores the step's interpolation vectors too (savevalues!(integrator, true)).
    auto save_forced = [&]() {
        if (a.k_out) save_dense(true);
        save_point(t, u, ulo);
    };

    // The model's ContinuousCallback after an accepted step: handle_callbacks!
    // (integrator_utils.jl:1081-1132) with find_callback_time, nudge_tprev,
    // check_event_occurrence and apply_callback! (lib/DiffEqBase/src/callbacks.jl:
    // 364-458, 557-643).  The event time is the left end of the sign change to
    // adjacent floats (LeftRootFind; the reference's ModAB runs with abstol =
    // reltol = 0); the condition between tprev and t comes from the step's
    // interpolant.  After moving to the event the reference recomputes the step's
    // interpolation data for the shortened step before saving the saveat points
    // that precede the event; here those points come from the accepted step's own
    // interpolant (the two differ by the local error).  Returns true when an event
    // was applied (its saves made).
    bool ev_last = false, terminated = false;
    double last_event_error = 0.0;
    auto handle_event = [&]() -> bool {
        if constexpr (Model::HAS_EVENT && event_len<Model>::value == 1) {
            auto cond_at = [&](double abst) -> double {
                if (abst == t) return Model::template event_condition<R, L, C>(u, ulo, a.p + j, N, TM(abst), g);
                if (abst == tprev)
                    return Model::template event_condition<R, L, C>(uprev, uprevlo, a.p + j, N, TM(abst), g);
                R v[C], vlo[C];
                Alg::template interpolate<Model, R, L, C>(cache, v, vlo, (abst - tprev) / dt, TM(dt), TM(tprev), uprev,
                                                          uprevlo, u, ulo, p, g);
                return Model::template event_condition<R, L, C>(v, vlo, a.p + j, N, TM(abst), g);
            };
            auto is_event = [](double bs, double ts) {
                return ((bs < 0.0 && Model::EVENT_AFFECT_POS) || (bs > 0.0 && Model::EVENT_AFFECT_NEG)) &&
                       bs * ts <= 0.0;
            };
            double bottom_t = tprev;
            double bc = cond_at(bottom_t);
            if (ev_last) {   // nudge_tprev: still at the last event's root -> look from just past it
                if (fabs(bc - last_event_error) <= kCbAbstol) bottom_t = tprev + dt * kCbRepeatNudge;
                bc = cond_at(bottom_t);
            }
            const double bs = dsign(bc);
            double top_t = t;
            double tv = cond_at(top_t);
            double ts = dsign(tv);
            bool occ = is_event(bs, ts);
            if (a.interp_points != 0 && !occ) {   // range(tprev, stop = t, length = interp_points)
                const int m = a.interp_points;
                for (int i = 2; i <= m; ++i) {
                    top_t = i == m ? t : tprev + (t - tprev) * ((double)(i - 1) / (double)(m - 1));
                    tv = cond_at(top_t);
                    ts = dsign(tv);
                    occ = is_event(bs, ts);
                    if (occ) break;
                }
            }
            if (!occ) {
                ev_last = false;
                return false;
            }
            double cb_t = top_t, residual = 0.0;
            if (ts != 0.0) {
                cb_t = bracket_left_root(cond_at, bottom_t, top_t, bc, tv);
                residual = cond_at(cb_t);
            }
            ev_last = true;
            last_event_error = residual;
            // apply_callback!: set_proposed_dt! (dtrelax = 1)
            dtpropose = pmax(nextafter(a.dtmin, __longlong_as_double(0x7ff0000000000000LL)), dt);
            // change_t_via_interpolation!
            const bool moved = cb_t != t;
            if (moved) {
                R v[C], vlo[C];
                Alg::template interpolate<Model, R, L, C>(cache, v, vlo, (cb_t - tprev) / dt, TM(dt), TM(tprev), uprev,
                                                          uprevlo, u, ulo, p, g);
#pragma unroll
                for (int c = 0; c < C; ++c) { u[c] = v[c]; ulo[c] = vlo[c]; }
                t = cb_t;
                recompute_step();
            }
            // saveat up to the event, then the pre-affect save unless one landed on t
            if (!savevalues(u, ulo)) save_forced();
            bool modified = false;
            if (bs < 0.0 && Model::EVENT_AFFECT_POS) {
                terminated = Model::template event_affect<R, L, C>(u, ulo, a.p + j, N, TM(t), true, g);
                modified = true;
            } else if (bs > 0.0 && Model::EVENT_AFFECT_NEG) {
                terminated = Model::template event_affect<R, L, C>(u, ulo, a.p + j, N, TM(t), false, g);
                modified = true;
            }
            if (modified) save_forced();   // save_positions[2]
            if (!terminated && (moved || modified)) Alg::template reset_fsal<Model, R, L, C>(cache, u, ulo, p, TM(t), g, st);
            return true;
        }
        return false;
    };

    // The model's VectorContinuousCallback of M conditions after an accepted step:
    // find_callback_time(integrator, ::VectorContinuousCallback, idx) (lib/DiffEqBase/
    // src/callbacks.jl:239-362) and apply_callback! (:557-643).  The bottom signs come
    // from tprev; the components of the last event (prev_mask) take theirs just past
    // it (nudge_tprev on the one whose condition is closest to zero); a component
    // fires on a sign change away from a nonzero bottom sign (findall_events!,
    // :495-523), checked at t and, unless every component fired there, at the
    // interp_points of the step; each firing component's root is bracketed to
    // adjacent floats, the earliest wins and ties fire together; affect! gets the
    // events' directions (+1 upcrossing, -1 downcrossing, 0 none).
    int prev_mask = 0;
    auto handle_vector_event = [&]() -> bool {
        if constexpr (Model::HAS_EVENT && event_len<Model>::value > 1) {
            constexpr int M = event_len<Model>::value;
            static_assert(M <= 32, "at most 32 conditions");
            auto conds_at = [&](double abst, double* out) {
                if (abst == t) {
                    Model::template event_conditions<R, L, C>(out, u, ulo, a.p + j, N, TM(abst), g);
                } else if (abst == tprev) {
                    Model::template event_conditions<R, L, C>(out, uprev, uprevlo, a.p + j, N, TM(abst), g);
                } else {
                    R v[C], vlo[C];
                    Alg::template interpolate<Model, R, L, C>(cache, v, vlo, (abst - tprev) / dt, TM(dt), TM(tprev),
                                                              uprev, uprevlo, u, ulo, p, g);
                    Model::template event_conditions<R, L, C>(out, v, vlo, a.p + j, N, TM(abst), g);
                }
            };
            double bc[M], bs[M], nc[M], tc[M];
            conds_at(tprev, bc);
#pragma unroll
            for (int i = 0; i < M; ++i) { bs[i] = dsign(bc[i]); nc[i] = bc[i]; }
            double nudged_t = tprev;
            if (ev_last) {
                double minc = 0.0, mina = __longlong_as_double(0x7ff0000000000000LL);
#pragma unroll
                for (int i = 0; i < M; ++i)
                    if (((prev_mask >> i) & 1) && fabs(bc[i]) < mina) { mina = fabs(bc[i]); minc = bc[i]; }
                if (fabs(minc - last_event_error) <= kCbAbstol) nudged_t = tprev + dt * kCbRepeatNudge;
                conds_at(nudged_t, nc);
#pragma unroll
                for (int i = 0; i < M; ++i)
                    if ((prev_mask >> i) & 1) bs[i] = dsign(nc[i]);
            }
            auto fired = [&](const double* top) {
                int m = 0;
#pragma unroll
                for (int i = 0; i < M; ++i)
                    if (bs[i] != 0.0 && bs[i] * dsign(top[i]) <= 0.0) m |= 1 << i;
                return m;
            };
            double top_t = t;
            conds_at(top_t, tc);
            int ev = fired(tc);
            constexpr int all = M == 32 ? -1 : (1 << M) - 1;
            if (a.interp_points != 0 && ev != all) {   // any(iszero, event_idx)
                const int m = a.interp_points;
                for (int i = 2; i <= m; ++i) {
                    top_t = i == m ? t : tprev + (t - tprev) * ((double)(i - 1) / (double)(m - 1));
                    conds_at(top_t, tc);
                    ev = fired(tc);
                    if (ev) break;
                }
            }
            if (!ev) {
                ev_last = false;
                return false;
            }
            // the earliest root among the firing components (rightfloat(top_t) to start)
            double cb_t = nextafter(top_t, __longlong_as_double(0x7ff0000000000000LL)), residual = 0.0;
            int sim = 0, dir[M];
#pragma unroll
            for (int i = 0; i < M; ++i) dir[i] = 0;
            // one copy of the root finder for every component (a rare path: events)
#pragma unroll 1
            for (int i = 0; i < M; ++i) {
                if (!((ev >> i) & 1)) continue;
                auto fi = [&](double s) {
                    double o[M];
                    conds_at(s, o);
                    return o[i];
                };
                double cbi;
                if (dsign(tc[i]) == 0.0) {
                    cbi = top_t;
                } else {
                    const bool from_nudge = ev_last && ((prev_mask >> i) & 1);
                    const double lo = from_nudge ? nudged_t : tprev;
                    cbi = bracket_left_root(fi, lo, top_t, from_nudge ? nc[i] : bc[i], tc[i]);
                }
                if (cbi < cb_t) {
                    sim = 0;
#pragma unroll
                    for (int k = 0; k < M; ++k) dir[k] = 0;
                }
                if (cbi <= cb_t) {
                    cb_t = cbi;
                    residual = fi(cbi);
                    sim |= 1 << i;
                    dir[i] = bs[i] < 0.0 ? 1 : -1;
                }
            }
            ev_last = true;
            last_event_error = residual;
            prev_mask = sim;
            // apply_callback!: set_proposed_dt! (dtrelax = 1), change_t_via_interpolation!,
            // saveat up to the event, the pre-affect save unless one landed on t, affect!
            // with the events' directions, the post-affect save
            dtpropose = pmax(nextafter(a.dtmin, __longlong_as_double(0x7ff0000000000000LL)), dt);
            const bool moved = cb_t != t;
            if (moved) {
                R v[C], vlo[C];
                Alg::template interpolate<Model, R, L, C>(cache, v, vlo, (cb_t - tprev) / dt, TM(dt), TM(tprev), uprev,
                                                          uprevlo, u, ulo, p, g);
#pragma unroll
                for (int c = 0; c < C; ++c) { u[c] = v[c]; ulo[c] = vlo[c]; }
                t = cb_t;
                recompute_step();
            }
            if (!savevalues(u, ulo)) save_forced();
            terminated = Model::template vector_event_affect<R, L, C>(u, ulo, a.p + j, N, TM(t), dir, g);
            save_forced();
            if (!terminated) Alg::template reset_fsal<Model, R, L, C>(cache, u, ulo, p, TM(t), g, st);
            return true;
        }
        return false;
    };

    // the tstops heap (initialize_tstops, solve.jl:1021-1040): the shared ascending
    // tstops inside (t0, tf), then tf.  Entries not after t leave it at each loop
    // header: the ones at t0 and, after a step landed on a tstop, every copy of it
    // (handle_tstop!, integrator_utils.jl:1290-1313); NaNs and out-of-order
    // entries are dropped the same way.
    int itst = 0;

    // Load trajectory j: its state, parameters, span and tolerances, the start
    // save, the method's initialisation and the initial step; every piece of
    // per-trajectory state starts afresh.
    auto start = [&]() {
#pragma unroll
        for (int c = 0; c < C; ++c) Acc<R>::split(a.u0[(size_t)(g.lane * C + c) * N + j], u[c], ulo[c]);
#pragma unroll
        for (int i = 0; i < NP; ++i) p[i] = make_param<R>(a.p[(size_t)i * N + j]);
        if constexpr (!FWD) {
            bwd = a.tspan[N + j] < a.tspan[j];
            bm = bwd ? -1 : 0;
        }
        t0 = TM(a.tspan[j]);
        tf = TM(a.tspan[N + j]);
        dtmax = a.dtmax > 0 ? a.dtmax : tf - t0;
        abstol = (R)(a.abstol_traj ? a.abstol_traj[j] : a.abstol);
        reltol = (R)(a.reltol_traj ? a.reltol_traj[j] : a.reltol);
        st = StepStats{0, 0, 0, 0, 0, 0};
        nsaved = 0;
        isave = 0;
        last_saved_t = dnan();
        // saveat entries outside (t0, tf] are skipped (initialize_saveat, solve.jl:1103-1124)
        while (isave < a.nsave && !(saveat_at(isave) > t0)) isave++;
#pragma unroll
        for (int c = 0; c < C; ++c) { uprev[c] = u[c]; uprevlo[c] = ulo[c]; }
        if (a.save_start) {
            if (a.k_out) save_dense(false);
            save_point(t0, u, ulo);
        }
        t = t0;
        tprev = t0;
        Alg::template initialize<Model, R, L, C>(cache, u, p, TM(t), g, st, a, j);
        if (!a.adaptive) {
            dt = fabs(a.dt);   // fixed steps: no initial-step heuristic (handle_dt!, solve.jl:968-985)
        } else if (a.dt > 0) {
            dt = a.dt;
        } else {
            // the initial step's dtmax is at most the distance to the first tstop
            // (_determine_initdt, integrator_interface.jl:644-656)
            int k0 = 0;
            while (k0 < a.ntstops && !(tstop_at(k0) > t0)) k0++;
            const double first_tstop = (k0 < a.ntstops && tstop_at(k0) < tf) ? tstop_at(k0) : tf;
            dt = initdt<Model, R, L, C, Alg::ORDER>(u, p, TM(t), bwd, jmin(fabs(dtmax), fabs(first_tstop - t0)),
                                                     a.dtmin, tol(), Alg::template fsal_slot<R, C>(cache), g);
            st.nf += 2;
        }
        dtpropose = dt;
        EEst = CT(1);
        q11 = CT(1);
        errold = kval<CT>(a, 0, KQOLD);
        bank_errold = errold;
        bank_q11 = CT(1);
        ln_errold = bank_ln_errold = ln_qoldinit;
        do_error_check = true;
        iter = 0;
        success_iter = 0;
        accept = false;
        next_tstop = false;
        isout = false;
        rc = (tf >= t0) ? RC_DEFAULT : RC_INITIALFAILURE;   // a NaN span is not stepped
        ev_last = false;
        terminated = false;
        last_event_error = 0.0;
        prev_mask = 0;
        itst = 0;
    };

    // The trajectory in hand has ended: the endpoint save
    // (solution_endpoint_match_cur_integrator!) and its counts, retcode and stats.
    auto finish = [&]() {
        if (rc == RC_DEFAULT) rc = RC_SUCCESS;
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
            if (need) {
                if (a.k_out) save_dense(st.naccept > 0);
                save_point(t, u, ulo);
            }
        }
        if (g.lane == 0) {
            a.nsaved[j] = nsaved < a.nsave_cap ? nsaved : a.nsave_cap;
            a.retcode[j] = rc;
            if (a.stats) {
                OdeStatsDev* s = a.stats + j;
                s->nf = st.nf; s->njacs = st.njacs; s->nw = st.nw; s->nsolve = st.nsolve;
                s->naccept = st.naccept; s->nreject = st.nreject;
            }
        }
    };

    // One step attempt per iteration for every group of the warp that holds a
    // trajectory; a group whose trajectory ended finishes it and loads the next.
    bool done = true;   // no trajectory in hand
    for (;;) {
        // the idle lanes of the warp take their next trajectories together once
        // a.refill_lanes of them are idle (or all are): loading one runs the
        // initial-step probe and the method's start, which the stepping lanes would
        // otherwise wait through once per trajectory.  Lanes also leave the loop
        // only together: a warp whose lanes left one by one ran the mixed
        // Robertson solve 3% slower than one that keeps them to the end.
        const unsigned live = __activemask();
        const unsigned idle = __ballot_sync(live, done);
        if (done) {
            if (__popc(idle) < a.refill_lanes && idle != live) continue;
            if (j >= 0) finish();
            j = next();
            if (j < 0) break;
            start();
            done = !(t < tf);
            continue;
        }
        // ---- loopheader!
        while (itst < a.ntstops && !(tstop_at(itst) > t)) itst++;
        const double tnext = (itst < a.ntstops && tstop_at(itst) < tf) ? tstop_at(itst) : tf;   // first_tstop
        const double dist = tnext - t;   // > 0 inside the loop
        if (iter > 0) {
            if (accept) {
                success_iter++;
#pragma unroll
                for (int c = 0; c < C; ++c) { uprev[c] = u[c]; uprevlo[c] = ulo[c]; }
                // apply_step!: dt = dtpropose, then modify_dt_for_tstops! (whose flag and
                // dtpropose the second call below overwrites; only the clip survives)
                dt = pmin(dtpropose, dist);
                Alg::template on_accept<R, C>(cache);
            } else if (!FWD && isout) {
                // handle_step_rejection! after an out-of-domain step: dt * qmin
                if constexpr (is_composite_alg<Alg>::value) dt = dt * a.kd[cache.current][KQMIN];
                else dt = dt * a.kd[0][KQMIN];
            } else {
                // step_reject_controller!: dt /= min(1/qmin, q11/gamma)
                const CT qmin_inv = KV(KQMININV);
                const CT qq = q11 / KV(KGAM);
                const CT f = (qmin_inv != qmin_inv || qq != qq) ? qq + qmin_inv : (qmin_inv < qq ? qmin_inv : qq);
                dt = Ctl<R>::scale_dt(dt, f);
            }
        }
        iter++;
        if constexpr (is_composite_alg<Alg>::value) {
            // choose_algorithm! (integrator_utils.jl:120-121): on a switch the controller
            // state of the method left is banked and the other's resumed
            // (CompositeController), then the new method is initialised
            if (Alg::choose(cache, dt, do_error_check)) {
                const int cur = cache.current;
                const CT e_old = errold, q_old = q11;   // swap with the other method's state
                errold = bank_errold;
                q11 = bank_q11;
                bank_errold = e_old;
                bank_q11 = q_old;
                const double l_old = ln_errold;
                ln_errold = bank_ln_errold;
                bank_ln_errold = l_old;
                using NSA = typename Alg::NonStiff;
                using SA = typename Alg::Stiff;
                Alg::template enter<Model, R, L, C>(cache, uprev, uprevlo, p, TM(t), g, st);
            }
        }
        // fix_dt_at_bounds!  (backward the reference takes min(dt, dtmin) of a negative
        // dt and a positive dtmin: the lower bound applies forward only)
        dt = pmin(dtmax, dt);
        dt = pmax(dt, __longlong_as_double(abs_bits(pmax(peps(t), a.dtmin)) & ~(long long)bm));
        {   // modify_dt_for_tstops!  (fixed steps: the given dt, dtcache, clipped instead;
            // without one, every step runs to the next tstop)
            const double tol = ptol100(pmax(pabs(t), pabs(tnext)));
            const double orig = a.adaptive ? pabs(dt) : (a.dt != 0 ? fabs(a.dt) : dist);
            if (a.adaptive) dtpropose = orig;
            next_tstop = !plt(orig + tol, dist);
            dt = pmin(orig, dist);
        }
        // ---- check_error (de_check_error), unless a composite's stiffness test
        // turned it off for this step (solve.jl:909)
        {
            int e = RC_SUCCESS;
            const long long db = __double_as_longlong(dt);
            if (!do_error_check) e = RC_SUCCESS;
            else if (bits_nan(db)) e = RC_DTNAN;
            else if (iter > a.maxiters) e = RC_MAXITERS;
            // t + dt < tdir * first(tstops) in the reference's own time
            else if (a.adaptive && (FWD || !a.force_dtmin) && ple(pabs(dt), pabs(a.dtmin)) &&
                     (!accept || (bwd ? t + dt > tnext : t + dt < tnext)))
                e = RC_DTLESSTHANMIN;
            else if (a.adaptive && (FWD || !a.force_dtmin) && !accept && ple(pabs(dt), peps(t))) e = RC_UNSTABLE;
            else if (accept) {
                bool bad = false;
#pragma unroll
                for (int c = 0; c < C; ++c) bad = bad || !isfinite(u[c]);
                if (g.any(bad)) e = RC_UNSTABLE;
            }
            if (e == RC_SUCCESS && a.abort_flag != nullptr && (iter & 63) == 0 && *a.abort_flag != 0)
                e = RC_ABORTED;
            if (e != RC_SUCCESS) {
                rc = e;
                done = true;
                continue;
            }
        }
        // ---- perform_step! (skipped for a step below eps(t) onto the tstop)
        if (!(next_tstop && plt(pabs(dt), peps(t)))) {
            EEst = Alg::template step<Model, R, L, C>(cache, u, ulo, uprev, uprevlo, p, TM(t), TM(dt), tol(),
                                                      iter, EEst > CT(1), g, st);
        }
        // ---- loopfooter!
        if constexpr (is_composite_alg<Alg>::value) do_error_check = true;
        const double ttmp = t + dt;
        const CT inv_qmaxc = success_iter == 0 ? KV(KIQMAXF) : KV(KIQMAX);
        CT q = CT(1);
        double ln_eest = dnan();   // FP64 form: ln(EEst) of this attempt when EEst is finite and positive
        if (!a.adaptive) {
            // fixed steps: every step is accepted and no controller runs
        } else if (EEst == CT(0)) {
            q = inv_qmaxc;
        } else {
            CT qq, den;
            if constexpr (sizeof(CT) == 8) {
                const bool fin = EEst > 0.0 && EEst < __longlong_as_double(0x7ff0000000000000LL);
                if (fin) ln_eest = series_ln(EEst);
                qq = fin ? series_exp(KV(KB1) * ln_eest) : Ctl<R>::pw(EEst, KV(KB1));
                den = ln_errold == ln_errold ? series_exp(KV(KB2) * ln_errold) : Ctl<R>::pw(errold, KV(KB2));
            } else {
                qq = Ctl<R>::pw(EEst, KV(KB1));
                den = Ctl<R>::pw(errold, KV(KB2));
            }
            q = qq / den;
            q11 = qq;
            const CT x = q / KV(KGAM);
            q = x > KV(KQMININV) ? KV(KQMININV) : (x < inv_qmaxc ? inv_qmaxc : x);
        }
        // isoutofdomain (the common any(x -> x < 0, u)) at the step's end, adaptive
        // steps only (integrator_utils.jl:612-615)
        isout = false;
        if (!FWD && a.isoutofdomain && a.adaptive) {
            bool neg = false;
#pragma unroll
            for (int c = 0; c < C; ++c) neg = neg || u[c] < R(0) || (u[c] == R(0) && ulo[c] < R(0));
            isout = g.any(neg);
        }
        accept = !a.adaptive || (!isout && EEst <= CT(1));
        // force_dtmin: a step at the smallest dt is taken whatever its error
        if (!FWD && !accept && a.force_dtmin) accept = ple(pabs(dt), pabs(pmax(peps(t), a.dtmin)));
        if (accept) {
            st.naccept++;
            tprev = t;
            if (next_tstop) {
                if (a.adaptive) dt = dtpropose;
                next_tstop = false;
                t = tnext;   // the tstop target
            } else {
                t = ttmp;
            }
            if (a.adaptive) {
                if (KV(KQSMIN) <= q && q <= KV(KQSMAX)) q = CT(1);
                errold = (EEst != EEst) ? EEst : (EEst > KV(KQOLD) ? EEst : KV(KQOLD));
                if constexpr (sizeof(CT) == 8)
                    ln_errold = (EEst != EEst) ? dnan() : (EEst > KV(KQOLD) ? ln_eest : ln_qoldinit);
                const double dtnew = Ctl<R>::scale_dt(dt, q);
                const double dtp = pmin(pabs(dtmax), pabs(dtnew));
                dtpropose = pmax(pabs(dtp), pabs(pmax(peps(t), a.dtmin)));
            } else {
                dtpropose = dt;   // the non-adaptive footer (integrator_utils.jl:660-677)
            }
            // ---- handle_callbacks! / savevalues!
            // handle_callbacks! (integrator_utils.jl:1081-1132): the continuous callback,
            // then the discrete one; savevalues! unless the last of them saved
            bool handled = false;
            if constexpr (Model::HAS_EVENT) {
                if (a.callback) handled = event_len<Model>::value == 1 ? handle_event() : handle_vector_event();
            }
            if constexpr (has_discrete_callback<Model>::value) {
                // apply_discrete_callback! (lib/DiffEqBase/src/callbacks.jl:645-682): the
                // condition is t in tstops (the step landed on the tstop the index points
                // at; entries before it were passed at the header) or the model's own
                bool fire = false;
                if (a.callback) {
                    if constexpr (discrete_at_tstops<Model>::value) fire = itst < a.ntstops && tstop_at(itst) == t;
                    else fire = Model::template discrete_condition<R, L, C>(u, ulo, a.p + j, N, TM(t), g);
                }
                if (fire) {
                    // saveat up to t and the every-step save, then save_positions[1]
                    // unless a save landed on t; affect!; save_positions[2]
                    if (!savevalues(u, ulo)) save_forced();
                    terminated = Model::template discrete_affect<R, L, C>(u, ulo, a.p + j, N, TM(t), g) || terminated;
                    save_forced();
                    // u changed: FSAL methods evaluate f(u) again (reeval_fsal)
                    if (!terminated) Alg::template reset_fsal<Model, R, L, C>(cache, u, ulo, p, TM(t), g, st);
                }
                handled = fire;   // saved_in_cb is the discrete callbacks' verdict
            }
            if (!handled) savevalues(u, ulo);
            Alg::template after_save<R, C>(cache);
            if (terminated) {   // terminate! (ReturnCode.Terminated)
                rc = RC_TERMINATED;
                done = true;
                continue;
            }
        } else {
            st.nreject++;
        }
        done = !(t < tf);
    }
}

// Ensemble kernel: static (one trajectory per group, the plain one-kernel-per-
// ensemble form) or persistent (groups pop trajectory indices from a device
// counter until the ensemble is exhausted).
template <class Alg, class Model, class R, int L, int C, bool FWD = false>
// Mixed kernels with up to 4 states per lane are held to 3 resident blocks of
// 128 (<= 170 registers; measured 10% faster than 2 on Robertson, no spills;
// 4 blocks cap them at 128 registers and spill 316 bytes: 4.92 against 4.24 ms);
// wider or FP64 kernels keep their registers.
#ifndef ODEGB_MIN_BLOCKS_F32
#define ODEGB_MIN_BLOCKS_F32 3
#endif
__global__ void __launch_bounds__(128, (sizeof(R) == 4 && C <= 4) ? ODEGB_MIN_BLOCKS_F32 : 1)
    ensemble_kernel(EnsembleArgs a) {
    Group<L> g;
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / L;
    bool first = true;
    solve_trajectories<Alg, Model, R, L, C, FWD>(a, g, [&]() -> long long {
        unsigned long long idx;
        if (!a.persistent) {   // static: this group's own trajectory, once
            idx = first ? (unsigned long long)gid : ~0ull;
            first = false;
        } else {               // persistent: the next index of the device queue
            idx = 0;
            if (g.lane == 0) idx = atomicAdd(a.queue, 1ull);
            idx = g.bcast(idx, 0);
        }
        if (idx >= (unsigned long long)a.count) return -1;
        return a.order ? a.order[idx] : (long long)idx;
    });
}

// Uneven-size ensembles in ONE persistent launch.  Trajectories were bucketed
// on the device by state count; every warp works through the size classes
// from the largest down (longest jobs first), its lane groups popping
// trajectories of the current class from that class's device counter, so a
// group that finishes a trajectory refills at once and the load balances
// across classes.  At a class change the warp regroups its lanes (L depends
// on the class), which needs the whole warp: __syncwarp between classes.
template <class Alg, class Model, class R, int L, int C, bool FWD>
__device__ __forceinline__ void drain_class(const EnsembleArgs& a, int cls) {
    Group<L> g;
    const unsigned long long cnt = a.class_count[cls], off = a.class_offset[cls];
    solve_trajectories<Alg, Model, R, L, C, FWD>(a, g, [&]() -> long long {
        unsigned long long idx = 0;
        if (g.lane == 0) idx = atomicAdd(a.class_next + cls, 1ull);
        idx = g.bcast(idx, 0);
        return idx < cnt ? a.order[off + idx] : -1;
    });
    __syncwarp();
}

// Classes n = 64, 32, 16, 8, 4 with C states per lane (L = n/C).
// The mixed one-launch kernel at 3 resident blocks (<= 168 registers, no
// spills): 227 ms against 295 ms at 2 blocks for 1M uneven Duffing chains.
#ifndef ODEGB_MIN_BLOCKS_FUSED_F32
#define ODEGB_MIN_BLOCKS_FUSED_F32 3
#endif
template <class Alg, class Model, class R, int C, bool FWD = false>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? ODEGB_MIN_BLOCKS_FUSED_F32 : 1) fused_class_kernel(EnsembleArgs a) {
    static_assert(C == 2 || C == 4, "class layouts hold 2 or 4 states per lane");
    drain_class<Alg, Model, R, 64 / C, C, FWD>(a, 4);
    drain_class<Alg, Model, R, 32 / C, C, FWD>(a, 3);
    drain_class<Alg, Model, R, 16 / C, C, FWD>(a, 2);
    drain_class<Alg, Model, R, 8 / C, C, FWD>(a, 1);
    drain_class<Alg, Model, R, 4 / C, C, FWD>(a, 0);
}

}  // namespace odegb
