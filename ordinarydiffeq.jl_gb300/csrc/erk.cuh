// Explicit Runge-Kutta steps on a lane group: Tsit5 and Vern7.
//
//  Tsit5: perform_step!(::Tsit5Cache)  lib/OrdinaryDiffEqTsit5/src/tsit_perform_step.jl:309-367,
//         initialize! :293-307 (FSAL), interpolant lib/OrdinaryDiffEqTsit5/src/interpolants.jl:25-65.
//  Vern7: perform_step!(::Vern7Cache)  lib/OrdinaryDiffEqVerner/src/verner_rk_perform_step.jl:412-570
//         (lazy: extra stages only when a save falls in the step, verner_addsteps.jl:80-195),
//         interpolant lib/OrdinaryDiffEqVerner/src/interpolants.jl:183-252.
// Stage sums come from rksum.cuh: reference nesting in FP64, compensated sums
// with split coefficients in the mixed mode.
#pragma once
#include "integrator.cuh"
#include "rksum.cuh"

namespace odegb {

#define HDC __host__ __device__ static constexpr
struct Tsit5Sol {
    HDC int last() { return 6; } HDC bool m(int j) { return j >= 1 && j <= 6; }
    HDC double w(int j) { return tab::TSIT5_A(7, j); }
    HDC float whi(int j) { return tab::TSIT5_A_HI(7, j); } HDC float wlo(int j) { return tab::TSIT5_A_LO(7, j); }
};
struct Tsit5Err {
    HDC int last() { return 7; } HDC bool m(int j) { return j >= 1 && j <= 7; }
    HDC double w(int j) { return tab::TSIT5_BT(j); }
    HDC float whi(int j) { return tab::TSIT5_BT_HI(j); } HDC float wlo(int j) { return tab::TSIT5_BT_LO(j); }
};
struct Vern7Sol {
    HDC int last() { return 9; } HDC bool m(int j) { return tab::VERN7_BM(j); }
    HDC double w(int j) { return tab::VERN7_B(j); }
    HDC float whi(int j) { return tab::VERN7_B_HI(j); } HDC float wlo(int j) { return tab::VERN7_B_LO(j); }
};
struct Vern7Err {
    HDC int last() { return 10; } HDC bool m(int j) { return tab::VERN7_BTM(j); }
    HDC double w(int j) { return tab::VERN7_BT(j); }
    HDC float whi(int j) { return tab::VERN7_BT_HI(j); } HDC float wlo(int j) { return tab::VERN7_BT_LO(j); }
};
#undef HDC

// Interpolation weights b_i(theta): Horner in FP64 (the reference's @evalpoly).
template <int NPOLY, class RF>
__device__ __forceinline__ double interp_weight(double th, int i, RF r, bool first) {
    double acc = r(i, NPOLY - 1);
#pragma unroll
    for (int q = NPOLY - 2; q >= (first ? 1 : 2); --q) acc = fma(th, acc, r(i, q));
    return first ? th * acc : (th * th) * acc;
}
// Derivative weights b_i'(theta) of the reference's Val{1} interpolants: Horner
// over the coefficients times their powers (b1: @evalpoly(th, r1, 2 r2, ...);
// the others th * @evalpoly(th, 2 r2, 3 r3, ...)), in FP64.
template <int NPOLY, class RF>
__device__ __forceinline__ double interp_dweight(double th, int i, RF r, bool first) {
    double acc = (double)(NPOLY - 1) * r(i, NPOLY - 1);
#pragma unroll
    for (int q = NPOLY - 2; q >= (first ? 1 : 2); --q) acc = fma(th, acc, (double)q * r(i, q));
    return first ? acc : th * acc;
}
// Mixed form: the weights stay FP64 (a save is rare and the FP64 pipe is
// otherwise idle there; a double-float Horner measured slower on the FP32
// issue path) and are split once into float pairs for the compensated sums.
__device__ __forceinline__ ff split_weight(double w) {
    const float h = (float)w;
    return ff(h, (float)(w - (double)h));
}

// Interpolation weights of a save computed lane-parallel within a lane group.
// Every lane of a group needs the same NW weights b_q(theta) (Horner in FP64);
// on GB300 an FP64 warp instruction occupies the FP64 pipe as long with one
// active lane as with 32, so a group of L lanes evaluates them L at a time --
// lane l the weights l, l + L, ... -- and shares them by shuffles: ceil(NW/L)
// rounds of FP64 work per save instead of NW.  The arithmetic of each weight is
// the sequential form's (interp_weight), so results are unchanged.  A table row
// holds the polynomial's coefficients, read at run time by the lane that owns it.
#define ODEGB_R5(i) {tab::TSIT5_R(i, 0), tab::TSIT5_R(i, 1), tab::TSIT5_R(i, 2), tab::TSIT5_R(i, 3), tab::TSIT5_R(i, 4)}
#define ODEGB_R8(i)                                                                                      \
    {tab::VERN7_R(i, 0), tab::VERN7_R(i, 1), tab::VERN7_R(i, 2), tab::VERN7_R(i, 3), tab::VERN7_R(i, 4), \
     tab::VERN7_R(i, 5), tab::VERN7_R(i, 6), tab::VERN7_R(i, 7)}
// weight q of Tsit5 belongs to stage q + 1; Vern7's 13 weights to stages 1, 4-9, 11-16
static __device__ double kTsit5InterpR[7][5] = {ODEGB_R5(1), ODEGB_R5(2), ODEGB_R5(3), ODEGB_R5(4),
                                                ODEGB_R5(5), ODEGB_R5(6), ODEGB_R5(7)};
static __device__ double kVern7InterpR[13][8] = {ODEGB_R8(1),  ODEGB_R8(4),  ODEGB_R8(5),  ODEGB_R8(6), ODEGB_R8(7),
                                                 ODEGB_R8(8),  ODEGB_R8(9),  ODEGB_R8(11), ODEGB_R8(12),
                                                 ODEGB_R8(13), ODEGB_R8(14), ODEGB_R8(15), ODEGB_R8(16)};
#undef ODEGB_R5
#undef ODEGB_R8
template <int NPOLY>
__device__ __forceinline__ double interp_weight_row(double th, const double* r, bool first) {
    double acc = r[NPOLY - 1];
#pragma unroll
    for (int q = NPOLY - 2; q >= 2; --q) acc = fma(th, acc, r[q]);
    if (first) acc = fma(th, acc, r[1]);
    return first ? th * acc : (th * th) * acc;
}
// b[q] for q < NW as double (FP64 form) or float pairs (mixed form); row(q) the
// coefficient row of weight q; weight 0 is the `first` one (degree from 1).
template <int NW, int NPOLY, int L, class B, class Row>
__device__ __forceinline__ void group_weights(B* b, double th, const Group<L>& g, Row row) {
#pragma unroll
    for (int q0 = 0; q0 < NW; q0 += L) {
        const int q = q0 + g.lane;
        double w = 0.0;
        if (q < NW) w = interp_weight_row<NPOLY>(th, row(q), q == 0);
        if constexpr (is_double<B>::value) {
#pragma unroll
            for (int k = 0; k < L; ++k)
                if (q0 + k < NW) b[q0 + k] = g.from(w, k);
        } else {                          // float pair, split by the owning lane
            const float hi = (float)w, lo = (float)(w - (double)hi);
#pragma unroll
            for (int k = 0; k < L; ++k)
                if (q0 + k < NW) b[q0 + k] = ff(g.from(hi, k), g.from(lo, k));
        }
    }
}
struct Tsit5Alg {
    static constexpr int ORDER = 5;
    static constexpr bool IMPLICIT = false;
    template <class R, int C> struct Cache {
        R k[7][C];   // k1..k7; k1 is the FSAL value
        R tmp[C];
        double eig;  // the stiffness estimate of the last step (composite steps only)
    };
    template <class R, int C> __device__ static R* fsal_slot(Cache<R, C>& c) { return c.tmp; }

    template <class Model, class R, int L, int C>
    __device__ static void initialize(Cache<R, C>& c, const R* u, const PR<R>* p, double t, const Group<L>& g,
                                      StepStats& st, const EnsembleArgs&, long long) {
        Model::template rhs<R, L, C>(c.k[0], u, p, t, g);
        st.nf += 1;
    }
    template <class R, int C> __device__ static void on_accept(Cache<R, C>& c) {
#pragma unroll
        for (int i = 0; i < C; ++i) c.k[0][i] = c.k[6][i];
    }
    template <class R, int C> __device__ static void after_save(Cache<R, C>&) {}

    // Dense output (dense = true): the step's k1..k7, the reference's integrator.k
    // for Tsit5 (tsit_perform_step.jl:293-307).
    static constexpr int NDENSE = 7;
    template <class R, int C> __device__ static void prepare_dense(Cache<R, C>&) {}
    template <class R, int C> __device__ static R* dense_slot(Cache<R, C>& c, int q) { return c.k[q]; }

    // A callback moved or modified u: the FSAL value is f(u) again (update_fsal! ->
    // reset_fsal!, integrator_utils.jl:216-235,1326-1340; one counted call).  k7
    // becomes the next step's k1 when it starts.
    template <class Model, class R, int L, int C>
    __device__ static void reset_fsal(Cache<R, C>& c, const R* u, const R*, const PR<R>* p, double t, const Group<L>& g,
                                      StepStats& st) {
        Model::template rhs<R, L, C>(c.k[6], u, p, t, g);
        st.nf += 1;
    }

    // EIG: also the stiffness estimate of a composite step (tsit_perform_step.jl:
    // 240-246, Hairer II p. 22 with the Inf norm): max_i |(k7 - k6) / (u - g6)|,
    // g6 the sixth stage's input, NaN propagating like Julia's maximum.
    template <class Model, class R, int L, int C, bool EIG = false>
    __device__ static typename Ctl<R>::T step(Cache<R, C>& c, R* u, R* ulo, const R* up, const R* uplo,
                                             const PR<R>* p, double t, double dt, const Tol<R>& tol, long long, bool,
                                             const Group<L>& g, StepStats& st) {
        static_assert(!EIG || L == 1, "the stiffness estimate is formed on one lane");
        using K = RK<Tsit5Tab, R, C>;
        const R d = (R)dt;
        const R dl = Acc<R>::dt_lo(dt, d);
        R* tmp = c.tmp;
        R g6[EIG ? C : 1];
        K::template stage<2>(tmp, c.k, d, up, uplo);
        Model::template rhs<R, L, C>(c.k[1], tmp, p, stage_time<Model>(Tsit5Tab::c(2), dt, t), g);
        K::template stage<3>(tmp, c.k, d, up, uplo);
        Model::template rhs<R, L, C>(c.k[2], tmp, p, stage_time<Model>(Tsit5Tab::c(3), dt, t), g);
        K::template stage<4>(tmp, c.k, d, up, uplo);
        Model::template rhs<R, L, C>(c.k[3], tmp, p, stage_time<Model>(Tsit5Tab::c(4), dt, t), g);
        K::template stage<5>(tmp, c.k, d, up, uplo);
        Model::template rhs<R, L, C>(c.k[4], tmp, p, stage_time<Model>(Tsit5Tab::c(5), dt, t), g);
        K::template stage<6>(tmp, c.k, d, up, uplo);
        if constexpr (EIG) {
#pragma unroll
            for (int i = 0; i < C; ++i) g6[i] = tmp[i];
        }
        Model::template rhs<R, L, C>(c.k[5], tmp, p, stage_time<Model>(1.0, dt, t), g);
        K::weights(tmp, c.k, Tsit5Sol());
#pragma unroll
        for (int i = 0; i < C; ++i) Acc<R>::update2(u[i], ulo[i], d, dl, tmp[i], up[i], uplo[i]);
        Model::template rhs<R, L, C>(c.k[6], u, p, stage_time<Model>(1.0, dt, t), g);
        st.nf += 6;
        if constexpr (EIG) {
            double e = 0.0;
#pragma unroll
            for (int i = 0; i < C; ++i) {
                const double v = fabs((double)(c.k[6][i] - c.k[5][i]) / (double)(u[i] - g6[i]));
                e = (e != e || v != v) ? dnan() : (v > e ? v : e);
            }
            c.eig = e;
        }
        K::weights(tmp, c.k, Tsit5Err());
#pragma unroll
        for (int i = 0; i < C; ++i) tmp[i] = d * tmp[i];
        return error_norm<R, L, C>(tmp, up, u, tol, g);
    }

    template <class Model, class R, int L, int C>
    __device__ static void interpolate(Cache<R, C>& c, R* out, R* outlo, double th, double dt, double,
                                       const R* y0, const R* y0lo, const R*, const R*, const PR<R>*,
                                       const Group<L>& g) {
        auto r = [](int i, int q) { return tab::TSIT5_R(i, q); };
        const R d = (R)dt;
        if constexpr (sizeof(R) == 8) {
            double b[8];
            if constexpr (L > 1) {
                group_weights<7, 5, L>(b + 1, th, g, [](int q) { return (const double*)kTsit5InterpR[q]; });
            } else {
                b[1] = interp_weight<5>(th, 1, r, true);
#pragma unroll
                for (int i = 2; i <= 7; ++i) b[i] = interp_weight<5>(th, i, r, false);
            }
#pragma unroll
            for (int i = 0; i < C; ++i) {
                R acc = c.k[6][i] * (R)b[7];
#pragma unroll
                for (int s = 6; s >= 1; --s) acc = FMA(c.k[s - 1][i], (R)b[s], acc);
                Acc<R>::update(out[i], outlo[i], d, acc, y0[i], y0lo[i]);
            }
        } else {
            const R dl = Acc<R>::dt_lo(dt, d);
            ff b[8];
            if constexpr (L > 1) {
                group_weights<7, 5, L>(b + 1, th, g, [](int q) { return (const double*)kTsit5InterpR[q]; });
            } else {
                b[1] = split_weight(interp_weight<5>((double)th, 1, r, true));
#pragma unroll
                for (int i = 2; i <= 7; ++i) b[i] = split_weight(interp_weight<5>((double)th, i, r, false));
            }
#pragma unroll
            for (int i = 0; i < C; ++i) {
                CSum cs;
#pragma unroll
                for (int s = 1; s <= 7; ++s) cs.add_pair(b[s].hi, b[s].lo, (float)c.k[s - 1][i]);
                Acc<R>::update2(out[i], outlo[i], d, dl, (R)cs.value(), y0[i], y0lo[i]);
            }
        }
    }
};

// sol(t, Val{1}) of a Tsit5 step (interpolants.jl:143-178): sum_i k_i b_i'(theta),
// FP64 (the dense-output evaluation).
template <int C>
__device__ __forceinline__ void tsit5_derivative(const double (*k)[C], double th, double* out) {
    auto r = [](int i, int q) { return tab::TSIT5_R(i, q); };
    double b[8];
    b[1] = interp_dweight<5>(th, 1, r, true);
#pragma unroll
    for (int i = 2; i <= 7; ++i) b[i] = interp_dweight<5>(th, i, r, false);
#pragma unroll
    for (int i = 0; i < C; ++i) {
        double acc = k[6][i] * b[7];
#pragma unroll
        for (int s = 6; s >= 1; --s) acc = fma(k[s - 1][i], b[s], acc);
        out[i] = acc;
    }
}

// Tsit5's second derivative (interpolants.jl: tsit5pre2, the Val{2} form):
// (sum_i k_i b_i''(th)) / dt with b_i'' = evalpoly(th, 2 r_i2, 6 r_i3, 12 r_i4).
template <int C>
__device__ __forceinline__ void tsit5_second_derivative(const double (*k)[C], double th, double dt, double* out) {
    double b[8];
#pragma unroll
    for (int i = 1; i <= 7; ++i)
        b[i] = fma(th, fma(th, 12.0 * tab::TSIT5_R(i, 4), 6.0 * tab::TSIT5_R(i, 3)), 2.0 * tab::TSIT5_R(i, 2));
    const double invdt = 1.0 / dt;
#pragma unroll
    for (int i = 0; i < C; ++i) {
        double acc = k[6][i] * b[7];
#pragma unroll
        for (int s = 6; s >= 1; --s) acc = fma(k[s - 1][i], b[s], acc);
        out[i] = acc * invdt;
    }
}

// Tsit5's third derivative (tsit5pre3, the Val{3} form): (sum_i k_i b_i'''(th)) /
// dt^2 with b_i''' = evalpoly(th, 6 r_i3, 24 r_i4) and inv(dt)^2.
template <int C>
__device__ __forceinline__ void tsit5_third_derivative(const double (*k)[C], double th, double dt, double* out) {
    double b[8];
#pragma unroll
    for (int i = 1; i <= 7; ++i) b[i] = fma(th, 24.0 * tab::TSIT5_R(i, 4), 6.0 * tab::TSIT5_R(i, 3));
    const double invdt = 1.0 / dt, invdt2 = invdt * invdt;
#pragma unroll
    for (int i = 0; i < C; ++i) {
        double acc = k[6][i] * b[7];
#pragma unroll
        for (int s = 6; s >= 1; --s) acc = fma(k[s - 1][i], b[s], acc);
        out[i] = acc * invdt2;
    }
}

struct Vern7Alg {
    static constexpr int ORDER = 7;
    static constexpr bool IMPLICIT = false;
    template <class R, int C> struct Cache {
        R s[13][C];   // slots, see Vern7Tab::slot
        R tmp[C];
        bool extra;
    };
    template <class R, int C> __device__ static R* fsal_slot(Cache<R, C>& c) { return c.tmp; }
    template <class Model, class R, int L, int C>
    __device__ static void initialize(Cache<R, C>& c, const R*, const PR<R>*, double, const Group<L>&, StepStats&,
                                      const EnsembleArgs&, long long) {
        c.extra = false;
    }
    template <class R, int C> __device__ static void on_accept(Cache<R, C>&) {}
    template <class R, int C> __device__ static void after_save(Cache<R, C>& c) { c.extra = false; }

    // Dense output: k1, k4..k9, the stages that the interpolant and the lazy extra
    // stages read (interpolants.jl:183-252, verner_addsteps.jl:137-193); of the
    // reference's integrator.k[1..10], k2, k3 and k10 are read by neither.
    static constexpr int NDENSE = 7;
    __host__ __device__ static constexpr int dense_stage(int q) { return q == 0 ? 1 : q + 3; }
    template <class R, int C> __device__ static void prepare_dense(Cache<R, C>&) {}
    template <class R, int C> __device__ static R* dense_slot(Cache<R, C>& c, int q) {
        return c.s[Vern7Tab::slot(dense_stage(q))];
    }

    template <int ROW, class Model, class R, int L, int C>
    __device__ static void eval_stage(Cache<R, C>& c, const R* up, const R* uplo, const PR<R>* p, double tstage, R d,
                                      const Group<L>& g) {
        RK<Vern7Tab, R, C>::template stage<ROW>(c.tmp, c.s, d, up, uplo);
        Model::template rhs<R, L, C>(c.s[Vern7Tab::slot(ROW)], c.tmp, p, tstage, g);
    }

    template <class Model, class R, int L, int C>
    __device__ static typename Ctl<R>::T step(Cache<R, C>& c, R* u, R* ulo, const R* up, const R* uplo,
                                             const PR<R>* p, double t, double dt, const Tol<R>& tol, long long, bool,
                                             const Group<L>& g, StepStats& st) {
        const R d = (R)dt;
        c.extra = false;
        Model::template rhs<R, L, C>(c.s[0], up, p, t, g);
        eval_stage<2, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(2), dt, t), d, g);
        eval_stage<3, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(3), dt, t), d, g);
        eval_stage<4, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(4), dt, t), d, g);
        eval_stage<5, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(5), dt, t), d, g);
        eval_stage<6, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(6), dt, t), d, g);
        eval_stage<7, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(7), dt, t), d, g);
        eval_stage<8, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(8), dt, t), d, g);
        eval_stage<9, Model>(c, up, uplo, p, stage_time<Model>(1.0, dt, t), d, g);
        eval_stage<10, Model>(c, up, uplo, p, stage_time<Model>(1.0, dt, t), d, g);
        RK<Vern7Tab, R, C>::weights(c.tmp, c.s, Vern7Sol());
        const R dl = Acc<R>::dt_lo(dt, d);
#pragma unroll
        for (int i = 0; i < C; ++i) Acc<R>::update2(u[i], ulo[i], d, dl, c.tmp[i], up[i], uplo[i]);
        st.nf += 10;
        RK<Vern7Tab, R, C>::weights(c.tmp, c.s, Vern7Err());
#pragma unroll
        for (int i = 0; i < C; ++i) c.tmp[i] = d * c.tmp[i];
        return error_norm<R, L, C>(c.tmp, up, u, tol, g);
    }

    // Extra stages k11..k16 (verner_addsteps.jl:80-195) at (tprev, uprev, dt).
    template <class Model, class R, int L, int C>
    __device__ static void extra_stages(Cache<R, C>& c, double tprev, double dt, const R* up, const R* uplo,
                                        const PR<R>* p, const Group<L>& g) {
        const R d = (R)dt;
        eval_stage<11, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(11), dt, tprev), d, g);
        eval_stage<12, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(12), dt, tprev), d, g);
        eval_stage<13, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(13), dt, tprev), d, g);
        eval_stage<14, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(14), dt, tprev), d, g);
        eval_stage<15, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(15), dt, tprev), d, g);
        eval_stage<16, Model>(c, up, uplo, p, stage_time<Model>(Vern7Tab::c(16), dt, tprev), d, g);
        c.extra = true;
    }

    // not FSAL (isfsal(::Vern7) = false): nothing to redo after a callback
    template <class Model, class R, int L, int C>
    __device__ static void reset_fsal(Cache<R, C>&, const R*, const R*, const PR<R>*, double, const Group<L>&,
                                      StepStats&) {}

    template <class Model, class R, int L, int C>
    __device__ static void interpolate(Cache<R, C>& c, R* out, R* outlo, double th, double dt,
                                       double tprev, const R* y0, const R* y0lo, const R*, const R*, const PR<R>* p,
                                       const Group<L>& g) {
        if (!c.extra) extra_stages<Model, R, L, C>(c, tprev, dt, y0, y0lo, p, g);
        // stages of the 7th-order interpolant, in the reference's summation order
        constexpr int idx[13] = {1, 4, 5, 6, 7, 8, 9, 11, 12, 13, 14, 15, 16};
        auto r = [](int i, int q) { return tab::VERN7_R(i, q); };
        const R d = (R)dt;
        if constexpr (sizeof(R) == 8) {
            double b[13];
            if constexpr (L > 1) {
                group_weights<13, 8, L>(b, th, g, [](int q) { return (const double*)kVern7InterpR[q]; });
            } else {
                b[0] = interp_weight<8>(th, 1, r, true);
#pragma unroll
                for (int q = 1; q < 13; ++q) b[q] = interp_weight<8>(th, idx[q], r, false);
            }
#pragma unroll
            for (int i = 0; i < C; ++i) {
                R acc = c.s[Vern7Tab::slot(16)][i] * (R)b[12];
#pragma unroll
                for (int q = 11; q >= 0; --q) acc = FMA(c.s[Vern7Tab::slot(idx[q])][i], (R)b[q], acc);
                Acc<R>::update(out[i], outlo[i], d, acc, y0[i], y0lo[i]);
            }
        } else {
            const R dl = Acc<R>::dt_lo(dt, d);
            ff b[13];
            if constexpr (L > 1) {
                group_weights<13, 8, L>(b, th, g, [](int q) { return (const double*)kVern7InterpR[q]; });
            } else {
                b[0] = split_weight(interp_weight<8>((double)th, 1, r, true));
#pragma unroll
                for (int q = 1; q < 13; ++q) b[q] = split_weight(interp_weight<8>((double)th, idx[q], r, false));
            }
#pragma unroll
            for (int i = 0; i < C; ++i) {
                CSum cs;
#pragma unroll
                for (int q = 0; q < 13; ++q) cs.add_pair(b[q].hi, b[q].lo, (float)c.s[Vern7Tab::slot(idx[q])][i]);
                Acc<R>::update2(out[i], outlo[i], d, dl, (R)cs.value(), y0[i], y0lo[i]);
            }
        }
    }

    // sol(t, Val{1}) (interpolants.jl:305-334): sum over the 13 stages of k_s b_s'(theta),
    // the extra stages formed first; FP64 (the dense-output evaluation).
    template <class Model, int L, int C>
    __device__ static void derivative(Cache<double, C>& c, double* out, double th, double dt, double tprev,
                                      const double* y0, const double* y0lo, const double* p, const Group<L>& g) {
        if (!c.extra) extra_stages<Model, double, L, C>(c, tprev, dt, y0, y0lo, p, g);
        constexpr int idx[13] = {1, 4, 5, 6, 7, 8, 9, 11, 12, 13, 14, 15, 16};
        auto r = [](int i, int q) { return tab::VERN7_R(i, q); };
        double b[13];
        b[0] = interp_dweight<8>(th, 1, r, true);
#pragma unroll
        for (int q = 1; q < 13; ++q) b[q] = interp_dweight<8>(th, idx[q], r, false);
#pragma unroll
        for (int i = 0; i < C; ++i) {
            double acc = c.s[Vern7Tab::slot(16)][i] * b[12];
#pragma unroll
            for (int q = 11; q >= 0; --q) acc = fma(c.s[Vern7Tab::slot(idx[q])][i], b[q], acc);
            out[i] = acc;
        }
    }
};

}  // namespace odegb
