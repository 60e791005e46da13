// Explicit Runge-Kutta steps on a lane group: Tsit5 and Vern7.
//
//  Tsit5: perform_step!(::Tsit5Cache)  lib/OrdinaryDiffEqTsit5/src/tsit_perform_step.jl:309-367,
//         initialize! :293-307 (FSAL), interpolant lib/OrdinaryDiffEqTsit5/src/interpolants.jl:25-65.
//  Vern7: perform_step!(::Vern7Cache)  lib/OrdinaryDiffEqVerner/src/verner_rk_perform_step.jl:412-570
//         (lazy: extra stages only when a save falls in the step, verner_addsteps.jl:80-195),
//         interpolant lib/OrdinaryDiffEqVerner/src/interpolants.jl:183-252.
// Stage sums use the reference's @muladd nesting: uprev + dt*(a1 k1 + ... + am km)
// = fma(dt, fma(a1,k1, fma(a2,k2, ... am*km)), uprev).
#pragma once
#include "integrator.cuh"
#include "tableaus.h"

namespace odegb {

#define T_(x) ((R)(tab::x))

struct Tsit5Alg {
    static constexpr int ORDER = 5;
    static constexpr bool IMPLICIT = false;
    template <class R, int C> struct Cache {
        R k[7][C];   // k1..k7; k1 is the FSAL value
        R tmp[C];
    };
    template <class R, int C> __device__ static R* fsal_slot(Cache<R, C>& c) { return c.tmp; }

    template <class Model, class R, int L, int C>
    __device__ static void initialize(Cache<R, C>& c, const R* u, const R* p, double t, const Group<L>& g,
                                      StepStats& st, const EnsembleArgs&) {
        Model::template rhs<R, L, C>(c.k[0], u, p, t, g);
        st.nf += 1;
    }
    template <class R, int C> __device__ static void on_accept(Cache<R, C>& c) {
#pragma unroll
        for (int i = 0; i < C; ++i) c.k[0][i] = c.k[6][i];
    }
    template <class R, int C> __device__ static void after_save(Cache<R, C>&) {}

    template <class Model, class R, int L, int C>
    __device__ static double step(Cache<R, C>& c, R* u, const R* up, const R* p, double t, double dt,
                                  R abstol, R reltol, long long, double, const Group<L>& g, StepStats& st) {
        const R d = (R)dt;
        R (*k)[C] = c.k;
        R* tmp = c.tmp;
        const R a = d * T_(TSIT5_a21);
#pragma unroll
        for (int i = 0; i < C; ++i) tmp[i] = FMA(a, k[0][i], up[i]);
        Model::template rhs<R, L, C>(k[1], tmp, p, fma(tab::TSIT5_c1, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i) tmp[i] = FMA(d, FMA(T_(TSIT5_a31), k[0][i], T_(TSIT5_a32) * k[1][i]), up[i]);
        Model::template rhs<R, L, C>(k[2], tmp, p, fma(tab::TSIT5_c2, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(TSIT5_a41), k[0][i], FMA(T_(TSIT5_a42), k[1][i], T_(TSIT5_a43) * k[2][i])), up[i]);
        Model::template rhs<R, L, C>(k[3], tmp, p, fma(tab::TSIT5_c3, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(TSIT5_a51), k[0][i], FMA(T_(TSIT5_a52), k[1][i],
                          FMA(T_(TSIT5_a53), k[2][i], T_(TSIT5_a54) * k[3][i]))), up[i]);
        Model::template rhs<R, L, C>(k[4], tmp, p, fma(tab::TSIT5_c4, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(TSIT5_a61), k[0][i], FMA(T_(TSIT5_a62), k[1][i], FMA(T_(TSIT5_a63), k[2][i],
                          FMA(T_(TSIT5_a64), k[3][i], T_(TSIT5_a65) * k[4][i])))), up[i]);
        Model::template rhs<R, L, C>(k[5], tmp, p, t + dt, g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            u[i] = FMA(d, FMA(T_(TSIT5_a71), k[0][i], FMA(T_(TSIT5_a72), k[1][i], FMA(T_(TSIT5_a73), k[2][i],
                       FMA(T_(TSIT5_a74), k[3][i], FMA(T_(TSIT5_a75), k[4][i], T_(TSIT5_a76) * k[5][i]))))), up[i]);
        Model::template rhs<R, L, C>(k[6], u, p, t + dt, g);
        st.nf += 6;
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = d * FMA(T_(TSIT5_btilde1), k[0][i], FMA(T_(TSIT5_btilde2), k[1][i], FMA(T_(TSIT5_btilde3), k[2][i],
                         FMA(T_(TSIT5_btilde4), k[3][i], FMA(T_(TSIT5_btilde5), k[4][i],
                         FMA(T_(TSIT5_btilde6), k[5][i], T_(TSIT5_btilde7) * k[6][i]))))));
        return error_norm<R, L, C>(tmp, up, u, abstol, reltol, g);
    }

    template <class Model, class R, int L, int C>
    __device__ static void interpolate(Cache<R, C>& c, R* out, double thd, double dt, double, const R* y0, const R*,
                                       const R*, const Group<L>&) {
        const R th = (R)thd, th2 = th * th, d = (R)dt;
        const R b1 = th * FMA(th, FMA(th, FMA(th, T_(TSIT5I_r14), T_(TSIT5I_r13)), T_(TSIT5I_r12)), T_(TSIT5I_r11));
        const R b2 = th2 * FMA(th, FMA(th, T_(TSIT5I_r24), T_(TSIT5I_r23)), T_(TSIT5I_r22));
        const R b3 = th2 * FMA(th, FMA(th, T_(TSIT5I_r34), T_(TSIT5I_r33)), T_(TSIT5I_r32));
        const R b4 = th2 * FMA(th, FMA(th, T_(TSIT5I_r44), T_(TSIT5I_r43)), T_(TSIT5I_r42));
        const R b5 = th2 * FMA(th, FMA(th, T_(TSIT5I_r54), T_(TSIT5I_r53)), T_(TSIT5I_r52));
        const R b6 = th2 * FMA(th, FMA(th, T_(TSIT5I_r64), T_(TSIT5I_r63)), T_(TSIT5I_r62));
        const R b7 = th2 * FMA(th, FMA(th, T_(TSIT5I_r74), T_(TSIT5I_r73)), T_(TSIT5I_r72));
        R (*k)[C] = c.k;
#pragma unroll
        for (int i = 0; i < C; ++i)
            out[i] = FMA(d, FMA(k[0][i], b1, FMA(k[1][i], b2, FMA(k[2][i], b3, FMA(k[3][i], b4,
                          FMA(k[4][i], b5, FMA(k[5][i], b6, k[6][i] * b7)))))), y0[i]);
    }
};

struct Vern7Alg {
    static constexpr int ORDER = 7;
    static constexpr bool IMPLICIT = false;
    // Slots: k1..k10 in s[0..9]; on a save step the extra stages k11..k16 are
    // computed into s[1], s[2], s[9] (k2, k3, k10 are not used by the
    // interpolant or the extra stages) and s[10..12].
    template <class R, int C> struct Cache {
        R s[13][C];
        R tmp[C];
        bool extra;
    };
    template <class R, int C> __device__ static R* fsal_slot(Cache<R, C>& c) { return c.tmp; }
    template <class Model, class R, int L, int C>
    __device__ static void initialize(Cache<R, C>& c, const R*, const R*, double, const Group<L>&, StepStats&,
                                      const EnsembleArgs&) {
        c.extra = false;
    }
    template <class R, int C> __device__ static void on_accept(Cache<R, C>&) {}
    template <class R, int C> __device__ static void after_save(Cache<R, C>& c) { c.extra = false; }

    template <class Model, class R, int L, int C>
    __device__ static double step(Cache<R, C>& c, R* u, const R* up, const R* p, double t, double dt,
                                  R abstol, R reltol, long long, double, const Group<L>& g, StepStats& st) {
        const R d = (R)dt;
        R (*k)[C] = c.s;
        R* tmp = c.tmp;
        c.extra = false;
        Model::template rhs<R, L, C>(k[0], up, p, t, g);
        const R a = d * T_(VERN7_a021);
#pragma unroll
        for (int i = 0; i < C; ++i) tmp[i] = FMA(a, k[0][i], up[i]);
        Model::template rhs<R, L, C>(k[1], tmp, p, fma(tab::VERN7_c2, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i) tmp[i] = FMA(d, FMA(T_(VERN7_a031), k[0][i], T_(VERN7_a032) * k[1][i]), up[i]);
        Model::template rhs<R, L, C>(k[2], tmp, p, fma(tab::VERN7_c3, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i) tmp[i] = FMA(d, FMA(T_(VERN7_a041), k[0][i], T_(VERN7_a043) * k[2][i]), up[i]);
        Model::template rhs<R, L, C>(k[3], tmp, p, fma(tab::VERN7_c4, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7_a051), k[0][i], FMA(T_(VERN7_a053), k[2][i], T_(VERN7_a054) * k[3][i])), up[i]);
        Model::template rhs<R, L, C>(k[4], tmp, p, fma(tab::VERN7_c5, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7_a061), k[0][i], FMA(T_(VERN7_a063), k[2][i], FMA(T_(VERN7_a064), k[3][i],
                          T_(VERN7_a065) * k[4][i]))), up[i]);
        Model::template rhs<R, L, C>(k[5], tmp, p, fma(tab::VERN7_c6, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7_a071), k[0][i], FMA(T_(VERN7_a073), k[2][i], FMA(T_(VERN7_a074), k[3][i],
                          FMA(T_(VERN7_a075), k[4][i], T_(VERN7_a076) * k[5][i])))), up[i]);
        Model::template rhs<R, L, C>(k[6], tmp, p, fma(tab::VERN7_c7, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7_a081), k[0][i], FMA(T_(VERN7_a083), k[2][i], FMA(T_(VERN7_a084), k[3][i],
                          FMA(T_(VERN7_a085), k[4][i], FMA(T_(VERN7_a086), k[5][i], T_(VERN7_a087) * k[6][i]))))), up[i]);
        Model::template rhs<R, L, C>(k[7], tmp, p, fma(tab::VERN7_c8, dt, t), g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7_a091), k[0][i], FMA(T_(VERN7_a093), k[2][i], FMA(T_(VERN7_a094), k[3][i],
                          FMA(T_(VERN7_a095), k[4][i], FMA(T_(VERN7_a096), k[5][i], FMA(T_(VERN7_a097), k[6][i],
                          T_(VERN7_a098) * k[7][i])))))), up[i]);
        Model::template rhs<R, L, C>(k[8], tmp, p, t + dt, g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7_a101), k[0][i], FMA(T_(VERN7_a103), k[2][i], FMA(T_(VERN7_a104), k[3][i],
                          FMA(T_(VERN7_a105), k[4][i], FMA(T_(VERN7_a106), k[5][i], T_(VERN7_a107) * k[6][i]))))), up[i]);
        Model::template rhs<R, L, C>(k[9], tmp, p, t + dt, g);
#pragma unroll
        for (int i = 0; i < C; ++i)
            u[i] = FMA(d, FMA(T_(VERN7_b1), k[0][i], FMA(T_(VERN7_b4), k[3][i], FMA(T_(VERN7_b5), k[4][i],
                       FMA(T_(VERN7_b6), k[5][i], FMA(T_(VERN7_b7), k[6][i], FMA(T_(VERN7_b8), k[7][i],
                       T_(VERN7_b9) * k[8][i])))))), up[i]);
        st.nf += 10;
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = d * FMA(T_(VERN7_btilde1), k[0][i], FMA(T_(VERN7_btilde4), k[3][i], FMA(T_(VERN7_btilde5), k[4][i],
                         FMA(T_(VERN7_btilde6), k[5][i], FMA(T_(VERN7_btilde7), k[6][i], FMA(T_(VERN7_btilde8), k[7][i],
                         FMA(T_(VERN7_btilde9), k[8][i], T_(VERN7_btilde10) * k[9][i])))))));
        return error_norm<R, L, C>(tmp, up, u, abstol, reltol, g);
    }

    // Extra stages k11..k16 (verner_addsteps.jl:80-195) at (tprev, uprev, dt).
    template <class Model, class R, int L, int C>
    __device__ static void extra_stages(Cache<R, C>& c, double tprev, double dt, const R* up, const R* p,
                                        const Group<L>& g) {
        const R d = (R)dt;
        R (*k)[C] = c.s;
        R* tmp = c.tmp;
        // k11 -> s[1]
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7X_a1101), k[0][i], FMA(T_(VERN7X_a1104), k[3][i], FMA(T_(VERN7X_a1105), k[4][i],
                          FMA(T_(VERN7X_a1106), k[5][i], FMA(T_(VERN7X_a1107), k[6][i], FMA(T_(VERN7X_a1108), k[7][i],
                          T_(VERN7X_a1109) * k[8][i])))))), up[i]);
        Model::template rhs<R, L, C>(k[1], tmp, p, fma(tab::VERN7X_c11, dt, tprev), g);
        // k12 -> s[2]
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7X_a1201), k[0][i], FMA(T_(VERN7X_a1204), k[3][i], FMA(T_(VERN7X_a1205), k[4][i],
                          FMA(T_(VERN7X_a1206), k[5][i], FMA(T_(VERN7X_a1207), k[6][i], FMA(T_(VERN7X_a1208), k[7][i],
                          FMA(T_(VERN7X_a1209), k[8][i], T_(VERN7X_a1211) * k[1][i]))))))), up[i]);
        Model::template rhs<R, L, C>(k[2], tmp, p, fma(tab::VERN7X_c12, dt, tprev), g);
        // k13 -> s[9]
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7X_a1301), k[0][i], FMA(T_(VERN7X_a1304), k[3][i], FMA(T_(VERN7X_a1305), k[4][i],
                          FMA(T_(VERN7X_a1306), k[5][i], FMA(T_(VERN7X_a1307), k[6][i], FMA(T_(VERN7X_a1308), k[7][i],
                          FMA(T_(VERN7X_a1309), k[8][i], FMA(T_(VERN7X_a1311), k[1][i], T_(VERN7X_a1312) * k[2][i])))))))), up[i]);
        Model::template rhs<R, L, C>(k[9], tmp, p, fma(tab::VERN7X_c13, dt, tprev), g);
        // k14 -> s[10]
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7X_a1401), k[0][i], FMA(T_(VERN7X_a1404), k[3][i], FMA(T_(VERN7X_a1405), k[4][i],
                          FMA(T_(VERN7X_a1406), k[5][i], FMA(T_(VERN7X_a1407), k[6][i], FMA(T_(VERN7X_a1408), k[7][i],
                          FMA(T_(VERN7X_a1409), k[8][i], FMA(T_(VERN7X_a1411), k[1][i], FMA(T_(VERN7X_a1412), k[2][i],
                          T_(VERN7X_a1413) * k[9][i]))))))))), up[i]);
        Model::template rhs<R, L, C>(k[10], tmp, p, fma(tab::VERN7X_c14, dt, tprev), g);
        // k15 -> s[11]
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7X_a1501), k[0][i], FMA(T_(VERN7X_a1504), k[3][i], FMA(T_(VERN7X_a1505), k[4][i],
                          FMA(T_(VERN7X_a1506), k[5][i], FMA(T_(VERN7X_a1507), k[6][i], FMA(T_(VERN7X_a1508), k[7][i],
                          FMA(T_(VERN7X_a1509), k[8][i], FMA(T_(VERN7X_a1511), k[1][i], FMA(T_(VERN7X_a1512), k[2][i],
                          T_(VERN7X_a1513) * k[9][i]))))))))), up[i]);
        Model::template rhs<R, L, C>(k[11], tmp, p, fma(tab::VERN7X_c15, dt, tprev), g);
        // k16 -> s[12]
#pragma unroll
        for (int i = 0; i < C; ++i)
            tmp[i] = FMA(d, FMA(T_(VERN7X_a1601), k[0][i], FMA(T_(VERN7X_a1604), k[3][i], FMA(T_(VERN7X_a1605), k[4][i],
                          FMA(T_(VERN7X_a1606), k[5][i], FMA(T_(VERN7X_a1607), k[6][i], FMA(T_(VERN7X_a1608), k[7][i],
                          FMA(T_(VERN7X_a1609), k[8][i], FMA(T_(VERN7X_a1611), k[1][i], FMA(T_(VERN7X_a1612), k[2][i],
                          T_(VERN7X_a1613) * k[9][i]))))))))), up[i]);
        Model::template rhs<R, L, C>(k[12], tmp, p, fma(tab::VERN7X_c16, dt, tprev), g);
        c.extra = true;
    }

    template <class R>
    __device__ static R poly6(R th, R r2, R r3, R r4, R r5, R r6, R r7) {
        return FMA(th, FMA(th, FMA(th, FMA(th, FMA(th, r7, r6), r5), r4), r3), r2);
    }

    template <class Model, class R, int L, int C>
    __device__ static void interpolate(Cache<R, C>& c, R* out, double thd, double dt, double tprev, const R* y0,
                                       const R*, const R* p, const Group<L>& g) {
        if (!c.extra) extra_stages<Model, R, L, C>(c, tprev, dt, y0, p, g);
        const R th = (R)thd, th2 = th * th, d = (R)dt;
        const R b1 = th * FMA(th, poly6<R>(th, T_(VERN7I_r012), T_(VERN7I_r013), T_(VERN7I_r014), T_(VERN7I_r015),
                                          T_(VERN7I_r016), T_(VERN7I_r017)), T_(VERN7I_r011));
#define VB(S) th2 * poly6<R>(th, T_(VERN7I_r##S##2), T_(VERN7I_r##S##3), T_(VERN7I_r##S##4), T_(VERN7I_r##S##5), \
                              T_(VERN7I_r##S##6), T_(VERN7I_r##S##7))
        const R b4 = VB(04), b5 = VB(05), b6 = VB(06), b7 = VB(07), b8 = VB(08), b9 = VB(09);
        const R b11 = VB(11), b12 = VB(12), b13 = VB(13), b14 = VB(14), b15 = VB(15), b16 = VB(16);
#undef VB
        R (*k)[C] = c.s;
#pragma unroll
        for (int i = 0; i < C; ++i)
            out[i] = FMA(d, FMA(k[0][i], b1, FMA(k[3][i], b4, FMA(k[4][i], b5, FMA(k[5][i], b6, FMA(k[6][i], b7,
                          FMA(k[7][i], b8, FMA(k[8][i], b9, FMA(k[1][i], b11, FMA(k[2][i], b12, FMA(k[9][i], b13,
                          FMA(k[10][i], b14, FMA(k[11][i], b15, k[12][i] * b16)))))))))))), y0[i]);
    }
};

#undef T_

}  // namespace odegb
