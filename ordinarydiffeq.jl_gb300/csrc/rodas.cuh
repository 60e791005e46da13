// Rodas5P on one lane per trajectory (small systems, W kept in registers).
//
//  perform_step!(::RosenbrockCache)  lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_perform_step.jl:729-847
//      fused accumulation helpers :581-727 (acc = base; acc = muladd(c_i, k_i, acc), left to right)
//  tableau                            lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:23-72
//  W = J - I/(dt*gamma)               lib/OrdinaryDiffEqDifferentiation/src/derivative_utils.jl:663-685
//  J reuse after a rejected step      derivative_utils.jl:535-557 (do_newJW), :1011-1041
//  time derivative                    derivative_utils.jl:181-227 (models are autonomous: dT = 0;
//                                     the reference's AD evaluation is counted as one f call)
//  interpolant (order 3)              rosenbrock_interpolants.jl:172-206
// The LU is Doolittle with partial pivoting (largest |pivot|, first on ties),
// the same algorithm the CPU oracle states; LinearSolve's LU (not vendored)
// pivots the same way.
//
// Mixed precision (R = float): J, W and the LU are FP32; every solve W x = b
// is followed by `a.ir_sweeps` refinement sweeps whose residual b - W x is
// formed in FP64 from an FP64 copy of W.
#pragma once
#include "integrator.cuh"
#include "tableaus.h"

namespace odegb {

template <class R, int N>
__device__ __forceinline__ void lu_factor_reg(R (*W)[N], int* piv) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
        int pr = c;
        R best = ABS(W[c][c]);
#pragma unroll
        for (int r = c + 1; r < N; ++r) {
            R v = ABS(W[r][c]);
            if (v > best) { best = v; pr = r; }
        }
        piv[c] = pr;
#pragma unroll
        for (int r = c + 1; r < N; ++r) {
            bool sw = (pr == r);
#pragma unroll
            for (int j = 0; j < N; ++j) {
                R a = W[c][j], b = W[r][j];
                W[c][j] = sw ? b : a;
                W[r][j] = sw ? a : b;
            }
        }
        R dgn = W[c][c];
        if (dgn != R(0)) {
            R inv = R(1) / dgn;
#pragma unroll
            for (int r = c + 1; r < N; ++r) {
                R l = W[r][c] * inv;
                W[r][c] = l;
#pragma unroll
                for (int j = c + 1; j < N; ++j) W[r][j] = FMA(-l, W[c][j], W[r][j]);
            }
        }
    }
}

template <class R, int N>
__device__ __forceinline__ void lu_solve_reg(const R (*LU)[N], const int* piv, R* b) {
#pragma unroll
    for (int c = 0; c < N; ++c) {
#pragma unroll
        for (int r = c + 1; r < N; ++r) {
            bool sw = (piv[c] == r);
            R x = b[c], y = b[r];
            b[c] = sw ? y : x;
            b[r] = sw ? x : y;
        }
    }
#pragma unroll
    for (int r = 1; r < N; ++r) {
        R acc = b[r];
#pragma unroll
        for (int j = 0; j < r; ++j) acc = FMA(-LU[r][j], b[j], acc);
        b[r] = acc;
    }
#pragma unroll
    for (int r = N - 1; r >= 0; --r) {
        R acc = b[r];
#pragma unroll
        for (int j = r + 1; j < N; ++j) acc = FMA(-LU[r][j], b[j], acc);
        b[r] = acc / LU[r][r];
    }
}

#define RP_(x) ((R)(tab::x))

struct Rodas5PAlg {
    static constexpr int ORDER = 5;
    static constexpr bool IMPLICIT = true;
    template <class R, int C> struct Cache {
        R J[C][C];
        R W[C][C];
        int piv[C];
        R ks[8][C];
        R dk[3][C];   // dense k1..k3
        R scratch[C];
        bool haveJ;
        int ir;
    };
    template <class R, int C> __device__ static R* fsal_slot(Cache<R, C>& c) { return c.scratch; }
    template <class Model, class R, int L, int C>
    __device__ static void initialize(Cache<R, C>& c, const R*, const R*, double, const Group<L>&, StepStats&,
                                      const EnsembleArgs& a) {
        c.haveJ = false;
        c.ir = a.ir_sweeps;
    }
    template <class R, int C> __device__ static void on_accept(Cache<R, C>&) {}
    template <class R, int C> __device__ static void after_save(Cache<R, C>&) {}

    // Solve W x = b in place (b -> x), with FP64-residual refinement in mixed mode.
    template <class R, int C>
    __device__ static void wsolve(Cache<R, C>& c, R* b, double invdtgamma, int sweeps) {
        if (sizeof(R) == 8 || sweeps <= 0) {
            lu_solve_reg<R, C>(c.W, c.piv, b);
            return;
        }
        double b64[C];
#pragma unroll
        for (int i = 0; i < C; ++i) b64[i] = (double)b[i];
        lu_solve_reg<R, C>(c.W, c.piv, b);
        double x[C];
#pragma unroll
        for (int i = 0; i < C; ++i) x[i] = (double)b[i];
        for (int s = 0; s < sweeps; ++s) {
            R r[C];
#pragma unroll
            for (int i = 0; i < C; ++i) {
                double acc = b64[i];
#pragma unroll
                for (int j = 0; j < C; ++j) {
                    double wij = (double)c.J[i][j] - (i == j ? invdtgamma : 0.0);
                    acc = fma(-wij, x[j], acc);
                }
                r[i] = (R)acc;
            }
            lu_solve_reg<R, C>(c.W, c.piv, r);
#pragma unroll
            for (int i = 0; i < C; ++i) x[i] += (double)r[i];
        }
#pragma unroll
        for (int i = 0; i < C; ++i) b[i] = (R)x[i];
    }

    template <class Model, class R, int L, int C>
    __device__ static double step(Cache<R, C>& c, R* u, const R* up, const R* p, double t, double dt,
                                  R abstol, R reltol, long long iter, double EEst_prev, const Group<L>& g,
                                  StepStats& st) {
        static_assert(L == 1, "register Rodas5P runs one trajectory per lane");
        const double invdt = 1.0 / dt;
        const double dtgamma = dt * tab::RODAS5P_GAMMA;
        R* fsal = c.scratch;
        Model::template rhs<R, L, C>(fsal, up, p, t, g);
        st.nf += 1;
        bool errorfail = EEst_prev > 1.0;
        bool new_jac = !(iter > 1 && errorfail) || !c.haveJ;
        if (new_jac) {
            Model::template jac<R, C>(c.J, up, p, t);
            st.njacs += 1;
            st.nf += 1;   // the reference's AD time derivative (dT = 0 for autonomous models)
            c.haveJ = true;
        }
        const double invdtgamma = 1.0 / dtgamma;
        const R idg = (R)invdtgamma;
#pragma unroll
        for (int i = 0; i < C; ++i)
#pragma unroll
            for (int j = 0; j < C; ++j) c.W[i][j] = (i == j) ? FMA(R(-1), idg, c.J[i][j]) : c.J[i][j];
        st.nw += 1;
        lu_factor_reg<R, C>(c.W, c.piv);
        R r[C];
#pragma unroll
        for (int i = 0; i < C; ++i) r[i] = fsal[i];
        wsolve<R, C>(c, r, invdtgamma, c.ir);
#pragma unroll
        for (int i = 0; i < C; ++i) c.ks[0][i] = -r[i];
        st.nsolve += 1;
#pragma unroll
        for (int s = 1; s < 8; ++s) {
#pragma unroll
            for (int i = 0; i < C; ++i) {
                R acc = up[i];
#pragma unroll
                for (int jj = 0; jj < s; ++jj) acc = FMA((R)tab::RODAS5P_A(s, jj), c.ks[jj][i], acc);
                u[i] = acc;
            }
            R du[C];
            Model::template rhs<R, L, C>(du, u, p, fma(tab::RODAS5P_c(s), dt, t), g);
            st.nf += 1;
#pragma unroll
            for (int i = 0; i < C; ++i) {
                R acc = du[i];
#pragma unroll
                for (int jj = 0; jj < s; ++jj) acc = FMA((R)(tab::RODAS5P_C(s, jj) * invdt), c.ks[jj][i], acc);
                r[i] = acc;
            }
            wsolve<R, C>(c, r, invdtgamma, c.ir);
#pragma unroll
            for (int i = 0; i < C; ++i) c.ks[s][i] = -r[i];
            st.nsolve += 1;
        }
#pragma unroll
        for (int i = 0; i < C; ++i) {
            R acc = up[i];
#pragma unroll
            for (int jj = 0; jj < 7; ++jj) acc = FMA((R)tab::RODAS5P_A(7, jj), c.ks[jj][i], acc);
            u[i] = FMA(R(1), c.ks[7][i], acc);
        }
        double EEst = error_norm<R, L, C>(c.ks[7], up, u, abstol, reltol, g);
#pragma unroll
        for (int jd = 0; jd < 3; ++jd)
#pragma unroll
            for (int i = 0; i < C; ++i) {
                R acc = R(0);
#pragma unroll
                for (int q = 0; q < 8; ++q) acc = FMA((R)tab::RODAS5P_H(jd, q), c.ks[q][i], acc);
                c.dk[jd][i] = acc;
            }
        return EEst;
    }

    template <class Model, class R, int L, int C>
    __device__ static void interpolate(Cache<R, C>& c, R* out, double thd, double, double, const R* y0,
                                       const R* y1, const R*, const Group<L>&) {
        const R th = (R)thd, th1 = R(1) - th;
#pragma unroll
        for (int i = 0; i < C; ++i) {
            R inner = FMA(th, c.dk[2][i], c.dk[1][i]);
            inner = FMA(th, inner, c.dk[0][i]);
            R v = FMA(th1, inner, y1[i]);
            out[i] = FMA(th1, y0[i], th * v);
        }
    }
};

#undef RP_

}  // namespace odegb
