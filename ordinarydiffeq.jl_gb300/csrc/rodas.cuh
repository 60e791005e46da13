// Rodas5P, with the linear algebra as a policy:
//   RegLA   one lane per trajectory, J, W and the LU in registers (n <= 8);
//   SmemLA  a lane group per trajectory, W and the LU in shared memory
//           (16 to 64 states, lu_group.cuh).
//
//  perform_step!(::RosenbrockCache)  lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_perform_step.jl:729-847
//      fused accumulation helpers :581-727 (acc = base; acc = muladd(c_i, k_i, acc), left to right)
//  tableau                            lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:23-72
//  W = J - I/(dt*gamma)               lib/OrdinaryDiffEqDifferentiation/src/derivative_utils.jl:663-685
//  J reuse after a rejected step      derivative_utils.jl:535-557 (do_newJW), :1011-1041
//  time derivative                    derivative_utils.jl:181-227: the model's analytic tgrad
//                                     (not an f call), formed with a fresh J only (:1040); an
//                                     autonomous model without one has dT = 0, and the reference's
//                                     AD evaluation of it is counted as one f call
//  dT in the stages                   linsolve_tmp = fsalfirst + dtd1 dT (:227, plain ops), then
//                                     muladd(dtd_s, dT, du) + sum dtC ks (_stage_rhs!, :637-652)
//  interpolant (order 3)              rosenbrock_interpolants.jl:172-206
// The LU is Doolittle with partial pivoting (largest |pivot|, first on ties),
// the same algorithm the CPU oracle states; LinearSolve's LU (not vendored)
// pivots the same way.
//
// Mixed precision (R = float): J, W, the LU, the solves and the stage sums are
// FP32; the right-hand side is evaluated in double-float (ff) on the
// compensated state, because stiff kinetics cancel inside f; `ir_sweeps`
// optional refinement sweeps per solve form the residual b - W x in FP64.
#pragma once
#include "integrator.cuh"
#include "lu_group.cuh"
#include "rksum.cuh"
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

// f(u) for a Rosenbrock stage: plain R in FP64 mode; in the mixed mode the
// state (hi + lo) and the parameters are lifted to double-float, f runs in
// double-float, and the result is rounded to FP32.
template <class Model, class R, int L, int C, int NP>
__device__ __forceinline__ void rhs_stage(R* du, const R* u, const R* ulo, const PR<R>* p, const ff* pff, double t,
                                          const Group<L>& g) {
    if (sizeof(R) == 8) {
        Model::template rhs<R, L, C>(du, u, p, t, g);
    } else {
        ff uu[C], dd[C];
#pragma unroll
        for (int i = 0; i < C; ++i) uu[i] = ff_fast2sum((float)u[i], (float)ulo[i]);
        Model::template rhs<ff, L, C>(dd, uu, pff, t, g);
#pragma unroll
        for (int i = 0; i < C; ++i) du[i] = (R)dd[i].f();
    }
}

// J, W and the LU in one lane's registers.
struct RegLA {
    template <class R, int C> struct Store {
        R J[C][C];
        R W[C][C];
        int piv[C];
    };
    template <class R, int L, int C> __host__ __device__ static constexpr int smem_bytes() { return 0; }
    template <class R, int L, int C> __device__ static void init(Store<R, C>&, const Group<L>&) {
        static_assert(L == 1, "register Rodas5P runs one trajectory per lane");
    }
    // J(uprev); kept across a rejected step (fresh = false)
    template <class Model, class R, int L, int C>
    __device__ static void jacobian(Store<R, C>& s, const R* up, const PR<R>* p, double t, bool fresh, const Group<L>&) {
        if (fresh) Model::template jac<R, C>(s.J, up, p, t);
    }
    // W = J - I/(dt*gamma), factorised in place
    template <class R, int L, int C>
    __device__ static void factor(Store<R, C>& s, R idg, const Group<L>&) {
#pragma unroll
        for (int i = 0; i < C; ++i)
#pragma unroll
            for (int jj = 0; jj < C; ++jj) s.W[i][jj] = (i == jj) ? FMA(R(-1), idg, s.J[i][jj]) : s.J[i][jj];
        lu_factor_reg<R, C>(s.W, s.piv);
    }
    // Solve W x = b in place (b -> x); in the mixed mode optionally refined with
    // FP64 residuals b - (J - idg I) x (idg = 1/(dt*gamma) as factored, in FP32).
    template <class Model, class R, int L, int C>
    __device__ static void wsolve(Store<R, C>& s, R* b, double, R idg, int ir, const R*, const R*,
                                  const ff*, const Group<L>&) {
        if constexpr (sizeof(R) == 8) {
            lu_solve_reg<R, C>(s.W, s.piv, b);
            return;
        }
        if (ir <= 0) {
            lu_solve_reg<R, C>(s.W, s.piv, b);
            return;
        }
        // the residual of the matrix that was factored: J - idg*I with the FP32 idg
        const double invdtgamma = (double)idg;
        double b64[C];
#pragma unroll
        for (int i = 0; i < C; ++i) b64[i] = (double)b[i];
        lu_solve_reg<R, C>(s.W, s.piv, b);
        double x[C];
#pragma unroll
        for (int i = 0; i < C; ++i) x[i] = (double)b[i];
        for (int sw = 0; sw < ir; ++sw) {
            R r[C];
#pragma unroll
            for (int i = 0; i < C; ++i) {
                double acc = b64[i];
#pragma unroll
                for (int jj = 0; jj < C; ++jj) {
                    double wij = (double)s.J[i][jj] - (i == jj ? invdtgamma : 0.0);
                    acc = fma(-wij, x[jj], acc);
                }
                r[i] = (R)acc;
            }
            lu_solve_reg<R, C>(s.W, s.piv, r);
#pragma unroll
            for (int i = 0; i < C; ++i) x[i] += (double)r[i];
        }
#pragma unroll
        for (int i = 0; i < C; ++i) b[i] = (R)x[i];
    }
};

template <class LA>
struct Rodas5PT {
    static constexpr int ORDER = 5;
    static constexpr bool IMPLICIT = true;
    // parameters kept in double-float (mixed mode); only the model's NP are
    // touched, so the unused entries take no registers
    static constexpr int MAXP = 32;
    template <class R, int C> struct Cache {
        typename LA::template Store<R, C> la;
        R ks[8][C];
        R dk[3][C];   // dense k1..k3
        R scratch[C];
        R dT[C];       // df/dt at (uprev, t), non-autonomous models
        ff pff[MAXP];  // parameters in double-float (mixed mode)
        bool haveJ;
        int ir;
    };
    template <class R, int L, int C> __host__ __device__ static constexpr int smem_bytes() {
        return LA::template smem_bytes<R, L, C>();
    }
    template <class R, int C> __device__ static R* fsal_slot(Cache<R, C>& c) { return c.scratch; }
    template <class Model, class R, int L, int C>
    __device__ static void initialize(Cache<R, C>& c, const R*, const PR<R>*, double, const Group<L>& g, StepStats&,
                                      const EnsembleArgs& a, long long j) {
        LA::template init<R, L, C>(c.la, g);
        c.haveJ = false;
        c.ir = a.ir_sweeps;
        if (sizeof(R) == 4) {
#pragma unroll
            for (int i = 0; i < Model::NP; ++i) c.pff[i] = ff(a.p[(size_t)i * a.N + j]);
            static_assert(Model::NP <= MAXP, "too many parameters for the double-float copy");
        }
    }
    template <class R, int C> __device__ static void on_accept(Cache<R, C>&) {}
    template <class R, int C> __device__ static void after_save(Cache<R, C>&) {}

    template <class Model, class R, int L, int C>
    __device__ static typename Ctl<R>::T step(Cache<R, C>& c, R* u, R* ulo, const R* up, const R* uplo,
                                             const PR<R>* p, double t, double dt, const Tol<R>& tol, long long iter,
                                             bool errorfail, const Group<L>& g, StepStats& st) {
        constexpr int NP = Model::NP;
        // dt-derived coefficients: FP64 like the reference; in the mixed mode they
        // scale FP32 stage terms, so they are formed in FP32 from dt (no FP64 work).
        const R dr = (R)dt;
        R invdt, idg;
        if constexpr (sizeof(R) == 8) {
            invdt = R(1.0 / dt);
            idg = R(1.0 / (dt * tab::RODAS5P_GAMMA));
        } else {
            invdt = R(1) / dr;
            idg = R(1) / (dr * (R)tab::RODAS5P_GAMMA);
        }
        R* fsal = c.scratch;
        rhs_stage<Model, R, L, C, NP>(fsal, up, uplo, p, c.pff, t, g);
        st.nf += 1;
        bool new_jac = !(iter > 1 && errorfail) || !c.haveJ;
        LA::template jacobian<Model, R, L, C>(c.la, up, p, t, new_jac, g);
        static_assert(Model::AUTONOMOUS || has_tgrad<Model>::value, "a non-autonomous model needs its tgrad");
        static_assert(Model::AUTONOMOUS || L == 1, "time derivatives are formed on one lane");
        if (new_jac) {
            st.njacs += 1;
            st.nf += jac_f_calls<Model>::value;
            if constexpr (has_tgrad<Model>::value) Model::template tgrad<R, C>(c.dT, up, p, t);
            else st.nf += 1;   // the reference's AD time derivative (dT = 0 for autonomous models)
            c.haveJ = true;
        }
        LA::template factor<R, L, C>(c.la, idg, g);
        st.nw += 1;
        R r[C];
#pragma unroll
        for (int i = 0; i < C; ++i) r[i] = fsal[i];
        if constexpr (!Model::AUTONOMOUS) {   // fsalfirst + dtd1 dT
            const R dtd0 = (R)(dt * tab::RODAS5P_d(0));
#pragma unroll
            for (int i = 0; i < C; ++i) r[i] = fsal[i] + dtd0 * c.dT[i];
        }
        LA::template wsolve<Model, R, L, C>(c.la, r, dt, idg, c.ir, up, uplo, c.pff, g);
#pragma unroll
        for (int i = 0; i < C; ++i) c.ks[0][i] = -r[i];
        st.nsolve += 1;
#pragma unroll
        for (int s = 1; s < 8; ++s) {
            R stlo[C];
#pragma unroll
            for (int i = 0; i < C; ++i) {
                if (sizeof(R) == 8) {   // reference: acc = uprev; acc = muladd(A[s,j], ks_j, acc)
                    R acc = up[i];
#pragma unroll
                    for (int jj = 0; jj < s; ++jj) acc = FMA((R)tab::RODAS5P_A(s, jj), c.ks[jj][i], acc);
                    u[i] = acc;
                    stlo[i] = R(0);
                } else {   // compensated sum, then the stage value as an exact pair up + sum + uplo
                    CSum cs;
#pragma unroll
                    for (int jj = 0; jj < s; ++jj) cs.add_pair(tab::RODAS5P_A_HI(s, jj), tab::RODAS5P_A_LO(s, jj), (float)c.ks[jj][i]);
                    Acc<R>::update(u[i], stlo[i], R(1), (R)cs.value(), up[i], uplo[i]);
                }
            }
            R du[C];
            rhs_stage<Model, R, L, C, NP>(du, u, stlo, p, c.pff, stage_time<Model>(tab::RODAS5P_c(s), dt, t), g);
            st.nf += 1;
#pragma unroll
            for (int i = 0; i < C; ++i) {
                if (sizeof(R) == 8) {
                    R acc = du[i];
                    if constexpr (!Model::AUTONOMOUS) acc = FMA((R)(dt * tab::RODAS5P_d(s)), c.dT[i], acc);
#pragma unroll
                    for (int jj = 0; jj < s; ++jj) acc = FMA((R)tab::RODAS5P_C(s, jj) * invdt, c.ks[jj][i], acc);
                    r[i] = acc;
                } else {   // du + sum_j (C[s,j]/dt) ks_j with C split at compile time and 1/dt exact in FP32 pairs
                    CSum cs;
                    cs.hi = (float)du[i];
                    if constexpr (!Model::AUTONOMOUS) {   // + dtd_s dT, dtd_s = dt d_s as a float pair
                        const double dd = dt * tab::RODAS5P_d(s);
                        const float dh = (float)dd;
                        cs.add_pair(dh, (float)(dd - (double)dh), (float)c.dT[i]);
                    }
#pragma unroll
                    for (int jj = 0; jj < s; ++jj) {
                        const float ch = tab::RODAS5P_C_HI(s, jj), cl = tab::RODAS5P_C_LO(s, jj);
                        const float wh = ch * (float)invdt;
                        const float wl = fmaf(cl, (float)invdt, fmaf(ch, (float)invdt, -wh));
                        cs.add_pair(wh, wl, (float)c.ks[jj][i]);
                    }
                    r[i] = (R)cs.value();
                }
            }
            LA::template wsolve<Model, R, L, C>(c.la, r, dt, idg, c.ir, up, uplo, c.pff, g);
#pragma unroll
            for (int i = 0; i < C; ++i) c.ks[s][i] = -r[i];
            st.nsolve += 1;
        }
#pragma unroll
        for (int i = 0; i < C; ++i) {
            if (sizeof(R) == 8) {   // reference order: acc = uprev; acc = muladd(b_j, ks_j, acc)
                R acc = up[i];
#pragma unroll
                for (int jj = 0; jj < 7; ++jj) acc = FMA((R)tab::RODAS5P_A(7, jj), c.ks[jj][i], acc);
                Acc<R>::set(u[i], ulo[i], FMA(R(1), c.ks[7][i], acc));
            } else {                // compensated increment, added to the compensated solution
                CSum cs;
#pragma unroll
                for (int jj = 0; jj < 7; ++jj) cs.add_pair(tab::RODAS5P_A_HI(7, jj), tab::RODAS5P_A_LO(7, jj), (float)c.ks[jj][i]);
                cs.add_pair(1.0f, 0.0f, (float)c.ks[7][i]);
                Acc<R>::update(u[i], ulo[i], R(1), (R)cs.value(), up[i], uplo[i]);
            }
        }
        return error_norm<R, L, C>(c.ks[7], up, u, tol, g);
    }

    // Dense coefficients k_j = sum_i H[j,i] ks_i (rosenbrock_perform_step.jl:811-815),
    // formed only on steps that interpolate a save (same operations as forming them
    // every step, since ks is still the accepted step's).
    template <class R, int C>
    __device__ static void dense(Cache<R, C>& c) {
#pragma unroll
        for (int jd = 0; jd < 3; ++jd)
#pragma unroll
            for (int i = 0; i < C; ++i) {
                if (sizeof(R) == 8) {
                    R acc = R(0);
#pragma unroll
                    for (int q = 0; q < 8; ++q) acc = FMA((R)tab::RODAS5P_H(jd, q), c.ks[q][i], acc);
                    c.dk[jd][i] = acc;
                } else {
                    CSum cs;
#pragma unroll
                    for (int q = 0; q < 8; ++q) cs.add_pair(tab::RODAS5P_H_HI(jd, q), tab::RODAS5P_H_LO(jd, q), (float)c.ks[q][i]);
                    c.dk[jd][i] = (R)cs.value();
                }
            }
    }

    // Dense output (dense = true): the step's dense k1..k3, the reference's
    // integrator.k for Rodas5P (rosenbrock_perform_step.jl:811-815).
    static constexpr int NDENSE = 3;
    template <class R, int C> __device__ static void prepare_dense(Cache<R, C>& c) { dense<R, C>(c); }
    template <class R, int C> __device__ static R* dense_slot(Cache<R, C>& c, int q) { return c.dk[q]; }

    // not FSAL (isfsal(::Rodas5P) = false, alg_utils.jl:60): f(uprev) is formed every step
    template <class Model, class R, int L, int C>
    __device__ static void reset_fsal(Cache<R, C>&, const R*, const R*, const PR<R>*, double, const Group<L>&,
                                      StepStats&) {}

    template <class Model, class R, int L, int C>
    __device__ static void interpolate(Cache<R, C>& c, R* out, R* outlo, double th, double, double,
                                       const R* y0, const R* y0lo, const R* y1, const R* y1lo, const PR<R>*,
                                       const Group<L>&) {
        dense<R, C>(c);
        interp_dense<R, C>(c, out, outlo, th, y0, y0lo, y1, y1lo);
    }

    // Interpolant on formed dense coefficients (rosenbrock_interpolants.jl:172-206);
    // theta in the stage precision.
    template <class R, int C>
    __device__ static void interp_dense(const Cache<R, C>& c, R* out, R* outlo, double thd, const R* y0,
                                        const R* y0lo, const R* y1, const R* y1lo) {
        const R th = (R)thd;
        const R th1 = R(1) - th;
#pragma unroll
        for (int i = 0; i < C; ++i) {
            R inner = FMA(th, c.dk[2][i], c.dk[1][i]);
            inner = FMA(th, inner, c.dk[0][i]);
            if constexpr (sizeof(R) == 8) {
                R v = FMA(th1, inner, y1[i]);
                Acc<R>::set(out[i], outlo[i], FMA(th1, y0[i], th * v));
            } else {   // (1-th) y0 + th (y1 + (1-th) inner) on the compensated end points, in double-float
                float ph, pl;
                ph = th1 * inner;
                pl = fmaf(th1, inner, -ph);
                const ff v = ff(y1[i], y1lo[i]) + ff_fast2sum(ph, pl);
                const ff o = ff_mul_f(ff(y0[i], y0lo[i]), th1) + ff_mul_f(v, th);
                out[i] = o.hi;
                outlo[i] = o.lo;
            }
        }
    }
};

using Rodas5PAlg = Rodas5PT<RegLA>;
using Rodas5PGroupAlg = Rodas5PT<SmemLA>;

}  // namespace odegb
