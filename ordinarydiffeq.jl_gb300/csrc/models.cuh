// Registered right-hand sides and analytic Jacobians.
//
// The reference takes an arbitrary Julia f(du, u, p, t) (and optional jac);
// a device ensemble cannot call Julia closures, so models are registered at
// compile time and selected by model_id.  Each is written for a lane group:
// a lane holds C consecutive state components, neighbours across lanes come
// from warp shuffles.  Operation order matches the oracle's restatement
// exactly (explicit products and sums, no contraction).
//
//  LINEAR       u_i' = p0 u_i                       (prob_ode_linear, test/Regression_I/ode_dense_tests.jl:30-38)
//  LORENZ       lib/OrdinaryDiffEqCore/src/precompilation_setup.jl:1-6, p = (sigma, rho, beta)
//  ROBERTSON    benchmark/benchmarks.jl:93-100, p = (k1, k2, k3)
//  DUFFING      chain of N oscillators, interleaved (x_i, v_i), walls x_0 = x_{N+1} = 0,
//               p = (k, delta, beta): v_i' = (k*lap_i - delta*v_i) - beta*x_i^3
//  BRUSSELATOR  1-D periodic, interleaved (u_i, v_i), p = (A, B, alpha), ae = alpha*ncells^2:
//               u' = ((A + u^2 v) - (B+1) u) + ae*lap u,  v' = (B u - u^2 v) + ae*lap v
//  FORCED_DUFFING  non-autonomous: x' = v, v' = ((g cos(w t) - delta v) - alpha x) - beta x^3,
//               p = (delta, alpha, beta, g, w), with its analytic time derivative (tgrad)
#pragma once
#include "common.cuh"

namespace odegb {

enum ModelId { M_LINEAR = 0, M_LORENZ = 1, M_ROBERTSON = 2, M_DUFFING = 3, M_BRUSSELATOR = 4, M_BOUNCING_BALL = 5,
               M_VANDERPOL = 6, M_PK1 = 7, M_FORCED_DUFFING = 8 };

// A forced (non-autonomous) Duffing oscillator, the standard driven nonlinear
// oscillator: u = (x, v), x' = v, v' = ((g cos(w t) - delta v) - alpha x) - beta x^3;
// p = (delta, alpha, beta, g, w).  With beta = 0 it is the driven damped linear
// oscillator, whose closed-form solution pins the oracle.  The forcing is
// evaluated in FP64 in every precision (t is FP64; w t in FP32 would lose the
// phase after a few periods) and rounded to the stage type.  tgrad is the
// analytic df/dt = (0, -g w sin(w t)) (ODEFunction's tgrad: the Rosenbrock
// methods take it instead of differentiating f in t, so it is not an f call).
struct ForcedDuffing {
    static constexpr int NP = 5;
    static constexpr bool AUTONOMOUS = false;
    static constexpr bool HAS_EVENT = false;
    static constexpr bool HAS_TGRAD = true;
    template <class P> __device__ static double forcing(const P* p, double t) {
        return pdouble(p[3]) * cos(pdouble(p[4]) * t);
    }
    template <class R, int L, int C, class P>
    __device__ static void rhs(R* du, const R* u, const P* p, double t, const Group<L>&) {
        static_assert(L == 1 && C == 2, "the forced oscillator has 2 states on one lane");
        const R fo = from_double<R>(forcing(p, t));
        du[0] = u[1];
        du[1] = ((fo - p[0] * u[1]) - p[1] * u[0]) - p[2] * (u[0] * u[0] * u[0]);
    }
    template <class R, int N, class P>
    __device__ static void jac(R (*J)[N], const R* u, const P* p, double) {
        J[0][0] = R(0);
        J[0][1] = R(1);
        J[1][0] = -p[1] - p[2] * (R(3) * (u[0] * u[0]));
        J[1][1] = -p[0];
    }
    template <class R, int C, class P>
    __device__ static void tgrad(R* dT, const R*, const P* p, double t) {
        const double w = pdouble(p[4]);
        dT[0] = R(0);
        dT[1] = from_double<R>(-(pdouble(p[3]) * w) * sin(w * t));
    }
};

// The van der Pol oscillator of the reference's stiffness-detection test
// (test/InterfaceI/stiffness_detection_test.jl:10-16): u = (x, y), x' = y,
// y' = mu ((1 - x^2) y - x), p = (mu).
struct VanDerPol {
    static constexpr int NP = 1;
    static constexpr bool AUTONOMOUS = true;
    static constexpr bool HAS_EVENT = false;
    template <class R, int L, int C, class P>
    __device__ static void rhs(R* du, const R* u, const P* p, double, const Group<L>&) {
        static_assert(L == 1 && C == 2, "van der Pol has 2 states on one lane");
        du[0] = u[1];
        du[1] = p[0] * ((R(1) - u[0] * u[0]) * u[1] - u[0]);
    }
    template <class R, int N, class P>
    __device__ static void jac(R (*J)[N], const R* u, const P* p, double) {
        J[0][0] = R(0);
        J[0][1] = R(1);
        J[1][0] = p[0] * (R(-2) * u[0] * u[1] - R(1));
        J[1][1] = p[0] * (R(1) - u[0] * u[0]);
    }
};

// One-compartment pharmacokinetics with first-order absorption, dosed by its
// registered DiscreteCallback: u = (depot, central), depot' = -ka depot,
// central' = ka depot - ke central; p = (ka, ke, dose).  Callback: condition
// t in tstops (the dose times are the solve's tstops, the pattern of
// DiffEqCallbacks' PresetTimeCallback), affect!: depot += dose.
struct PKOneCompartment {
    static constexpr int NP = 3;
    static constexpr bool AUTONOMOUS = true;
    static constexpr bool HAS_EVENT = false;
    static constexpr bool HAS_DISCRETE = true;
    template <class R, int L, int C, class P>
    __device__ static void rhs(R* du, const R* u, const P* p, double, const Group<L>&) {
        static_assert(L == 1 && C == 2, "the one-compartment model has 2 states on one lane");
        du[0] = -p[0] * u[0];
        du[1] = p[0] * u[0] - p[1] * u[1];
    }
    template <class R, int N, class P>
    __device__ static void jac(R (*J)[N], const R*, const P* p, double) {
        J[0][0] = -p[0]; J[0][1] = R(0);
        J[1][0] = p[0];  J[1][1] = -p[1];
    }
    // affect!: the dose into the depot, in FP64 on the state pair (no terminate!)
    template <class R, int L, int C>
    __device__ static bool discrete_affect(R* u, R* ulo, const double* p, long long stride, double,
                                           const Group<L>&) {
        const double v = ((double)u[0] + (double)ulo[0]) + p[2 * stride];
        u[0] = (R)v;
        ulo[0] = (R)(v - (double)u[0]);
        return false;
    }
};

// A ball under gravity with its registered ContinuousCallback (the reference's
// event tests, test/Integrators_I/ode_event_tests.jl:100-113 and 283-360):
// u = (x, v), x' = v, v' = -g; p = (g, e, t_stop).  Callback: condition x,
// affect! = nothing, affect_neg!: terminate! once t >= t_stop, else v <- -e v.
struct BouncingBall {
    static constexpr int NP = 3;
    static constexpr bool AUTONOMOUS = true;
    static constexpr bool HAS_EVENT = true;
    static constexpr bool EVENT_AFFECT_POS = false;   // affect! = nothing
    static constexpr bool EVENT_AFFECT_NEG = true;    // affect_neg!
    template <class R, int L, int C, class P>
    __device__ static void rhs(R* du, const R* u, const P* p, double, const Group<L>&) {
        static_assert(L == 1 && C == 2, "the ball has 2 states on one lane");
        du[0] = u[1];
        du[1] = -p[0];
    }
    template <class R, int N, class P>
    __device__ static void jac(R (*J)[N], const R*, const P*, double) {
        J[0][0] = R(0); J[0][1] = R(1);
        J[1][0] = R(0); J[1][1] = R(0);
    }
    // condition(u, t, integrator) = u[1] (the height), in FP64 from the state pair
    template <class R, int L, int C>
    __device__ static double event_condition(const R* u, const R* ulo, const double*, long long, double,
                                             const Group<L>&) {
        return (double)u[0] + (double)ulo[0];
    }
    // the affect for a crossing from below (upcrossing) or above; true: terminate!
    template <class R, int L, int C>
    __device__ static bool event_affect(R* u, R* ulo, const double* p, long long stride, double t, bool,
                                        const Group<L>&) {
        if (t >= p[2 * stride]) return true;
        const double v = -p[stride] * ((double)u[1] + (double)ulo[1]);
        u[1] = (R)v;
        ulo[1] = (R)(v - (double)u[1]);
        return false;
    }
};

struct Linear {
    static constexpr int NP = 1;
    static constexpr bool AUTONOMOUS = true;   // f(u, p) does not read t
    static constexpr bool HAS_EVENT = false;   // no registered callback
    template <class R, int L, int C, class P>
    __device__ static void rhs(R* du, const R* u, const P* p, double, const Group<L>&) {
#pragma unroll
        for (int c = 0; c < C; ++c) du[c] = p[0] * u[c];
    }
    template <class R, int N, class P>
    __device__ static void jac(R (*J)[N], const R*, const P* p, double) {
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = 0; j < N; ++j) J[i][j] = (i == j) ? p[0] : R(0);
    }
};

struct Lorenz {
    static constexpr int NP = 3;
    static constexpr bool AUTONOMOUS = true;   // f(u, p) does not read t
    static constexpr bool HAS_EVENT = false;   // no registered callback
    template <class R, int L, int C, class P>
    __device__ static void rhs(R* du, const R* u, const P* p, double, const Group<L>&) {
        static_assert(L == 1 && C == 3, "Lorenz has 3 states on one lane");
        du[0] = p[0] * (u[1] - u[0]);
        du[1] = u[0] * (p[1] - u[2]) - u[1];
        du[2] = u[0] * u[1] - p[2] * u[2];
    }
    template <class R, int N, class P>
    __device__ static void jac(R (*J)[N], const R* u, const P* p, double) {
        J[0][0] = -p[0]; J[0][1] = p[0]; J[0][2] = R(0);
        J[1][0] = p[1] - u[2]; J[1][1] = R(-1); J[1][2] = -u[0];
        J[2][0] = u[1]; J[2][1] = u[0]; J[2][2] = -p[2];
    }
};

struct Robertson {
    static constexpr int NP = 3;
    static constexpr bool AUTONOMOUS = true;   // f(u, p) does not read t
    static constexpr bool HAS_EVENT = false;   // no registered callback
    template <class R, int L, int C, class P>
    __device__ static void rhs(R* du, const R* u, const P* p, double, const Group<L>&) {
        static_assert(L == 1 && C == 3, "Robertson has 3 states on one lane");
        R y1 = u[0], y2 = u[1], y3 = u[2];
        du[0] = -p[0] * y1 + p[2] * y2 * y3;
        du[1] = p[0] * y1 - p[1] * (y2 * y2) - p[2] * y2 * y3;
        du[2] = p[1] * (y2 * y2);
    }
    template <class R, int N, class P>
    __device__ static void jac(R (*J)[N], const R* u, const P* p, double) {
        R y2 = u[1], y3 = u[2];
        J[0][0] = -p[0]; J[0][1] = p[2] * y3; J[0][2] = p[2] * y2;
        J[1][0] = p[0]; J[1][1] = R(-2) * p[1] * y2 - p[2] * y3; J[1][2] = -p[2] * y2;
        J[2][0] = R(0); J[2][1] = R(2) * p[1] * y2; J[2][2] = R(0);
    }
};

// Neighbour values across lanes for the chain models: x of the last pair of
// the previous lane and of the first pair of the next lane (wrapping).
template <class R, int L, int C>
__device__ __forceinline__ void chain_halo(const R* u, const Group<L>& g, int off, R& left, R& right) {
    left = g.from(u[C - 2 + off], (g.lane + L - 1) % L);
    right = g.from(u[0 + off], (g.lane + 1) % L);
}

struct Duffing {
    static constexpr int NP = 3;
    static constexpr bool AUTONOMOUS = true;   // f(u, p) does not read t
    static constexpr bool HAS_EVENT = false;   // no registered callback
    template <class R, int L, int C, class P>
    __device__ static void rhs(R* du, const R* u, const P* p, double, const Group<L>& g) {
        static_assert(C % 2 == 0, "Duffing lanes hold whole (x, v) pairs");
        R xl, xr;
        chain_halo<R, L, C>(u, g, 0, xl, xr);
        if (g.lane == 0) xl = R(0);
        if (g.lane == L - 1) xr = R(0);
#pragma unroll
        for (int q = 0; q < C / 2; ++q) {
            R x = u[2 * q], v = u[2 * q + 1];
            R left = q > 0 ? u[2 * q - 2] : xl;
            R right = q < C / 2 - 1 ? u[2 * q + 2] : xr;
            R lap = (left + right) - R(2) * x;
            du[2 * q] = v;
            du[2 * q + 1] = (p[0] * lap - p[1] * v) - p[2] * (x * x * x);
        }
    }
    template <class R, int N, class P>
    __device__ static void jac(R (*J)[N], const R* u, const P* p, double) {
#pragma unroll
        for (int i = 0; i < N; ++i)
#pragma unroll
            for (int j = 0; j < N; ++j) J[i][j] = R(0);
#pragma unroll
        for (int i = 0; i < N / 2; ++i) {
            R x = u[2 * i];
            J[2 * i][2 * i + 1] = R(1);
            J[2 * i + 1][2 * i] = R(-2) * p[0] - p[2] * (R(3) * (x * x));
            J[2 * i + 1][2 * i + 1] = -p[1];
            if (i > 0) J[2 * i + 1][2 * i - 2] = p[0];
            if (i < N / 2 - 1) J[2 * i + 1][2 * i + 2] = p[0];
        }
    }
};

struct Brusselator {
    static constexpr int NP = 3;
    static constexpr bool AUTONOMOUS = true;   // f(u, p) does not read t
    static constexpr bool HAS_EVENT = false;   // no registered callback
    template <class R, int L, int C, class P>
    __device__ static void rhs(R* du, const R* u, const P* p, double, const Group<L>& g) {
        static_assert(C % 2 == 0, "Brusselator lanes hold whole (u, v) cells");
        constexpr int NC = L * C / 2;
        R ae = p[2] * (R(NC) * R(NC));
        R ul, ur, vl, vr;
        chain_halo<R, L, C>(u, g, 0, ul, ur);
        chain_halo<R, L, C>(u, g, 1, vl, vr);
#pragma unroll
        for (int q = 0; q < C / 2; ++q) {
            R uu = u[2 * q], vv = u[2 * q + 1];
            R uL = q > 0 ? u[2 * q - 2] : ul, uR = q < C / 2 - 1 ? u[2 * q + 2] : ur;
            R vL = q > 0 ? u[2 * q - 1] : vl, vR = q < C / 2 - 1 ? u[2 * q + 3] : vr;
            R lu = (uL + uR) - R(2) * uu;
            R lv = (vL + vR) - R(2) * vv;
            R u2v = uu * uu * vv;
            du[2 * q] = ((p[0] + u2v) - (p[1] + R(1)) * uu) + ae * lu;
            du[2 * q + 1] = (p[1] * uu - u2v) + ae * lv;
        }
    }
    // Nonzeros of the lane's own rows (cells lane*C/2 ...) of J(u), in the
    // oracle's arithmetic; put(i, col, v) with i the lane-local row.  The
    // neighbour columns are distinct from the cell's own for 3 cells or more.
    template <class R, int L, int C, class P, class Put>
    __device__ static void jac_rows(const R* u, const P* p, const Group<L>& g, Put&& put) {
        constexpr int NC = L * C / 2;
        static_assert(NC >= 3, "group Jacobian assumes distinct neighbour cells");
        const R ae = p[2] * (R(NC) * R(NC));
#pragma unroll
        for (int q = 0; q < C / 2; ++q) {
            const int cell = g.lane * (C / 2) + q;
            const int il = cell == 0 ? NC - 1 : cell - 1, ir = cell == NC - 1 ? 0 : cell + 1;
            const R uu = u[2 * q], vv = u[2 * q + 1];
            put(2 * q, 2 * cell, (R(2) * uu * vv - (p[1] + R(1))) - R(2) * ae);
            put(2 * q, 2 * cell + 1, uu * uu);
            put(2 * q, 2 * il, ae);
            put(2 * q, 2 * ir, ae);
            put(2 * q + 1, 2 * cell, p[1] - R(2) * uu * vv);
            put(2 * q + 1, 2 * cell + 1, -(uu * uu) - R(2) * ae);
            put(2 * q + 1, 2 * il + 1, ae);
            put(2 * q + 1, 2 * ir + 1, ae);
        }
    }
    // J(u) x in double-float for the lane's rows (x in FP32, u and p in
    // double-float): the refinement residual of the mixed Rosenbrock solve.
    template <int L, int C>
    __device__ static void jvp(ff* out, const float* x, const ff* u, const ff* p, const Group<L>& g) {
        constexpr int NC = L * C / 2;
        const ff ae = p[2] * (ff(NC) * ff(NC));
        float xul, xur, xvl, xvr;
        chain_halo<float, L, C>(x, g, 0, xul, xur);
        chain_halo<float, L, C>(x, g, 1, xvl, xvr);
#pragma unroll
        for (int q = 0; q < C / 2; ++q) {
            const ff uu = u[2 * q], vv = u[2 * q + 1];
            const float xuL = q > 0 ? x[2 * q - 2] : xul, xuR = q < C / 2 - 1 ? x[2 * q + 2] : xur;
            const float xvL = q > 0 ? x[2 * q - 1] : xvl, xvR = q < C / 2 - 1 ? x[2 * q + 3] : xvr;
            const ff uv2 = ff(2) * uu * vv, u2 = uu * uu, ae2 = ff(2) * ae;
            const ff xu = ff(x[2 * q]), xv = ff(x[2 * q + 1]);
            out[2 * q] = (((uv2 - (p[1] + ff(1))) - ae2) * xu + u2 * xv) + ae * (ff(xuL) + ff(xuR));
            out[2 * q + 1] = ((p[1] - uv2) * xu - (u2 + ae2) * xv) + ae * (ff(xvL) + ff(xvR));
        }
    }
};

}  // namespace odegb
