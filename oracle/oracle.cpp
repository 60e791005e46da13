// TEST INFRASTRUCTURE — CPU FP64 restatement of the reference's ensemble
// solve path, used only as the checker (tests/, smoke(), bench.py's CPU
// baseline).  Never linked into the product.
//
// Parity status: pinned at the solution level against the reference's own
// tolerance tests (tests/test_oracle.py); not pinned bit-for-bit against Julia
// (the reference cannot run here).  Every routine cites the reference file it
// restates; paths are relative to the OrdinaryDiffEq.jl checkout.
//
// Floating-point order: every `a*b + c` the reference writes under @muladd is
// written here as fma(a, b, c) with the same nesting (MuladdMacro rewrites
// `a1*k1 + a2*k2 + a3*k3` as muladd(a1,k1, muladd(a2,k2, a3*k3))).  The file
// is compiled with -ffp-contract=off so no other contraction happens.
#include "oracle.h"
#include "oracle_tableaus.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- helpers
// Julia's min/max propagate NaN (Base.min/max on Float64).
inline double jmin(double a, double b) { return (a != a || b != b) ? NAN : (a < b ? a : b); }
inline double jmax(double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : b); }
// Julia eps(x): spacing of doubles at |x|.
inline double jeps(double x) {
    double ax = std::fabs(x);
    if (!std::isfinite(ax)) return NAN;
    return std::nextafter(ax, INFINITY) - ax;
}

// x^y as used by the PI controller and initdt.  The reference calls
// FastPower.fastpower (package FastPower, compat floor 1.1.2, not vendored;
// lib/OrdinaryDiffEqCore/Project.toml:70), i.e. exp2(y*log2(x)).  Restated as
// exp(y*ln x) with ln from the atanh series ln m = 2 atanh((m-1)/(m+1)) on
// m in [1/sqrt2, sqrt2) and exp from range reduction by ln2 plus a Taylor
// series (textbook methods, e.g. Muller, "Elementary Functions", ch. 5-6).
const double LNC[13] = {2.0, 0.6666666666666666, 0.4, 0.2857142857142857, 0.2222222222222222,
                        0.18181818181818182, 0.15384615384615385, 0.13333333333333333,
                        0.11764705882352941, 0.10526315789473684, 0.09523809523809523,
                        0.08695652173913043, 0.08};
const double EXC[18] = {1.0, 1.0, 0.5, 0.16666666666666666, 0.041666666666666664,
                        0.008333333333333333, 0.001388888888888889, 0.0001984126984126984,
                        2.48015873015873e-05, 2.7557319223985893e-06, 2.755731922398589e-07,
                        2.505210838544172e-08, 2.08767569878681e-09, 1.6059043836821613e-10,
                        1.1470745597729725e-11, 7.647163731819816e-13, 4.779477332387385e-14,
                        2.8114572543455206e-15};
const double LN2 = 0.6931471805599453, LN2LO = 2.3190468138462996e-17;
const double INVLN2 = 1.4426950408889634, SQRT1_2 = 0.7071067811865476;

double series_ln(double x) {  // x > 0 finite
    int e;
    double m = std::frexp(x, &e);
    if (m < SQRT1_2) { m = m * 2.0; e -= 1; }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s;
    double poly = LNC[12];
    for (int k = 11; k >= 0; --k) poly = std::fma(poly, s2, LNC[k]);
    double de = (double)e;
    return std::fma(de, LN2, std::fma(de, LN2LO, s * poly));
}
double series_exp(double t) {
    if (t != t) return t;
    if (t > 709.0) return INFINITY;
    if (t < -745.0) return 0.0;
    double k = std::rint(t * INVLN2);
    double r = std::fma(-k, LN2, t);
    r = std::fma(-k, LN2LO, r);
    double e = EXC[17];
    for (int i = 16; i >= 0; --i) e = std::fma(e, r, EXC[i]);
    return std::ldexp(e, (int)k);
}
double ctrl_pow(double x, double y) {
    if (x == 0.0) return 0.0;
    if (x != x || y != y) return NAN;
    if (std::isinf(x)) return INFINITY;
    return series_exp(y * series_ln(x));
}

// ---------------------------------------------------------------- models
// Lorenz: lib/OrdinaryDiffEqCore/src/precompilation_setup.jl:1-6 with p = (sigma, rho, beta).
// Robertson: benchmark/benchmarks.jl:93-100 with p = (k1, k2, k3).
// Duffing chain (defined by the workload, not the reference): N oscillators,
//   state interleaved (x1, v1, ..., xN, vN), fixed walls x0 = x_{N+1} = 0,
//   p = (k stiffness, delta damping, beta cubic):
//   x_i' = v_i,  v_i' = (k*lap_i - delta*v_i) - beta*(x_i*x_i*x_i),
//   lap_i = (x_{i-1} + x_{i+1}) - 2 x_i.
// Brusselator 1-D periodic, 32 cells on [0,1), interleaved (u1, v1, ...),
//   p = (A, B, alpha), ae = alpha*ncells^2 (alpha/dx^2 as in
//   benchmark/benchmarks.jl:243-247):
//   u' = ((A + u*u*v) - (B+1)*u) + ae*lap(u),  v' = (B*u - u*u*v) + ae*lap(v).
// Linear: u_i' = p0 * u_i (prob_ode_linear with p0 = 1.01, test/Regression_I/ode_dense_tests.jl:30-38).
// Bouncing ball: x' = v, v' = -g (p = (g, e, t_stop); test/Integrators_I/ode_event_tests.jl:100-104),
//   with its event below.
// Forced Duffing (non-autonomous, defined by this build's tests): x' = v,
//   v' = ((g cos(w t) - delta v) - alpha x) - beta x^3, p = (delta, alpha, beta, g, w),
//   with the analytic time derivative (tgrad) below.
// Two models that the library does not compile in, for the tests of models
// registered at run time (the GPU side gets them as source through
// ode_register_model):
//   Lotka-Volterra, benchmark/benchmarks.jl:13-26: x' = a x - b x y,
//     y' = d x y - c y, p = (a, b, c, d);
//   the Oregonator (Field-Koros-Noyes, the stiff test problem of Hairer and
//     Wanner's "Solving ODEs II", sec. IV.10): y1' = s (y2 + y1 (1 - q y1 - y2)),
//     y2' = (y3 - (1 + y1) y2) / s, y3' = w (y1 - y3), p = (s, w, q).
// Two models for the tests of callbacks registered with a model (defined by
// those tests, not the reference):
//   a ball in a box, u = (x, y, vx, vy), p = (g, e, W): x' = vx, y' = vy,
//     vx' = 0, vy' = -g, with a VectorContinuousCallback of three conditions
//     (y: the floor; x and W - x: the walls) whose affect! reflects vy with
//     restitution e at the floor and vx at a wall;
//   a state-triggered dose, u = (c), p = (k, threshold, dose): c' = -k c, with a
//     DiscreteCallback whose condition is c < threshold and whose affect! adds
//     the dose.
void rhs(int model, int n, const double* u, const double* p, double t, double* du) {
    switch (model) {
    case ORC_BALL_BOX:
        du[0] = u[2];
        du[1] = u[3];
        du[2] = 0.0;
        du[3] = -p[0];
        break;
    case ORC_THRESHOLD_DOSE:
        du[0] = -p[0] * u[0];
        break;
    case ORC_LOTKA_VOLTERRA:
        du[0] = p[0] * u[0] - p[1] * u[0] * u[1];
        du[1] = p[3] * u[0] * u[1] - p[2] * u[1];
        break;
    case ORC_OREGONATOR:
        du[0] = p[0] * (u[1] + u[0] * (1.0 - p[2] * u[0] - u[1]));
        du[1] = (u[2] - (1.0 + u[0]) * u[1]) / p[0];
        du[2] = p[1] * (u[0] - u[2]);
        break;
    case ORC_FORCED_DUFFING:
        du[0] = u[1];
        du[1] = ((p[3] * std::cos(p[4] * t) - p[0] * u[1]) - p[1] * u[0]) - p[2] * (u[0] * u[0] * u[0]);
        break;
    case ORC_BOUNCING_BALL:
        du[0] = u[1];
        du[1] = -p[0];
        break;
    case ORC_VANDERPOL:   // test/InterfaceI/stiffness_detection_test.jl:10-16: mu ((1 - x^2) y - x)
        du[0] = u[1];
        du[1] = p[0] * ((1.0 - u[0] * u[0]) * u[1] - u[0]);
        break;
    case ORC_PK1:   // one-compartment PK, first-order absorption: p = (ka, ke, dose)
        du[0] = -p[0] * u[0];
        du[1] = p[0] * u[0] - p[1] * u[1];
        break;
    case ORC_LINEAR:
        for (int i = 0; i < n; ++i) du[i] = p[0] * u[i];
        break;
    case ORC_LORENZ:
        du[0] = p[0] * (u[1] - u[0]);
        du[1] = u[0] * (p[1] - u[2]) - u[1];
        du[2] = u[0] * u[1] - p[2] * u[2];
        break;
    case ORC_ROBERTSON: {
        double y1 = u[0], y2 = u[1], y3 = u[2];
        du[0] = -p[0] * y1 + p[2] * y2 * y3;
        du[1] = p[0] * y1 - p[1] * (y2 * y2) - p[2] * y2 * y3;
        du[2] = p[1] * (y2 * y2);
        break;
    }
    case ORC_DUFFING: {
        int N = n / 2;
        for (int i = 0; i < N; ++i) {
            double x = u[2 * i], v = u[2 * i + 1];
            double xl = i > 0 ? u[2 * i - 2] : 0.0;
            double xr = i < N - 1 ? u[2 * i + 2] : 0.0;
            double lap = (xl + xr) - 2.0 * x;
            du[2 * i] = v;
            du[2 * i + 1] = (p[0] * lap - p[1] * v) - p[2] * (x * x * x);
        }
        break;
    }
    case ORC_BRUSSELATOR: {
        int N = n / 2;
        double ae = p[2] * ((double)N * (double)N);
        for (int i = 0; i < N; ++i) {
            int il = i == 0 ? N - 1 : i - 1, ir = i == N - 1 ? 0 : i + 1;
            double uu = u[2 * i], vv = u[2 * i + 1];
            double lu = (u[2 * il] + u[2 * ir]) - 2.0 * uu;
            double lv = (u[2 * il + 1] + u[2 * ir + 1]) - 2.0 * vv;
            double u2v = uu * uu * vv;
            du[2 * i] = ((p[0] + u2v) - (p[1] + 1.0) * uu) + ae * lu;
            du[2 * i + 1] = (p[1] * uu - u2v) + ae * lv;
        }
        break;
    }
    }
}

// Parameters each model reads (the dense record keeps a copy for the Vern7 extra stages).
int model_nparams(int model) {
    switch (model) {
    case ORC_LINEAR: case ORC_VANDERPOL: return 1;
    case ORC_LOTKA_VOLTERRA: return 4;
    case ORC_FORCED_DUFFING: return 5;
    default: return 3;   // ORC_THRESHOLD_DOSE and ORC_BALL_BOX read at most 3 (callbacks included)
    }
}

// Analytic Jacobians (row-major J[i*n + j] = d f_i / d u_j).
void jac(int model, int n, const double* u, const double* p, double t, double* J) {
    (void)t;
    std::memset(J, 0, sizeof(double) * n * n);
    switch (model) {
    case ORC_BALL_BOX:
        J[2] = 1.0;
        J[7] = 1.0;
        break;
    case ORC_THRESHOLD_DOSE:
        J[0] = -p[0];
        break;
    case ORC_LOTKA_VOLTERRA:
        J[0] = p[0] - p[1] * u[1]; J[1] = -p[1] * u[0];
        J[2] = p[3] * u[1];        J[3] = p[3] * u[0] - p[2];
        break;
    case ORC_OREGONATOR:
        J[0] = p[0] * (1.0 - 2.0 * p[2] * u[0] - u[1]); J[1] = p[0] * (1.0 - u[0]); J[2] = 0.0;
        J[3] = -u[1] / p[0]; J[4] = -(1.0 + u[0]) / p[0]; J[5] = 1.0 / p[0];
        J[6] = p[1]; J[7] = 0.0; J[8] = -p[1];
        break;
    case ORC_FORCED_DUFFING:
        J[1] = 1.0;
        J[2] = -p[1] - p[2] * (3.0 * (u[0] * u[0]));
        J[3] = -p[0];
        break;
    case ORC_BOUNCING_BALL:
        J[1] = 1.0;
        break;
    case ORC_VANDERPOL:
        J[1] = 1.0;
        J[2] = p[0] * (-2.0 * u[0] * u[1] - 1.0);
        J[3] = p[0] * (1.0 - u[0] * u[0]);
        break;
    case ORC_PK1:
        J[0] = -p[0];
        J[2] = p[0];
        J[3] = -p[1];
        break;
    case ORC_LINEAR:
        for (int i = 0; i < n; ++i) J[i * n + i] = p[0];
        break;
    case ORC_LORENZ:
        J[0] = -p[0]; J[1] = p[0]; J[2] = 0.0;
        J[3] = p[1] - u[2]; J[4] = -1.0; J[5] = -u[0];
        J[6] = u[1]; J[7] = u[0]; J[8] = -p[2];
        break;
    case ORC_ROBERTSON: {
        double y2 = u[1], y3 = u[2];
        J[0] = -p[0]; J[1] = p[2] * y3; J[2] = p[2] * y2;
        J[3] = p[0]; J[4] = -2.0 * p[1] * y2 - p[2] * y3; J[5] = -p[2] * y2;
        J[6] = 0.0; J[7] = 2.0 * p[1] * y2; J[8] = 0.0;
        break;
    }
    case ORC_DUFFING: {
        int N = n / 2;
        for (int i = 0; i < N; ++i) {
            double x = u[2 * i];
            int rx = 2 * i, rv = 2 * i + 1;
            J[rx * n + rv] = 1.0;
            J[rv * n + rx] = -2.0 * p[0] - p[2] * (3.0 * (x * x));
            J[rv * n + rv] = -p[1];
            if (i > 0) J[rv * n + rx - 2] = p[0];
            if (i < N - 1) J[rv * n + rx + 2] = p[0];
        }
        break;
    }
    case ORC_BRUSSELATOR: {
        int N = n / 2;
        double ae = p[2] * ((double)N * (double)N);
        for (int i = 0; i < N; ++i) {
            int il = i == 0 ? N - 1 : i - 1, ir = i == N - 1 ? 0 : i + 1;
            double uu = u[2 * i], vv = u[2 * i + 1];
            int ru = 2 * i, rv = 2 * i + 1;
            J[ru * n + ru] = (2.0 * uu * vv - (p[1] + 1.0)) - 2.0 * ae;
            J[ru * n + rv] = uu * uu;
            J[ru * n + 2 * il] += ae;
            J[ru * n + 2 * ir] += ae;
            J[rv * n + ru] = p[1] - 2.0 * uu * vv;
            J[rv * n + rv] = -(uu * uu) - 2.0 * ae;
            J[rv * n + 2 * il + 1] += ae;
            J[rv * n + 2 * ir + 1] += ae;
        }
        break;
    }
    }
}

// Analytic time derivative df/dt (ODEFunction's tgrad) of the non-autonomous
// models; false for the others (autonomous: the reference differentiates f in t
// by AD, one counted f call, and gets 0).
bool tgrad(int model, int n, const double* u, const double* p, double t, double* dT) {
    (void)u;
    if (model != ORC_FORCED_DUFFING) return false;
    std::fill(dT, dT + n, 0.0);
    dT[1] = -(p[3] * p[4]) * std::sin(p[4] * t);
    return true;
}

// ---------------------------------------------------------------- integrator
struct Step {  // one accepted step for dense output
    double tprev, tend;
    std::vector<double> y0, y1, k;  // k: nk * n (Vern7: k1..k10; the extra stages are formed when evaluated)
};

struct Dense {
    int alg, model, n;
    std::vector<double> p;
    std::vector<Step> steps;
};

struct Integ {
    int alg, model, n;
    const double* p;
    double t0, tf;
    double tdir;   // sign(tf - t0) (solve.jl:273); +1 for t0 == tf
    orc_opts o;
    double t, dt, tprev, dtpropose, dtcache;
    double EEst, q11, errold;
    double beta1, beta2, qmin, qmax, qmax_first, gamma, qsteady_min, qsteady_max, qoldinit;
    int order;
    int64_t iter, success_iter;
    bool isout = false;   // the last attempt ended out of the domain (isoutofdomain)
    bool accept_step, next_step_tstop;
    double tstop_target;
    std::vector<double> u, uprev, tmp, utilde, atmp, fsalfirst, fsallast;
    std::vector<double> k;  // up to 16 stage vectors (or Rodas dense k1..k3), row k[s*n + i]
    int nk_valid;          // Vern7 lazy: 10 until extra stages computed
    // Rodas
    std::vector<double> J, W, dT, ks, rhs, du;
    std::vector<int> piv;
    bool have_J;
    // Rosenbrock23's JacReuseState (rosenbrock_caches.jl:25-60)
    double jr_last_dtgamma, jr_pending_dtgamma;
    int64_t jr_last_naccept, jr_last_step_iter;
    bool recomputing;   // inside recompute_step_k (ode_addsteps! after an event)
    std::vector<double> tstops;  // tdir * t, ascending (the reference's directional heap)
    size_t itstop;
    std::vector<double> dtimes;  // the tstops as given, sorted: the discrete callback's times
    std::vector<double> saveat;  // tdir * t, ascending
    size_t isave;
    double* t_out;
    double* u_out;
    int cap, nsaved;
    double last_saved_t;
    orc_stats st;
    Dense* dense;
    std::vector<double> dense_last_u;   // u of the last save (the next dense interval's start)
    std::vector<double> interp_out;
    // AutoTsit5(Rosenbrock23()): the composite's state (AutoSwitchCache,
    // composite_algs.jl:55-94) and one PI controller state per method
    int current;                 // 0 Tsit5, 1 Rosenbrock23
    int as_count, successive_switches;
    bool is_stiffalg, do_error_check;
    double eigen_est;
    double ctl_errold[2], ctl_q11[2];
    std::vector<double> g6;
    std::vector<int32_t> alg_choice;
    // continuous callback state (integrator.event_last_time, last_event_error)
    int event_last_time;
    double last_event_error;
    bool prev_events[8];   // the components of the last vector event
    bool reeval_fsal, terminated;
    std::vector<double> cb_tmp;
};

thread_local int64_t g_rhs_calls = 0;  // counts every RHS call (the reference's counting-wrapper tests)
thread_local std::vector<double> g_eval_times;   // the t of every RHS call, while recording
thread_local bool g_record_times = false;

inline void f_eval(Integ& I, const double* u, double t, double* du) {
    ++g_rhs_calls;
    if (g_record_times) g_eval_times.push_back(t);
    rhs(I.model, I.n, u, I.p, t, du);
}

// calculate_residuals + ODE_DEFAULT_NORM:
// lib/DiffEqBase/src/calculate_residuals.jl:9-14,117-125 and
// lib/DiffEqBase/src/common_defaults.jl:69-75 (sqrt(sum(abs2)/n)).  Array
// tolerances (the broadcast over abstol and reltol) give state i its own.
inline double abstol_at(const Integ& I, int i) { return I.o.abstol_vec ? I.o.abstol_vec[i] : I.o.abstol; }
inline double reltol_at(const Integ& I, int i) { return I.o.reltol_vec ? I.o.reltol_vec[i] : I.o.reltol; }

double residual_norm(Integ& I, const double* ut, const double* u0, const double* u1) {
    double acc = 0.0;
    for (int i = 0; i < I.n; ++i) {
        double sc = std::fma(jmax(std::fabs(u0[i]), std::fabs(u1[i])), reltol_at(I, i), abstol_at(I, i));
        double e = ut[i] / sc;
        acc = std::fma(e, e, acc);
    }
    return std::sqrt(acc / (double)(I.n > 1 ? I.n : 1));
}

// Hairer initial step: lib/OrdinaryDiffEqCore/src/initdt.jl:17-298 (iip); the
// result carries the direction tdir.  Its dtmax is the distance to the first
// tstop when that is smaller (_determine_initdt, integrator_interface.jl:644-656),
// so the trial evaluation stays before it.
double initdt(Integ& I) {
    int n = I.n;
    const double* u0 = I.u.data();
    double t = I.t;
    const double tdir = I.tdir;
    const double first_tstop = I.itstop < I.tstops.size() ? I.tstops[I.itstop] : tdir * I.tf;
    double dtmax = jmin(std::fabs(I.o.dtmax), std::fabs(first_tstop - tdir * t));   // dtmax_tdir
    double dtmin = std::nextafter(jmax(I.o.dtmin, jeps(t)), INFINITY);
    double smalldt = jmax(dtmin, 1e-6);
    std::vector<double> sk(n), f0(n), f1(n), u1(n), tmp(n);
    for (int i = 0; i < n; ++i) sk[i] = std::fma(std::fabs(u0[i]), reltol_at(I, i), abstol_at(I, i));
    f_eval(I, u0, t, f0.data());
    if (I.alg == ORC_TSIT5) I.fsallast = f0;
    auto nrm = [&](const std::vector<double>& v) {
        double a = 0.0;
        for (int i = 0; i < n; ++i) a = std::fma(v[i], v[i], a);
        return std::sqrt(a / (double)n);
    };
    for (int i = 0; i < n; ++i) tmp[i] = u0[i] / sk[i];
    double d0 = nrm(tmp);
    for (int i = 0; i < n; ++i) tmp[i] = f0[i] / sk[i];
    double d1 = nrm(tmp);
    if (d1 != d1) return tdir * dtmin;
    double dt0 = (d0 < 1e-5 || d1 < 1e-5) ? smalldt : (d0 / d1) / 100.0;
    dt0 = jmin(dt0, dtmax);
    if (dt0 < 10.0 * 2.220446049250313e-16) return tdir * jmax(smalldt, dtmin);
    const double dt0_tdir = tdir * dt0;
    for (int i = 0; i < n; ++i) u1[i] = std::fma(dt0_tdir, f0[i], u0[i]);
    f_eval(I, u1.data(), t + dt0_tdir, f1.data());
    bool same = true;
    for (int i = 0; i < n; ++i) same = same && (f0[i] == f1[i]);
    if (n > 0 && same) return tdir * jmax(dtmin, 100.0 * dt0);
    for (int i = 0; i < n; ++i) tmp[i] = (f1[i] - f0[i]) / sk[i];
    double d2 = nrm(tmp) / dt0;
    double mx = jmax(d1, d2);
    double dt1;
    if (mx <= 1e-15) {
        dt1 = jmax(1e-6, dt0 * 1e-3);
    } else {
        // 10^(-(2 + log10 mx)/order) = exp(-(2 ln10 + ln mx)/order)
        const double LN10 = 2.302585092994046;
        dt1 = series_exp(-(2.0 * LN10 + series_ln(mx)) / (double)I.order);
    }
    return tdir * jmax(dtmin, jmin(jmin(100.0 * dt0, dt1), dtmax));
}

// ---------------------------------------------------------------- Tsit5
// perform_step!(::Tsit5Cache): lib/OrdinaryDiffEqTsit5/src/tsit_perform_step.jl:309-367.
void tsit5_step(Integ& I) {
    int n = I.n;
    double t = I.t, dt = I.dt;
    const double* up = I.uprev.data();
    double* K = I.k.data();
    auto k = [&](int s) { return K + (s - 1) * n; };
    std::memcpy(k(1), I.fsalfirst.data(), sizeof(double) * n);
    double* tmp = I.tmp.data();
    double a = dt * TSIT5_A[2][1];
    for (int i = 0; i < n; ++i) tmp[i] = std::fma(a, k(1)[i], up[i]);
    f_eval(I, tmp, std::fma(TSIT5_c[2], dt, t), k(2));
    for (int s = 3; s <= 7; ++s) {
        for (int i = 0; i < n; ++i) {
            double acc = TSIT5_A[s][s - 1] * k(s - 1)[i];
            for (int j = s - 2; j >= 1; --j) acc = std::fma(TSIT5_A[s][j], k(j)[i], acc);
            tmp[i] = std::fma(dt, acc, up[i]);
        }
        if (s < 7) {
            if (s == 6 && I.alg == ORC_AUTOTSIT5_ROSENBROCK23) I.g6.assign(tmp, tmp + n);
            f_eval(I, tmp, std::fma(TSIT5_c[s], dt, t), k(s));
        } else {
            std::memcpy(I.u.data(), tmp, sizeof(double) * n);
            f_eval(I, I.u.data(), t + dt, k(7));
        }
    }
    std::memcpy(I.fsallast.data(), k(7), sizeof(double) * n);
    I.st.nf += 6;
    if (I.alg == ORC_AUTOTSIT5_ROSENBROCK23) {
        // stiffness estimate of a composite step (tsit_perform_step.jl:240-246, Hairer II p. 22,
        // Inf norm): max_i |(k7 - k6) / (g7 - g6)|, NaN propagating like Julia's maximum
        double e = 0.0;
        for (int i = 0; i < n; ++i) e = jmax(e, std::fabs((k(7)[i] - k(6)[i]) / (I.u[i] - I.g6[i])));
        I.eigen_est = e;
    }
    if (I.o.adaptive) {
        for (int i = 0; i < n; ++i) {
            double acc = TSIT5_bt[7] * k(7)[i];
            for (int j = 6; j >= 1; --j) acc = std::fma(TSIT5_bt[j], k(j)[i], acc);
            I.utilde[i] = dt * acc;
        }
        I.EEst = residual_norm(I, I.utilde.data(), up, I.u.data());
    }
    I.nk_valid = 7;
}

// Tsit5 interpolant: lib/OrdinaryDiffEqTsit5/src/interpolants.jl:25-65 with
// Tsit5Interp (tsit_tableaus.jl:244-276); @evalpoly is Horner with muladd.
void tsit5_interp(double th, double dt, const double* y0, const double* K, int n, double* out) {
    double b[8];
    double th2 = th * th;
    b[1] = th * std::fma(th, std::fma(th, std::fma(th, TSIT5_R[1][4], TSIT5_R[1][3]), TSIT5_R[1][2]), TSIT5_R[1][1]);
    for (int s = 2; s <= 7; ++s)
        b[s] = th2 * std::fma(th, std::fma(th, TSIT5_R[s][4], TSIT5_R[s][3]), TSIT5_R[s][2]);
    for (int i = 0; i < n; ++i) {
        double acc = K[6 * n + i] * b[7];
        for (int s = 6; s >= 1; --s) acc = std::fma(K[(s - 1) * n + i], b[s], acc);
        out[i] = std::fma(dt, acc, y0[i]);
    }
}

// ---------------------------------------------------------------- Vern7 / Vern9
// Generic explicit RK stage: tmp = uprev + dt * sum_{j in mask} A[s][j] k_j with
// the reference's muladd nesting (last term is the innermost product).
template <int S>
void erk_stage(int n, const double (&A)[S][S], const unsigned char (&Am)[S][S], int s,
               const double* K, const double* up, double dt, double* out) {
    int js[S];
    int nj = 0;
    for (int j = 1; j < s; ++j)
        if (Am[s][j]) js[nj++] = j;
    for (int i = 0; i < n; ++i) {
        double acc = A[s][js[nj - 1]] * K[(js[nj - 1] - 1) * n + i];
        for (int q = nj - 2; q >= 0; --q) acc = std::fma(A[s][js[q]], K[(js[q] - 1) * n + i], acc);
        out[i] = std::fma(dt, acc, up[i]);
    }
}

template <int S>
void erk_combo(int n, const double (&w)[S], const unsigned char (&wm)[S], const double* K,
               double* out_acc) {
    int js[S];
    int nj = 0;
    for (int j = 1; j < S; ++j)
        if (wm[j]) js[nj++] = j;
    for (int i = 0; i < n; ++i) {
        double acc = w[js[nj - 1]] * K[(js[nj - 1] - 1) * n + i];
        for (int q = nj - 2; q >= 0; --q) acc = std::fma(w[js[q]], K[(js[q] - 1) * n + i], acc);
        out_acc[i] = acc;
    }
}

// perform_step!(::Vern7Cache): lib/OrdinaryDiffEqVerner/src/verner_rk_perform_step.jl:412-570 (lazy).
void vern7_step(Integ& I) {
    int n = I.n;
    double t = I.t, dt = I.dt;
    const double* up = I.uprev.data();
    double* K = I.k.data();
    double* tmp = I.tmp.data();
    f_eval(I, up, t, K);
    double a = dt * VERN7_A[2][1];
    for (int i = 0; i < n; ++i) tmp[i] = std::fma(a, K[i], up[i]);
    f_eval(I, tmp, std::fma(VERN7_c[2], dt, t), K + n);
    for (int s = 3; s <= 10; ++s) {
        erk_stage<17>(n, VERN7_A, VERN7_A_m, s, K, up, dt, tmp);
        double ts = (s <= 8) ? std::fma(VERN7_c[s], dt, t) : t + dt;
        f_eval(I, tmp, ts, K + (s - 1) * n);
    }
    std::vector<double> acc(n);
    erk_combo<17>(n, VERN7_b, VERN7_b_m, K, acc.data());
    for (int i = 0; i < n; ++i) I.u[i] = std::fma(dt, acc[i], up[i]);
    I.st.nf += 10;
    if (I.o.adaptive) {
        erk_combo<17>(n, VERN7_bt, VERN7_bt_m, K, acc.data());
        for (int i = 0; i < n; ++i) I.utilde[i] = dt * acc[i];
        I.EEst = residual_norm(I, I.utilde.data(), up, I.u.data());
    }
    I.nk_valid = 10;
}

// Lazy extra stages: lib/OrdinaryDiffEqVerner/src/verner_addsteps.jl:80-195
// (called with tprev, uprev, dt of the step).  Not counted in nf.
void vern7_extra(int model, int n, const double* p, double tprev, double dt, const double* up, double* K) {
    std::vector<double> tmp(n);
    for (int s = 11; s <= 16; ++s) {
        erk_stage<17>(n, VERN7_A, VERN7_A_m, s, K, up, dt, tmp.data());
        rhs(model, n, tmp.data(), p, std::fma(VERN7_c[s], dt, tprev), K + (s - 1) * n);
    }
}

// Vern7 interpolant: lib/OrdinaryDiffEqVerner/src/interpolants.jl:183-252.
void vern7_interp(double th, double dt, const double* y0, const double* K, int n, double* out) {
    static const int idx[13] = {1, 4, 5, 6, 7, 8, 9, 11, 12, 13, 14, 15, 16};
    double b[17];
    double th2 = th * th;
    {
        double acc = VERN7_R[1][7];
        for (int p = 6; p >= 1; --p) acc = std::fma(th, acc, VERN7_R[1][p]);
        b[1] = th * acc;
    }
    for (int q = 1; q < 13; ++q) {
        int s = idx[q];
        double acc = VERN7_R[s][7];
        for (int p = 6; p >= 2; --p) acc = std::fma(th, acc, VERN7_R[s][p]);
        b[s] = th2 * acc;
    }
    for (int i = 0; i < n; ++i) {
        double acc = K[(16 - 1) * n + i] * b[16];
        for (int q = 11; q >= 0; --q) acc = std::fma(K[(idx[q] - 1) * n + i], b[idx[q]], acc);
        out[i] = std::fma(dt, acc, y0[i]);
    }
}

// perform_step!(::Vern9Cache): lib/OrdinaryDiffEqVerner/src/verner_rk_perform_step.jl:1272-1420
// (used only as the high-accuracy ground truth; saves are hit as tstops).
void vern9_step(Integ& I) {
    int n = I.n;
    double t = I.t, dt = I.dt;
    const double* up = I.uprev.data();
    double* K = I.k.data();
    double* tmp = I.tmp.data();
    f_eval(I, up, t, K);
    double a = dt * VERN9_A[2][1];
    for (int i = 0; i < n; ++i) tmp[i] = std::fma(a, K[i], up[i]);
    f_eval(I, tmp, std::fma(VERN9_c[2], dt, t), K + n);
    for (int s = 3; s <= 16; ++s) {
        erk_stage<17>(n, VERN9_A, VERN9_A_m, s, K, up, dt, tmp);
        double ts = (s <= 14) ? std::fma(VERN9_c[s], dt, t) : t + dt;
        f_eval(I, tmp, ts, K + (s - 1) * n);
    }
    std::vector<double> acc(n);
    erk_combo<17>(n, VERN9_b, VERN9_b_m, K, acc.data());
    for (int i = 0; i < n; ++i) I.u[i] = std::fma(dt, acc[i], up[i]);
    I.st.nf += 16;
    if (I.o.adaptive) {
        erk_combo<17>(n, VERN9_bt, VERN9_bt_m, K, acc.data());
        for (int i = 0; i < n; ++i) I.utilde[i] = dt * acc[i];
        I.EEst = residual_norm(I, I.utilde.data(), up, I.u.data());
    }
    I.nk_valid = 16;
}

// ---------------------------------------------------------------- Rodas5P
// LU with partial pivoting (row of largest |pivot|, first on ties) and the
// triangular solves; stands in for LinearSolve's dense LU (not vendored).
bool lu_factor(int n, double* W, int* piv) {
    bool ok = true;
    for (int c = 0; c < n; ++c) {
        int pr = c;
        double best = std::fabs(W[c * n + c]);
        for (int r = c + 1; r < n; ++r) {
            double v = std::fabs(W[r * n + c]);
            if (v > best) { best = v; pr = r; }
        }
        piv[c] = pr;
        if (pr != c)
            for (int j = 0; j < n; ++j) std::swap(W[c * n + j], W[pr * n + j]);
        double d = W[c * n + c];
        if (d == 0.0) { ok = false; continue; }
        double inv = 1.0 / d;
        for (int r = c + 1; r < n; ++r) {
            double l = W[r * n + c] * inv;
            W[r * n + c] = l;
            for (int j = c + 1; j < n; ++j) W[r * n + j] = std::fma(-l, W[c * n + j], W[r * n + j]);
        }
    }
    return ok;
}
void lu_solve(int n, const double* LU, const int* piv, double* b) {
    for (int c = 0; c < n; ++c)
        if (piv[c] != c) std::swap(b[c], b[piv[c]]);
    for (int r = 1; r < n; ++r) {
        double acc = b[r];
        for (int j = 0; j < r; ++j) acc = std::fma(-LU[r * n + j], b[j], acc);
        b[r] = acc;
    }
    for (int r = n - 1; r >= 0; --r) {
        double acc = b[r];
        for (int j = r + 1; j < n; ++j) acc = std::fma(-LU[r * n + j], b[j], acc);
        b[r] = acc / LU[r * n + r];
    }
}

// perform_step!(::RosenbrockCache): lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_perform_step.jl:729-847,
// fused helpers :581-727 (left-to-right muladd accumulation), W = J - I/dtgamma
// (lib/OrdinaryDiffEqDifferentiation/src/derivative_utils.jl:663-685), J reused
// after a rejected step (do_newJW, :535-557).  Autonomous models: dT = 0; the
// reference evaluates it by AD (one counted f call per fresh J, :181-227).
void rodas5p_step(Integ& I) {
    int n = I.n;
    double t = I.t, dt = I.dt;
    const double* up = I.uprev.data();
    double invdt = 1.0 / dt;
    double dtC[8][7], dtd[8];
    for (int s = 0; s < 8; ++s) {
        for (int j = 0; j < 7; ++j) dtC[s][j] = RODAS5P_C[s][j] * invdt;
        dtd[s] = dt * RODAS5P_d[s];
    }
    double dtgamma = dt * RODAS5P_GAMMA;
    double* fsal = I.fsalfirst.data();
    f_eval(I, up, t, fsal);
    I.st.nf += 1;
    bool errorfail = I.EEst > 1.0;
    bool new_jac = !(I.iter > 1 && errorfail) || !I.have_J;
    if (I.iter <= 1) new_jac = true;
    if (new_jac) {
        jac(I.model, n, up, I.p, t, I.J.data());
        I.st.njacs += 1;
        // calc_tderivative! (derivative_utils.jl:181-227), with a fresh J only
        // (:1040): the model's tgrad, else the reference differentiates f in t by
        // AD (one counted call), exactly zero for the autonomous models here.
        if (!tgrad(I.model, n, up, I.p, t, I.dT.data())) {
            f_eval(I, up, t, I.du.data());
            std::fill(I.dT.begin(), I.dT.end(), 0.0);
            I.st.nf += 1;
        }
        I.have_J = true;
    }
    double invdtgamma = 1.0 / dtgamma;
    for (int i = 0; i < n * n; ++i) I.W[i] = I.J[i];
    for (int i = 0; i < n; ++i) I.W[i * n + i] = std::fma(-1.0, invdtgamma, I.J[i * n + i]);
    I.st.nw += 1;
    lu_factor(n, I.W.data(), I.piv.data());
    double* ks = I.ks.data();
    double* r = I.rhs.data();
    for (int i = 0; i < n; ++i) r[i] = fsal[i] + dtd[0] * I.dT[i];
    lu_solve(n, I.W.data(), I.piv.data(), r);
    for (int i = 0; i < n; ++i) ks[i] = -r[i];
    I.st.nsolve += 1;
    double* u = I.u.data();
    double* du = I.du.data();
    for (int s = 1; s < 8; ++s) {
        for (int i = 0; i < n; ++i) {
            double acc = up[i];
            for (int j = 0; j < s; ++j) acc = std::fma(RODAS5P_A[s][j], ks[j * n + i], acc);
            u[i] = acc;
        }
        f_eval(I, u, std::fma(RODAS5P_cc[s], dt, t), du);
        I.st.nf += 1;
        for (int i = 0; i < n; ++i) {
            double acc = std::fma(dtd[s], I.dT[i], du[i]);
            for (int j = 0; j < s; ++j) acc = std::fma(dtC[s][j], ks[j * n + i], acc);
            r[i] = acc;
        }
        lu_solve(n, I.W.data(), I.piv.data(), r);
        for (int i = 0; i < n; ++i) ks[s * n + i] = -r[i];
        I.st.nsolve += 1;
    }
    // b = (A[8,1:7]..., 1), btilde = e_8 (rosenbrock_tableaus.jl:64-72)
    for (int i = 0; i < n; ++i) {
        double acc = up[i];
        for (int j = 0; j < 7; ++j) acc = std::fma(RODAS5P_A[7][j], ks[j * n + i], acc);
        acc = std::fma(1.0, ks[7 * n + i], acc);
        u[i] = acc;
    }
    if (I.o.adaptive) {
        for (int i = 0; i < n; ++i) I.utilde[i] = ks[7 * n + i];
        I.EEst = residual_norm(I, I.utilde.data(), up, u);
    }
    // dense k_j = sum_i H[j,i] ks_i
    double* K = I.k.data();
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < n; ++i) {
            double acc = 0.0;
            for (int q = 0; q < 8; ++q) acc = std::fma(RODAS5P_H[j][q], ks[q * n + i], acc);
            K[j * n + i] = acc;
        }
    I.nk_valid = 3;
}

// Rodas interpolant (interp_order 3): lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_interpolants.jl:172-206.
void rodas_interp(double th, const double* y0, const double* y1, const double* K, int n, double* out) {
    double th1 = 1.0 - th;
    for (int i = 0; i < n; ++i) {
        double inner = std::fma(th, K[2 * n + i], K[n + i]);            // k2 + th*k3
        inner = std::fma(th, inner, K[i]);                              // k1 + th*(...)
        double v = std::fma(th1, inner, y1[i]);                         // y1 + th1*(...)
        out[i] = std::fma(th1, y0[i], th * v);                          // th1*y0 + th*(...)
    }
}

// _rosenbrock_jac_reuse_decision (lib/OrdinaryDiffEqDifferentiation/src/derivative_utils.jl:
// 46-170) for Rosenbrock23, a W-method with reuse state, no mass matrix and not linear:
// true when J (and W) must be fresh.  derivative_discontinuity is false here: the
// callbacks' reeval_internals_due_to_modification! clears it before the next step.
bool jac_reuse_decision(Integ& I, double dtgamma) {
    if (I.iter <= 1) return true;
    if (!I.o.adaptive) return true;
    const int64_t naccept = I.st.naccept;
    if (naccept > I.jr_last_naccept) I.jr_last_dtgamma = I.jr_pending_dtgamma;
    if (I.jr_last_dtgamma == 0.0) return true;
    if (I.jr_last_step_iter != 0 && I.iter > I.jr_last_step_iter + 1) return true;
    if (I.EEst > 1.0) return true;
    const double tol = I.o.jac_reuse_gamma_tol < 0 ? 0.03 : I.o.jac_reuse_gamma_tol;
    if (std::fabs(dtgamma / I.jr_last_dtgamma - 1.0) > tol) return true;
    if (naccept - I.jr_last_naccept >= I.o.max_jac_age) {
        I.jr_last_naccept = naccept;
        return true;
    }
    return false;
}

// perform_step!(::Rosenbrock23Cache): lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_perform_step.jl:34-146,
// tableau rosenbrock_tableaus.jl:6-10 (c32 = 6 + sqrt(2), d = 1/(2 + sqrt(2))).  A W-method
// whose default max_jac_age = 1 (algorithms.jl:108-115) makes the reuse decision
// (derivative_utils.jl:46-170) take a fresh J and W on every attempt, rejected or
// not.  FSAL: fsalfirst is f(uprev), carried from the last accepted step.
// Multiply-adds follow @muladd: a - b*c -> muladd(-b, c, a).
void rosenbrock23_step(Integ& I) {
    const int n = I.n;
    const double t = I.t, dt = I.dt;
    const double c32 = 6.0 + std::sqrt(2.0), d = 1.0 / (2.0 + std::sqrt(2.0));
    const double* up = I.uprev.data();
    const double dtgamma = dt * d;
    const double neginvdtgamma = -(1.0 / dtgamma);
    const double dto2 = dt / 2.0, dto6 = dt / 6.0;
    // calc_rosenbrock_differentiation! (derivative_utils.jl:1011-1041): the reuse
    // decision (a composite always takes a fresh J); J and dT only when fresh.  An
    // event's recomputation (the in-place ode_addsteps!) keeps the cached J and dT.
    bool new_jac = true;
    if (I.recomputing) {
        new_jac = false;
    } else if (I.alg == ORC_ROSENBROCK23) {
        new_jac = jac_reuse_decision(I, dtgamma);
        I.jr_last_step_iter = I.iter;
        if (new_jac) I.jr_pending_dtgamma = dtgamma;
    }
    if (new_jac) {
        jac(I.model, n, up, I.p, t, I.J.data());
        I.st.njacs += 1;
        // the model's tgrad, else the reference differentiates f in t by AD (one counted
        // call; autonomous models: dT = 0)
        if (!tgrad(I.model, n, up, I.p, t, I.dT.data())) {
            f_eval(I, up, t, I.du.data());
            std::fill(I.dT.begin(), I.dT.end(), 0.0);
            I.st.nf += 1;
        }
    }
    const double invdtgamma = 1.0 / dtgamma;
    for (int i = 0; i < n * n; ++i) I.W[i] = I.J[i];
    for (int i = 0; i < n; ++i) I.W[i * n + i] = std::fma(-1.0, invdtgamma, I.J[i * n + i]);
    I.st.nw += 1;
    lu_factor(n, I.W.data(), I.piv.data());
    const double* fsal0 = I.fsalfirst.data();
    double* r = I.rhs.data();
    double* k1 = I.ks.data();
    double* k2 = k1 + n;
    double* k3 = k1 + 2 * n;
    double* f1 = k1 + 3 * n;
    // fsalfirst + dtd1 dT: calc_tderivative! is not under @muladd (plain ops)
    for (int i = 0; i < n; ++i) r[i] = fsal0[i] + dtgamma * I.dT[i];
    lu_solve(n, I.W.data(), I.piv.data(), r);
    for (int i = 0; i < n; ++i) k1[i] = r[i] * neginvdtgamma;
    I.st.nsolve += 1;
    double* u = I.u.data();
    for (int i = 0; i < n; ++i) u[i] = std::fma(dto2, k1[i], up[i]);
    f_eval(I, u, t + dto2, f1);
    I.st.nf += 1;
    for (int i = 0; i < n; ++i) r[i] = f1[i] - k1[i];
    lu_solve(n, I.W.data(), I.piv.data(), r);
    for (int i = 0; i < n; ++i) k2[i] = std::fma(r[i], neginvdtgamma, k1[i]);
    I.st.nsolve += 1;
    for (int i = 0; i < n; ++i) u[i] = std::fma(dt, k2[i], up[i]);
    if (I.o.adaptive) {
        double* fl = I.fsallast.data();
        f_eval(I, u, t + dt, fl);
        I.st.nf += 1;
        for (int i = 0; i < n; ++i) {
            double acc = std::fma(-c32, k2[i] - f1[i], fl[i]);
            acc = std::fma(-2.0, k1[i] - fsal0[i], acc);
            r[i] = std::fma(dt, I.dT[i], acc);
        }
        lu_solve(n, I.W.data(), I.piv.data(), r);
        for (int i = 0; i < n; ++i) k3[i] = r[i] * neginvdtgamma;
        I.st.nsolve += 1;
        for (int i = 0; i < n; ++i) I.utilde[i] = dto6 * (std::fma(-2.0, k2[i], k1[i]) + k3[i]);
        I.EEst = residual_norm(I, I.utilde.data(), up, u);
    } else {
        f_eval(I, u, t + dt, I.fsallast.data());
        I.st.nf += 1;
    }
    // integrator.k = [k1, k2] (initialize!, rosenbrock_perform_step.jl:1-14)
    std::memcpy(I.k.data(), k1, sizeof(double) * n);
    std::memcpy(I.k.data() + n, k2, sizeof(double) * n);
    I.nk_valid = 2;
}

// Rosenbrock23 interpolant: lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_interpolants.jl:39-67
// (c1 = th(1-th)/(1-2d), c2 = th(th-2d)/(1-2d); y0 + dt (c1 k1 + c2 k2)).
void ros23_interp(double th, double dt, const double* y0, const double* K, int n, double* out) {
    const double d = 1.0 / (2.0 + std::sqrt(2.0));
    const double c1 = th * (1.0 - th) / (1.0 - 2.0 * d);
    const double c2 = th * (th - 2.0 * d) / (1.0 - 2.0 * d);
    for (int i = 0; i < n; ++i) out[i] = std::fma(dt, std::fma(c1, K[i], c2 * K[n + i]), y0[i]);
}

// sol(t, Val{1}): the derivatives of the interpolants in t.
// Tsit5 (lib/OrdinaryDiffEqTsit5/src/interpolants.jl:143-178): sum_i k_i b_i'(th) with
// b1' = @evalpoly(th, r11, 2 r12, 3 r13, 4 r14), bi' = th @evalpoly(th, 2 ri2, 3 ri3, 4 ri4).
void tsit5_interp_d1(double th, const double* K, int n, double* out) {
    double b[8];
    b[1] = std::fma(th, std::fma(th, std::fma(th, 4.0 * TSIT5_R[1][4], 3.0 * TSIT5_R[1][3]), 2.0 * TSIT5_R[1][2]),
                    TSIT5_R[1][1]);
    for (int s = 2; s <= 7; ++s)
        b[s] = th * std::fma(th, std::fma(th, 4.0 * TSIT5_R[s][4], 3.0 * TSIT5_R[s][3]), 2.0 * TSIT5_R[s][2]);
    for (int i = 0; i < n; ++i) {
        double acc = K[6 * n + i] * b[7];
        for (int s = 6; s >= 1; --s) acc = std::fma(K[(s - 1) * n + i], b[s], acc);
        out[i] = acc;
    }
}

// Tsit5's second derivative (interpolants.jl: tsit5pre2, Val{2}): sum_i k_i b_i''(th) / dt,
// b_i'' = evalpoly(th, 2 r_i2, 6 r_i3, 12 r_i4).
void tsit5_interp_d2(double th, double dt, const double* K, int n, double* out) {
    double b[8];
    for (int s = 1; s <= 7; ++s)
        b[s] = std::fma(th, std::fma(th, 12.0 * TSIT5_R[s][4], 6.0 * TSIT5_R[s][3]), 2.0 * TSIT5_R[s][2]);
    const double invdt = 1.0 / dt;
    for (int i = 0; i < n; ++i) {
        double acc = K[6 * n + i] * b[7];
        for (int s = 6; s >= 1; --s) acc = std::fma(K[(s - 1) * n + i], b[s], acc);
        out[i] = acc * invdt;
    }
}

// Tsit5's third derivative (tsit5pre3, Val{3}): sum_i k_i b_i'''(th) inv(dt)^2,
// b_i''' = evalpoly(th, 6 r_i3, 24 r_i4).
void tsit5_interp_d3(double th, double dt, const double* K, int n, double* out) {
    double b[8];
    for (int s = 1; s <= 7; ++s) b[s] = std::fma(th, 24.0 * TSIT5_R[s][4], 6.0 * TSIT5_R[s][3]);
    const double invdt = 1.0 / dt, invdt2 = invdt * invdt;
    for (int i = 0; i < n; ++i) {
        double acc = K[6 * n + i] * b[7];
        for (int s = 6; s >= 1; --s) acc = std::fma(K[(s - 1) * n + i], b[s], acc);
        out[i] = acc * invdt2;
    }
}

// Rodas5P's third derivative (rosenbrock_interpolants.jl:644-653, interp_order 3):
// (-6 k2 + 6 k3 - 24 th k3) / dt^3
void rodas_interp_d3(double th, double dt, const double* K, int n, double* out) {
    for (int i = 0; i < n; ++i) {
        const double k2 = K[n + i], k3 = K[2 * n + i];
        out[i] = std::fma(-6.0, k2, std::fma(6.0, k3, -24.0 * th * k3)) / (dt * dt * dt);
    }
}

// Rodas5P's second derivative (rosenbrock_interpolants.jl:544-560, interp_order 3):
// (-2 k1 + 2 k2 + th (-6 k2 + 6 k3 - 12 th k3)) / dt^2
void rodas_interp_d2(double th, double dt, const double* K, int n, double* out) {
    for (int i = 0; i < n; ++i) {
        const double k1 = K[i], k2 = K[n + i], k3 = K[2 * n + i];
        const double in2 = std::fma(-6.0, k2, std::fma(6.0, k3, -12.0 * th * k3));
        out[i] = std::fma(th, in2, std::fma(-2.0, k1, 2.0 * k2)) / (dt * dt);
    }
}

// Vern7 (lib/OrdinaryDiffEqVerner/src/interpolants.jl:305-334), the extra stages formed.
void vern7_interp_d1(double th, const double* K, int n, double* out) {
    static const int idx[13] = {1, 4, 5, 6, 7, 8, 9, 11, 12, 13, 14, 15, 16};
    double b[17];
    {
        double acc = 7.0 * VERN7_R[1][7];
        for (int p = 6; p >= 1; --p) acc = std::fma(th, acc, (double)p * VERN7_R[1][p]);
        b[1] = acc;
    }
    for (int q = 1; q < 13; ++q) {
        const int s = idx[q];
        double acc = 7.0 * VERN7_R[s][7];
        for (int p = 6; p >= 2; --p) acc = std::fma(th, acc, (double)p * VERN7_R[s][p]);
        b[s] = th * acc;
    }
    for (int i = 0; i < n; ++i) {
        double acc = K[(16 - 1) * n + i] * b[16];
        for (int q = 11; q >= 0; --q) acc = std::fma(K[(idx[q] - 1) * n + i], b[idx[q]], acc);
        out[i] = acc;
    }
}

// Rodas5P, interp_order 3 (lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_interpolants.jl:444-470):
// (k1 + th (-2 k1 + 2 k2 + th (-3 k2 + 3 k3 - 4 th k3)) - y0 + y1) / dt
void rodas_interp_d1(double th, double dt, const double* y0, const double* y1, const double* K, int n,
                     double* out) {
    for (int i = 0; i < n; ++i) {
        const double k1 = K[i], k2 = K[n + i], k3 = K[2 * n + i];
        const double in2 = std::fma(-3.0, k2, std::fma(3.0, k3, -4.0 * th * k3));
        const double in1 = std::fma(th, in2, std::fma(-2.0, k1, 2.0 * k2));
        out[i] = ((std::fma(th, in1, k1) - y0[i]) + y1[i]) / dt;
    }
}

// Rosenbrock23 (rosenbrock_interpolants.jl:111-127): c1' k1 + c2' k2 with
// c1' = (1 - 2 th)/(1 - 2d), c2' = (2 th - 2d)/(1 - 2d).
void ros23_interp_d1(double th, const double* K, int n, double* out) {
    const double d = 1.0 / (2.0 + std::sqrt(2.0));
    const double c1 = (1.0 - 2.0 * th) / (1.0 - 2.0 * d);
    const double c2 = (2.0 * th - 2.0 * d) / (1.0 - 2.0 * d);
    for (int i = 0; i < n; ++i) out[i] = std::fma(c1, K[i], c2 * K[n + i]);
}

void do_step(Integ& I) {
    switch (I.alg) {
    case ORC_AUTOTSIT5_ROSENBROCK23:   // perform_step!(::CompositeCache): the current method
        if (I.current == 0) tsit5_step(I);
        else rosenbrock23_step(I);
        break;
    case ORC_TSIT5: tsit5_step(I); break;
    case ORC_VERN7: vern7_step(I); break;
    case ORC_VERN9: vern9_step(I); break;
    case ORC_RODAS5P: rodas5p_step(I); break;
    case ORC_ROSENBROCK23: rosenbrock23_step(I); break;
    }
}

void interpolate(Integ& I, double th, double* out) {
    int n = I.n;
    const int alg = I.alg == ORC_AUTOTSIT5_ROSENBROCK23 ? (I.current == 0 ? ORC_TSIT5 : ORC_ROSENBROCK23) : I.alg;
    switch (alg) {
    case ORC_TSIT5: tsit5_interp(th, I.dt, I.uprev.data(), I.k.data(), n, out); break;
    case ORC_VERN7:
        if (I.nk_valid < 16) {
            vern7_extra(I.model, n, I.p, I.tprev, I.dt, I.uprev.data(), I.k.data());
            I.nk_valid = 16;
        }
        vern7_interp(th, I.dt, I.uprev.data(), I.k.data(), n, out);
        break;
    case ORC_RODAS5P: rodas_interp(th, I.uprev.data(), I.u.data(), I.k.data(), n, out); break;
    case ORC_ROSENBROCK23: ros23_interp(th, I.dt, I.uprev.data(), I.k.data(), n, out); break;
    default: {  // Vern9 ground truth: linear (only reached if a save is not a tstop)
        for (int i = 0; i < n; ++i) out[i] = (1.0 - th) * I.uprev[i] + th * I.u[i];
    }
    }
}

void record_dense(Integ& I, double t, const double* v);

void push_save(Integ& I, double t, const double* v) {
    if (I.dense) {   // dense output saves every step: each save after the start is an interval
        if (I.nsaved > 0) record_dense(I, t, v);
        I.dense_last_u.assign(v, v + I.n);
    }
    const int slot = I.nsaved < I.cap ? I.nsaved : ((I.o.save_everystep || I.o.callback) ? I.cap - 1 : -1);
    if (slot >= 0) {
        if (I.t_out) I.t_out[slot] = t;
        if (I.u_out) std::memcpy(I.u_out + (size_t)slot * I.n, v, sizeof(double) * I.n);
    }
    if (I.alg == ORC_AUTOTSIT5_ROSENBROCK23) I.alg_choice.push_back(I.current + 1);   // sol.alg_choice
    I.nsaved++;
    I.last_saved_t = t;
}

// _savevalues!: lib/OrdinaryDiffEqCore/src/integrators/integrator_utils.jl:340-414.
void savevalues(Integ& I) {
    while (I.isave < I.saveat.size() && I.saveat[I.isave] <= I.tdir * I.t) {
        double curt = I.tdir * I.saveat[I.isave++];
        if (curt != I.t) {
            double th = (curt - I.tprev) / I.dt;
            interpolate(I, th, I.interp_out.data());
            push_save(I, curt, I.interp_out.data());
        } else {
            if (curt == I.tf && !I.o.save_end) continue;
            push_save(I, I.t, I.u.data());
        }
    }
    // save_everystep: the accepted step unless it repeats the last save (t === sol.t[end]
    // with dt != 0) or is tf with save_end off (integrator_utils.jl:397-404)
    if (I.o.save_everystep &&
        (I.nsaved == 0 || ((I.t != I.last_saved_t || I.dt == 0.0) && (I.o.save_end || I.t != I.tf))))
        push_save(I, I.t, I.u.data());
    if (I.alg == ORC_VERN7 && I.nk_valid > 10) I.nk_valid = 10;  // post_savevalues! resize
}

// modify_dt_for_tstops!: integrator_utils.jl:268-324.
void modify_dt_for_tstops(Integ& I) {
    if (I.itstop >= I.tstops.size()) { I.next_step_tstop = false; return; }
    const double tdir_tstop = I.tstops[I.itstop];
    const double tdir_t = I.tdir * I.t;
    double dist = std::fabs(tdir_tstop - tdir_t);
    double tol = (std::isfinite(tdir_tstop) && std::isfinite(I.t))
                     ? 100.0 * jeps(jmax(std::fabs(I.t), std::fabs(tdir_tstop))) : 0.0;
    if (I.o.adaptive) {
        double orig = std::fabs(I.dt);
        I.dtpropose = I.tdir * orig;
        if (orig + tol < dist) {
            I.next_step_tstop = false;
        } else {
            I.next_step_tstop = true;
            I.tstop_target = I.tdir * tdir_tstop;
        }
        I.dt = I.tdir * jmin(orig, dist);
    } else if (I.dtcache == 0.0) {   // fixed steps without a dt: to the next tstop
        I.next_step_tstop = true;
        I.tstop_target = I.tdir * tdir_tstop;
        I.dt = I.tdir * dist;
    } else {
        if (std::fabs(I.dtcache) + tol < dist) {
            I.next_step_tstop = false;
        } else {
            I.next_step_tstop = true;
            I.tstop_target = I.tdir * tdir_tstop;
        }
        I.dt = I.tdir * jmin(std::fabs(I.dtcache), dist);
    }
}

inline double dtmin_t(const Integ& I) { return std::fabs(jmax(jeps(I.t), I.o.dtmin)); }

// fix_dt_at_bounds!: integrator_utils.jl:1243-1256.  Backward, the reference
// bounds dt by min(dt, dtmin) with the positive dtmin, which leaves a negative dt
// as it is: the lower bound applies forward only.
void fix_dt_at_bounds(Integ& I) {
    if (I.tdir > 0) {
        I.dt = jmin(I.o.dtmax, I.dt);
        I.dt = jmax(I.dt, dtmin_t(I));
    } else {
        I.dt = jmax(I.o.dtmax, I.dt);
        I.dt = jmin(I.dt, dtmin_t(I));
    }
}

// PI controller: lib/OrdinaryDiffEqCore/src/integrators/controllers.jl:805-843.
double stepsize_controller(Integ& I) {
    double qmax = I.success_iter == 0 ? I.qmax_first : I.qmax;
    double q;
    if (I.EEst == 0.0) {
        q = 1.0 / qmax;
    } else {
        double q11 = ctrl_pow(I.EEst, I.beta1);
        q = q11 / ctrl_pow(I.errold, I.beta2);
        I.q11 = q11;
        double x = q / I.gamma, lo = 1.0 / qmax, hi = 1.0 / I.qmin;
        q = x > hi ? hi : (x < lo ? lo : x);
    }
    return q;
}

void record_dense(Integ& I, double t, const double* v) {
    // sol.t / sol.u / sol.k of a step save or a callback's save (save_dense_at_t!,
    // integrator_utils.jl:455-473; savevalues!(integrator, true) in apply_callback!):
    // the interval from the previous save, with the interpolation data of the step
    // as it stands (an event's step is the shortened one)
    Step s;
    s.tprev = I.last_saved_t;
    s.tend = t;
    s.y0 = I.dense_last_u;
    s.y1.assign(v, v + I.n);
    const int alg = I.alg == ORC_AUTOTSIT5_ROSENBROCK23 ? (I.current == 0 ? ORC_TSIT5 : ORC_ROSENBROCK23) : I.alg;
    int nk = alg == ORC_TSIT5 ? 7 : alg == ORC_VERN7 ? 10 : alg == ORC_RODAS5P ? 3 : alg == ORC_ROSENBROCK23 ? 2 : 0;
    s.k.assign(I.k.begin(), I.k.begin() + (size_t)nk * I.n);
    I.dense->steps.push_back(std::move(s));
}

// ---------------------------------------------------------------- callbacks
// The models' registered ContinuousCallback (SciMLBase's ContinuousCallback, not
// vendored; its defaults: interp_points = 10, rootfind = LeftRootFind,
// save_positions = (true, true), abstol = 10eps(), repeat_nudge = 1//100,
// dtrelax = 1).  Bouncing ball: condition u[1] (the height), affect! = nothing,
// affect_neg!: terminate! once t >= p[3], else v = -e v (p[2] = e = 1 gives the
// reference's ode_event_tests.jl:100-113 and 332-346 callbacks).
constexpr double CB_ABSTOL = 10.0 * 2.220446049250313e-16;
constexpr double CB_REPEAT_NUDGE = 0.01;

bool model_has_event(int model) { return model == ORC_BOUNCING_BALL; }
// the ball in a box's VectorContinuousCallback, its number of conditions
bool model_has_vector_event(int model) { return model == ORC_BALL_BOX; }
constexpr int BOX_EVENTS = 3;
double event_condition(int model, const double* u) { (void)model; return u[0]; }
bool event_has_affect(int) { return false; }
bool event_has_affect_neg(int) { return true; }
// affect (upcrossing) / affect_neg (downcrossing) on the integrator state; true: terminate!
bool event_apply(Integ& I, bool upcrossing) {
    (void)upcrossing;
    if (I.t >= I.p[2]) return true;
    I.u[1] = -I.p[1] * I.u[1];
    return false;
}

inline double jsign(double x) { return x > 0 ? 1.0 : (x < 0 ? -1.0 : (x == 0 ? 0.0 : x)); }

// get_condition (lib/DiffEqBase/src/callbacks.jl:91-137): u at t, uprev at tprev,
// else the current step's interpolant at abst.
double cond_at(Integ& I, double abst) {
    const double* v;
    if (abst == I.t) {
        v = I.u.data();
    } else if (abst == I.tprev) {
        v = I.uprev.data();
    } else {
        interpolate(I, (abst - I.tprev) / I.dt, I.cb_tmp.data());
        v = I.cb_tmp.data();
    }
    return event_condition(I.model, v);
}

// is_event_occurrence (callbacks.jl:525-530)
bool is_event(const Integ& I, double bs, double ts) {
    return ((bs < 0 && event_has_affect(I.model)) || (bs > 0 && event_has_affect_neg(I.model))) && bs * ts <= 0;
}

// find_root with LeftRootFind (callbacks.jl:480-492): the reference runs ModAB
// (BracketingNonlinearSolve, not vendored) with abstol = reltol = 0, i.e. to
// adjacent floats, and returns the left end (or a point where the condition is
// exactly 0).  Any bracketing method run to adjacent floats ends at the same
// pair where the sign change is unique; this one is Anderson-Bjorck false
// position (the secant point; when the same end is replaced twice in a row the
// retained end's value is scaled by 1 - f_new/f_replaced, or 1/2 when that is
// not positive) with a bisection whenever the bracket has not halved over two
// steps or the secant point is not strictly inside.  fa = f(a), fb = f(b) of
// opposite signs, nonzero.  a is the end first in the integration direction
// (a > b backward); the iteration runs on tdir * t and returns the root's side
// towards a.
double find_root_left(Integ& I, double a, double b, double fa, double fb) {
    const double d = I.tdir;
    a *= d;
    b *= d;
    int side = 0;
    double w_prev = b - a, w_prev2 = 2.0 * (b - a);
    for (int it = 0; it < 2200; ++it) {
        const double w = b - a;
        double m = (w > 0.5 * w_prev2) ? a + w * 0.5 : a + w * (fa / (fa - fb));
        if (!(m > a && m < b)) m = a + w * 0.5;
        if (!(m > a && m < b)) break;
        const double fm = cond_at(I, d * m);
        if (fm == 0.0) return d * m;
        w_prev2 = w_prev;
        w_prev = w;
        if ((fm > 0.0) == (fa > 0.0)) {
            if (side == -1) {
                const double g = 1.0 - fm / fa;
                fb *= g > 0.0 ? g : 0.5;
            }
            a = m;
            fa = fm;
            side = -1;
        } else {
            if (side == +1) {
                const double g = 1.0 - fm / fb;
                fa *= g > 0.0 ? g : 0.5;
            }
            b = m;
            fb = fm;
            side = +1;
        }
    }
    return d * a;
}

// find_callback_time(integrator, ::ContinuousCallback, idx) (callbacks.jl:364-412),
// with nudge_tprev (:414-426) and check_event_occurrence (:428-458).
bool find_callback_time(Integ& I, double& cb_t, double& bottom_sign, double& residual) {
    double bottom_t = I.tprev;
    double bc = cond_at(I, bottom_t);
    if (I.event_last_time == 1) {
        if (std::fabs(bc - I.last_event_error) <= CB_ABSTOL) bottom_t = I.tprev + I.dt * CB_REPEAT_NUDGE;
        bc = cond_at(I, bottom_t);
    }
    const double bs = jsign(bc);
    double top_t = I.t;
    double tv = cond_at(I, top_t);
    double ts = jsign(tv);
    bool occ = is_event(I, bs, ts);
    if (I.o.interp_points != 0 && !occ) {
        // range(tprev, stop = t, length = interp_points)
        const int m = I.o.interp_points;
        for (int i = 2; i <= m; ++i) {
            top_t = i == m ? I.t : I.tprev + (I.t - I.tprev) * ((double)(i - 1) / (double)(m - 1));
            tv = cond_at(I, top_t);
            ts = jsign(tv);
            occ = is_event(I, bs, ts);
            if (occ) break;
        }
    }
    bottom_sign = bs;
    residual = 0.0;
    if (!occ) {
        cb_t = I.t;
        return false;
    }
    if (ts == 0.0) {
        cb_t = top_t;
    } else {
        cb_t = find_root_left(I, bottom_t, top_t, bc, tv);
        residual = cond_at(I, cb_t);
    }
    return true;
}

// ode_addsteps!(integrator, f, always_calc_begin = true): the step's
// interpolation data recomputed from (tprev, uprev) with the current dt
// (reeval_internals_due_to_modification!, integrator_interface.jl:54-79).  The
// reference does not count these evaluations; u, the error estimate and the
// counters are kept.
void recompute_step_k(Integ& I) {
    const std::vector<double> u = I.u, fsf = I.fsalfirst, fsl = I.fsallast, ut = I.utilde, J = I.J;
    const double EEst = I.EEst, t = I.t;
    const orc_stats st = I.st;
    const bool have_J = I.have_J;
    I.t = I.tprev;
    if (I.alg == ORC_TSIT5 || I.alg == ORC_ROSENBROCK23 || I.alg == ORC_AUTOTSIT5_ROSENBROCK23)
        f_eval(I, I.uprev.data(), I.t, I.fsalfirst.data());
    const double eig = I.eigen_est;
    I.recomputing = true;
    do_step(I);
    I.recomputing = false;
    I.eigen_est = eig;
    I.u = u;
    I.fsalfirst = fsf;
    I.fsallast = fsl;
    I.utilde = ut;
    I.J = J;
    I.have_J = have_J;
    I.EEst = EEst;
    I.t = t;
    I.st = st;
}

// apply_callback! (callbacks.jl:557-643) for a ContinuousCallback.
void apply_callback(Integ& I, double cb_t, double bottom_sign) {
    if (I.o.adaptive) {   // set_proposed_dt! (integrator_interface.jl:180-182), dtrelax = 1
        I.dtpropose = I.tdir * jmax(std::nextafter(I.o.dtmin, INFINITY), I.tdir * 1.0 * I.dt);
        I.dtcache = I.dtpropose;
    }
    // change_t_via_interpolation! (integrator_interface.jl:5-40)
    if (cb_t != I.t) {
        interpolate(I, (cb_t - I.tprev) / I.dt, I.u.data());
        I.t = cb_t;
        I.dt = I.t - I.tprev;
        recompute_step_k(I);
        I.reeval_fsal = true;
    }
    // savevalues! with saveat up to the event, then the pre-affect save unless saved exactly
    const int before = I.nsaved;
    const double last_before = I.last_saved_t;
    savevalues(I);
    const bool savedexactly = I.nsaved > before && I.last_saved_t == I.t && !(last_before == I.t);
    if (!savedexactly) push_save(I, I.t, I.u.data());
    // affect! (upcrossing) or affect_neg! (downcrossing); a nothing affect makes no change
    bool modified = false;
    if (bottom_sign < 0 && event_has_affect(I.model)) {
        I.terminated = event_apply(I, true);
        modified = true;
    } else if (bottom_sign > 0 && event_has_affect_neg(I.model)) {
        I.terminated = event_apply(I, false);
        modified = true;
    }
    if (modified) {
        recompute_step_k(I);
        I.reeval_fsal = true;
        push_save(I, I.t, I.u.data());   // save_positions[2]
    }
}

// apply_discrete_callback! (lib/DiffEqBase/src/callbacks.jl:645-682) for the
// dosing model's DiscreteCallback: condition t in the dose times (the solve's
// tstops as given), affect! depot += dose, save_positions = (true, true); the
// modification sets reeval_fsal (reeval_internals_due_to_modification! with
// continuous_modification = false: the step's k are kept).
void apply_discrete_callback(Integ& I) {
    if (!std::binary_search(I.dtimes.begin(), I.dtimes.end(), I.t)) {
        savevalues(I);
        return;
    }
    const int before = I.nsaved;
    const double last_before = I.last_saved_t;
    savevalues(I);
    const bool savedexactly = I.nsaved > before && I.last_saved_t == I.t && !(last_before == I.t);
    if (!savedexactly) push_save(I, I.t, I.u.data());
    I.u[0] += I.p[2];
    I.reeval_fsal = true;
    push_save(I, I.t, I.u.data());
}

// ---- VectorContinuousCallback (the ball in a box)
void vector_conditions(Integ& I, const double* v, double* out) {
    out[0] = v[1];
    out[1] = v[0];
    out[2] = I.p[2] - v[0];
}
// get_condition for a vector callback: u at t, uprev at tprev, else the interpolant
void vcond_at(Integ& I, double abst, double* out) {
    const double* v;
    if (abst == I.t) {
        v = I.u.data();
    } else if (abst == I.tprev) {
        v = I.uprev.data();
    } else {
        interpolate(I, (abst - I.tprev) / I.dt, I.cb_tmp.data());
        v = I.cb_tmp.data();
    }
    vector_conditions(I, v, out);
}
// one component of the vector condition, as a function of t (find_root's zero_func)
double find_root_left_component(Integ& I, int k, double a, double b, double fa, double fb) {
    const double d = I.tdir;
    a *= d;
    b *= d;
    int side = 0;
    double w_prev = b - a, w_prev2 = 2.0 * (b - a);
    double o[BOX_EVENTS];
    for (int it = 0; it < 2200; ++it) {
        const double w = b - a;
        double m = (w > 0.5 * w_prev2) ? a + w * 0.5 : a + w * (fa / (fa - fb));
        if (!(m > a && m < b)) m = a + w * 0.5;
        if (!(m > a && m < b)) break;
        vcond_at(I, d * m, o);
        const double fm = o[k];
        if (fm == 0.0) return d * m;
        w_prev2 = w_prev;
        w_prev = w;
        if ((fm > 0.0) == (fa > 0.0)) {
            if (side == -1) {
                const double g = 1.0 - fm / fa;
                fb *= g > 0.0 ? g : 0.5;
            }
            a = m;
            fa = fm;
            side = -1;
        } else {
            if (side == +1) {
                const double g = 1.0 - fm / fb;
                fa *= g > 0.0 ? g : 0.5;
            }
            b = m;
            fb = fm;
            side = +1;
        }
    }
    return d * a;
}

// find_callback_time(integrator, ::VectorContinuousCallback, idx)
// (lib/DiffEqBase/src/callbacks.jl:239-362), check_event_occurrence (:428-458)
// and findall_events! (:495-523).  events[k]: -sign(bottom sign) for the
// components that fire at the earliest root, 0 else.
bool find_vector_callback_time(Integ& I, double& cb_t, int* events, double& residual) {
    const int M = BOX_EVENTS;
    double bc[M], bs[M], nc[M], tc[M];
    vcond_at(I, I.tprev, bc);
    for (int i = 0; i < M; ++i) {
        bs[i] = jsign(bc[i]);
        nc[i] = bc[i];
        events[i] = 0;
    }
    double nudged_t = I.tprev;
    if (I.event_last_time == 1) {
        double minc = 0.0, mina = INFINITY;
        for (int i = 0; i < M; ++i)
            if (I.prev_events[i] && std::fabs(bc[i]) < mina) {
                mina = std::fabs(bc[i]);
                minc = bc[i];
            }
        if (std::fabs(minc - I.last_event_error) <= CB_ABSTOL) nudged_t = I.tprev + I.dt * CB_REPEAT_NUDGE;
        vcond_at(I, nudged_t, nc);
        for (int i = 0; i < M; ++i)
            if (I.prev_events[i]) bs[i] = jsign(nc[i]);
    }
    bool ev[M];
    auto fire = [&](const double* top) {
        bool any = false;
        for (int i = 0; i < M; ++i) {
            ev[i] = bs[i] != 0.0 && bs[i] * jsign(top[i]) <= 0.0;
            any = any || ev[i];
        }
        return any;
    };
    double top_t = I.t;
    vcond_at(I, top_t, tc);
    bool occ = fire(tc);
    bool any_zero = false;
    for (int i = 0; i < M; ++i) any_zero = any_zero || !ev[i];
    if (I.o.interp_points != 0 && any_zero) {
        const int m = I.o.interp_points;
        for (int i = 2; i <= m; ++i) {
            top_t = i == m ? I.t : I.tprev + (I.t - I.tprev) * ((double)(i - 1) / (double)(m - 1));
            vcond_at(I, top_t, tc);
            occ = fire(tc);
            if (occ) break;
        }
    }
    residual = 0.0;
    if (!occ) {
        cb_t = I.t;
        return false;
    }
    cb_t = std::nextafter(top_t, I.tdir * INFINITY);   // rightfloat(top_t, tdir)
    for (int i = 0; i < M; ++i) {
        if (!ev[i]) continue;
        double cbi;
        if (jsign(tc[i]) == 0.0) {
            cbi = top_t;
        } else if (I.event_last_time == 1 && I.prev_events[i]) {
            cbi = find_root_left_component(I, i, nudged_t, top_t, nc[i], tc[i]);
        } else {
            cbi = find_root_left_component(I, i, I.tprev, top_t, bc[i], tc[i]);
        }
        if (I.tdir * cbi < I.tdir * cb_t)
            for (int k = 0; k < M; ++k) events[k] = 0;
        if (I.tdir * cbi <= I.tdir * cb_t) {
            cb_t = cbi;
            double o[M];
            vcond_at(I, cbi, o);
            residual = o[i];
            events[i] = bs[i] < 0.0 ? 1 : -1;
        }
    }
    return true;
}

// apply_callback! (callbacks.jl:557-643) for the VectorContinuousCallback: affect!
// gets the events' directions; the ball reflects vy at the floor (restitution
// e = p[2]) and vx at a wall.
void apply_vector_callback(Integ& I, double cb_t, const int* events) {
    if (I.o.adaptive) {
        I.dtpropose = I.tdir * jmax(std::nextafter(I.o.dtmin, INFINITY), I.tdir * 1.0 * I.dt);
        I.dtcache = I.dtpropose;
    }
    if (cb_t != I.t) {
        interpolate(I, (cb_t - I.tprev) / I.dt, I.u.data());
        I.t = cb_t;
        I.dt = I.t - I.tprev;
        recompute_step_k(I);
        I.reeval_fsal = true;
    }
    const int before = I.nsaved;
    const double last_before = I.last_saved_t;
    savevalues(I);
    const bool savedexactly = I.nsaved > before && I.last_saved_t == I.t && !(last_before == I.t);
    if (!savedexactly) push_save(I, I.t, I.u.data());
    if (events[0] != 0) I.u[3] = -I.p[1] * I.u[3];
    if (events[1] != 0 || events[2] != 0) I.u[2] = -I.u[2];
    recompute_step_k(I);
    I.reeval_fsal = true;
    push_save(I, I.t, I.u.data());
}

// apply_discrete_callback! (callbacks.jl:645-682) for the state-triggered dose:
// condition c < threshold, affect! c += dose.  Returns saved_in_cb.
bool apply_threshold_callback(Integ& I) {
    if (!(I.u[0] < I.p[1])) return false;
    const int before = I.nsaved;
    const double last_before = I.last_saved_t;
    savevalues(I);
    const bool savedexactly = I.nsaved > before && I.last_saved_t == I.t && !(last_before == I.t);
    if (!savedexactly) push_save(I, I.t, I.u.data());
    I.u[0] += I.p[2];
    I.reeval_fsal = true;
    push_save(I, I.t, I.u.data());
    return true;
}

// handle_callbacks! (integrator_utils.jl:1081-1132): the model's continuous
// callback (scalar or vector), then its discrete one; savevalues! unless the
// discrete callbacks (if any), else the continuous one, saved.
void handle_callbacks(Integ& I) {
    if (I.o.callback && I.model == ORC_PK1) {
        apply_discrete_callback(I);
        return;
    }
    bool saved_in_cb = false;
    if (I.o.callback && model_has_event(I.model)) {
        double cb_t, bs, residual;
        if (find_callback_time(I, cb_t, bs, residual)) {
            I.event_last_time = 1;
            I.last_event_error = residual;
            apply_callback(I, cb_t, bs);
            saved_in_cb = true;
        } else {
            I.event_last_time = 0;
        }
    }
    if (I.o.callback && model_has_vector_event(I.model)) {
        double cb_t, residual;
        int events[BOX_EVENTS];
        if (find_vector_callback_time(I, cb_t, events, residual)) {
            I.event_last_time = 1;
            I.last_event_error = residual;
            for (int k = 0; k < BOX_EVENTS; ++k) I.prev_events[k] = events[k] != 0;
            apply_vector_callback(I, cb_t, events);
            saved_in_cb = true;
        } else {
            I.event_last_time = 0;
        }
    }
    if (I.o.callback && I.model == ORC_THRESHOLD_DOSE) saved_in_cb = apply_threshold_callback(I);
    if (!saved_in_cb) savevalues(I);
}

// _loopfooter!: integrator_utils.jl:597-677.
void loopfooter(Integ& I) {
    I.do_error_check = true;   // _loopfooter! (integrator_utils.jl:597-599)
    double ttmp = I.t + I.dt;
    if (I.o.adaptive) {
        double q = stepsize_controller(I);
        // isoutofdomain (here the common any(x -> x < 0, u)) at the step's end, then
        // accept_step_controller, or force_dtmin at abs(dt) <= timedepentdtmin
        // (integrator_utils.jl:612-623, utils.jl:93: abs(max(eps(t), dtmin)))
        I.isout = false;
        if (I.o.isoutofdomain)
            for (int i = 0; i < I.n; ++i) I.isout = I.isout || I.u[i] < 0.0;
        I.accept_step = (!I.isout && I.EEst <= 1.0) ||
                        (I.o.force_dtmin && std::fabs(I.dt) <= std::fabs(jmax(jeps(I.t), I.o.dtmin)));
        if (I.accept_step) {
            I.st.naccept++;
            I.tprev = I.t;
            if (I.next_step_tstop) I.dt = I.dtpropose;
            if (I.next_step_tstop) {
                I.next_step_tstop = false;
                I.t = I.tstop_target;
            } else {
                I.t = ttmp;
            }
            if (I.qsteady_min <= q && q <= I.qsteady_max) q = 1.0;
            I.errold = jmax(I.EEst, I.qoldinit);
            double dtnew = I.dt / q;   // calc_dt_propose! (integrator_utils.jl:1199-1209)
            double dtp = I.tdir * jmin(std::fabs(I.o.dtmax), std::fabs(dtnew));
            dtp = I.tdir * jmax(std::fabs(dtp), dtmin_t(I));
            I.dtpropose = dtp;
            handle_callbacks(I);
        } else {
            I.st.nreject++;
        }
    } else {
        I.st.naccept++;
        I.tprev = I.t;
        if (I.next_step_tstop) {
            I.next_step_tstop = false;
            I.t = I.tstop_target;
        } else {
            I.t = ttmp;
        }
        I.accept_step = true;
        I.dtpropose = I.dt;
        handle_callbacks(I);
    }
}

// Controller defaults of one method (alg_utils.jl:407-879): beta1 = 7/(10 order),
// beta2 = 2/(5 order), qsteady_max 6/5 for the adaptive implicit family.
// The caller's PIController knobs (controllers.jl:751-774: beta1, beta2,
// qoldinit and the CommonControllerOptions qmin, gamma, qsteady_min,
// qsteady_max) over the defaults, for every method of a composite.
void apply_controller_knobs(Integ& I) {
    if (!I.o.ctrl_given) return;
    auto set = [](double& f, double v) { if (!std::isnan(v)) f = v; };
    set(I.beta1, I.o.c_beta1);
    set(I.beta2, I.o.c_beta2);
    set(I.qoldinit, I.o.c_qoldinit);
    set(I.qmin, I.o.c_qmin);
    set(I.gamma, I.o.c_gamma);
    set(I.qsteady_min, I.o.c_qsteady_min);
    set(I.qsteady_max, I.o.c_qsteady_max);
}

void set_controller(Integ& I, int order, bool implicit) {
    I.order = order;
    I.beta2 = 2.0 / (5.0 * order);
    I.beta1 = 7.0 / (10.0 * order);
    I.qsteady_max = implicit ? 1.2 : 1.0;
    apply_controller_knobs(I);
}

// choose_algorithm! for AutoTsit5(Rosenbrock23()) (composite_perform_step.jl:181-221)
// with its AutoSwitch choice function (composite_algs.jl:17-94; defaults maxstiffstep
// 10, maxnonstiffstep 3, nonstifftol = stifftol = 9//10, dtfac 2, stiffalgfirst false,
// switch_max 5).  The composite's controller is one PI controller per method
// (CompositeController, controllers.jl:1263-1345): switching banks the old
// method's controller state and resumes the new one's.
void choose_algorithm(Integ& I) {
    if (I.alg != ORC_AUTOTSIT5_ROSENBROCK23) return;
    // is_stiff: |eigen_est dt / alg_stability_size(Tsit5)| with alg_stability_size(::Tsit5) = 3.5068
    // (lib/OrdinaryDiffEqTsit5/src/alg_utils.jl:3); `stiffness <= 9//10` compares exactly,
    // which for a double is `< 0.9` (0.9 lies above 9/10)
    const double stiffness = std::fabs(I.eigen_est * I.dt / 3.5068);
    const bool stiff = !(stiffness < 0.9);
    if (!stiff) I.successive_switches++;
    else I.successive_switches = 0;
    I.do_error_check = (I.successive_switches > 5 || !stiff) || I.is_stiffalg;
    I.as_count = stiff ? (I.as_count < 0 ? 1 : I.as_count + 1) : (I.as_count > 0 ? -1 : I.as_count - 1);
    if (!I.is_stiffalg && I.as_count > 10) {
        I.dt = I.dt * 2.0;
        I.is_stiffalg = true;
    } else if (I.is_stiffalg && I.as_count < -3) {
        I.dt = I.dt / 2.0;
        I.is_stiffalg = false;
    }
    const int next = I.is_stiffalg ? 1 : 0;
    if (next != I.current) {
        I.ctl_errold[I.current] = I.errold;
        I.ctl_q11[I.current] = I.q11;
        I.current = next;
        I.errold = I.ctl_errold[next];
        I.q11 = I.ctl_q11[next];
        if (next == 0) set_controller(I, 5, false);
        else set_controller(I, 2, true);
        // initialize! of the method switched to: its FSAL value f(uprev, t)
        f_eval(I, I.uprev.data(), I.t, I.fsalfirst.data());
        I.st.nf += 1;
    }
}

// loopheader!: integrator_utils.jl:84-127 (apply_step! :175-203, handle_step_rejection! :130-150).
void loopheader(Integ& I) {
    if (I.iter > 0) {
        if (!I.o.adaptive || I.accept_step) {
            I.success_iter++;
            I.uprev = I.u;
            I.dt = I.dtpropose;
            if (I.alg == ORC_TSIT5 || I.alg == ORC_ROSENBROCK23 || I.alg == ORC_AUTOTSIT5_ROSENBROCK23) {
                if (I.reeval_fsal) {   // update_fsal! -> reset_fsal! (integrator_utils.jl:216-235,1326-1340)
                    f_eval(I, I.u.data(), I.t, I.fsalfirst.data());
                    I.st.nf += 1;
                } else {
                    I.fsalfirst = I.fsallast;
                }
            }
            I.reeval_fsal = false;
            modify_dt_for_tstops(I);
        } else {
            // handle_step_rejection! (integrator_utils.jl:135-139)
            if (I.isout) I.dt = I.dt * I.qmin;
            else I.dt = I.dt / jmin(1.0 / I.qmin, I.q11 / I.gamma);
        }
    }
    I.iter++;
    choose_algorithm(I);
    fix_dt_at_bounds(I);
    modify_dt_for_tstops(I);
}

// de_check_error: lib/DiffEqBase/src/check_error.jl:70-118.
int check_error(Integ& I) {
    if (I.dt != I.dt) return ORC_RC_DTNAN;
    if (I.iter > I.o.maxiters) return ORC_RC_MAXITERS;
    bool acc = I.accept_step;
    if (I.o.adaptive && !I.o.force_dtmin) {   // check_error.jl:91
        // t + dt < tdir * first(tstops), as the reference writes it for either direction
        double next_tstop = I.itstop < I.tstops.size() ? I.tdir * I.tstops[I.itstop] : I.tdir * INFINITY;
        if (std::fabs(I.dt) <= std::fabs(I.o.dtmin) && (!acc || I.t + I.dt < next_tstop))
            return ORC_RC_DTLESSTHANMIN;
        if (!acc && std::fabs(I.dt) <= std::fabs(jeps(I.t))) return ORC_RC_UNSTABLE;
    }
    if (acc)
        for (int i = 0; i < I.n; ++i)
            if (!std::isfinite(I.u[i])) return ORC_RC_UNSTABLE;
    return ORC_RC_SUCCESS;
}

// solution_endpoint_match_cur_integrator!: integrator_utils.jl:540-588.
void postamble(Integ& I) {
    if (!I.o.save_end) return;
    bool need;
    if (I.nsaved == 0) {
        need = true;
    } else {
        bool in_saveat = false;
        if (I.o.saveat_given) {
            if (I.o.saveat_scalar) {
                in_saveat = false;
            } else {
                for (double s : I.saveat) in_saveat = in_saveat || (I.tdir * s == I.t);
            }
        }
        need = I.last_saved_t != I.t &&
               (I.o.save_end_user == 1 || in_saveat || I.t == I.tf || !I.o.saveat_given);
    }
    if (need) push_save(I, I.t, I.u.data());
}

int solve_one(Integ& I, const double* u0) {
    int n = I.n;
    I.u.assign(u0, u0 + n);
    I.uprev = I.u;
    I.tmp.assign(n, 0.0);
    I.utilde.assign(n, 0.0);
    I.atmp.assign(n, 0.0);
    I.fsalfirst.assign(n, 0.0);
    I.fsallast.assign(n, 0.0);
    I.k.assign((size_t)16 * n, 0.0);
    I.interp_out.assign(n, 0.0);
    I.current = 0;   // AutoSwitch: stiffalgfirst = false -> Tsit5 first
    I.as_count = 0;
    I.successive_switches = 0;
    I.is_stiffalg = false;
    I.do_error_check = true;
    I.eigen_est = 1.0;   // solve.jl:697
    I.alg_choice.clear();
    if (I.alg == ORC_AUTOTSIT5_ROSENBROCK23) {
        I.ctl_errold[0] = I.ctl_errold[1] = I.qoldinit;
        I.ctl_q11[0] = I.ctl_q11[1] = 1.0;
        set_controller(I, 5, false);
    }
    if (I.alg == ORC_RODAS5P || I.alg == ORC_ROSENBROCK23 || I.alg == ORC_AUTOTSIT5_ROSENBROCK23) {
        I.J.assign((size_t)n * n, 0.0);
        I.W.assign((size_t)n * n, 0.0);
        I.dT.assign(n, 0.0);
        I.ks.assign((size_t)8 * n, 0.0);
        I.rhs.assign(n, 0.0);
        I.du.assign(n, 0.0);
        I.piv.assign(n, 0);
        I.have_J = false;
    }
    I.jr_last_dtgamma = I.jr_pending_dtgamma = 0.0;
    I.jr_last_naccept = I.jr_last_step_iter = 0;
    I.recomputing = false;
    I.t = I.t0;
    I.tprev = I.t0;
    I.nk_valid = 0;
    I.iter = 0;
    I.success_iter = 0;
    I.accept_step = false;
    I.isout = false;
    I.next_step_tstop = false;
    I.EEst = 1.0;
    I.q11 = 1.0;
    I.errold = I.qoldinit;
    I.nsaved = 0;
    I.last_saved_t = NAN;
    I.event_last_time = 0;
    I.last_event_error = 0.0;
    for (bool& b : I.prev_events) b = false;
    I.reeval_fsal = false;
    I.terminated = false;
    I.cb_tmp.assign(n, 0.0);
    std::memset(&I.st, 0, sizeof(I.st));
    if (I.o.save_start) push_save(I, I.t0, I.u.data());
    if (I.alg == ORC_TSIT5 || I.alg == ORC_ROSENBROCK23 || I.alg == ORC_AUTOTSIT5_ROSENBROCK23) {
        // initialize!: FSAL pre-start (tsit_perform_step.jl:293-307, rosenbrock_perform_step.jl:1-14)
        f_eval(I, I.u.data(), I.t, I.fsalfirst.data());
        I.st.nf += 1;
    }
    if (!I.o.adaptive) {
        I.dt = I.tdir * std::fabs(I.o.dt);   // fixed steps: no heuristic (handle_dt!, solve.jl:968-985)
    } else if (I.o.dt > 0.0) {
        I.dt = I.tdir * I.o.dt;   // a positive dt is taken in the direction (handle_dt!, solve.jl:949-966)
    } else {
        I.dt = initdt(I);
        I.st.nf += 2;
    }
    I.dtpropose = I.dt;
    I.dtcache = I.dt;
    int rc = ORC_RC_DEFAULT;
    while (I.itstop < I.tstops.size()) {
        double first_tstop = I.tstops[I.itstop];
        while (I.tdir * I.t < first_tstop) {
            loopheader(I);
            int e = I.do_error_check ? check_error(I) : ORC_RC_SUCCESS;   // solve.jl:909
            if (e != ORC_RC_SUCCESS) {
                postamble(I);
                return e;
            }
            bool tiny = I.next_step_tstop && std::fabs(I.dt) < jeps(std::fabs(I.t));
            if (!tiny) do_step(I);
            bool should_exit = I.next_step_tstop;
            loopfooter(I);
            if (I.terminated) {   // terminate! (ReturnCode.Terminated); postamble as the reference's
                postamble(I);
                return ORC_RC_TERMINATED;
            }
            if (I.itstop >= I.tstops.size() || should_exit) break;
        }
        // handle_tstop!: integrator_utils.jl:1290-1314
        if (I.itstop < I.tstops.size() && I.tdir * I.t == I.tstops[I.itstop]) {
            while (I.itstop < I.tstops.size() && I.tstops[I.itstop] == I.tdir * I.t) I.itstop++;
        }
    }
    postamble(I);
    rc = ORC_RC_SUCCESS;
    return rc;
}

void setup(Integ& I, int alg, int model, int n, const double* p, double t0, double tf, const orc_opts* o,
           const double* saveat, int nsave, const double* tstops, int ntstops) {
    I.alg = alg;
    I.model = model;
    I.n = n;
    I.p = p;
    I.t0 = t0;
    I.tf = tf;
    I.tdir = tf < t0 ? -1.0 : 1.0;
    I.o = *o;
    // default tf - t0; a positive dtmax is taken in the direction (solve.jl:153,401)
    if (I.o.dtmax <= 0.0) I.o.dtmax = tf - t0;
    else I.o.dtmax *= I.tdir;
    if (I.o.maxiters <= 0) I.o.maxiters = 1000000;
    I.order = alg == ORC_VERN7 ? 7 : alg == ORC_VERN9 ? 9 : alg == ORC_ROSENBROCK23 ? 2 : 5;   // composite: Tsit5's
    // controller defaults: lib/OrdinaryDiffEqCore/src/alg_utils.jl:407-879
    I.beta2 = 2.0 / (5.0 * I.order);
    I.beta1 = 7.0 / (10.0 * I.order);
    I.qmin = 0.2;
    I.qmax = o->qmax > 0 ? o->qmax : 10.0;
    I.qmax_first = o->qmax_first_step > 0 ? o->qmax_first_step : 10000.0;
    I.gamma = 0.9;
    I.qsteady_min = 1.0;
    I.qsteady_max = (alg == ORC_RODAS5P || alg == ORC_ROSENBROCK23) ? 1.2 : 1.0;   // AdaptiveImplicit: 6/5
    I.qoldinit = 1e-4;
    apply_controller_knobs(I);
    // initialize_tstops / initialize_saveat (solve.jl:1021-1040, 1103-1124): tdir * t
    // inside the span, ascending
    const double d = I.tdir, dt0 = d * t0, dtf = d * tf;
    I.tstops.clear();
    for (int i = 0; i < ntstops; ++i)
        if (dt0 < d * tstops[i] && d * tstops[i] < dtf) I.tstops.push_back(d * tstops[i]);
    I.tstops.push_back(dtf);
    std::sort(I.tstops.begin(), I.tstops.end());
    I.itstop = 0;
    I.saveat.clear();
    for (int i = 0; i < nsave; ++i)
        if (dt0 < d * saveat[i] && d * saveat[i] <= dtf) I.saveat.push_back(d * saveat[i]);
    std::sort(I.saveat.begin(), I.saveat.end());
    I.isave = 0;
    I.dense = nullptr;
}

}  // namespace

extern "C" {

int64_t orc_rhs_calls(int reset) {
    int64_t v = g_rhs_calls;
    if (reset) g_rhs_calls = 0;
    return v;
}

int orc_record_eval_times(int enable) {
    g_record_times = enable != 0;
    g_eval_times.clear();
    return 0;
}

int orc_eval_times(double* out, int cap) {
    const int m = (int)g_eval_times.size() < cap ? (int)g_eval_times.size() : cap;
    for (int i = 0; i < m; ++i) out[i] = g_eval_times[i];
    return (int)g_eval_times.size();
}

void orc_rhs(int model, int n, const double* u, const double* p, double t, double* du) {
    rhs(model, n, u, p, t, du);
}
void orc_jac(int model, int n, const double* u, const double* p, double t, double* J) {
    jac(model, n, u, p, t, J);
}
int orc_tgrad(int model, int n, const double* u, const double* p, double t, double* dT) {
    return tgrad(model, n, u, p, t, dT) ? 1 : 0;
}

thread_local std::vector<int32_t> g_last_alg_choice;

int orc_solve(int alg, int model, int n, const double* p, double t0, double tf, const double* u0,
              const orc_opts* o, const double* saveat, int nsave_in, const double* tstops, int ntstops,
              double* t_out, double* u_out, int cap, int32_t* retcode, orc_stats* st, void** dense_handle) {
    Integ I;
    setup(I, alg, model, n, p, t0, tf, o, saveat, nsave_in, tstops, ntstops);
    I.dtimes.assign(tstops, tstops + (tstops ? ntstops : 0));
    std::sort(I.dtimes.begin(), I.dtimes.end());
    I.t_out = t_out;
    I.u_out = u_out;
    I.cap = cap;
    Dense* D = nullptr;
    if (dense_handle) {
        D = new Dense();
        D->alg = alg;
        D->model = model;
        D->n = n;
        D->p.assign(p, p + model_nparams(model));
        I.dense = D;
        *dense_handle = D;
    }
    int rc = solve_one(I, u0);
    if (retcode) *retcode = rc;
    if (st) *st = I.st;
    g_last_alg_choice = I.alg_choice;
    return I.nsaved;
}

double orc_initdt(int alg, int model, int n, const double* p, double t0, double tf, const double* u0,
                  const orc_opts* o, const double* tstops, int ntstops) {
    Integ I;
    setup(I, alg, model, n, p, t0, tf, o, nullptr, 0, tstops, tstops ? ntstops : 0);
    I.u.assign(u0, u0 + n);
    I.t = t0;
    I.fsallast.assign(n, 0.0);
    return initdt(I);
}

int orc_last_alg_choice(int32_t* out, int cap) {
    const int m = (int)g_last_alg_choice.size() < cap ? (int)g_last_alg_choice.size() : cap;
    for (int i = 0; i < m; ++i) out[i] = g_last_alg_choice[i];
    return m;
}

int orc_dense_nsteps(void* h) { return h ? (int)((Dense*)h)->steps.size() : 0; }

// sol(t) on the recorded steps: ode_interpolation(tval::Number, ...) with left
// continuity (lib/OrdinaryDiffEqCore/src/dense/generic_dense.jl:1094-1190).  The
// saved times are ts = [tprev of step 0, tend of each step]; i+ is the first
// index >= 1 (0-based) with ts[i+] >= t, clamped to the last; dt = ts[i+] -
// ts[i-] and theta = (t - ts[i-]) / dt; Vern7's extra stages are formed by
// _ode_addsteps! with that dt (verner_addsteps.jl:137-193).
// A query equal to a saved time returns that save for deriv 0 (the first at
// that time; with `right`, continuity = :right, the next one when it is at the
// same time), as ode_interpolation does before interpolating.
int orc_dense_eval_ex(void* h, const double* tq, int nq, int deriv, int right, double* out);

int orc_dense_eval(void* h, const double* tq, int nq, double* out) { return orc_dense_eval_ex(h, tq, nq, 0, 0, out); }

int orc_dense_eval_deriv(void* h, const double* tq, int nq, int deriv, double* out) {
    return orc_dense_eval_ex(h, tq, nq, deriv, 0, out);
}

int orc_dense_eval_ex(void* h, const double* tq, int nq, int deriv, int right, double* out) {
    Dense* D = (Dense*)h;
    // Val{2}: the forms the reference has (Tsit5, Rodas5P)
    if (deriv < 0 || deriv > 3 || (deriv >= 2 && D->alg != ORC_TSIT5 && D->alg != ORC_RODAS5P)) return -2;
    const int n = D->n;
    if (D->steps.empty()) return -1;
    const size_t ns = D->steps.size() + 1;
    auto ts = [&](size_t i) { return i == 0 ? D->steps[0].tprev : D->steps[i - 1].tend; };
    const double tdir = ts(ns - 1) < ts(0) ? -1.0 : 1.0;   // sign(ts[end] - ts[1])
    std::vector<double> K;
    for (int q = 0; q < nq; ++q) {
        const double t = tq[q];
        if (deriv == 0) {   // the exact-time rule (searchsortedfirst, then ts[i] == t)
            size_t i0 = 0;
            while (i0 < ns && tdir * ts(i0) < tdir * t) ++i0;
            if (i0 < ns && ts(i0) == t) {
                const size_t k = (right && i0 + 1 < ns && ts(i0 + 1) == t) ? i0 + 1 : i0;
                const double* v = k == 0 ? D->steps[0].y0.data() : D->steps[k - 1].y1.data();
                std::copy(v, v + n, out + (size_t)q * n);
                continue;
            }
        }
        size_t ip = 1;
        while (ip < ns && tdir * ts(ip) < tdir * t) ++ip;
        if (ip > ns - 1) ip = ns - 1;
        const size_t im = ip - 1;
        const Step& S = D->steps[ip - 1];
        const double dt = ts(ip) - ts(im);
        const double th = dt == 0.0 ? 1.0 : (t - ts(im)) / dt;
        double* o = out + (size_t)q * n;
        switch (D->alg) {
        case ORC_TSIT5:
            if (deriv == 3) tsit5_interp_d3(th, dt, S.k.data(), n, o);
            else if (deriv == 2) tsit5_interp_d2(th, dt, S.k.data(), n, o);
            else if (deriv) tsit5_interp_d1(th, S.k.data(), n, o);
            else tsit5_interp(th, dt, S.y0.data(), S.k.data(), n, o);
            break;
        case ORC_VERN7:
            K.assign((size_t)16 * n, 0.0);
            std::copy(S.k.begin(), S.k.end(), K.begin());
            vern7_extra(D->model, n, D->p.data(), ts(im), dt, S.y0.data(), K.data());
            if (deriv) vern7_interp_d1(th, K.data(), n, o);
            else vern7_interp(th, dt, S.y0.data(), K.data(), n, o);
            break;
        case ORC_RODAS5P:
            if (deriv == 3) rodas_interp_d3(th, dt, S.k.data(), n, o);
            else if (deriv == 2) rodas_interp_d2(th, dt, S.k.data(), n, o);
            else if (deriv) rodas_interp_d1(th, dt, S.y0.data(), S.y1.data(), S.k.data(), n, o);
            else rodas_interp(th, S.y0.data(), S.y1.data(), S.k.data(), n, o);
            break;
        case ORC_ROSENBROCK23:
            if (deriv) ros23_interp_d1(th, S.k.data(), n, o);
            else ros23_interp(th, dt, S.y0.data(), S.k.data(), n, o);
            break;
        default:
            for (int i = 0; i < n; ++i) o[i] = deriv ? (S.y1[i] - S.y0[i]) / dt : (1.0 - th) * S.y0[i] + th * S.y1[i];
        }
    }
    return 0;
}

// Step s of a dense record: tprev and tend, y0, y1 (n each) and the stored
// interpolation vectors in the library's order (Tsit5 k1..k7, Vern7 k1 and
// k4..k9, Rodas5P dense k1..k3; q-major, n each).  Returns the vector count.
int orc_dense_step(void* h, int s, double* t2, double* y0, double* y1, double* k) {
    Dense* D = (Dense*)h;
    if (s < 0 || (size_t)s >= D->steps.size()) return -1;
    const Step& S = D->steps[s];
    const int n = D->n;
    t2[0] = S.tprev;
    t2[1] = S.tend;
    std::copy(S.y0.begin(), S.y0.end(), y0);
    std::copy(S.y1.begin(), S.y1.end(), y1);
    static const int vern7_stage[7] = {1, 4, 5, 6, 7, 8, 9};
    const int nk = D->alg == ORC_VERN7 ? 7 : (int)(S.k.size() / (size_t)n);
    for (int q = 0; q < nk; ++q) {
        const int src = D->alg == ORC_VERN7 ? vern7_stage[q] - 1 : q;
        std::copy(S.k.begin() + (size_t)src * n, S.k.begin() + (size_t)(src + 1) * n, k + (size_t)q * n);
    }
    return nk;
}

void orc_dense_free(void* h) { delete (Dense*)h; }

int orc_solve_ensemble(int alg, int model, int nmax, const int32_t* n_per_traj, int np, int64_t N,
                       const double* u0, const double* p, const double* tspan, const orc_opts* o,
                       const double* saveat, int nsave, int saveat_per_traj, double* t_out, double* u_out,
                       int32_t* nsaved, int32_t* retcode, orc_stats* stats, int nthreads) {
    if (nthreads <= 0) nthreads = (int)std::thread::hardware_concurrency();
    if (nthreads <= 0) nthreads = 1;
    // saves plus possible start and end saves, and two per event (before and after its affect)
    int cap = nsave + (o->save_everystep ? o->max_step_saves : 0) + 2 + (o->callback ? 2 * o->max_events : 0);
    std::atomic<int64_t> next(0);
    auto worker = [&]() {
        std::vector<double> uj(nmax), pj(np), sv(nsave > 0 ? nsave : 1), tl(cap), ul((size_t)cap * nmax);
        std::vector<double> ts;
        Integ I;
        for (;;) {
            int64_t j = next.fetch_add(1);
            if (j >= N) break;
            int n = n_per_traj ? n_per_traj[j] : nmax;
            for (int i = 0; i < n; ++i) uj[i] = u0[(size_t)i * N + j];
            for (int i = 0; i < np; ++i) pj[i] = p[(size_t)i * N + j];
            for (int s = 0; s < nsave; ++s) sv[s] = saveat_per_traj ? saveat[(size_t)s * N + j] : saveat[s];
            double t0 = tspan[j], tf = tspan[N + j];
            ts.clear();
            if (o->saveat_as_tstops) ts.insert(ts.end(), sv.begin(), sv.begin() + nsave);
            if (o->ntstops > 0 && o->tstops) ts.insert(ts.end(), o->tstops, o->tstops + o->ntstops);
            setup(I, alg, model, n, pj.data(), t0, tf, o, sv.data(), nsave, ts.empty() ? nullptr : ts.data(),
                  (int)ts.size());
            I.dtimes.assign(o->tstops, o->tstops + (o->tstops ? o->ntstops : 0));
            std::sort(I.dtimes.begin(), I.dtimes.end());
            I.t_out = tl.data();
            I.u_out = ul.data();
            I.cap = cap;
            int rc = solve_one(I, uj.data());
            int ns = I.nsaved < cap ? I.nsaved : cap;
            if (nsaved) nsaved[j] = ns;
            if (retcode) retcode[j] = rc;
            if (stats) stats[j] = I.st;
            for (int s = 0; s < ns; ++s) {
                if (t_out) t_out[(size_t)s * N + j] = tl[s];
                if (u_out)
                    for (int i = 0; i < n; ++i) u_out[((size_t)s * nmax + i) * N + j] = ul[(size_t)s * n + i];
            }
        }
    };
    std::vector<std::thread> th;
    for (int i = 0; i < nthreads; ++i) th.emplace_back(worker);
    for (auto& x : th) x.join();
    return 0;
}

}  // extern "C"
