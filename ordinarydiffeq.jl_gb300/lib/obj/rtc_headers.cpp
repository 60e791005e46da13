// Generated by odegb300/build.py: the device headers, for NVRTC.
namespace odegb {
extern const char* const kRtcHeaderNames[] = {"common.cuh", "ensemble_args.h", "integrator.cuh", "rksum.cuh", "tableaus.h", "erk.cuh", "lu_group.cuh", "rodas.cuh", "ros23.cuh", "autoswitch.cuh", "user_model.cuh"};
extern const char* const kRtcHeaderSources[] = {
R"ODEGBRTC(// Device helpers shared by every integrator kernel.
//
// All kernels are compiled with -fmad=false: every fused multiply-add is
// written explicitly (fma / fmaf) in the nesting the reference's @muladd code
// produces, so the FP64 path follows the reference's operation order.
#pragma once
// The device headers also compile under NVRTC (registered models' kernels are
// compiled at run time), which has no standard or CUDA runtime headers.
#ifndef __CUDACC_RTC__
#include <cstdint>
#include <cuda_runtime.h>
#else
typedef signed char int8_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;
#endif

namespace odegb {

// the two type traits the kernels use (std's, which NVRTC lacks)
template <bool B> struct bool_constant { static constexpr bool value = B; };
template <class...> using void_t = void;
template <class T> struct is_double : bool_constant<false> {};
template <> struct is_double<double> : bool_constant<true> {};

// ------------------------------------------------------------------ scalars
template <class T> struct Arith;
template <> struct Arith<double> {
    static __device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
    static __device__ __forceinline__ double abs_(double a) { return fabs(a); }
};
template <> struct Arith<float> {
    static __device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
    static __device__ __forceinline__ float abs_(float a) { return fabsf(a); }
};
template <class T> __device__ __forceinline__ T FMA(T a, T b, T c) { return Arith<T>::fma_(a, b, c); }
template <class T> __device__ __forceinline__ T ABS(T a) { return Arith<T>::abs_(a); }

// |x| as a bit pattern, on the integer pipe.  Written in inline PTX because
// the optimizer recognises a masked sign bit as a floating-point abs (an FP64
// instruction on GB300's narrow FP64 pipe) and masked-bit comparisons as
// floating-point tests; the time and pivot helpers below rely on this.
__device__ __forceinline__ long long abs_bits_i(long long b) {
    long long r;
    asm("and.b64 %0, %1, %2;" : "=l"(r) : "l"(b), "l"(0x7fffffffffffffffLL));
    return r;
}
__device__ __forceinline__ long long abs_bits(double x) { return abs_bits_i(__double_as_longlong(x)); }

// Julia's Base.min/max on floats propagate NaN.
__device__ __forceinline__ double jmin(double a, double b) { return (a != a || b != b) ? __longlong_as_double(0x7ff8000000000000LL) : (a < b ? a : b); }
__device__ __forceinline__ double jmax(double a, double b) { return (a != a || b != b) ? __longlong_as_double(0x7ff8000000000000LL) : (a > b ? a : b); }
template <class T> __device__ __forceinline__ T tmax(T a, T b) { return (a != a || b != b) ? a + b : (a > b ? a : b); }
// Julia eps(x): spacing of doubles at |x|.
__device__ __forceinline__ double jeps(double x) {
    double ax = fabs(x);
    if (!isfinite(ax)) return __longlong_as_double(0x7ff8000000000000LL);
    return nextafter(ax, __longlong_as_double(0x7ff0000000000000LL)) - ax;
}

// x^y for the step-size controller and the initial-step heuristic: the
// reference calls FastPower.fastpower (exp2(y*log2 x)).  Evaluated here as
// exp(y ln x): ln from the atanh series ln m = 2 atanh((m-1)/(m+1)) with
// m in [1/sqrt2, sqrt2), exp by reduction modulo ln2 and a Taylor series
// (textbook methods; Muller, "Elementary Functions", ch. 5-6).  Only +, *,
// fma, IEEE division and exact scaling are used, so the result is identical
// on every IEEE-754 machine that evaluates the same sequence.
__device__ __forceinline__ double series_ln(double x) {
    const double LN2 = 0.6931471805599453, LN2LO = 2.3190468138462996e-17, SQRT1_2 = 0.7071067811865476;
    int e;
    double m = frexp(x, &e);
    if (m < SQRT1_2) { m = m * 2.0; e -= 1; }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s;
    double poly = 0.08;
    poly = fma(poly, s2, 0.08695652173913043);
    poly = fma(poly, s2, 0.09523809523809523);
    poly = fma(poly, s2, 0.10526315789473684);
    poly = fma(poly, s2, 0.11764705882352941);
    poly = fma(poly, s2, 0.13333333333333333);
    poly = fma(poly, s2, 0.15384615384615385);
    poly = fma(poly, s2, 0.18181818181818182);
    poly = fma(poly, s2, 0.2222222222222222);
    poly = fma(poly, s2, 0.2857142857142857);
    poly = fma(poly, s2, 0.4);
    poly = fma(poly, s2, 0.6666666666666666);
    poly = fma(poly, s2, 2.0);
    double de = (double)e;
    return fma(de, LN2, fma(de, LN2LO, s * poly));
}
__device__ __forceinline__ double series_exp(double t) {
    const double LN2 = 0.6931471805599453, LN2LO = 2.3190468138462996e-17, INVLN2 = 1.4426950408889634;
    if (t != t) return t;
    if (t > 709.0) return __longlong_as_double(0x7ff0000000000000LL);
    if (t < -745.0) return 0.0;
    double k = rint(t * INVLN2);
    double r = fma(-k, LN2, t);
    r = fma(-k, LN2LO, r);
    double e = 2.8114572543455206e-15;
    e = fma(e, r, 4.779477332387385e-14);
    e = fma(e, r, 7.647163731819816e-13);
    e = fma(e, r, 1.1470745597729725e-11);
    e = fma(e, r, 1.6059043836821613e-10);
    e = fma(e, r, 2.08767569878681e-09);
    e = fma(e, r, 2.505210838544172e-08);
    e = fma(e, r, 2.755731922398589e-07);
    e = fma(e, r, 2.7557319223985893e-06);
    e = fma(e, r, 2.48015873015873e-05);
    e = fma(e, r, 0.0001984126984126984);
    e = fma(e, r, 0.001388888888888889);
    e = fma(e, r, 0.008333333333333333);
    e = fma(e, r, 0.041666666666666664);
    e = fma(e, r, 0.16666666666666666);
    e = fma(e, r, 0.5);
    e = fma(e, r, 1.0);
    e = fma(e, r, 1.0);
    return ldexp(e, (int)k);
}
__device__ __forceinline__ double ctrl_pow(double x, double y) {
    if (x == 0.0) return 0.0;
    if (x != x || y != y) return __longlong_as_double(0x7ff8000000000000LL);
    if (isinf(x)) return __longlong_as_double(0x7ff0000000000000LL);
    return series_exp(y * series_ln(x));
}

// ------------------------------------------------------------------ solution accumulator
// The state u is carried as a pair (hi, lo).  In FP64 mode lo is always zero
// and every formula reduces to the reference's single-rounding expression.
// In the mixed mode (R = float) the pair is a compensated FP32 sum
// (hi + lo, about 48 significant bits, Dekker/Knuth two-sum): stage values and
// increments are FP32, but the running solution does not lose a float ulp per
// step, which at reltol 1e-6 would otherwise dominate the error.  On GB300 a
// two-sum costs a handful of FP32 instructions where an FP64 add runs on a
// far slower pipe.
template <class R> struct Acc;
template <> struct Acc<double> {
    // stage input uprev + d*S (reference: muladd(d, S, uprev))
    static __device__ __forceinline__ double stage(double d, double S, double up, double) { return fma(d, S, up); }
    // new solution u = uprev + d*S
    static __device__ __forceinline__ void update(double& hi, double& lo, double d, double S, double up, double) {
        hi = fma(d, S, up);
        lo = 0.0;
    }
    // u = uprev + dt*S with dt as a pair (dh, dl); in FP64 dl is 0 and this is update
    static __device__ __forceinline__ void update2(double& hi, double& lo, double dh, double, double S, double up,
                                                   double) {
        hi = fma(dh, S, up);
        lo = 0.0;
    }
    // the low part of dt as a float pair: none in FP64
    static __device__ __forceinline__ double dt_lo(double, double) { return 0.0; }
    // u = uprev + inc where inc was accumulated starting from uprev already
    static __device__ __forceinline__ void set(double& hi, double& lo, double v) { hi = v; lo = 0.0; }
    static __device__ __forceinline__ void set_pair(double& hi, double& lo, double v) { hi = v; lo = 0.0; }
    static __device__ __forceinline__ void split(double x, double& hi, double& lo) { hi = x; lo = 0.0; }
    static __device__ __forceinline__ double join(double hi, double) { return hi; }
};
template <> struct Acc<float> {
    static __device__ __forceinline__ float stage(float d, float S, float up, float uplo) {
        return fmaf(d, S, up) + uplo;
    }
    static __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
        s = a + b;
        float bb = s - a;
        e = (a - (s - bb)) + (b - bb);
    }
    static __device__ __forceinline__ void update(float& hi, float& lo, float d, float S, float up, float uplo) {
        float inc = d * S + uplo;
        two_sum(up, inc, hi, lo);
    }
    // u = uprev + dt*S with the FP64 dt as a float pair dh + dl (dh = float(dt)):
    // the remainder dl*S joins the increment, so the state advances by the step
    // that t advances by (with dh alone the state drifts by up to 2^-24 of each
    // increment, which shifts event times and accumulates over long runs)
    static __device__ __forceinline__ void update2(float& hi, float& lo, float dh, float dl, float S, float up,
                                                   float uplo) {
        float inc = fmaf(dh, S, fmaf(dl, S, uplo));
        two_sum(up, inc, hi, lo);
    }
    static __device__ __forceinline__ float dt_lo(double dt, float dh) { return (float)(dt - (double)dh); }
    static __device__ __forceinline__ void set(float& hi, float& lo, float v) { hi = v; lo = 0.0f; }
    static __device__ __forceinline__ void split(double x, float& hi, float& lo) {
        hi = (float)x;
        lo = (float)(x - (double)hi);
    }
    static __device__ __forceinline__ double join(float hi, float lo) { return (double)hi + (double)lo; }
};

// ------------------------------------------------------------------ double-float
// An unevaluated sum hi + lo of two floats (about 48 significant bits),
// evaluated with error-free transformations on the FP32 pipe (Dekker 1971;
// Joldes, Muller, Popescu 2017, "Tight and rigorous error bounds for basic
// building blocks of double-word arithmetic", algorithms 1-4 and 10-12).  The
// mixed Rosenbrock path evaluates stiff right-hand sides in it: their terms
// cancel (ROBER's k1 y1 - k2 y2^2 - k3 y2 y3), and FP32 arithmetic there alone
// leaves ~70x reltol of error at reltol 1e-6.
struct ff {
    float hi, lo;
    __device__ __forceinline__ ff() : hi(0.0f), lo(0.0f) {}
    __device__ __forceinline__ ff(float h) : hi(h), lo(0.0f) {}
    __device__ __forceinline__ ff(int h) : hi((float)h), lo(0.0f) {}
    __device__ __forceinline__ ff(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ explicit ff(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    __device__ __forceinline__ float f() const { return hi + lo; }
};
__device__ __forceinline__ ff ff_fast2sum(float a, float b) {
    float s = a + b;
    return ff(s, b - (s - a));
}
__device__ __forceinline__ ff operator+(ff a, ff b) {
    float s = a.hi + b.hi;
    float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    return ff_fast2sum(s, e + (a.lo + b.lo));
}
__device__ __forceinline__ ff operator-(ff a) { return ff(-a.hi, -a.lo); }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
// a * b for a float b (error-free product of the leading part plus the tail)
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return ff_fast2sum(p, e);
}
__device__ __forceinline__ ff operator*(ff a, ff b) {
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    return ff_fast2sum(p, e);
}

// ------------------------------------------------------------------ parameters
// A parameter in the mixed form: its FP64 value as a float pair hi + lo
// (hi = float(p)).  A product with an FP32 state value folds lo in before its
// one rounding, fma(hi, x, lo x), so the right-hand side sees the FP64
// parameter rather than float(p): rounding a parameter to FP32 changes the
// problem itself by up to 2^-25 relative, a systematic error that
// ill-conditioned trajectories (random Duffing chains) amplify far past the
// tolerance.  Sums fold lo in after the leading rounding.  Converts to float
// (hi) where a model's Jacobian takes a parameter as an entry.
struct fpair {
    float hi, lo;
    __device__ __forceinline__ fpair() : hi(0.0f), lo(0.0f) {}
    __device__ __forceinline__ fpair(float h, float l) : hi(h), lo(l) {}
    __device__ __forceinline__ explicit fpair(double x) : hi((float)x), lo((float)(x - (double)(float)x)) {}
    __device__ __forceinline__ operator float() const { return hi; }
};
__device__ __forceinline__ float operator*(fpair a, float x) { return fmaf(a.hi, x, a.lo * x); }
__device__ __forceinline__ float operator*(float x, fpair a) { return fmaf(a.hi, x, a.lo * x); }
__device__ __forceinline__ float operator*(fpair a, fpair b) { return fmaf(a.hi, b.hi, fmaf(a.hi, b.lo, a.lo * b.hi)); }
__device__ __forceinline__ float operator+(fpair a, float x) { return (a.hi + x) + a.lo; }
__device__ __forceinline__ float operator+(float x, fpair a) { return (x + a.hi) + a.lo; }
__device__ __forceinline__ float operator-(fpair a, float x) { return (a.hi - x) + a.lo; }
__device__ __forceinline__ float operator-(float x, fpair a) { return (x - a.hi) - a.lo; }
__device__ __forceinline__ fpair operator-(fpair a) { return fpair(-a.hi, -a.lo); }

// Parameter type of a precision: double in FP64, a float pair in the mixed form.
template <class R> struct ParamOf { using type = R; };
template <> struct ParamOf<float> { using type = fpair; };
template <class R> using PR = typename ParamOf<R>::type;
template <class R> __device__ __forceinline__ PR<R> make_param(double x) { return PR<R>(x); }

// A parameter's FP64 value from any precision's parameter type, and an FP64
// value in a stage type (float, double-float or double).
__device__ __forceinline__ double pdouble(double x) { return x; }
__device__ __forceinline__ double pdouble(fpair x) { return (double)x.hi + (double)x.lo; }
__device__ __forceinline__ double pdouble(ff x) { return (double)x.hi + (double)x.lo; }
template <class R> __device__ __forceinline__ R from_double(double x) { return (R)x; }
template <> __device__ __forceinline__ ff from_double<ff>(double x) { return ff(x); }

// ------------------------------------------------------------------ lane groups
// A trajectory is owned by a group of L consecutive lanes of one warp; each
// lane holds C state components (component index = lane_in_group*C + c).
template <int L> struct Group {
    unsigned mask;
    int lane;   // lane within the group
    int base;   // warp lane of the group's lane 0
    __device__ __forceinline__ Group() {
        int wl = threadIdx.x & 31;
        lane = wl % L;
        base = wl - lane;
        mask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << base);
    }
    // bit l set when lane l of the group has b
    __device__ __forceinline__ unsigned ballot(bool b) const {
        if (L == 1) return b ? 1u : 0u;
        unsigned m = __ballot_sync(mask, b);
        return L == 32 ? m : (m >> base) & ((1u << L) - 1u);
    }
    template <class T> __device__ __forceinline__ T sum(T v) const {
#pragma unroll
        for (int off = L / 2; off > 0; off >>= 1) v += __shfl_xor_sync(mask, v, off, L);
        return v;
    }
    template <class T> __device__ __forceinline__ T bcast(T v, int src) const {
        if (L == 1) return v;
        return __shfl_sync(mask, v, src, L);
    }
    template <class T> __device__ __forceinline__ T from(T v, int src_lane) const {
        if (L == 1) return v;
        return __shfl_sync(mask, v, src_lane, L);
    }
    __device__ __forceinline__ ff from(ff v, int src_lane) const {
        if (L == 1) return v;
        return ff(__shfl_sync(mask, v.hi, src_lane, L), __shfl_sync(mask, v.lo, src_lane, L));
    }
    __device__ __forceinline__ bool any(bool b) const {
        if (L == 1) return b;
        return __any_sync(mask, b);
    }
    __device__ __forceinline__ void sync() const {
        if (L > 1) __syncwarp(mask);
    }
};

}  // namespace odegb
)ODEGBRTC",
R"ODEGBRTC(// The parameter block of one ensemble launch, shared by the kernels, the host
// runtime and the runtime-compiled kernels of registered models (plain types
// only, so the header also compiles under NVRTC, which has no standard headers).
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

namespace odegb {

struct OdeStatsDev {
    long long nf, njacs, nw, nsolve, naccept, nreject;
};

// Everything one ensemble launch needs.  Device pointers; SoA layouts:
//   u0[i*N + j], p[i*N + j], tspan[j] / tspan[N + j],
//   saveat[s] (shared) or saveat[s*N + j] (per trajectory),
//   t_out[s*N + j], u_out[(s*nmax + i)*N + j].
struct EnsembleArgs {
    long long N;            // trajectories in the arrays
    long long count;        // trajectories this launch integrates (entries of order, or N)
    const long long* order; // optional trajectory indices (size-class buckets); nullptr = identity
    int nmax;               // state stride
    const double* u0;
    const double* p;
    const double* tspan;
    const double* saveat;
    int nsave;
    int saveat_per_traj;
    int nsave_cap;          // save slots per trajectory in t_out/u_out
    double* t_out;
    double* u_out;
    int32_t* nsaved;
    int32_t* retcode;
    OdeStatsDev* stats;
    // options
    double reltol, abstol, dtmax, dtmin, dt;
    const double* reltol_traj;   // per-trajectory tolerances (nullptr: reltol/abstol for all)
    const double* abstol_traj;
    long long maxiters;
    int save_start, save_end, save_end_user, saveat_given, saveat_scalar;
    int save_everystep;     // save every accepted step (saveat empty); nsave_cap bounds the slots
    int callback;           // 1: the model's ContinuousCallback (models with HAS_EVENT)
    int interp_points;      // its interp_points
    const double* tstops;   // the solve's tstops, ascending, shared by every trajectory
    int ntstops;
    double* k_out;          // dense output (nullptr: none): k_out[((s*NDENSE + q)*nmax + i)*N + j], the
                            // method's NDENSE interpolation vectors of the step ending at save s
    double qmax_first_step, qmax;
    int ir_sweeps;          // mixed Rosenbrock: refinement sweeps per solve
    // scheduling
    int persistent;
    unsigned long long* queue;     // persistent work counter (zeroed before launch)
    const volatile int* abort_flag;  // host-settable early stop (nullptr: none)
    // size classes of an uneven ensemble (one launch over all classes):
    // class k holds class_count[k] trajectories at order[class_offset[k] ...]
    const unsigned long long* class_count;
    const unsigned long long* class_offset;
    unsigned long long* class_next;  // per-class work counters (zeroed before launch)
};

}  // namespace odegb
)ODEGBRTC",
R"ODEGBRTC(// The per-trajectory integrator loop, run by one lane group on the device.
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

// Residual norm sqrt(sum_i (ut_i / (abstol + max(|u0_i|,|u1_i|) reltol))^2 / n).
// FP64 mode: the sum in FP64 (sequentially within a lane, then across the
// group).  Mixed mode: the same sum carried in double-float (an exact square
// by fma, a two-sum per term; FP64-class precision on the FP32 pipe), since
// on GB300 each FP64 add/fma or float<->double conversion per component would
// cost the FP64 pipe more time than the whole FP32 stage work of a small system.
template <class R, int L, int C>
__device__ __forceinline__ typename Ctl<R>::T error_norm(const R* ut, const R* u0, const R* u1, R abstol, R reltol,
                                                         const Group<L>& g) {
    if (sizeof(R) == 8) {
        double acc = 0.0;
#pragma unroll
        for (int c = 0; c < C; ++c) {
            R sc = FMA(tmax(ABS(u0[c]), ABS(u1[c])), reltol, abstol);
            double e = (double)(ut[c] / sc);
            acc = fma(e, e, acc);
        }
        acc = g.sum(acc);
        return (typename Ctl<R>::T)sqrt(acc / (double)(L * C));
    }
    float hi = 0.0f, lo = 0.0f;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const float sc = fmaf(tmax(fabsf((float)u0[c]), fabsf((float)u1[c])), (float)reltol, (float)abstol);
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
template <class Model, class R, int L, int C, int ORDER>
__device__ double initdt(const R* u0, const PR<R>* p, double t, double dtmax, double dtmin_user, R abstol, R reltol,
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
        // 10^(-(2 + log10 mx)/order) = exp(-(2 ln10 + ln mx)/order)
        const double LN10 = 2.302585092994046;
        dt1 = series_exp(-(2.0 * LN10 + series_ln(mx)) / (double)ORDER);
    }
    return jmax(dtmin, jmin(jmin(100.0 * dt0, dt1), dtmax));
}

// One trajectory, start to finish, on lane group g.  Alg provides the cache,
// the step, the interpolant and the FSAL hooks.
template <class Alg, class Model, class R, int L, int C>
__device__ void solve_trajectory(const EnsembleArgs& a, long long j, const Group<L>& g) {
    using CT = typename Ctl<R>::T;
    constexpr int NP = Model::NP;
    const long long N = a.N;
    R u[C], uprev[C], ulo[C], uprevlo[C];   // solution as (hi, lo) pairs, see Acc
    PR<R> p[NP > 0 ? NP : 1];   // FP64, or float pairs in the mixed form (fpair)
#pragma unroll
    for (int c = 0; c < C; ++c) Acc<R>::split(a.u0[(size_t)(g.lane * C + c) * N + j], u[c], ulo[c]);
#pragma unroll
    for (int i = 0; i < NP; ++i) p[i] = make_param<R>(a.p[(size_t)i * N + j]);
    const double t0 = a.tspan[j], tf = a.tspan[N + j];
    const double dtmax = a.dtmax > 0 ? a.dtmax : tf - t0;
    // the ensemble's tolerances, or per trajectory (requests merged into one
    // launch by the serving loop keep their own)
    const R abstol = (R)(a.abstol_traj ? a.abstol_traj[j] : a.abstol);
    const R reltol = (R)(a.reltol_traj ? a.reltol_traj[j] : a.reltol);
    const Ctrl K = make_ctrl<Alg::ORDER, Alg::IMPLICIT>(a);
    // beta1, beta2 and qsteady_max change with a composite's current method
    CT beta1 = (CT)K.beta1, beta2 = (CT)K.beta2, qsteady_max = (CT)K.qsteady_max;
    const CT gam = (CT)K.gamma, qmin_inv = (CT)K.qmin_inv;
    const CT qoldinit = (CT)K.qoldinit;
    const CT inv_qmax = (CT)(1.0 / K.qmax), inv_qmax_first = (CT)(1.0 / K.qmax_first);

    typename Alg::template Cache<R, C> cache;
    StepStats st = {0, 0, 0, 0, 0, 0};
    int nsaved = 0;
    int isave = 0;
    double last_saved_t = dnan();

    auto save_point = [&](double ts, const R* v, const R* vlo) {
        // past the capacity, step saves keep the latest point in the last slot
        const int slot = nsaved < a.nsave_cap ? nsaved : ((a.save_everystep || a.callback) ? a.nsave_cap - 1 : -1);
        if (slot >= 0) {
            if (g.lane == 0 && a.t_out) a.t_out[(size_t)slot * N + j] = ts;
#pragma unroll
            for (int c = 0; c < C; ++c)
                a.u_out[((size_t)slot * a.nmax + g.lane * C + c) * N + j] = Acc<R>::join(v[c], vlo[c]);
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
    auto saveat_at = [&](int s) -> double {
        return a.saveat_per_traj ? a.saveat[(size_t)s * N + j] : a.saveat[s];
    };

    // saveat entries outside (t0, tf] are skipped (initialize_saveat, solve.jl:1103-1124)
    while (isave < a.nsave && !(saveat_at(isave) > t0)) isave++;

#pragma unroll
    for (int c = 0; c < C; ++c) { uprev[c] = u[c]; uprevlo[c] = ulo[c]; }
    if (a.save_start) {
        if (a.k_out) save_dense(false);
        save_point(t0, u, ulo);
    }

    double t = t0, tprev = t0;
    Alg::template initialize<Model, R, L, C>(cache, u, p, t, g, st, a, j);
    double dt;
    if (a.dt > 0) {
        dt = a.dt;
    } else {
        dt = initdt<Model, R, L, C, Alg::ORDER>(u, p, t, dtmax, a.dtmin, abstol, reltol,
                                                 Alg::template fsal_slot<R, C>(cache), g);
        st.nf += 2;
    }
    double dtpropose = dt;
    CT EEst = CT(1), q11 = CT(1), errold = qoldinit;
    CT bank_errold = qoldinit, bank_q11 = CT(1);   // composite: the other method's controller state
    bool do_error_check = true;
    long long iter = 0, success_iter = 0;
    bool accept = false, next_tstop = false;
    // forward integration only: tf < t0 (or a NaN span) is not stepped
    int rc = (tf >= t0) ? RC_DEFAULT : RC_INITIALFAILURE;

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
                Alg::template interpolate<Model, R, L, C>(cache, out, outlo, th, dt, tprev, uprev, uprevlo, y1, y1lo,
                                                          p, g);
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
                if (abst == t) return Model::template event_condition<R, L, C>(u, ulo, a.p + j, N, abst, g);
                if (abst == tprev)
                    return Model::template event_condition<R, L, C>(uprev, uprevlo, a.p + j, N, abst, g);
                R v[C], vlo[C];
                Alg::template interpolate<Model, R, L, C>(cache, v, vlo, (abst - tprev) / dt, dt, tprev, uprev,
                                                          uprevlo, u, ulo, p, g);
                return Model::template event_condition<R, L, C>(v, vlo, a.p + j, N, abst, g);
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
            // change_t_via_interpolation!  (the step's end state stays for the saveat
            // points before the event)
            const bool moved = cb_t != t;
            R uend[C], uendlo[C];
#pragma unroll
            for (int c = 0; c < C; ++c) { uend[c] = u[c]; uendlo[c] = ulo[c]; }
            if (moved) {
                R v[C], vlo[C];
                Alg::template interpolate<Model, R, L, C>(cache, v, vlo, (cb_t - tprev) / dt, dt, tprev, uprev,
                                                          uprevlo, u, ulo, p, g);
#pragma unroll
                for (int c = 0; c < C; ++c) { u[c] = v[c]; ulo[c] = vlo[c]; }
                t = cb_t;
            }
            // saveat up to the event, then the pre-affect save unless one landed on t
            if (!savevalues(uend, uendlo)) save_point(t, u, ulo);
            bool modified = false;
            if (bs < 0.0 && Model::EVENT_AFFECT_POS) {
                terminated = Model::template event_affect<R, L, C>(u, ulo, a.p + j, N, t, true, g);
                modified = true;
            } else if (bs > 0.0 && Model::EVENT_AFFECT_NEG) {
                terminated = Model::template event_affect<R, L, C>(u, ulo, a.p + j, N, t, false, g);
                modified = true;
            }
            if (modified) save_point(t, u, ulo);   // save_positions[2]
            if (!terminated && (moved || modified)) Alg::template reset_fsal<Model, R, L, C>(cache, u, ulo, p, t, g, st);
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
                    Model::template event_conditions<R, L, C>(out, u, ulo, a.p + j, N, abst, g);
                } else if (abst == tprev) {
                    Model::template event_conditions<R, L, C>(out, uprev, uprevlo, a.p + j, N, abst, g);
                } else {
                    R v[C], vlo[C];
                    Alg::template interpolate<Model, R, L, C>(cache, v, vlo, (abst - tprev) / dt, dt, tprev, uprev,
                                                              uprevlo, u, ulo, p, g);
                    Model::template event_conditions<R, L, C>(out, v, vlo, a.p + j, N, abst, g);
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
            R uend[C], uendlo[C];
#pragma unroll
            for (int c = 0; c < C; ++c) { uend[c] = u[c]; uendlo[c] = ulo[c]; }
            if (moved) {
                R v[C], vlo[C];
                Alg::template interpolate<Model, R, L, C>(cache, v, vlo, (cb_t - tprev) / dt, dt, tprev, uprev,
                                                          uprevlo, u, ulo, p, g);
#pragma unroll
                for (int c = 0; c < C; ++c) { u[c] = v[c]; ulo[c] = vlo[c]; }
                t = cb_t;
            }
            if (!savevalues(uend, uendlo)) save_point(t, u, ulo);
            terminated = Model::template vector_event_affect<R, L, C>(u, ulo, a.p + j, N, t, dir, g);
            save_point(t, u, ulo);
            if (!terminated) Alg::template reset_fsal<Model, R, L, C>(cache, u, ulo, p, t, g, st);
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
    while (t < tf) {
        // ---- loopheader!
        while (itst < a.ntstops && !(a.tstops[itst] > t)) itst++;
        const double tnext = (itst < a.ntstops && a.tstops[itst] < tf) ? a.tstops[itst] : tf;   // first_tstop
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
            } else {
                // step_reject_controller!: dt /= min(1/qmin, q11/gamma)
                const CT qq = q11 / gam;
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
                using NSA = typename Alg::NonStiff;
                using SA = typename Alg::Stiff;
                const Ctrl K2 = cur == 0 ? make_ctrl<NSA::ORDER, NSA::IMPLICIT>(a) : make_ctrl<SA::ORDER, SA::IMPLICIT>(a);
                beta1 = (CT)K2.beta1;
                beta2 = (CT)K2.beta2;
                qsteady_max = (CT)K2.qsteady_max;
                Alg::template enter<Model, R, L, C>(cache, uprev, uprevlo, p, t, g, st);
            }
        }
        // fix_dt_at_bounds!
        dt = pmin(dtmax, dt);
        dt = pmax(dt, pabs(pmax(peps(t), a.dtmin)));
        {   // modify_dt_for_tstops!
            const double tol = ptol100(pmax(pabs(t), pabs(tnext)));
            const double orig = pabs(dt);
            dtpropose = orig;
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
            else if (ple(pabs(dt), pabs(a.dtmin)) && (!accept || t + dt < tnext)) e = RC_DTLESSTHANMIN;
            else if (!accept && ple(pabs(dt), peps(t))) e = RC_UNSTABLE;
            else if (accept) {
                bool bad = false;
#pragma unroll
                for (int c = 0; c < C; ++c) bad = bad || !isfinite(u[c]);
                if (g.any(bad)) e = RC_UNSTABLE;
            }
            if (e == RC_SUCCESS && a.abort_flag != nullptr && (iter & 63) == 0 && *a.abort_flag != 0)
                e = RC_ABORTED;
            if (e != RC_SUCCESS) { rc = e; break; }
        }
        // ---- perform_step! (skipped for a step below eps(t) onto the tstop)
        if (!(next_tstop && plt(pabs(dt), peps(t)))) {
            EEst = Alg::template step<Model, R, L, C>(cache, u, ulo, uprev, uprevlo, p, t, dt, abstol, reltol, iter,
                                                      EEst > CT(1), g, st);
        }
        // ---- loopfooter!
        if constexpr (is_composite_alg<Alg>::value) do_error_check = true;
        const double ttmp = t + dt;
        const CT inv_qmaxc = success_iter == 0 ? inv_qmax_first : inv_qmax;
        CT q;
        if (EEst == CT(0)) {
            q = inv_qmaxc;
        } else {
            const CT qq = Ctl<R>::pw(EEst, beta1);
            q = qq / Ctl<R>::pw(errold, beta2);
            q11 = qq;
            const CT x = q / gam;
            q = x > qmin_inv ? qmin_inv : (x < inv_qmaxc ? inv_qmaxc : x);
        }
        accept = EEst <= CT(1);
        if (accept) {
            st.naccept++;
            tprev = t;
            if (next_tstop) {
                dt = dtpropose;
                next_tstop = false;
                t = tnext;   // the tstop target
            } else {
                t = ttmp;
            }
            if (CT(1) <= q && q <= qsteady_max) q = CT(1);
            errold = (EEst != EEst) ? EEst : (EEst > qoldinit ? EEst : qoldinit);
            const double dtnew = Ctl<R>::scale_dt(dt, q);
            const double dtp = pmin(pabs(dtmax), pabs(dtnew));
            dtpropose = pmax(pabs(dtp), pabs(pmax(peps(t), a.dtmin)));
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
                    if constexpr (discrete_at_tstops<Model>::value) fire = itst < a.ntstops && a.tstops[itst] == t;
                    else fire = Model::template discrete_condition<R, L, C>(u, ulo, a.p + j, N, t, g);
                }
                if (fire) {
                    // saveat up to t and the every-step save, then save_positions[1]
                    // unless a save landed on t; affect!; save_positions[2]
                    if (!savevalues(u, ulo)) save_point(t, u, ulo);
                    terminated = Model::template discrete_affect<R, L, C>(u, ulo, a.p + j, N, t, g) || terminated;
                    save_point(t, u, ulo);
                    // u changed: FSAL methods evaluate f(u) again (reeval_fsal)
                    if (!terminated) Alg::template reset_fsal<Model, R, L, C>(cache, u, ulo, p, t, g, st);
                }
                handled = fire;   // saved_in_cb is the discrete callbacks' verdict
            }
            if (!handled) savevalues(u, ulo);
            Alg::template after_save<R, C>(cache);
            if (terminated) {   // terminate! (ReturnCode.Terminated)
                rc = RC_TERMINATED;
                break;
            }
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
}

// Ensemble kernel: static (one trajectory per group, the plain one-kernel-per-
// ensemble form) or persistent (groups pop trajectory indices from a device
// counter until the ensemble is exhausted).
template <class Alg, class Model, class R, int L, int C>
// Mixed kernels with up to 4 states per lane are held to 3 resident blocks of
// 128 (<= 170 registers; measured 10% faster than 2 on Robertson, no spills);
// wider or FP64 kernels keep their registers.
#ifndef ODEGB_MIN_BLOCKS_F32
#define ODEGB_MIN_BLOCKS_F32 3
#endif
__global__ void __launch_bounds__(128, (sizeof(R) == 4 && C <= 4) ? ODEGB_MIN_BLOCKS_F32 : 1)
    ensemble_kernel(EnsembleArgs a) {
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

// Uneven-size ensembles in ONE persistent launch.  Trajectories were bucketed
// on the device by state count; every warp works through the size classes
// from the largest down (longest jobs first), its lane groups popping
// trajectories of the current class from that class's device counter, so a
// group that finishes a trajectory refills at once and the load balances
// across classes.  At a class change the warp regroups its lanes (L depends
// on the class), which needs the whole warp: __syncwarp between classes.
template <class Alg, class Model, class R, int L, int C>
__device__ __forceinline__ void drain_class(const EnsembleArgs& a, int cls) {
    Group<L> g;
    const unsigned long long cnt = a.class_count[cls], off = a.class_offset[cls];
    for (;;) {
        unsigned long long idx = 0;
        if (g.lane == 0) idx = atomicAdd(a.class_next + cls, 1ull);
        idx = g.bcast(idx, 0);
        if (idx >= cnt) break;
        solve_trajectory<Alg, Model, R, L, C>(a, a.order[off + idx], g);
    }
    __syncwarp();
}

// Classes n = 64, 32, 16, 8, 4 with C states per lane (L = n/C).
// The mixed one-launch kernel at 3 resident blocks (<= 168 registers, no
// spills): 227 ms against 295 ms at 2 blocks for 1M uneven Duffing chains.
#ifndef ODEGB_MIN_BLOCKS_FUSED_F32
#define ODEGB_MIN_BLOCKS_FUSED_F32 3
#endif
template <class Alg, class Model, class R, int C>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? ODEGB_MIN_BLOCKS_FUSED_F32 : 1) fused_class_kernel(EnsembleArgs a) {
    static_assert(C == 2 || C == 4, "class layouts hold 2 or 4 states per lane");
    drain_class<Alg, Model, R, 64 / C, C>(a, 4);
    drain_class<Alg, Model, R, 32 / C, C>(a, 3);
    drain_class<Alg, Model, R, 16 / C, C>(a, 2);
    drain_class<Alg, Model, R, 8 / C, C>(a, 1);
    drain_class<Alg, Model, R, 4 / C, C>(a, 0);
}

}  // namespace odegb
)ODEGBRTC",
R"ODEGBRTC(// Tableau-driven stage sums for the explicit methods, in two arithmetic forms.
//
// FP64 (R = double): the reference's order.  A row  uprev + dt*(a1 k1 + ... + am km)
// is muladd(dt, muladd(a1,k1, muladd(a2,k2, ... am*km)), uprev) (MuladdMacro
// nesting, the last term innermost); a single-term row is uprev + (dt*a)*k1.
//
// Mixed (R = float): each coefficient is split at compile time into
// a_hi + a_lo (two floats) and the sum is accumulated with an error-free
// product (fma) and two-sum, i.e. compensated (Ogita-Rump-Oishi Dot2).  Vern7
// rows carry coefficients up to |a| ~ 190 that cancel to O(1); plain FP32
// rounding of those coefficients and partial sums leaves errors of ~100x
// reltol at reltol 1e-6, the compensated form stays at the FP64 level.
#pragma once
#include "common.cuh"
#include "tableaus.h"

namespace odegb {

// ---- tableau descriptions (1-based stages; slot(j) = storage slot of k_j)
struct Tsit5Tab {
    static constexpr int S = 7;
    __host__ __device__ static constexpr double a(int i, int j) { return tab::TSIT5_A(i, j); }
    __host__ __device__ static constexpr float ahi(int i, int j) { return tab::TSIT5_A_HI(i, j); }
    __host__ __device__ static constexpr float alo(int i, int j) { return tab::TSIT5_A_LO(i, j); }
    __host__ __device__ static constexpr bool am(int i, int j) { return tab::TSIT5_AM(i, j); }
    __host__ __device__ static constexpr double c(int i) { return tab::TSIT5_CS(i); }
    __host__ __device__ static constexpr double bt(int j) { return tab::TSIT5_BT(j); }
    __host__ __device__ static constexpr bool btm(int j) { return j >= 1 && j <= 7; }
    __host__ __device__ static constexpr int slot(int j) { return j - 1; }
};

struct Vern7Tab {
    static constexpr int S = 16;
    __host__ __device__ static constexpr double a(int i, int j) { return tab::VERN7_A(i, j); }
    __host__ __device__ static constexpr float ahi(int i, int j) { return tab::VERN7_A_HI(i, j); }
    __host__ __device__ static constexpr float alo(int i, int j) { return tab::VERN7_A_LO(i, j); }
    __host__ __device__ static constexpr bool am(int i, int j) { return tab::VERN7_AM(i, j); }
    __host__ __device__ static constexpr double c(int i) { return tab::VERN7_CS(i); }
    __host__ __device__ static constexpr double b(int j) { return tab::VERN7_B(j); }
    __host__ __device__ static constexpr bool bm(int j) { return tab::VERN7_BM(j); }
    __host__ __device__ static constexpr double bt(int j) { return tab::VERN7_BT(j); }
    __host__ __device__ static constexpr bool btm(int j) { return tab::VERN7_BTM(j); }
    // k1..k10 in slots 0..9; the lazy stages k11..k16 reuse the slots of
    // k2, k3, k10 (unused by the interpolant) and 10..12.
    __host__ __device__ static constexpr int slot(int j) {
        return j <= 10 ? j - 1 : (j == 11 ? 1 : j == 12 ? 2 : j == 13 ? 9 : j - 4);
    }
};

template <class Tab>
__host__ __device__ constexpr int row_last(int row) {
    int l = 0;
    for (int j = 1; j < row; ++j)
        if (Tab::am(row, j)) l = j;
    return l;
}
template <class Tab>
__host__ __device__ constexpr int row_terms(int row) {
    int n = 0;
    for (int j = 1; j < row; ++j)
        if (Tab::am(row, j)) ++n;
    return n;
}

struct CSum {
    float hi = 0.0f, lo = 0.0f;
    // weight given as a float pair wh + wl
    __device__ __forceinline__ void add_pair(float wh, float wl, float k) {
        float p = wh * k;
        float e = fmaf(wh, k, -p);
        e = fmaf(wl, k, e);
        float s = hi + p;
        float bb = s - hi;
        float e2 = (hi - (s - bb)) + (p - bb);
        hi = s;
        lo += e + e2;
    }
    __device__ __forceinline__ float value() const { return hi + lo; }
};

template <class Tab, class R, int C> struct RK;

template <class Tab, int C> struct RK<Tab, double, C> {
    // out = uprev + d * sum_j a(ROW, j) k_j
    template <int ROW>
    __device__ static void stage(double* out, double (*k)[C], double d, const double* up, const double*) {
        constexpr int last = row_last<Tab>(ROW);
        constexpr int nt = row_terms<Tab>(ROW);
        if (nt == 1) {
            const double a = d * Tab::a(ROW, last);
#pragma unroll
            for (int i = 0; i < C; ++i) out[i] = fma(a, k[Tab::slot(last)][i], up[i]);
            return;
        }
#pragma unroll
        for (int i = 0; i < C; ++i) {
            double acc = Tab::a(ROW, last) * k[Tab::slot(last)][i];
#pragma unroll
            for (int j = last - 1; j >= 1; --j)
                if (Tab::am(ROW, j)) acc = fma(Tab::a(ROW, j), k[Tab::slot(j)][i], acc);
            out[i] = fma(d, acc, up[i]);
        }
    }
    // S_i = sum_j w(j) k_j (reference nesting), for the solution and error weights
    template <class W>
    __device__ static void weights(double* out, double (*k)[C], W) {
        constexpr int last = W::last();
#pragma unroll
        for (int i = 0; i < C; ++i) {
            double acc = W::w(last) * k[Tab::slot(last)][i];
#pragma unroll
            for (int j = last - 1; j >= 1; --j)
                if (W::m(j)) acc = fma(W::w(j), k[Tab::slot(j)][i], acc);
            out[i] = acc;
        }
    }
};

template <class Tab>
__host__ __device__ constexpr double row_maxabs(int row) {
    double m = 0.0;
    for (int j = 1; j < row; ++j)
        if (Tab::am(row, j)) m = (Tab::a(row, j) < 0 ? -Tab::a(row, j) : Tab::a(row, j)) > m
                                     ? (Tab::a(row, j) < 0 ? -Tab::a(row, j) : Tab::a(row, j)) : m;
    return m;
}

template <class Tab, int C> struct RK<Tab, float, C> {
    // Rows whose coefficients stay below 4 in magnitude lose at most a few
    // float ulps in a plain FMA chain; only the large-coefficient rows (Vern7
    // stages 6-10, |a| up to 187) need the compensated sum.
    template <int ROW>
    __device__ static void stage(float* out, float (*k)[C], float d, const float* up, const float* uplo) {
        constexpr bool comp = row_maxabs<Tab>(ROW) > 4.0;
#pragma unroll
        for (int i = 0; i < C; ++i) {
            float S;
            if (comp) {
                CSum s;
#pragma unroll
                for (int j = 1; j < ROW; ++j)
                    if (Tab::am(ROW, j)) s.add_pair(Tab::ahi(ROW, j), Tab::alo(ROW, j), k[Tab::slot(j)][i]);
                S = s.value();
            } else {
                S = 0.0f;
#pragma unroll
                for (int j = 1; j < ROW; ++j)
                    if (Tab::am(ROW, j)) S = fmaf(Tab::ahi(ROW, j), k[Tab::slot(j)][i], S);
            }
            out[i] = fmaf(d, S, up[i]) + uplo[i];
        }
    }
    template <class W>
    __device__ static void weights(float* out, float (*k)[C], W) {
        constexpr int last = W::last();
#pragma unroll
        for (int i = 0; i < C; ++i) {
            CSum s;
#pragma unroll
            for (int j = 1; j <= last; ++j)
                if (W::m(j)) s.add_pair(W::whi(j), W::wlo(j), k[Tab::slot(j)][i]);
            out[i] = s.value();
        }
    }
};

}  // namespace odegb
)ODEGBRTC",
R"ODEGBRTC(// Generated by gen_tableaus.py from the reference's Julia tableau sources; do not edit.
// Tsit5: lib/OrdinaryDiffEqTsit5/src/tsit_tableaus.jl:45-101,244-276
// Vern7: lib/OrdinaryDiffEqVerner/src/verner_tableaus.jl:648-716,880-972,1129-1205
// Rodas5P: lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:23-72
// Rosenbrock23: lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_tableaus.jl:6-10
#pragma once
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#endif
namespace odegb {
namespace tab {
// TSIT5
constexpr double TSIT5_c1 = 0.161;
constexpr double TSIT5_c2 = 0.327;
constexpr double TSIT5_c3 = 0.9;
constexpr double TSIT5_c4 = 0.9800255409045097;
constexpr double TSIT5_c5 = 1.0;
constexpr double TSIT5_c6 = 1.0;
constexpr double TSIT5_a21 = 0.161;
constexpr double TSIT5_a31 = -0.008480655492356989;
constexpr double TSIT5_a32 = 0.335480655492357;
constexpr double TSIT5_a41 = 2.8971530571054935;
constexpr double TSIT5_a42 = -6.359448489975075;
constexpr double TSIT5_a43 = 4.3622954328695815;
constexpr double TSIT5_a51 = 5.325864828439257;
constexpr double TSIT5_a52 = -11.748883564062828;
constexpr double TSIT5_a53 = 7.4955393428898365;
constexpr double TSIT5_a54 = -0.09249506636175525;
constexpr double TSIT5_a61 = 5.86145544294642;
constexpr double TSIT5_a62 = -12.92096931784711;
constexpr double TSIT5_a63 = 8.159367898576159;
constexpr double TSIT5_a64 = -0.071584973281401;
constexpr double TSIT5_a65 = -0.028269050394068383;
constexpr double TSIT5_a71 = 0.09646076681806523;
constexpr double TSIT5_a72 = 0.01;
constexpr double TSIT5_a73 = 0.4798896504144996;
constexpr double TSIT5_a74 = 1.379008574103742;
constexpr double TSIT5_a75 = -3.290069515436081;
constexpr double TSIT5_a76 = 2.324710524099774;
constexpr double TSIT5_btilde1 = -0.00178001105222577714;
constexpr double TSIT5_btilde2 = -0.0008164344596567469;
constexpr double TSIT5_btilde3 = 0.007880878010261995;
constexpr double TSIT5_btilde4 = -0.1447110071732629;
constexpr double TSIT5_btilde5 = 0.5823571654525552;
constexpr double TSIT5_btilde6 = -0.45808210592918697;
constexpr double TSIT5_btilde7 = 0.015151515151515152;
// TSIT5I
constexpr double TSIT5I_r11 = 1.0;
constexpr double TSIT5I_r12 = -2.763706197274826;
constexpr double TSIT5I_r13 = 2.9132554618219126;
constexpr double TSIT5I_r14 = -1.0530884977290216;
constexpr double TSIT5I_r22 = 0.13169999999999998;
constexpr double TSIT5I_r23 = -0.2234;
constexpr double TSIT5I_r24 = 0.1017;
constexpr double TSIT5I_r32 = 3.9302962368947516;
constexpr double TSIT5I_r33 = -5.941033872131505;
constexpr double TSIT5I_r34 = 2.490627285651253;
constexpr double TSIT5I_r42 = -12.411077166933676;
constexpr double TSIT5I_r43 = 30.33818863028232;
constexpr double TSIT5I_r44 = -16.548102889244902;
constexpr double TSIT5I_r52 = 37.50931341651104;
constexpr double TSIT5I_r53 = -88.1789048947664;
constexpr double TSIT5I_r54 = 47.37952196281928;
constexpr double TSIT5I_r62 = -27.896526289197286;
constexpr double TSIT5I_r63 = 65.09189467479366;
constexpr double TSIT5I_r64 = -34.87065786149661;
constexpr double TSIT5I_r72 = 1.5;
constexpr double TSIT5I_r73 = -4.0;
constexpr double TSIT5I_r74 = 2.5;
// VERN7
constexpr double VERN7_c2 = 0.005;
constexpr double VERN7_c3 = 0.10888888888888888;
constexpr double VERN7_c4 = 0.16333333333333333;
constexpr double VERN7_c5 = 0.4555;
constexpr double VERN7_c6 = 0.6095094489978381;
constexpr double VERN7_c7 = 0.884;
constexpr double VERN7_c8 = 0.925;
constexpr double VERN7_a021 = 0.005;
constexpr double VERN7_a031 = -1.07679012345679;
constexpr double VERN7_a032 = 1.185679012345679;
constexpr double VERN7_a041 = 0.04083333333333333;
constexpr double VERN7_a043 = 0.1225;
constexpr double VERN7_a051 = 0.6389139236255726;
constexpr double VERN7_a053 = -2.455672638223657;
constexpr double VERN7_a054 = 2.272258714598084;
constexpr double VERN7_a061 = -2.6615773750187572;
constexpr double VERN7_a063 = 10.804513886456137;
constexpr double VERN7_a064 = -8.3539146573962;
constexpr double VERN7_a065 = 0.820487594956657;
constexpr double VERN7_a071 = 6.067741434696772;
constexpr double VERN7_a073 = -24.711273635911088;
constexpr double VERN7_a074 = 20.427517930788895;
constexpr double VERN7_a075 = -1.9061579788166472;
constexpr double VERN7_a076 = 1.006172249242068;
constexpr double VERN7_a081 = 12.054670076253203;
constexpr double VERN7_a083 = -49.75478495046899;
constexpr double VERN7_a084 = 41.142888638604674;
constexpr double VERN7_a085 = -4.461760149974004;
constexpr double VERN7_a086 = 2.042334822239175;
constexpr double VERN7_a087 = -0.09834843665406107;
constexpr double VERN7_a091 = 10.138146522881808;
constexpr double VERN7_a093 = -42.6411360317175;
constexpr double VERN7_a094 = 35.76384003992257;
constexpr double VERN7_a095 = -4.3480228403929075;
constexpr double VERN7_a096 = 2.0098622683770357;
constexpr double VERN7_a097 = 0.3487490460338272;
constexpr double VERN7_a098 = -0.27143900510483127;
constexpr double VERN7_a101 = -45.030072034298676;
constexpr double VERN7_a103 = 187.3272437654589;
constexpr double VERN7_a104 = -154.02882369350186;
constexpr double VERN7_a105 = 18.56465306347536;
constexpr double VERN7_a106 = -7.141809679295079;
constexpr double VERN7_a107 = 1.3088085781613787;
constexpr double VERN7_b1 = 0.04715561848627222;
constexpr double VERN7_b4 = 0.25750564298434153;
constexpr double VERN7_b5 = 0.26216653977412624;
constexpr double VERN7_b6 = 0.15216092656738558;
constexpr double VERN7_b7 = 0.4939969170032485;
constexpr double VERN7_b8 = -0.29430311714032503;
constexpr double VERN7_b9 = 0.08131747232495111;
constexpr double VERN7_btilde1 = 0.002547011879931045;
constexpr double VERN7_btilde4 = -0.00965839487279575;
constexpr double VERN7_btilde5 = 0.04206470975639691;
constexpr double VERN7_btilde6 = -0.0666822437469301;
constexpr double VERN7_btilde7 = 0.2650097464621281;
constexpr double VERN7_btilde8 = -0.29430311714032503;
constexpr double VERN7_btilde9 = 0.08131747232495111;
constexpr double VERN7_btilde10 = -0.02029518466335628;
// VERN7X
constexpr double VERN7X_c11 = 1.0;
constexpr double VERN7X_a1101 = 0.04715561848627222;
constexpr double VERN7X_a1104 = 0.25750564298434153;
constexpr double VERN7X_a1105 = 0.2621665397741262;
constexpr double VERN7X_a1106 = 0.15216092656738558;
constexpr double VERN7X_a1107 = 0.49399691700324844;
constexpr double VERN7X_a1108 = -0.29430311714032503;
constexpr double VERN7X_a1109 = 0.0813174723249511;
constexpr double VERN7X_c12 = 0.29;
constexpr double VERN7X_a1201 = 0.0523222769159969;
constexpr double VERN7X_a1204 = 0.22495861826705715;
constexpr double VERN7X_a1205 = 0.017443709248776376;
constexpr double VERN7X_a1206 = -0.007669379876829393;
constexpr double VERN7X_a1207 = 0.03435896044073285;
constexpr double VERN7X_a1208 = -0.0410209723009395;
constexpr double VERN7X_a1209 = 0.025651133005205617;
constexpr double VERN7X_a1211 = -0.0160443457;
constexpr double VERN7X_c13 = 0.125;
constexpr double VERN7X_a1301 = 0.053053341257859085;
constexpr double VERN7X_a1304 = 0.12195301011401886;
constexpr double VERN7X_a1305 = 0.017746840737602496;
constexpr double VERN7X_a1306 = -0.0005928372667681495;
constexpr double VERN7X_a1307 = 0.008381833970853752;
constexpr double VERN7X_a1308 = -0.01293369259698612;
constexpr double VERN7X_a1309 = 0.009412056815253861;
constexpr double VERN7X_a1311 = -0.005353253107275676;
constexpr double VERN7X_a1312 = -0.06666729992455811;
constexpr double VERN7X_c14 = 0.25;
constexpr double VERN7X_a1401 = 0.03887903257436304;
constexpr double VERN7X_a1404 = -0.0024403203308301317;
constexpr double VERN7X_a1405 = -0.0013928917214672623;
constexpr double VERN7X_a1406 = -0.00047446291558680135;
constexpr double VERN7X_a1407 = 0.00039207932413159514;
constexpr double VERN7X_a1408 = -0.00040554733285128004;
constexpr double VERN7X_a1409 = 0.00019897093147716726;
constexpr double VERN7X_a1411 = -0.00010278198793179169;
constexpr double VERN7X_a1412 = 0.03385661513870267;
constexpr double VERN7X_a1413 = 0.1814893063199928;
constexpr double VERN7X_c15 = 0.53;
constexpr double VERN7X_a1501 = 0.05723681204690013;
constexpr double VERN7X_a1504 = 0.22265948066761182;
constexpr double VERN7X_a1505 = 0.12344864200186899;
constexpr double VERN7X_a1506 = 0.04006332526666491;
constexpr double VERN7X_a1507 = -0.05269894848581452;
constexpr double VERN7X_a1508 = 0.04765971214244523;
constexpr double VERN7X_a1509 = -0.02138895885042213;
constexpr double VERN7X_a1511 = 0.015193891064036402;
constexpr double VERN7X_a1512 = 0.12060546716289655;
constexpr double VERN7X_a1513 = -0.022779423016187374;
constexpr double VERN7X_c16 = 0.79;
constexpr double VERN7X_a1601 = 0.051372038802756814;
constexpr double VERN7X_a1604 = 0.5414214473439406;
constexpr double VERN7X_a1605 = 0.350399806692184;
constexpr double VERN7X_a1606 = 0.14193112269692182;
constexpr double VERN7X_a1607 = 0.10527377478429423;
constexpr double VERN7X_a1608 = -0.031081847805874016;
constexpr double VERN7X_a1609 = -0.007401883149519145;
constexpr double VERN7X_a1611 = -0.006377932504865363;
constexpr double VERN7X_a1612 = -0.17325495908361865;
constexpr double VERN7X_a1613 = -0.18228156777622026;
// VERN7I
constexpr double VERN7I_r011 = 1.0;
constexpr double VERN7I_r012 = -8.413387198332767;
constexpr double VERN7I_r013 = 33.675508884490895;
constexpr double VERN7I_r014 = -70.80159089484886;
constexpr double VERN7I_r015 = 80.64695108301298;
constexpr double VERN7I_r016 = -47.19413969837522;
constexpr double VERN7I_r017 = 11.133813442539243;
constexpr double VERN7I_r042 = 8.754921980674396;
constexpr double VERN7I_r043 = -88.4596828699771;
constexpr double VERN7I_r044 = 346.9017638429916;
constexpr double VERN7I_r045 = -629.2580030059837;
constexpr double VERN7I_r046 = 529.6773755604193;
constexpr double VERN7I_r047 = -167.35886986514018;
constexpr double VERN7I_r052 = 8.913387586637922;
constexpr double VERN7I_r053 = -90.06081846893218;
constexpr double VERN7I_r054 = 353.1807459217058;
constexpr double VERN7I_r055 = -640.6476819744374;
constexpr double VERN7I_r056 = 539.2646279047156;
constexpr double VERN7I_r057 = -170.38809442991547;
constexpr double VERN7I_r062 = 5.1733120298478;
constexpr double VERN7I_r063 = -52.271115900055385;
constexpr double VERN7I_r064 = 204.9853867374073;
constexpr double VERN7I_r065 = -371.8306118563603;
constexpr double VERN7I_r066 = 312.9880934374529;
constexpr double VERN7I_r067 = -98.89290352172495;
constexpr double VERN7I_r072 = 16.79537744079696;
constexpr double VERN7I_r073 = -169.70040000059728;
constexpr double VERN7I_r074 = 665.4937727009246;
constexpr double VERN7I_r075 = -1207.1638892336007;
constexpr double VERN7I_r076 = 1016.1291515818546;
constexpr double VERN7I_r077 = -321.06001557237494;
constexpr double VERN7I_r082 = -10.005997536098665;
constexpr double VERN7I_r083 = 101.1005433052275;
constexpr double VERN7I_r084 = -396.47391512378437;
constexpr double VERN7I_r085 = 719.1787707014183;
constexpr double VERN7I_r086 = -605.3681033918824;
constexpr double VERN7I_r087 = 191.27439892797935;
constexpr double VERN7I_r092 = 2.764708833638599;
constexpr double VERN7I_r093 = -27.934602637390462;
constexpr double VERN7I_r094 = 109.54779186137893;
constexpr double VERN7I_r095 = -198.7128113064482;
constexpr double VERN7I_r096 = 167.26633571640318;
constexpr double VERN7I_r097 = -52.85010499525706;
constexpr double VERN7I_r112 = -2.1696320280163506;
constexpr double VERN7I_r113 = 22.016696037569876;
constexpr double VERN7I_r114 = -86.90152427798948;
constexpr double VERN7I_r115 = 159.22388973861476;
constexpr double VERN7I_r116 = -135.9618306534588;
constexpr double VERN7I_r117 = 43.792401183280006;
constexpr double VERN7I_r122 = -4.890070188793804;
constexpr double VERN7I_r123 = 22.75407737425176;
constexpr double VERN7I_r124 = -30.78034218537731;
constexpr double VERN7I_r125 = -2.797194317207249;
constexpr double VERN7I_r126 = 31.369456637508403;
constexpr double VERN7I_r127 = -15.655927320381801;
constexpr double VERN7I_r132 = 10.862170929551967;
constexpr double VERN7I_r133 = -50.542971417827104;
constexpr double VERN7I_r134 = 68.37148040407511;
constexpr double VERN7I_r135 = 6.213326521632409;
constexpr double VERN7I_r136 = -69.68006323194157;
constexpr double VERN7I_r137 = 34.776056794509195;
constexpr double VERN7I_r142 = -11.37286691922923;
constexpr double VERN7I_r143 = 130.79058078246717;
constexpr double VERN7I_r144 = -488.65113677785604;
constexpr double VERN7I_r145 = 832.2148793276441;
constexpr double VERN7I_r146 = -664.7743368554426;
constexpr double VERN7I_r147 = 201.79288044241662;
constexpr double VERN7I_r152 = -5.919778732715007;
constexpr double VERN7I_r153 = 63.27679965889219;
constexpr double VERN7I_r154 = -265.432682088738;
constexpr double VERN7I_r155 = 520.1009254140611;
constexpr double VERN7I_r156 = -467.412109533902;
constexpr double VERN7I_r157 = 155.3868452824017;
constexpr double VERN7I_r162 = -10.492146197961823;
constexpr double VERN7I_r163 = 105.35538525188011;
constexpr double VERN7I_r164 = -409.43975011988937;
constexpr double VERN7I_r165 = 732.831448907654;
constexpr double VERN7I_r166 = -606.3044574733512;
constexpr double VERN7I_r167 = 188.0495196316683;
// RODAS5P (8 stages): A lower triangular 8x8, C 8x7, c 8, d 8, H 3x8.
// Accessors are constexpr functions so device code folds them to immediates.
constexpr double RODAS5P_GAMMA = 0.21193756319429014;
__host__ __device__ constexpr double RODAS5P_A(int i, int j) {
    constexpr double t[8][8] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {3.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {2.849394379747939, 0.45842242204463923, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {-6.954028509809101, 2.489845061869568, -10.358996098473584, 0.0, 0.0, 0.0, 0.0, 0.0}, {2.8029986275628964, 0.5072464736228206, -0.3988312541770524, -0.04721187230404641, 0.0, 0.0, 0.0, 0.0}, {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946, 0.0, 0.0, 0.0}, {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946, 1.0, 0.0, 0.0}, {-7.502846399306121, 2.561846144803919, -11.627539656261098, -0.18268767659942256, 0.030198172008377946, 1.0, 1.0, 0.0}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_A_HI(int i, int j) {
    constexpr float t[8][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.8000000000000p+1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.6cb8f40000000p+1f, 0x1.d56cb00000000p-2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.bd0ece0000000p+2f, 0x1.3eb33e0000000p+1f, -0x1.4b7ce60000000p+3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.66c8a80000000p+1f, 0x1.03b5d00000000p-1f, -0x1.9867380000000p-2f, -0x1.82c2780000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.e02ea20000000p+2f, 0x1.47ea940000000p+1f, -0x1.7414ce0000000p+3f, -0x1.7624f40000000p-3f, 0x1.eec4500000000p-6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.e02ea20000000p+2f, 0x1.47ea940000000p+1f, -0x1.7414ce0000000p+3f, -0x1.7624f40000000p-3f, 0x1.eec4500000000p-6f, 0x1.0000000000000p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.e02ea20000000p+2f, 0x1.47ea940000000p+1f, -0x1.7414ce0000000p+3f, -0x1.7624f40000000p-3f, 0x1.eec4500000000p-6f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_A_LO(int i, int j) {
    constexpr float t[8][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.f4d8e20000000p-25f, -0x1.90aea80000000p-32f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.9eeb160000000p-24f, 0x1.a358fa0000000p-26f, 0x1.3a6a840000000p-22f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.6c1d940000000p-24f, -0x1.631d580000000p-26f, -0x1.9502780000000p-28f, -0x1.e1d7fc0000000p-30f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.53f7300000000p-23f, -0x1.deaef80000000p-24f, -0x1.7256860000000p-26f, -0x1.c607260000000p-28f, 0x1.2cca900000000p-32f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.53f7300000000p-23f, -0x1.deaef80000000p-24f, -0x1.7256860000000p-26f, -0x1.c607260000000p-28f, 0x1.2cca900000000p-32f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.53f7300000000p-23f, -0x1.deaef80000000p-24f, -0x1.7256860000000p-26f, -0x1.c607260000000p-28f, 0x1.2cca900000000p-32f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr double RODAS5P_C(int i, int j) {
    constexpr double t[8][7] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {-14.155112264123755, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {-17.97296035885952, -2.859693295451294, 0.0, 0.0, 0.0, 0.0, 0.0}, {147.12150275711716, -1.41221402718213, 71.68940251302358, 0.0, 0.0, 0.0, 0.0}, {165.43517024871676, -0.4592823456491126, 42.90938336958603, -5.961986721573306, 0.0, 0.0, 0.0}, {24.854864614690072, -3.0009227002832186, 47.4931110020768, 5.5814197821558125, -0.6610691825249471, 0.0, 0.0}, {30.91273214028599, -3.1208243349937974, 77.79954646070892, 34.28646028294783, -19.097331116725623, -28.087943162872662, 0.0}, {37.80277123390563, -3.2571969029072276, 112.26918849496327, 66.9347231244047, -40.06618937091002, -54.66780262877968, -9.48861652309627}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_C_HI(int i, int j) {
    constexpr float t[8][7] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.c4f6ae0000000p+3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.1f913e0000000p+4f, -0x1.6e0a6e0000000p+1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.263e360000000p+7f, -0x1.6986dc0000000p+0f, 0x1.1ec1f20000000p+6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.4adece0000000p+7f, -0x1.d64e1c0000000p-2f, 0x1.57466a0000000p+5f, -0x1.7d91300000000p+2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.8dad860000000p+4f, -0x1.801e3c0000000p+1f, 0x1.7bf1e40000000p+5f, 0x1.6535fc0000000p+2f, -0x1.5277a80000000p-1f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.ee9a8e0000000p+4f, -0x1.8f772c0000000p+1f, 0x1.3732bc0000000p+6f, 0x1.124aac0000000p+5f, -0x1.318eac0000000p+4f, -0x1.c168380000000p+4f, 0x0.0p+0f}, {0x1.2e6c140000000p+5f, -0x1.a0ebd40000000p+1f, 0x1.c113a60000000p+6f, 0x1.0bbd280000000p+6f, -0x1.40878e0000000p+5f, -0x1.b557a80000000p+5f, -0x1.2fa2c00000000p+3f}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_C_LO(int i, int j) {
    constexpr float t[8][7] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.4c28a00000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.c333640000000p-21f, -0x1.c8dc420000000p-28f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.8ffe760000000p-19f, 0x1.d267020000000p-27f, 0x1.76f9bc0000000p-19f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.4509b80000000p-18f, -0x1.e316f60000000p-28f, 0x1.937e600000000p-20f, -0x1.822bfc0000000p-23f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x1.0953400000000p-21f, -0x1.5e29680000000p-26f, 0x1.72cdee0000000p-22f, -0x1.5d32580000000p-23f, -0x1.dd5a380000000p-26f, 0x0.0p+0f, 0x0.0p+0f}, {-0x1.f76ed60000000p-21f, 0x1.14808c0000000p-29f, 0x1.3ac60a0000000p-20f, -0x1.3ea45c0000000p-21f, 0x1.da98f80000000p-21f, 0x1.d1f1c40000000p-21f, 0x0.0p+0f}, {-0x1.59c34a0000000p-20f, 0x1.6187400000000p-32f, 0x1.30ca740000000p-21f, 0x1.e1110a0000000p-23f, -0x1.2becd80000000p-21f, -0x1.cf2caa0000000p-20f, 0x1.c3410a0000000p-22f}};
    return t[i][j];
}
__host__ __device__ constexpr double RODAS5P_c(int i) {
    constexpr double t[8] = {0.0, 0.6358126895828704, 0.4095798393397535, 0.9769306725060716, 0.4288403609558664, 1.0, 1.0, 1.0};
    return t[i];
}
__host__ __device__ constexpr float RODAS5P_c_HI(int i) {
    constexpr float t[8] = {0x0.0p+0f, 0x1.45893e0000000p-1f, 0x1.a368e60000000p-2f, 0x1.f430420000000p-1f, 0x1.b721ee0000000p-2f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f};
    return t[i];
}
__host__ __device__ constexpr float RODAS5P_c_LO(int i) {
    constexpr float t[8] = {0x0.0p+0f, -0x1.5ee0d00000000p-27f, -0x1.0ef50a0000000p-28f, -0x1.7208c00000000p-28f, -0x1.13eaf20000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr double RODAS5P_d(int i) {
    constexpr double t[8] = {0.21193756319429014, -0.42387512638858027, -0.3384627126235924, 1.8046452872882734, 2.325825639765069, 0.0, 0.0, 0.0};
    return t[i];
}
__host__ __device__ constexpr float RODAS5P_d_HI(int i) {
    constexpr float t[8] = {0x1.b20c520000000p-3f, -0x1.b20c520000000p-2f, -0x1.5a95f80000000p-2f, 0x1.cdfd3c0000000p+0f, 0x1.29b4a80000000p+1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr float RODAS5P_d_LO(int i) {
    constexpr float t[8] = {0x1.ada8800000000p-30f, -0x1.ada8800000000p-29f, -0x1.3447e40000000p-29f, -0x1.b1bb100000000p-27f, -0x1.ba05820000000p-25f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr double RODAS5P_H(int i, int j) {
    constexpr double t[3][8] = {{25.948786856663858, -2.5579724845846235, 10.433815404888879, -2.3679251022685204, 0.524948541321073, 1.1241088310450404, 0.4272876194431874, -0.17202221070155493}, {-9.91568850695171, -0.9689944594115154, 3.0438037242978453, -24.495224566215796, 20.176138334709044, 15.98066361424651, -6.789040303419874, -6.710236069923372}, {11.419903575922262, 2.8879645146136994, 72.92137995996029, 80.12511834622643, -52.072871366152654, -59.78993625266729, -0.15582684282751913, 4.883087185713722}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_H_HI(int i, int j) {
    constexpr float t[3][8] = {{0x1.9f2e3c0000000p+4f, -0x1.476ba40000000p+1f, 0x1.4de1d00000000p+3f, -0x1.2f182c0000000p+1f, 0x1.0cc60e0000000p-1f, 0x1.1fc5980000000p+0f, 0x1.b58ae20000000p-2f, -0x1.604d2e0000000p-3f}, {-0x1.3d4d520000000p+3f, -0x1.f0200a0000000p-1f, 0x1.859b5c0000000p+1f, -0x1.87ec700000000p+4f, 0x1.42d1760000000p+4f, 0x1.ff61980000000p+3f, -0x1.b27fa20000000p+2f, -0x1.ad74820000000p+2f}, {0x1.6d6fda0000000p+3f, 0x1.71a8d20000000p+1f, 0x1.23af7e0000000p+6f, 0x1.4080200000000p+6f, -0x1.a0953e0000000p+5f, -0x1.de51ca0000000p+5f, -0x1.3f22240000000p-3f, 0x1.3884800000000p+2f}};
    return t[i][j];
}
__host__ __device__ constexpr float RODAS5P_H_LO(int i, int j) {
    constexpr float t[3][8] = {{-0x1.bef8220000000p-21f, -0x1.cab7b80000000p-25f, 0x1.b01fec0000000p-22f, 0x1.1661160000000p-24f, 0x1.10e91e0000000p-28f, 0x1.54f76c0000000p-25f, 0x1.7bf4160000000p-27f, -0x1.24c2f80000000p-29f}, {0x1.0a8e000000000p-27f, -0x1.64b5ec0000000p-26f, 0x1.169ac00000000p-25f, -0x1.3082540000000p-21f, 0x1.b8c96c0000000p-22f, 0x1.51e4380000000p-22f, -0x1.cd35080000000p-23f, 0x1.67aa600000000p-29f}, {-0x1.80f8600000000p-23f, 0x1.d918f00000000p-26f, 0x1.d367040000000p-21f, -0x1.f3d6a00000000p-19f, 0x1.ab31e80000000p-21f, -0x1.9190be0000000p-23f, -0x1.9c87b00000000p-28f, 0x1.d8a0e40000000p-26f}};
    return t[i][j];
}
__host__ __device__ constexpr double TSIT5_A(int i, int j) {
    constexpr double t[8][8] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.161, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -0.008480655492356989, 0.335480655492357, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 2.8971530571054935, -6.359448489975075, 4.3622954328695815, 0.0, 0.0, 0.0, 0.0}, {0.0, 5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0.0, 0.0, 0.0}, {0.0, 5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0.0, 0.0}, {0.0, 0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774, 0.0}};
    return t[i][j];
}
__host__ __device__ constexpr float TSIT5_A_HI(int i, int j) {
    constexpr float t[8][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.49ba5e0000000p-3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.15e4e40000000p-7f, 0x1.57883e0000000p-2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.72d5ea0000000p+1f, -0x1.9701340000000p+2f, 0x1.172fda0000000p+2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.54daf80000000p+2f, -0x1.77f6da0000000p+3f, 0x1.dfb6ea0000000p+2f, -0x1.7adc1c0000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.7722160000000p+2f, -0x1.9d78940000000p+3f, 0x1.05198a0000000p+3f, -0x1.2536480000000p-4f, -0x1.cf28fe0000000p-6f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.8b1a720000000p-4f, 0x1.47ae140000000p-7f, 0x1.eb68320000000p-2f, 0x1.6106b40000000p+0f, -0x1.a521000000000p+1f, 0x1.29901e0000000p+1f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr float TSIT5_A_LO(int i, int j) {
    constexpr float t[8][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.a9fbe80000000p-30f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.fd02480000000p-32f, -0x1.4383d40000000p-28f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.6039ba0000000p-24f, -0x1.ea143e0000000p-25f, -0x1.a22ae00000000p-23f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.3a20640000000p-25f, -0x1.540a5a0000000p-22f, 0x1.4bcbee0000000p-23f, 0x1.5deacc0000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.4d50700000000p-29f, -0x1.4b31740000000p-22f, 0x1.6a1aae0000000p-22f, -0x1.e41de80000000p-29f, 0x1.11893e0000000p-32f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.2b59120000000p-32f, 0x1.eb851e0000000p-33f, -0x1.6e3f300000000p-27f, 0x1.6d5bbc0000000p-25f, 0x1.15a2ae0000000p-24f, -0x1.6653100000000p-24f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr bool TSIT5_AM(int i, int j) {
    constexpr bool t[8][8] = {{false, false, false, false, false, false, false, false}, {false, false, false, false, false, false, false, false}, {false, true, false, false, false, false, false, false}, {false, true, true, false, false, false, false, false}, {false, true, true, true, false, false, false, false}, {false, true, true, true, true, false, false, false}, {false, true, true, true, true, true, false, false}, {false, true, true, true, true, true, true, false}};
    return t[i][j];
}
__host__ __device__ constexpr double TSIT5_CS(int i) {
    constexpr double t[8] = {0.0, 0.0, 0.161, 0.327, 0.9, 0.9800255409045097, 1.0, 1.0};
    return t[i];
}
__host__ __device__ constexpr float TSIT5_CS_HI(int i) {
    constexpr float t[8] = {0x0.0p+0f, 0x0.0p+0f, 0x1.49ba5e0000000p-3f, 0x1.4ed9160000000p-2f, 0x1.cccccc0000000p-1f, 0x1.f5c5e80000000p-1f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f};
    return t[i];
}
__host__ __device__ constexpr float TSIT5_CS_LO(int i) {
    constexpr float t[8] = {0x0.0p+0f, 0x0.0p+0f, 0x1.a9fbe80000000p-30f, 0x1.0e56040000000p-27f, 0x1.99999a0000000p-26f, 0x1.7b6fc80000000p-27f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr double TSIT5_BT(int i) {
    constexpr double t[8] = {0.0, -0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995, -0.1447110071732629, 0.5823571654525552, -0.45808210592918697, 0.015151515151515152};
    return t[i];
}
__host__ __device__ constexpr float TSIT5_BT_HI(int i) {
    constexpr float t[8] = {0x0.0p+0f, -0x1.d29e860000000p-10f, -0x1.ac0bfa0000000p-11f, 0x1.023d980000000p-7f, -0x1.285e3e0000000p-3f, 0x1.2a2ab80000000p-1f, -0x1.d5137a0000000p-2f, 0x1.f07c200000000p-7f};
    return t[i];
}
__host__ __device__ constexpr float TSIT5_BT_LO(int i) {
    constexpr float t[8] = {0x0.0p+0f, 0x1.f410500000000p-35f, -0x1.b6b51e0000000p-37f, 0x1.515e040000000p-32f, -0x1.32e2dc0000000p-28f, -0x1.7947cc0000000p-29f, 0x1.026bde0000000p-28f, -0x1.f07c200000000p-32f};
    return t[i];
}
__host__ __device__ constexpr double TSIT5_R(int i, int j) {
    constexpr double t[8][5] = {{0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 1.0, -2.763706197274826, 2.9132554618219126, -1.0530884977290216}, {0.0, 0.0, 0.13169999999999998, -0.2234, 0.1017}, {0.0, 0.0, 3.9302962368947516, -5.941033872131505, 2.490627285651253}, {0.0, 0.0, -12.411077166933676, 30.33818863028232, -16.548102889244902}, {0.0, 0.0, 37.50931341651104, -88.1789048947664, 47.37952196281928}, {0.0, 0.0, -27.896526289197286, 65.09189467479366, -34.87065786149661}, {0.0, 0.0, 1.5, -4.0, 2.5}};
    return t[i][j];
}
__host__ __device__ constexpr float TSIT5_R_HI(int i, int j) {
    constexpr float t[8][5] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.0000000000000p+0f, -0x1.61c1200000000p+1f, 0x1.74e58e0000000p+1f, -0x1.0d97360000000p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.0db8ba0000000p-3f, -0x1.c985f00000000p-3f, 0x1.a0902e0000000p-4f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.f713f20000000p+1f, -0x1.7c39e60000000p+2f, 0x1.3ecce00000000p+1f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.8d278c0000000p+3f, 0x1.e569380000000p+4f, -0x1.08c5080000000p+4f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.2c13120000000p+5f, -0x1.60b7320000000p+6f, 0x1.7b09420000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.be582c0000000p+4f, 0x1.045e1a0000000p+6f, -0x1.16f71c0000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.8000000000000p+0f, -0x1.0000000000000p+2f, 0x1.4000000000000p+1f}};
    return t[i][j];
}
__host__ __device__ constexpr float TSIT5_R_LO(int i, int j) {
    constexpr float t[8][5] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.579de60000000p-27f, 0x1.2b59120000000p-27f, 0x1.9ceb900000000p-25f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.8e21960000000p-28f, -0x1.bda5120000000p-29f, -0x1.ff2e480000000p-32f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.d21c120000000p-25f, -0x1.1277540000000p-25f, -0x1.b348a80000000p-29f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.64f8ce0000000p-22f, 0x1.ecbc440000000p-22f, 0x1.dbf6680000000p-22f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.d335440000000p-20f, -0x1.b080ee0000000p-19f, 0x1.9f26c20000000p-20f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.97c96e0000000p-25f, -0x1.73115a0000000p-20f, 0x1.0fedde0000000p-20f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr double VERN7_A(int i, int j) {
    constexpr double t[17][17] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.005, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -1.07679012345679, 1.185679012345679, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.04083333333333333, 0.0, 0.1225, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.6389139236255726, 0.0, -2.455672638223657, 2.272258714598084, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -2.6615773750187572, 0.0, 10.804513886456137, -8.3539146573962, 0.820487594956657, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 6.067741434696772, 0.0, -24.711273635911088, 20.427517930788895, -1.9061579788166472, 1.006172249242068, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 12.054670076253203, 0.0, -49.75478495046899, 41.142888638604674, -4.461760149974004, 2.042334822239175, -0.09834843665406107, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 10.138146522881808, 0.0, -42.6411360317175, 35.76384003992257, -4.3480228403929075, 2.0098622683770357, 0.3487490460338272, -0.27143900510483127, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, -45.030072034298676, 0.0, 187.3272437654589, -154.02882369350186, 18.56465306347536, -7.141809679295079, 1.3088085781613787, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.04715561848627222, 0.0, 0.0, 0.25750564298434153, 0.2621665397741262, 0.15216092656738558, 0.49399691700324844, -0.29430311714032503, 0.0813174723249511, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0523222769159969, 0.0, 0.0, 0.22495861826705715, 0.017443709248776376, -0.007669379876829393, 0.03435896044073285, -0.0410209723009395, 0.025651133005205617, 0.0, -0.0160443457, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.053053341257859085, 0.0, 0.0, 0.12195301011401886, 0.017746840737602496, -0.0005928372667681495, 0.008381833970853752, -0.01293369259698612, 0.009412056815253861, 0.0, -0.005353253107275676, -0.06666729992455811, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.03887903257436304, 0.0, 0.0, -0.0024403203308301317, -0.0013928917214672623, -0.00047446291558680135, 0.00039207932413159514, -0.00040554733285128004, 0.00019897093147716726, 0.0, -0.00010278198793179169, 0.03385661513870267, 0.1814893063199928, 0.0, 0.0, 0.0}, {0.0, 0.05723681204690013, 0.0, 0.0, 0.22265948066761182, 0.12344864200186899, 0.04006332526666491, -0.05269894848581452, 0.04765971214244523, -0.02138895885042213, 0.0, 0.015193891064036402, 0.12060546716289655, -0.022779423016187374, 0.0, 0.0, 0.0}, {0.0, 0.051372038802756814, 0.0, 0.0, 0.5414214473439406, 0.350399806692184, 0.14193112269692182, 0.10527377478429423, -0.031081847805874016, -0.007401883149519145, 0.0, -0.006377932504865363, -0.17325495908361865, -0.18228156777622026, 0.0, 0.0, 0.0}};
    return t[i][j];
}
__host__ __device__ constexpr float VERN7_A_HI(int i, int j) {
    constexpr float t[17][17] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.47ae140000000p-8f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.13a8840000000p+0f, 0x1.2f88a80000000p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.4e81b40000000p-5f, 0x0.0p+0f, 0x1.f5c2900000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.471fba0000000p-1f, 0x0.0p+0f, -0x1.3a537c0000000p+1f, 0x1.22d9600000000p+1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.54ae920000000p+1f, 0x0.0p+0f, 0x1.59be940000000p+3f, -0x1.0b53440000000p+3f, 0x1.a416f40000000p-1f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.8455e00000000p+2f, 0x0.0p+0f, -0x1.8b61600000000p+4f, 0x1.46d71e0000000p+4f, -0x1.e7f9f80000000p+0f, 0x1.0194820000000p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.81bfdc0000000p+3f, 0x0.0p+0f, -0x1.8e09cc0000000p+5f, 0x1.4924a20000000p+5f, -0x1.1d8d7a0000000p+2f, 0x1.056b3a0000000p+1f, -0x1.92d5d00000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.446bb20000000p+3f, 0x0.0p+0f, -0x1.55210c0000000p+5f, 0x1.1e1c580000000p+5f, -0x1.1646020000000p+2f, 0x1.01432a0000000p+1f, 0x1.651e780000000p-2f, -0x1.15f41c0000000p-2f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.683d960000000p+5f, 0x0.0p+0f, 0x1.76a78c0000000p+7f, -0x1.340ec20000000p+7f, 0x1.2908d20000000p+4f, -0x1.c913680000000p+2f, 0x1.4f0e140000000p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.824c800000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.07af900000000p-2f, 0x1.0c75620000000p-2f, 0x1.37a0260000000p-3f, 0x1.f9da540000000p-2f, -0x1.2d5dcc0000000p-2f, 0x1.4d138c0000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.ac9fc40000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.ccb71a0000000p-3f, 0x1.1dcc380000000p-6f, -0x1.f69ed80000000p-8f, 0x1.1977f60000000p-5f, -0x1.500b360000000p-5f, 0x1.a444a60000000p-6f, 0x0.0p+0f, -0x1.06dede0000000p-6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.b29cec0000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.f385000000000p-4f, 0x1.22c3a60000000p-6f, -0x1.36d1460000000p-11f, 0x1.12a7ec0000000p-7f, -0x1.a7cfae0000000p-7f, 0x1.346a0e0000000p-7f, 0x0.0p+0f, -0x1.5ed4b00000000p-8f, -0x1.1111bc0000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.3e7f3e0000000p-5f, 0x0.0p+0f, 0x0.0p+0f, -0x1.3fdb900000000p-9f, -0x1.6d23620000000p-10f, -0x1.f182ac0000000p-12f, 0x1.9b1ffe0000000p-12f, -0x1.a93f480000000p-12f, 0x1.a145b40000000p-13f, 0x0.0p+0f, -0x1.af19520000000p-14f, 0x1.155a780000000p-5f, 0x1.73b0aa0000000p-3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.d4e24c0000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.c801b20000000p-3f, 0x1.f9a5480000000p-4f, 0x1.4832e20000000p-5f, -0x1.afb5b40000000p-5f, 0x1.866daa0000000p-5f, -0x1.5e6fcc0000000p-6f, 0x0.0p+0f, 0x1.f1df980000000p-7f, 0x1.ee00000000000p-4f, -0x1.7537d40000000p-6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.a4d6fa0000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.1535320000000p-1f, 0x1.66cf340000000p-2f, 0x1.22acc80000000p-3f, 0x1.af338e0000000p-4f, -0x1.fd3eb80000000p-6f, -0x1.e516fe0000000p-8f, 0x0.0p+0f, -0x1.a1fbf40000000p-8f, -0x1.62d37e0000000p-3f, -0x1.75500a0000000p-3f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr float VERN7_A_LO(int i, int j) {
    constexpr float t[17][17] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.eb851e0000000p-34f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.f39c620000000p-26f, 0x1.cb28140000000p-25f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.d0369c0000000p-30f, 0x0.0p+0f, -0x1.47ae140000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.911b220000000p-28f, 0x0.0p+0f, 0x1.b925b80000000p-24f, -0x1.79801e0000000p-25f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.7a855a0000000p-24f, 0x0.0p+0f, -0x1.80fc700000000p-25f, -0x1.a9c5de0000000p-22f, -0x1.938cc40000000p-26f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.5d36a80000000p-25f, 0x0.0p+0f, -0x1.db2fb00000000p-22f, -0x1.ea99dc0000000p-21f, -0x1.2037380000000p-27f, -0x1.aeb9a20000000p-25f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.149b0c0000000p-22f, 0x0.0p+0f, -0x1.625c700000000p-20f, 0x1.98dc6e0000000p-20f, -0x1.c6bc020000000p-24f, 0x1.d3ff360000000p-26f, 0x1.1ea8980000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.06eab00000000p-23f, 0x0.0p+0f, 0x1.27be380000000p-23f, 0x1.55b5f00000000p-22f, 0x1.a2405e0000000p-24f, 0x1.6824cc0000000p-24f, 0x1.339fb00000000p-28f, 0x1.71ba500000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.a07ac80000000p-21f, 0x0.0p+0f, 0x1.fab3ba0000000p-19f, 0x1.5587a00000000p-23f, -0x1.65b2600000000p-22f, -0x1.cf6a100000000p-23f, 0x1.bf6b480000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.8ebfe40000000p-33f, 0x0.0p+0f, 0x0.0p+0f, -0x1.a6c6400000000p-27f, 0x1.537b9c0000000p-27f, -0x1.2a7f540000000p-30f, -0x1.495bb20000000p-30f, 0x1.18afb20000000p-29f, 0x1.8754600000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.0d36ae0000000p-30f, 0x0.0p+0f, 0x0.0p+0f, 0x1.4690d40000000p-28f, 0x1.7d25920000000p-33f, 0x1.fcc22e0000000p-35f, 0x1.b570d00000000p-31f, -0x1.9ee3da0000000p-30f, 0x1.5cda300000000p-32f, 0x0.0p+0f, 0x1.f765640000000p-31f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.2d4ed00000000p-31f, 0x0.0p+0f, 0x0.0p+0f, -0x1.e95a240000000p-32f, -0x1.b65bce0000000p-31f, 0x1.3cf39e0000000p-36f, -0x1.36f55a0000000p-32f, 0x1.47888c0000000p-32f, 0x1.ad479c0000000p-35f, 0x0.0p+0f, 0x1.f43eaa0000000p-33f, 0x1.e390960000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.4be72a0000000p-31f, 0x0.0p+0f, 0x0.0p+0f, -0x1.9f79d00000000p-39f, 0x1.c038960000000p-36f, 0x1.6ba4540000000p-37f, -0x1.b545b00000000p-44f, -0x1.02ac400000000p-37f, 0x1.2fe8860000000p-38f, 0x0.0p+0f, 0x1.249fc00000000p-40f, -0x1.39dc060000000p-32f, 0x1.66faa20000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.0866a60000000p-30f, 0x0.0p+0f, 0x0.0p+0f, -0x1.8c6ca60000000p-29f, 0x1.0446c60000000p-29f, -0x1.af70780000000p-35f, -0x1.11ee2c0000000p-30f, -0x1.c0bb2a0000000p-30f, 0x1.3df0400000000p-32f, 0x0.0p+0f, 0x1.3811e40000000p-32f, -0x1.b4427a0000000p-30f, 0x1.8fd63e0000000p-31f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, -0x1.5a73c80000000p-30f, 0x0.0p+0f, 0x0.0p+0f, -0x1.b9381a0000000p-26f, 0x1.f224260000000p-27f, 0x1.a449160000000p-28f, -0x1.0b32fc0000000p-30f, 0x1.656ba80000000p-35f, -0x1.cabcc00000000p-37f, 0x0.0p+0f, 0x1.e6eb8c0000000p-34f, -0x1.f224b40000000p-28f, 0x1.de67440000000p-31f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}};
    return t[i][j];
}
__host__ __device__ constexpr bool VERN7_AM(int i, int j) {
    constexpr bool t[17][17] = {{false, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, false, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, true, false, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, false, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, false, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, false, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, true, false, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, true, true, false, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, true, true, true, false, false, false, false, false, false, false, false}, {false, true, false, true, true, true, true, true, false, false, false, false, false, false, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, false, false, false, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, false, false, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, true, false, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, true, true, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, true, true, false, false, false}, {false, true, false, false, true, true, true, true, true, true, false, true, true, true, false, false, false}};
    return t[i][j];
}
__host__ __device__ constexpr double VERN7_CS(int i) {
    constexpr double t[17] = {0.0, 0.0, 0.005, 0.10888888888888888, 0.16333333333333333, 0.4555, 0.6095094489978381, 0.884, 0.925, 1.0, 1.0, 1.0, 0.29, 0.125, 0.25, 0.53, 0.79};
    return t[i];
}
__host__ __device__ constexpr float VERN7_CS_HI(int i) {
    constexpr float t[17] = {0x0.0p+0f, 0x0.0p+0f, 0x1.47ae140000000p-8f, 0x1.be02460000000p-4f, 0x1.4e81b40000000p-3f, 0x1.d26e980000000p-2f, 0x1.3811a00000000p-1f, 0x1.c49ba60000000p-1f, 0x1.d9999a0000000p-1f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f, 0x1.0000000000000p+0f, 0x1.28f5c20000000p-2f, 0x1.0000000000000p-3f, 0x1.0000000000000p-2f, 0x1.0f5c280000000p-1f, 0x1.947ae20000000p-1f};
    return t[i];
}
__host__ __device__ constexpr float VERN7_CS_LO(int i) {
    constexpr float t[17] = {0x0.0p+0f, 0x0.0p+0f, 0x1.eb851e0000000p-34f, 0x1.159e260000000p-29f, 0x1.d0369c0000000p-28f, -0x1.cac0840000000p-28f, -0x1.47ce240000000p-26f, -0x1.cac0840000000p-29f, -0x1.99999a0000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x1.1eb8520000000p-27f, 0x0.0p+0f, 0x0.0p+0f, 0x1.eb851e0000000p-26f, -0x1.70a3d80000000p-26f};
    return t[i];
}
__host__ __device__ constexpr double VERN7_B(int i) {
    constexpr double t[17] = {0.0, 0.04715561848627222, 0.0, 0.0, 0.25750564298434153, 0.26216653977412624, 0.15216092656738558, 0.4939969170032485, -0.29430311714032503, 0.08131747232495111, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    return t[i];
}
__host__ __device__ constexpr float VERN7_B_HI(int i) {
    constexpr float t[17] = {0x0.0p+0f, 0x1.824c800000000p-5f, 0x0.0p+0f, 0x0.0p+0f, 0x1.07af900000000p-2f, 0x1.0c75620000000p-2f, 0x1.37a0260000000p-3f, 0x1.f9da540000000p-2f, -0x1.2d5dcc0000000p-2f, 0x1.4d138c0000000p-4f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr float VERN7_B_LO(int i) {
    constexpr float t[17] = {0x0.0p+0f, -0x1.8ebfe40000000p-33f, 0x0.0p+0f, 0x0.0p+0f, -0x1.a6c6400000000p-27f, 0x1.537b9c0000000p-27f, -0x1.2a7f540000000p-30f, -0x1.495bb00000000p-30f, 0x1.18afb20000000p-29f, 0x1.8754600000000p-29f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr double VERN7_BT(int i) {
    constexpr double t[17] = {0.0, 0.002547011879931045, 0.0, 0.0, -0.00965839487279575, 0.04206470975639691, -0.0666822437469301, 0.2650097464621281, -0.29430311714032503, 0.08131747232495111, -0.02029518466335628, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    return t[i];
}
__host__ __device__ constexpr float VERN7_BT_HI(int i) {
    constexpr float t[17] = {0x0.0p+0f, 0x1.4dd78a0000000p-9f, 0x0.0p+0f, 0x0.0p+0f, -0x1.3c7c7e0000000p-7f, 0x1.5898180000000p-5f, -0x1.1121660000000p-4f, 0x1.0f5eb80000000p-2f, -0x1.2d5dcc0000000p-2f, 0x1.4d138c0000000p-4f, -0x1.4c842c0000000p-6f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr float VERN7_BT_LO(int i) {
    constexpr float t[17] = {0x0.0p+0f, -0x1.17ba940000000p-34f, 0x0.0p+0f, 0x0.0p+0f, 0x1.e3b5800000000p-32f, -0x1.d1f46c0000000p-30f, -0x1.03be2e0000000p-29f, -0x1.ee975e0000000p-27f, 0x1.18afb20000000p-29f, 0x1.8754600000000p-29f, -0x1.329c560000000p-31f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f};
    return t[i];
}
__host__ __device__ constexpr bool VERN7_BM(int j) {
    constexpr bool t[17] = {false, true, false, false, true, true, true, true, true, true, false, false, false, false, false, false, false};
    return t[j];
}
__host__ __device__ constexpr bool VERN7_BTM(int j) {
    constexpr bool t[17] = {false, true, false, false, true, true, true, true, true, true, true, false, false, false, false, false, false};
    return t[j];
}
__host__ __device__ constexpr double VERN7_R(int i, int j) {
    constexpr double t[17][8] = {{0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 1.0, -8.413387198332767, 33.675508884490895, -70.80159089484886, 80.64695108301298, -47.19413969837522, 11.133813442539243}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 8.754921980674396, -88.4596828699771, 346.9017638429916, -629.2580030059837, 529.6773755604193, -167.35886986514018}, {0.0, 0.0, 8.913387586637922, -90.06081846893218, 353.1807459217058, -640.6476819744374, 539.2646279047156, -170.38809442991547}, {0.0, 0.0, 5.1733120298478, -52.271115900055385, 204.9853867374073, -371.8306118563603, 312.9880934374529, -98.89290352172495}, {0.0, 0.0, 16.79537744079696, -169.70040000059728, 665.4937727009246, -1207.1638892336007, 1016.1291515818546, -321.06001557237494}, {0.0, 0.0, -10.005997536098665, 101.1005433052275, -396.47391512378437, 719.1787707014183, -605.3681033918824, 191.27439892797935}, {0.0, 0.0, 2.764708833638599, -27.934602637390462, 109.54779186137893, -198.7128113064482, 167.26633571640318, -52.85010499525706}, {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, -2.1696320280163506, 22.016696037569876, -86.90152427798948, 159.22388973861476, -135.9618306534588, 43.792401183280006}, {0.0, 0.0, -4.890070188793804, 22.75407737425176, -30.78034218537731, -2.797194317207249, 31.369456637508403, -15.655927320381801}, {0.0, 0.0, 10.862170929551967, -50.542971417827104, 68.37148040407511, 6.213326521632409, -69.68006323194157, 34.776056794509195}, {0.0, 0.0, -11.37286691922923, 130.79058078246717, -488.65113677785604, 832.2148793276441, -664.7743368554426, 201.79288044241662}, {0.0, 0.0, -5.919778732715007, 63.27679965889219, -265.432682088738, 520.1009254140611, -467.412109533902, 155.3868452824017}, {0.0, 0.0, -10.492146197961823, 105.35538525188011, -409.43975011988937, 732.831448907654, -606.3044574733512, 188.0495196316683}};
    return t[i][j];
}
__host__ __device__ constexpr float VERN7_R_HI(int i, int j) {
    constexpr float t[17][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x1.0000000000000p+0f, -0x1.0d3a780000000p+3f, 0x1.0d67720000000p+5f, -0x1.1b34d40000000p+6f, 0x1.42967a0000000p+6f, -0x1.798d9a0000000p+5f, 0x1.6448340000000p+3f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.1828520000000p+3f, -0x1.61d6b80000000p+6f, 0x1.5ae6da0000000p+8f, -0x1.3aa1060000000p+9f, 0x1.08d6b40000000p+9f, -0x1.4eb7be0000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.1d3a780000000p+3f, -0x1.683e480000000p+6f, 0x1.612e460000000p+8f, -0x1.4052e80000000p+9f, 0x1.0da1e00000000p+9f, -0x1.54c6b40000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.4b178c0000000p+2f, -0x1.a22b3e0000000p+5f, 0x1.99f8840000000p+7f, -0x1.73d4a20000000p+8f, 0x1.38fcf40000000p+8f, -0x1.8b92560000000p+6f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.0cb9de0000000p+4f, -0x1.53669a0000000p+7f, 0x1.4cbf340000000p+9f, -0x1.2dca7e0000000p+10f, 0x1.fc10880000000p+9f, -0x1.410f5e0000000p+8f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.4031220000000p+3f, 0x1.9466f40000000p+6f, -0x1.8c79520000000p+8f, 0x1.6796e20000000p+9f, -0x1.2eaf1e0000000p+9f, 0x1.7e8c7e0000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.61e1fa0000000p+1f, -0x1.bef4220000000p+4f, 0x1.b630f00000000p+6f, -0x1.8d6cf60000000p+7f, 0x1.4e885e0000000p+7f, -0x1.a6cd040000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.15b6800000000p+1f, 0x1.6044640000000p+4f, -0x1.5b9b2a0000000p+6f, 0x1.3e72a20000000p+7f, -0x1.0fec760000000p+7f, 0x1.5e56d60000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.38f6e80000000p+2f, 0x1.6c10b40000000p+4f, -0x1.ec7c480000000p+4f, -0x1.660a760000000p+1f, 0x1.f5e94c0000000p+4f, -0x1.f4fd5c0000000p+3f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.5b96e80000000p+3f, -0x1.9458020000000p+5f, 0x1.117c660000000p+6f, 0x1.8da7240000000p+2f, -0x1.16b8620000000p+6f, 0x1.16355e0000000p+5f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.6bee860000000p+3f, 0x1.0594c80000000p+7f, -0x1.e8a6b00000000p+8f, 0x1.a01b820000000p+9f, -0x1.4c631e0000000p+9f, 0x1.9395f40000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.7adda80000000p+2f, 0x1.fa36e20000000p+5f, -0x1.096ec40000000p+8f, 0x1.040cec0000000p+9f, -0x1.d369800000000p+8f, 0x1.36c6100000000p+7f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.4fbfaa0000000p+3f, 0x1.a56bea0000000p+6f, -0x1.9970940000000p+8f, 0x1.6e6a6c0000000p+9f, -0x1.2f26f80000000p+9f, 0x1.78195a0000000p+7f}};
    return t[i][j];
}
__host__ __device__ constexpr float VERN7_R_LO(int i, int j) {
    constexpr float t[17][8] = {{0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.ae93600000000p-24f, -0x1.988f440000000p-20f, -0x1.f2c4b60000000p-21f, 0x1.60fa700000000p-20f, 0x1.c589f80000000p-20f, -0x1.be21d80000000p-22f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.2207300000000p-24f, 0x1.c997560000000p-19f, -0x1.39a2c00000000p-24f, -0x1.f0a3e00000000p-18f, 0x1.f05c700000000p-18f, 0x1.ac1b400000000p-20f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.354baa0000000p-22f, 0x1.9b478c0000000p-19f, -0x1.4542c60000000p-17f, 0x1.839d960000000p-16f, -0x1.587ba40000000p-16f, -0x1.40a1fa0000000p-19f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.51e6700000000p-23f, -0x1.a0429e0000000p-20f, 0x1.388c4e0000000p-18f, -0x1.f50d7a0000000p-17f, -0x1.3be2fe0000000p-18f, 0x1.65fdaa0000000p-19f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.37f3420000000p-22f, -0x1.a862bc0000000p-18f, -0x1.cbddf00000000p-20f, 0x1.ad76c20000000p-15f, 0x1.3fc4ac0000000p-20f, 0x1.a38ecc0000000p-17f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.054cc20000000p-23f, 0x1.a5fe460000000p-19f, -0x1.00cb780000000p-17f, -0x1.553ece0000000p-20f, -0x1.876ba00000000p-22f, 0x1.0add480000000p-23f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.4770aa0000000p-24f, 0x1.ada7120000000p-24f, 0x1.661a340000000p-20f, 0x1.95f4b00000000p-19f, -0x1.b0a12a0000000p-18f, 0x1.37cd1a0000000p-22f}, {0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f, 0x0.0p+0f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.2caf340000000p-24f, -0x1.df15440000000p-21f, 0x1.a3abe20000000p-19f, -0x1.4bf5ea0000000p-19f, 0x1.dd7c6a0000000p-18f, 0x1.b9effa0000000p-21f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.e801c80000000p-23f, -0x1.205dec0000000p-21f, -0x1.65e27c0000000p-24f, -0x1.40f6520000000p-24f, -0x1.4613900000000p-21f, 0x1.6a9a100000000p-22f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.0580ca0000000p-22f, 0x1.33dc520000000p-20f, -0x1.482b240000000p-19f, 0x1.21c7d80000000p-24f, -0x1.fbc66c0000000p-20f, -0x1.787bea0000000p-20f}, {0x0.0p+0f, 0x0.0p+0f, -0x1.35f6640000000p-22f, -0x1.fdc9d40000000p-18f, -0x1.ccbc3a0000000p-17f, -0x1.ab1b2e0000000p-16f, 0x1.0f51ca0000000p-16f, 0x1.b38e8a0000000p-19f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.876ec60000000p-24f, 0x1.7aa7c60000000p-20f, -0x1.0372c80000000p-18f, -0x1.c087460000000p-16f, -0x1.553d500000000p-23f, 0x1.2b721c0000000p-18f}, {0x0.0p+0f, 0x0.0p+0f, 0x1.3bb9ce0000000p-22f, 0x1.c893920000000p-22f, 0x1.1281540000000p-17f, 0x1.d5eaac0000000p-16f, -0x1.d996220000000p-17f, 0x1.463a1a0000000p-18f}};
    return t[i][j];
}
// ROSENBROCK23: c32 = 6 + sqrt(2), d = 1 / (2 + sqrt(2)) in Float64
constexpr double ROS23_C32 = 0x1.da827999fcef3p+2;  // 7.414213562373095
constexpr float ROS23_C32_HI = 0x1.da827a0000000p+2f;
constexpr float ROS23_C32_LO = -0x1.980c440000000p-24f;
constexpr double ROS23_D = 0x1.2bec333018867p-2;  // 0.2928932188134525
constexpr float ROS23_D_HI = 0x1.2bec340000000p-2f;
constexpr float ROS23_D_LO = -0x1.9fcef40000000p-27f;
}  // namespace tab
}  // namespace odegb
)ODEGBRTC",
R"ODEGBRTC(// Explicit Runge-Kutta steps on a lane group: Tsit5 and Vern7.
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
                                             const PR<R>* p, double t, double dt, R abstol, R reltol, long long, bool,
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
        return error_norm<R, L, C>(tmp, up, u, abstol, reltol, g);
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
                                             const PR<R>* p, double t, double dt, R abstol, R reltol, long long, bool,
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
        return error_norm<R, L, C>(c.tmp, up, u, abstol, reltol, g);
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
};

}  // namespace odegb
)ODEGBRTC",
R"ODEGBRTC(// W = J - I/(dt*gamma) and its LU in shared memory, for a lane group of L
// lanes that owns one trajectory of n = L*C states (16 to 64).
//
// The reference builds a dense W (lib/OrdinaryDiffEqDifferentiation/src/
// derivative_utils.jl:663-685) and factors it with LinearSolve's dense LU
// (partial pivoting).  Here:
//   * Lane l owns rows l*C .. l*C+C-1 (the state components it integrates).
//     The matrix is stored column-major (column stride n+1) with the rows in
//     component-major order (row l*C+i at slot i*L+l): the lanes of a group
//     touch consecutive words of one column, and a row read across columns
//     has an odd word stride, so neither access has bank conflicts.
//   * Doolittle with partial pivoting, right-looking.  Rows are never moved:
//     `rowat[pos]` maps a pivot position to its physical row and each lane
//     keeps the positions of its own rows, which is the same factorisation
//     as swapping rows (each row carries its multipliers).  The pivot is the
//     largest |W[r][c]| over the rows at positions >= c, first position on
//     ties, found by a butterfly arg-max over the group's lanes (warp shuffles).
//   * The rank-1 update skips the columns where the pivot row is zero (a
//     group-wide ballot of the row), which leaves every entry unchanged
//     (w - l*0 = w); the periodic band of the chain models keeps most of each
//     pivot row zero.
//   * Solves are column-oriented: the entry of the row at position c is
//     broadcast from its owner lane and every lane updates its own rows.
//   * Zero tests and the pivot comparison run on integer bit patterns (warp
//     reductions for a full-warp group), keeping the FP64 form off the narrow
//     FP64 pipe wherever the arithmetic allows.
//   * When the factorisation exchanged no rows (the usual case for a
//     diagonally dominant W) the solves take a path whose ownership pattern
//     is known at compile time: no position table, no permutation at the end.
// Mixed precision (R = float): W, the LU and the solves are FP32; optional
// refinement sweeps form the residual b - (J(u) x - x/(dt*gamma)) in
// double-float through the model's Jacobian-vector product at the compensated
// state, and correct x with one more FP32 solve.
#pragma once
#include "common.cuh"

namespace odegb {

extern __shared__ __align__(16) unsigned char odegb_dyn_smem[];

// Zero tests and pivot magnitudes on the integer pipe (FP64 comparisons would
// occupy GB300's narrow FP64 pipe, which costs a full warp instruction even for
// one active lane).  mag_key orders like |x| and maps NaN to the key of zero.
template <class R> struct Bits;
template <> struct Bits<double> {
    using U = unsigned long long;
    static __device__ __forceinline__ bool nz(double x) { return abs_bits(x) != 0; }
    static __device__ __forceinline__ U mag_key(double x) {
        const U a = (U)abs_bits(x);
        return a > 0x7ff0000000000000ULL ? U(0) : a;
    }
};
template <> struct Bits<float> {
    using U = unsigned;
    static __device__ __forceinline__ bool nz(float x) { return (__float_as_int(x) << 1) != 0; }
    static __device__ __forceinline__ U mag_key(float x) {
        const U a = (U)__float_as_int(x) & 0x7fffffffu;
        return a > 0x7f800000u ? U(0) : a;
    }
};

// Group-wide arg-max of (key, -position): the largest key, first position on
// ties.  Lanes without a candidate pass key 0 and position n.
template <int L>
__device__ __forceinline__ int group_argmax(unsigned key, int pos, const Group<L>& g) {
    if (L == 32) {
        const unsigned km = __reduce_max_sync(0xffffffffu, key);
        return (int)__reduce_min_sync(0xffffffffu, key == km ? (unsigned)pos : 0xffffffffu);
    }
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1) {
        const unsigned ok = __shfl_xor_sync(g.mask, key, off, L);
        const int op = __shfl_xor_sync(g.mask, pos, off, L);
        if (ok > key || (ok == key && op < pos)) { key = ok; pos = op; }
    }
    return pos;
}
template <int L>
__device__ __forceinline__ int group_argmax(unsigned long long key, int pos, const Group<L>& g) {
    if (L == 32) {
        const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
        const unsigned kh = __reduce_max_sync(0xffffffffu, hi);
        const unsigned kl = __reduce_max_sync(0xffffffffu, hi == kh ? lo : 0u);
        return (int)__reduce_min_sync(0xffffffffu, (hi == kh && lo == kl) ? (unsigned)pos : 0xffffffffu);
    }
#pragma unroll
    for (int off = L / 2; off > 0; off >>= 1) {
        const unsigned long long ok = __shfl_xor_sync(g.mask, key, off, L);
        const int op = __shfl_xor_sync(g.mask, pos, off, L);
        if (ok > key || (ok == key && op < pos)) { key = ok; pos = op; }
    }
    return pos;
}

struct SmemLA {
    template <class R, int C> struct Store {
        R* W;        // n columns of stride n+1, component-major rows
        R* dinv;     // 1 / pivot, by position
        R* xs;       // permutation scratch
        int* rowat;  // physical row at each pivot position
        int pos[C];  // pivot position of each own row
        bool ident;  // no row exchange happened (position = row)
    };
    template <class R, int L, int C> __host__ __device__ static constexpr int smem_bytes() {
        return (L * C * (L * C + 1) + 2 * L * C) * (int)sizeof(R) + L * C * (int)sizeof(int);
    }
    // slot of row (lane*C + i), column col
    template <int L, int C> __device__ static __forceinline__ int at(int i, int lane, int col) {
        return col * (L * C + 1) + i * L + lane;
    }
    template <int L, int C> __device__ static __forceinline__ int at_row(int row, int col) {
        return col * (L * C + 1) + (row % C) * L + row / C;
    }

    template <class R, int L, int C> __device__ static void init(Store<R, C>& s, const Group<L>&) {
        constexpr int n = L * C;
        unsigned char* b = odegb_dyn_smem + (size_t)(threadIdx.x / L) * smem_bytes<R, L, C>();
        s.W = reinterpret_cast<R*>(b);
        s.dinv = s.W + n * (n + 1);
        s.xs = s.dinv + n;
        s.rowat = reinterpret_cast<int*>(s.xs + n);
        s.ident = true;
    }

    // J(uprev) into W.  A rejected step keeps uprev, so recomputing J there
    // reproduces the reference's reused J exactly; `fresh` only drives the count.
    template <class Model, class R, int L, int C>
    __device__ static void jacobian(Store<R, C>& s, const R* up, const PR<R>* p, double, bool, const Group<L>& g) {
        constexpr int n = L * C;
        R* W = s.W;
#pragma unroll 8
        for (int col = 0; col < n; ++col)
#pragma unroll
            for (int i = 0; i < C; ++i) W[at<L, C>(i, g.lane, col)] = R(0);
        Model::template jac_rows<R, L, C>(up, p, g, [&](int i, int col, R v) { W[at<L, C>(i, g.lane, col)] = v; });
    }

    template <class R, int L, int C>
    __device__ static void factor(Store<R, C>& s, R idg, const Group<L>& g) {
        using K = typename Bits<R>::U;
        constexpr int n = L * C;
        R* W = s.W;
#pragma unroll
        for (int i = 0; i < C; ++i) {
            const int r = g.lane * C + i;
            const int k = at<L, C>(i, g.lane, r);
            W[k] = FMA(R(-1), idg, W[k]);
            s.pos[i] = r;
            s.rowat[r] = r;
        }
        g.sync();
#pragma unroll 1
        for (int c = 0; c < n; ++c) {
            // pivot: largest |W[r][c]| over positions >= c, first position on ties
            K best = 0;
            int bpos = n;
#pragma unroll
            for (int i = 0; i < C; ++i) {
                if (s.pos[i] >= c) {
                    const K v = Bits<R>::mag_key(W[at<L, C>(i, g.lane, c)]);
                    if (bpos == n || v > best || (v == best && s.pos[i] < bpos)) { best = v; bpos = s.pos[i]; }
                }
            }
            bpos = group_argmax<L>(best, bpos, g);
            const int q = s.rowat[c];
            const int pr = s.rowat[bpos];
            const R d = W[at_row<L, C>(pr, c)];
            const R inv = R(1) / d;
            g.sync();   // rowat reads above complete before it changes
#pragma unroll
            for (int i = 0; i < C; ++i) {
                const int r = g.lane * C + i;
                if (r == pr) s.pos[i] = c;
                else if (r == q) s.pos[i] = bpos;
            }
            if (g.lane == 0) {
                s.rowat[c] = pr;
                s.rowat[bpos] = q;
                s.dinv[c] = inv;
            }
            if (Bits<R>::nz(d)) {
                R l[C];
                bool act[C];
#pragma unroll
                for (int i = 0; i < C; ++i) {
                    const int k = at<L, C>(i, g.lane, c);
                    const R w = W[k];
                    // a zero below the pivot stays zero (multiplier 0, no update)
                    act[i] = s.pos[i] > c && Bits<R>::nz(w);
                    l[i] = R(0);
                    if (act[i]) {
                        l[i] = w * inv;
                        W[k] = l[i];
                    }
                }
                // columns right of c where the pivot row is nonzero, C slices of L columns
#pragma unroll
                for (int kk = 0; kk < C; ++kk) {
                    const int jl = kk * L + g.lane;
                    unsigned m = g.ballot(jl > c && Bits<R>::nz(W[at_row<L, C>(pr, jl)]));
                    while (m) {
                        const int b = __ffs(m) - 1;
                        m &= m - 1;
                        const int j = kk * L + b;
                        const R urow = W[at_row<L, C>(pr, j)];
#pragma unroll
                        for (int i = 0; i < C; ++i) {
                            if (act[i]) {
                                const int k = at<L, C>(i, g.lane, j);
                                W[k] = FMA(-l[i], urow, W[k]);
                            }
                        }
                    }
                }
            }
            g.sync();
        }
        bool moved = false;
#pragma unroll
        for (int i = 0; i < C; ++i) moved = moved || s.pos[i] != g.lane * C + i;
        s.ident = !g.any(moved);
    }

    // x = W^{-1} b for the lane's components, in place.
    template <class R, int L, int C>
    __device__ static void solve(const Store<R, C>& s, R* b, const Group<L>& g) {
        constexpr int n = L * C;
        const R* W = s.W;
        if (s.ident) {
            // No row exchange: row r is position r, owned by lane r/C.  Block
            // columns: lane q solves its C x C diagonal block locally, the C
            // results go out in C independent shuffles, and every lane below
            // updates its rows.  Each row receives its updates in the same
            // column order as the column-by-column form (identical results)
            // with 1/C of the dependent shuffle rounds.
            // The lane's C x C entries of block column q are loaded one round
            // ahead (wn), so the shared-memory latency stays off the chain of
            // dependent rounds (for C <= 2; wider rows would spill registers).
            constexpr bool PF = C <= 2;
            R wn[C][C];
#pragma unroll
            for (int i = 0; i < C; ++i)
#pragma unroll
                for (int k = 0; k < C; ++k) wn[i][k] = W[at<L, C>(i, g.lane, k)];
#pragma unroll 1
            for (int q = 0; q < L; ++q) {
                R w[C][C];
#pragma unroll
                for (int i = 0; i < C; ++i)
#pragma unroll
                    for (int k = 0; k < C; ++k) w[i][k] = PF ? wn[i][k] : W[at<L, C>(i, g.lane, q * C + k)];
                if (PF && q + 1 < L) {
#pragma unroll
                    for (int i = 0; i < C; ++i)
#pragma unroll
                        for (int k = 0; k < C; ++k) wn[i][k] = W[at<L, C>(i, g.lane, (q + 1) * C + k)];
                }
                R y[C];
#pragma unroll
                for (int i = 0; i < C; ++i) {
                    R acc = b[i];
#pragma unroll
                    for (int k = 0; k < i; ++k) acc = FMA(-w[i][k], y[k], acc);
                    y[i] = acc;
                }
#pragma unroll
                for (int k = 0; k < C; ++k) y[k] = g.from(y[k], q);
                if (g.lane == q) {
#pragma unroll
                    for (int i = 0; i < C; ++i) b[i] = y[i];
                } else if (g.lane > q) {
#pragma unroll
                    for (int i = 0; i < C; ++i)
#pragma unroll
                        for (int k = 0; k < C; ++k) b[i] = FMA(-w[i][k], y[k], b[i]);
                }
            }
#pragma unroll
            for (int i = 0; i < C; ++i)
#pragma unroll
                for (int k = 0; k < C; ++k) wn[i][k] = W[at<L, C>(i, g.lane, (L - 1) * C + k)];
            R dn[C];
#pragma unroll
            for (int i = 0; i < C; ++i) dn[i] = s.dinv[(L - 1) * C + i];
#pragma unroll 1
            for (int q = L - 1; q >= 0; --q) {
                R w[C][C], dv[C];
#pragma unroll
                for (int i = 0; i < C; ++i) {
                    dv[i] = PF ? dn[i] : s.dinv[q * C + i];
#pragma unroll
                    for (int k = 0; k < C; ++k) w[i][k] = PF ? wn[i][k] : W[at<L, C>(i, g.lane, q * C + k)];
                }
                if (PF && q > 0) {
#pragma unroll
                    for (int i = 0; i < C; ++i) {
                        dn[i] = s.dinv[(q - 1) * C + i];
#pragma unroll
                        for (int k = 0; k < C; ++k) wn[i][k] = W[at<L, C>(i, g.lane, (q - 1) * C + k)];
                    }
                }
                R x[C];
#pragma unroll
                for (int i = C - 1; i >= 0; --i) {
                    R acc = b[i];
#pragma unroll
                    for (int k = C - 1; k > i; --k) acc = FMA(-w[i][k], x[k], acc);
                    x[i] = acc * dv[i];
                }
#pragma unroll
                for (int k = 0; k < C; ++k) x[k] = g.from(x[k], q);
                if (g.lane == q) {
#pragma unroll
                    for (int i = 0; i < C; ++i) b[i] = x[i];
                } else if (g.lane < q) {
#pragma unroll
                    for (int i = 0; i < C; ++i)
#pragma unroll
                        for (int k = C - 1; k >= 0; --k) b[i] = FMA(-w[i][k], x[k], b[i]);
                }
            }
            return;
        }
        // forward: rows at positions > c take the entry at position c
#pragma unroll 4
        for (int c = 0; c < n - 1; ++c) {
            const int pr = s.rowat[c];
            const int comp = pr % C;
            R v = b[0];
#pragma unroll
            for (int i = 1; i < C; ++i) v = (comp == i) ? b[i] : v;
            const R y = g.from(v, pr / C);
#pragma unroll
            for (int i = 0; i < C; ++i)
                if (s.pos[i] > c) b[i] = FMA(-W[at<L, C>(i, g.lane, c)], y, b[i]);
        }
        // backward: the entry at position c scaled by 1/pivot
#pragma unroll 4
        for (int c = n - 1; c >= 0; --c) {
            const int pr = s.rowat[c];
            const int comp = pr % C;
            R v = b[0];
#pragma unroll
            for (int i = 1; i < C; ++i) v = (comp == i) ? b[i] : v;
            const R x = g.from(v * s.dinv[c], pr / C);
#pragma unroll
            for (int i = 0; i < C; ++i) {
                if (s.pos[i] == c) b[i] = x;
                else if (s.pos[i] < c) b[i] = FMA(-W[at<L, C>(i, g.lane, c)], x, b[i]);
            }
        }
        // b[i] is the unknown at position pos[i]; unknown c belongs to component c
#pragma unroll
        for (int i = 0; i < C; ++i) s.xs[s.pos[i]] = b[i];
        g.sync();
#pragma unroll
        for (int i = 0; i < C; ++i) b[i] = s.xs[g.lane * C + i];
        g.sync();
    }

    template <class Model, class R, int L, int C>
    __device__ static void wsolve(Store<R, C>& s, R* b, double, R idg, int ir, const R* up, const R* uplo,
                                  const ff* pff, const Group<L>& g) {
        if constexpr (sizeof(R) == 8) {
            solve<R, L, C>(s, b, g);
            return;
        }
        if (ir <= 0) {
            solve<R, L, C>(s, b, g);
            return;
        }
        float b0[C];
#pragma unroll
        for (int i = 0; i < C; ++i) b0[i] = (float)b[i];
        solve<R, L, C>(s, b, g);
        ff uu[C];
#pragma unroll
        for (int i = 0; i < C; ++i) uu[i] = ff_fast2sum((float)up[i], (float)uplo[i]);
        for (int sw = 0; sw < ir; ++sw) {
            float x[C];
#pragma unroll
            for (int i = 0; i < C; ++i) x[i] = (float)b[i];
            ff jx[C];
            Model::template jvp<L, C>(jx, x, uu, pff, g);
            R r[C];
#pragma unroll
            for (int i = 0; i < C; ++i) {
                const ff res = (ff(b0[i]) - jx[i]) + ff((float)idg) * ff(x[i]);
                r[i] = (R)res.f();
            }
            solve<R, L, C>(s, r, g);
#pragma unroll
            for (int i = 0; i < C; ++i) b[i] = b[i] + r[i];
        }
    }
};

}  // namespace odegb
)ODEGBRTC",
R"ODEGBRTC(// Rodas5P, with the linear algebra as a policy:
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
                                             const PR<R>* p, double t, double dt, R abstol, R reltol, long long iter,
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
        return error_norm<R, L, C>(c.ks[7], up, u, abstol, reltol, g);
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
)ODEGBRTC",
R"ODEGBRTC(// Rosenbrock23 (Shampine's ode23s pair), with the linear algebra as a policy
// (RegLA: registers, n <= 8; SmemLA: shared memory, 16-64 states).
//
//  perform_step!(::Rosenbrock23Cache)  lib/OrdinaryDiffEqRosenbrock/src/rosenbrock_perform_step.jl:34-146
//  initialize! (FSAL, k = [k1, k2])   rosenbrock_perform_step.jl:1-14
//  tableau                             rosenbrock_tableaus.jl:6-10 (c32 = 6 + sqrt(2), d = 1/(2 + sqrt(2)))
//  interpolant                         rosenbrock_interpolants.jl:39-74
//  J and W on every attempt            a W-method whose default max_jac_age = 1
//                                      (algorithms.jl:108-115) makes _rosenbrock_jac_reuse_decision
//                                      (OrdinaryDiffEqDifferentiation/src/derivative_utils.jl:46-170)
//                                      return a fresh J and W each time, rejected or not
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

    template <class Model, class R, int L, int C>
    __device__ static typename Ctl<R>::T step(Cache<R, C>& c, R* u, R* ulo, const R* up, const R* uplo,
                                             const PR<R>* p, double t, double dt, R abstol, R reltol, long long,
                                             bool, const Group<L>& g, StepStats& st) {
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
        LA::template jacobian<Model, R, L, C>(c.la, up, p, t, true, g);
        st.njacs += 1;
        st.nf += jac_f_calls<Model>::value;
        // the time derivative (calc_tderivative!, derivative_utils.jl:181-227): the model's
        // analytic tgrad (not an f call); else dT = 0 for an autonomous model, whose AD
        // evaluation in the reference counts as one f call
        if constexpr (has_tgrad<Model>::value) Model::template tgrad<R, C>(c.dT, up, p, t);
        else st.nf += 1;
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
        return error_norm<R, L, C>(tmp, up, u, abstol, reltol, g);
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
)ODEGBRTC",
R"ODEGBRTC(// AutoTsit5(Rosenbrock23()): a CompositeAlgorithm of a non-stiff and a stiff
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
                                             const PR<R>* p, double t, double dt, R abstol, R reltol, long long iter,
                                             bool errorfail, const Group<L>& g, StepStats& st) {
        if (c.current == 0) {
            const typename Ctl<R>::T e = NS::template step<Model, R, L, C, true>(c.ns, u, ulo, up, uplo, p, t, dt,
                                                                                abstol, reltol, iter, errorfail, g, st);
            c.eigen_est = c.ns.eig;
            return e;
        }
        return S::template step<Model, R, L, C>(c.s, u, ulo, up, uplo, p, t, dt, abstol, reltol, iter, errorfail, g,
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
)ODEGBRTC",
R"ODEGBRTC(// Device side of registered models: a model supplied at run time as CUDA C++
// source (ode_register_model) is compiled by NVRTC together with these
// headers.  The source defines, for a model named NAME,
//
//   template <class T, class P>
//   __device__ void NAME_f(T* du, const T* u, const P* p, double t);       // required
//   template <class T, class P>
//   __device__ void NAME_jac(T* J, const T* u, const P* p, double t);      // optional, J row-major n x n
//   template <class T, class P>
//   __device__ void NAME_tgrad(T* dT, const T* u, const P* p, double t);   // optional, df/dt
//
// the reference's f(du, u, p, t), ODEFunction's jac and tgrad.  T is the stage
// type (double; float or a double-float pair in the mixed form) and P the
// parameter type (double; a float pair in the mixed form), so the functions are
// written once as templates with +, -, *, / and the usual math functions.
//
// Without NAME_jac the Rosenbrock methods take J by forward-mode automatic
// differentiation of NAME_f: one evaluation with every state seeded as its own
// dual direction (the reference's ForwardDiff Jacobian with one chunk for up to
// 12 states: lib/OrdinaryDiffEqDifferentiation/src/derivative_wrappers.jl:195-
// 241, one counted f call per Jacobian).
#pragma once
#include "common.cuh"

namespace odegb {

// A value with N partial derivatives (forward-mode AD).  Operations with plain
// values are hidden friends, so a parameter type that converts to T (a float
// pair to float) takes part without a template of its own.
template <class T, int N> struct dualn {
    T v;
    T d[N];
    __device__ __forceinline__ dualn() : v(T(0)) {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = T(0);
    }
    __device__ __forceinline__ dualn(T x) : v(x) {
#pragma unroll
        for (int i = 0; i < N; ++i) d[i] = T(0);
    }
    friend __device__ __forceinline__ dualn operator+(dualn a, dualn b) {
        dualn r;
        r.v = a.v + b.v;
#pragma unroll
        for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
        return r;
    }
    friend __device__ __forceinline__ dualn operator-(dualn a, dualn b) {
        dualn r;
        r.v = a.v - b.v;
#pragma unroll
        for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
        return r;
    }
    friend __device__ __forceinline__ dualn operator-(dualn a) {
        dualn r;
        r.v = -a.v;
#pragma unroll
        for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
        return r;
    }
    friend __device__ __forceinline__ dualn operator*(dualn a, dualn b) {
        dualn r;
        r.v = a.v * b.v;
#pragma unroll
        for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
        return r;
    }
    friend __device__ __forceinline__ dualn operator/(dualn a, dualn b) {
        dualn r;
        r.v = a.v / b.v;
        const T ib = T(1) / b.v;
#pragma unroll
        for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
        return r;
    }
    friend __device__ __forceinline__ dualn operator+(dualn a, T b) { a.v = a.v + b; return a; }
    friend __device__ __forceinline__ dualn operator+(T b, dualn a) { a.v = b + a.v; return a; }
    friend __device__ __forceinline__ dualn operator-(dualn a, T b) { a.v = a.v - b; return a; }
    friend __device__ __forceinline__ dualn operator-(T b, dualn a) {
        dualn r = -a;
        r.v = b - a.v;
        return r;
    }
    friend __device__ __forceinline__ dualn operator*(dualn a, T b) {
        a.v = a.v * b;
#pragma unroll
        for (int i = 0; i < N; ++i) a.d[i] = a.d[i] * b;
        return a;
    }
    friend __device__ __forceinline__ dualn operator*(T b, dualn a) { return a * b; }
    friend __device__ __forceinline__ dualn operator/(dualn a, T b) {
        const T ib = T(1) / b;
        a.v = a.v / b;
#pragma unroll
        for (int i = 0; i < N; ++i) a.d[i] = a.d[i] * ib;
        return a;
    }
    friend __device__ __forceinline__ dualn operator/(T b, dualn a) { return dualn(b) / a; }
    // chain rule for a function with value fv and derivative dv at a.v
    __device__ __forceinline__ dualn chain(T fv, T dv) const {
        dualn r;
        r.v = fv;
#pragma unroll
        for (int i = 0; i < N; ++i) r.d[i] = dv * d[i];
        return r;
    }
    friend __device__ __forceinline__ dualn exp(dualn a) { const T e = exp(a.v); return a.chain(e, e); }
    friend __device__ __forceinline__ dualn log(dualn a) { return a.chain(log(a.v), T(1) / a.v); }
    friend __device__ __forceinline__ dualn sqrt(dualn a) { const T s = sqrt(a.v); return a.chain(s, T(0.5) / s); }
    friend __device__ __forceinline__ dualn sin(dualn a) { return a.chain(sin(a.v), cos(a.v)); }
    friend __device__ __forceinline__ dualn cos(dualn a) { return a.chain(cos(a.v), -sin(a.v)); }
    friend __device__ __forceinline__ dualn tanh(dualn a) {
        const T th = tanh(a.v);
        return a.chain(th, T(1) - th * th);
    }
    friend __device__ __forceinline__ dualn pow(dualn a, T y) {
        const T pv = pow(a.v, y);
        return a.chain(pv, y * pow(a.v, y - T(1)));
    }
    friend __device__ __forceinline__ dualn fabs(dualn a) { return a.v < T(0) ? -a : a; }
};

// A float-pair parameter with a double operand (t, or a float stage value
// promoted by an FP64 constant in f, as in 1.0 - x) is used at its FP64 value:
// p w t keeps t's precision.  That arithmetic runs on the FP64 pipe; writing
// constants as T(c) keeps the mixed form's right-hand side in FP32.
__device__ __forceinline__ double operator*(fpair a, double x) { return pdouble(a) * x; }
__device__ __forceinline__ double operator*(double x, fpair a) { return x * pdouble(a); }
__device__ __forceinline__ double operator+(fpair a, double x) { return pdouble(a) + x; }
__device__ __forceinline__ double operator+(double x, fpair a) { return x + pdouble(a); }
__device__ __forceinline__ double operator-(fpair a, double x) { return pdouble(a) - x; }
__device__ __forceinline__ double operator-(double x, fpair a) { return x - pdouble(a); }
__device__ __forceinline__ double operator/(fpair a, double x) { return pdouble(a) / x; }
__device__ __forceinline__ double operator/(double x, fpair a) { return x / pdouble(a); }
__device__ __forceinline__ float operator/(fpair a, float x) { return (float)a / x; }
__device__ __forceinline__ float operator/(float x, fpair a) { return x / (float)a; }
__device__ __forceinline__ float operator/(fpair a, fpair b) { return (float)a / (float)b; }

// Division and the common functions for double-float stage values (the mixed
// Rosenbrock right-hand side): the quotient by one correction step; the
// functions through FP64 (a registered model's mixed Rosenbrock solve is not the
// fast path; this keeps it correct for any f written with them).
__device__ __forceinline__ ff operator/(ff a, ff b) {
    const float q1 = a.hi / b.hi;
    const ff r = a - ff_mul_f(b, q1);
    const float q2 = r.hi / b.hi;
    return ff_fast2sum(q1, q2);
}
// FP64 constants in f keep their full value: (double, ff) operations split the
// constant into a pair instead of rounding it to float
__device__ __forceinline__ ff operator+(ff a, double b) { return a + ff(b); }
__device__ __forceinline__ ff operator+(double a, ff b) { return ff(a) + b; }
__device__ __forceinline__ ff operator-(ff a, double b) { return a - ff(b); }
__device__ __forceinline__ ff operator-(double a, ff b) { return ff(a) - b; }
__device__ __forceinline__ ff operator*(ff a, double b) { return a * ff(b); }
__device__ __forceinline__ ff operator*(double a, ff b) { return ff(a) * b; }
__device__ __forceinline__ ff operator/(ff a, double b) { return a / ff(b); }
__device__ __forceinline__ ff operator/(double a, ff b) { return ff(a) / b; }
__device__ __forceinline__ double ffd(ff a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ ff exp(ff a) { return ff(::exp(ffd(a))); }
__device__ __forceinline__ ff log(ff a) { return ff(::log(ffd(a))); }
__device__ __forceinline__ ff sqrt(ff a) { return ff(::sqrt(ffd(a))); }
__device__ __forceinline__ ff sin(ff a) { return ff(::sin(ffd(a))); }
__device__ __forceinline__ ff cos(ff a) { return ff(::cos(ffd(a))); }
__device__ __forceinline__ ff tanh(ff a) { return ff(::tanh(ffd(a))); }
__device__ __forceinline__ ff pow(ff a, ff y) { return ff(::pow(ffd(a), ffd(y))); }
__device__ __forceinline__ ff fabs(ff a) { return a.hi < 0.0f ? -a : a; }

// J of f at u by forward-mode AD: every state its own direction, one evaluation.
template <class R, int N, class F, class P>
__device__ __forceinline__ void ad_jacobian(F f, R (*J)[N], const R* u, const P* p, double t) {
    dualn<R, N> x[N], y[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        x[i] = dualn<R, N>(u[i]);
        x[i].d[i] = R(1);
    }
    f(y, x, p, t);
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) J[i][j] = y[i].d[j];
}

}  // namespace odegb
)ODEGBRTC",
};
extern const int kRtcNumHeaders = 11;
}  // namespace odegb
