// Device helpers shared by every integrator kernel.
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
