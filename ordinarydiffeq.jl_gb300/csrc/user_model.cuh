// Device side of registered models: a model supplied at run time as CUDA C++
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
