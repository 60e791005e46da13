// Dense-output evaluation sol(t): the method's interpolant on the saved steps,
// in FP64.
//
// Follows ode_interpolation(tval::Number, ...) (lib/OrdinaryDiffEqCore/src/dense/
// generic_dense.jl:1094-1190) with left continuity: i+ is the first saved index
// >= 2 (1-based) with tdir ts[i+] >= tdir t (tdir = sign(ts[end] - ts[1])),
// clamped to the last index, i- = i+ - 1; dt =
// ts[i+] - ts[i-]; theta = (t - ts[i-]) / dt (1 when dt is 0); then the
// interpolant on (ts[i-], u[i-]) -> (ts[i+], u[i+]) with the vectors stored for
// the step ending at i+ (ks[i+]).  Vern7's lazy extra stages are formed from
// those vectors first, as _ode_addsteps! does (verner_addsteps.jl:137-193).
// The interpolants themselves are the integrator's own (erk.cuh, rodas.cuh).
#include "erk.cuh"
#include "ode_kernels.h"
#include "rodas.cuh"
#include "ros23.cuh"
#include "models.cuh"

namespace odegb {

static_assert(kDenseVectors[0] == Tsit5Alg::NDENSE && kDenseVectors[1] == Vern7Alg::NDENSE &&
                  kDenseVectors[2] == Rodas5PAlg::NDENSE && kDenseVectors[3] == Rosenbrock23Alg::NDENSE,
              "dense vector counts of the runtime and the kernels");

struct Interval {
    int im, ip;
    double th, dt, tprev;
};

__device__ __forceinline__ Interval dense_locate(const DenseArgs& a, long long j, int ns, double t) {
    const long long N = a.N;
    // the saved times run in the integration direction: sign(ts[end] - ts[1])
    const bool bwd = a.ts[(size_t)(ns - 1) * N + j] < a.ts[j];
    int lo = 1, hi = ns;   // first s in [1, ns) with tdir ts[s] >= tdir t, else ns
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const double ts = a.ts[(size_t)mid * N + j];
        if (bwd ? ts <= t : ts >= t) hi = mid;
        else lo = mid + 1;
    }
    Interval v;
    v.ip = lo < ns - 1 ? lo : ns - 1;
    v.im = v.ip > 0 ? v.ip - 1 : v.ip;
    v.tprev = a.ts[(size_t)v.im * N + j];
    v.dt = a.ts[(size_t)v.ip * N + j] - v.tprev;
    v.th = v.dt == 0.0 ? 1.0 : (t - v.tprev) / v.dt;
    return v;
}

// ode_interpolation's exact-time rule for sol(t) (generic_dense.jl:1094-1190): a
// query equal to a saved time returns that save, not the interpolant -- the
// first save at that time, or with continuity = :right the next one when it is
// at the same time (an event's post-affect save).  Returns the save index, or -1.
__device__ __forceinline__ int exact_save(const DenseArgs& a, long long j, int ns, double t) {
    const long long N = a.N;
    const bool bwd = a.ts[(size_t)(ns - 1) * N + j] < a.ts[j];
    int lo = 0, hi = ns;   // first s with tdir ts[s] >= tdir t (searchsortedfirst)
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const double ts = a.ts[(size_t)mid * N + j];
        if (bwd ? ts <= t : ts >= t) hi = mid;
        else lo = mid + 1;
    }
    if (lo >= ns || a.ts[(size_t)lo * N + j] != t) return -1;
    return (a.right && lo + 1 < ns && a.ts[(size_t)(lo + 1) * N + j] == t) ? lo + 1 : lo;
}

__device__ __forceinline__ double query_time(const DenseArgs& a, long long j, int r) {
    return a.tq_per_traj ? a.tq[(size_t)r * a.N + j] : a.tq[r];
}

// Tsit5, Rodas5P and Rosenbrock23: componentwise interpolants, one thread per
// (query, trajectory).
template <int ALG>
__global__ void dense_eval_pointwise(DenseArgs a) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= a.N * (long long)a.nq) return;
    const long long N = a.N, j = idx % N;
    const int r = (int)(idx / N), n = a.n;
    const int ns = min(a.nsaved[j], a.cap);
    if (ns <= 0) {
        for (int i = 0; i < n; ++i) a.out[((size_t)r * n + i) * N + j] = dnan();
        return;
    }
    const double tq = query_time(a, j, r);
    if (a.deriv == 0) {
        const int k = exact_save(a, j, ns, tq);
        if (k >= 0) {
            for (int i = 0; i < n; ++i) a.out[((size_t)r * n + i) * N + j] = a.us[((size_t)k * n + i) * N + j];
            return;
        }
    }
    const Interval v = dense_locate(a, j, ns, tq);
    constexpr int NK = kDenseVectors[ALG];
    Group<1> g;
    for (int i = 0; i < n; ++i) {
        double y0 = a.us[((size_t)v.im * n + i) * N + j], y1 = a.us[((size_t)v.ip * n + i) * N + j];
        double z = 0.0, o, olo;
        const double* kp = a.ks + ((size_t)v.ip * NK * n + i) * N + j;
        if constexpr (ALG == 0) {
            Tsit5Alg::Cache<double, 1> c;
#pragma unroll
            for (int q = 0; q < NK; ++q) c.k[q][0] = kp[(size_t)q * n * N];
            if (a.deriv == 3) tsit5_third_derivative<1>(c.k, v.th, v.dt, &o);
            else if (a.deriv == 2) tsit5_second_derivative<1>(c.k, v.th, v.dt, &o);
            else if (a.deriv) tsit5_derivative<1>(c.k, v.th, &o);
            else Tsit5Alg::interpolate<Linear, double, 1, 1>(c, &o, &olo, v.th, v.dt, v.tprev, &y0, &z, &y1, &z,
                                                             nullptr, g);
        } else if constexpr (ALG == 2) {
            Rodas5PAlg::Cache<double, 1> c;
#pragma unroll
            for (int q = 0; q < NK; ++q) c.dk[q][0] = kp[(size_t)q * n * N];
            if (a.deriv == 3) {
                // the Val{3} form (rosenbrock_interpolants.jl:644-653, interp_order 3):
                // (-6 k2 + 6 k3 - 24 th k3) / dt^3
                const double k2 = c.dk[1][0], k3 = c.dk[2][0], th = v.th;
                o = fma(-6.0, k2, fma(6.0, k3, -24.0 * th * k3)) / (v.dt * v.dt * v.dt);
            } else if (a.deriv == 2) {
                // the Val{2} form (rosenbrock_interpolants.jl:544-560, interp_order 3):
                // (-2 k1 + 2 k2 + th (-6 k2 + 6 k3 - 12 th k3)) / dt^2
                const double k1 = c.dk[0][0], k2 = c.dk[1][0], k3 = c.dk[2][0], th = v.th;
                const double in2 = fma(-6.0, k2, fma(6.0, k3, -12.0 * th * k3));
                o = fma(th, in2, fma(-2.0, k1, 2.0 * k2)) / (v.dt * v.dt);
            } else if (a.deriv) {
                // rosenbrock_interpolants.jl:444-470 (interp_order 3):
                // (k1 + th (-2 k1 + 2 k2 + th (-3 k2 + 3 k3 - 4 th k3)) - y0 + y1) / dt
                const double k1 = c.dk[0][0], k2 = c.dk[1][0], k3 = c.dk[2][0], th = v.th;
                const double in2 = fma(-3.0, k2, fma(3.0, k3, -4.0 * th * k3));
                const double in1 = fma(th, in2, fma(-2.0, k1, 2.0 * k2));
                o = ((fma(th, in1, k1) - y0) + y1) / v.dt;
            } else {
                Rodas5PAlg::interp_dense<double, 1>(c, &o, &olo, v.th, &y0, &z, &y1, &z);
            }
        } else {
            Rosenbrock23Alg::Cache<double, 1> c;
#pragma unroll
            for (int q = 0; q < NK; ++q) c.k[q][0] = kp[(size_t)q * n * N];
            if (a.deriv) {
                // rosenbrock_interpolants.jl:111-127: c1' k1 + c2' k2, c1' = (1 - 2 th)/(1 - 2d),
                // c2' = (2 th - 2d)/(1 - 2d)
                const double d = tab::ROS23_D, th = v.th;
                const double c1 = (1.0 - 2.0 * th) / (1.0 - 2.0 * d), c2 = (2.0 * th - 2.0 * d) / (1.0 - 2.0 * d);
                o = fma(c1, c.k[0][0], c2 * c.k[1][0]);
            } else {
                Rosenbrock23Alg::interpolate<Linear, double, 1, 1>(c, &o, &olo, v.th, v.dt, v.tprev, &y0, &z, &y1, &z,
                                                                   nullptr, g);
            }
        }
        a.out[((size_t)r * n + i) * N + j] = o;
    }
}

// Vern7: the extra stages need the right-hand side, so one lane group (the
// integrator's layout) per (query, trajectory).
template <class Model, int L, int C>
__global__ void dense_eval_vern7(DenseArgs a) {
    Group<L> g;
    const long long gid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / L;
    if (gid >= a.N * (long long)a.nq) return;
    const long long N = a.N, j = gid % N;
    const int r = (int)(gid / N), n = a.n;
    const int ns = min(a.nsaved[j], a.cap);
    double out[C], outlo[C];
    if (ns <= 0) {
#pragma unroll
        for (int c = 0; c < C; ++c) a.out[((size_t)r * n + g.lane * C + c) * N + j] = dnan();
        return;
    }
    const double tq = query_time(a, j, r);
    if (a.deriv == 0) {
        const int k = exact_save(a, j, ns, tq);
        if (k >= 0) {
#pragma unroll
            for (int c = 0; c < C; ++c)
                a.out[((size_t)r * n + g.lane * C + c) * N + j] = a.us[((size_t)k * n + g.lane * C + c) * N + j];
            return;
        }
    }
    const Interval v = dense_locate(a, j, ns, tq);
    double p[Model::NP];
#pragma unroll
    for (int k = 0; k < Model::NP; ++k) p[k] = a.p[(size_t)k * N + j];
    double y0[C], y1[C], z[C];
    Vern7Alg::Cache<double, C> cache;
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const int i = g.lane * C + c;
        y0[c] = a.us[((size_t)v.im * n + i) * N + j];
        y1[c] = a.us[((size_t)v.ip * n + i) * N + j];
        z[c] = 0.0;
#pragma unroll
        for (int q = 0; q < Vern7Alg::NDENSE; ++q)
            Vern7Alg::dense_slot<double, C>(cache, q)[c] =
                a.ks[(((size_t)v.ip * Vern7Alg::NDENSE + q) * n + i) * N + j];
    }
    cache.extra = false;
    if (a.deriv) Vern7Alg::derivative<Model, L, C>(cache, out, v.th, v.dt, v.tprev, y0, z, p, g);
    else Vern7Alg::interpolate<Model, double, L, C>(cache, out, outlo, v.th, v.dt, v.tprev, y0, z, y1, z, p, g);
#pragma unroll
    for (int c = 0; c < C; ++c) a.out[((size_t)r * n + g.lane * C + c) * N + j] = out[c];
}

#define PW(ALG, NAME)                                                                                  \
    {ALG, -1, -1, 1,                                                                                   \
     [](const DenseArgs& a, int g, int b, cudaStream_t st) { dense_eval_pointwise<ALG><<<g, b, 0, st>>>(a); }, \
     "dense/" NAME}
#define V7(MODEL, MID, L, C)                                                                           \
    {1, MID, (L) * (C), L,                                                                             \
     [](const DenseArgs& a, int g, int b, cudaStream_t st) { dense_eval_vern7<MODEL, L, C><<<g, b, 0, st>>>(a); }, \
     "dense/vern7/" #MODEL "/L" #L "C" #C}

// Vern7 shapes: the FP64 integrator's (kernels_vern7.cu).
static const DenseVariant kDense[] = {
    PW(0, "tsit5"), PW(2, "rodas5p"), PW(3, "rosenbrock23"),
    V7(BouncingBall, M_BOUNCING_BALL, 1, 2), V7(PKOneCompartment, M_PK1, 1, 2),
    V7(ForcedDuffing, M_FORCED_DUFFING, 1, 2),
    V7(Linear, M_LINEAR, 1, 1), V7(Linear, M_LINEAR, 1, 2), V7(Linear, M_LINEAR, 1, 8),
    V7(Lorenz, M_LORENZ, 1, 3),
    V7(Duffing, M_DUFFING, 1, 4), V7(Duffing, M_DUFFING, 1, 8), V7(Duffing, M_DUFFING, 2, 4),
    V7(Duffing, M_DUFFING, 4, 4), V7(Duffing, M_DUFFING, 8, 4), V7(Duffing, M_DUFFING, 16, 4),
};

const DenseVariant* dense_variants(int* count) {
    *count = (int)(sizeof(kDense) / sizeof(kDense[0]));
    return kDense;
}

}  // namespace odegb
