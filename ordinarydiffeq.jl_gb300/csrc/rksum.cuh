// Tableau-driven stage sums for the explicit methods, in two arithmetic forms.
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
