// W = J - I/(dt*gamma) and its LU in shared memory, for a lane group of L
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
