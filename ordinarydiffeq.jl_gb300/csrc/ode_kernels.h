// Kernel-side parameter block and the launcher table shared by the CUDA
// translation units and the host runtime (ode_capi.cu).  Plain C++ types only.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "ensemble_args.h"

namespace odegb {

// Size classes of uneven ensembles: state counts 4, 8, 16, 32, 64.
constexpr int kNumClasses = 5;
constexpr int kClassStates[kNumClasses] = {4, 8, 16, 32, 64};

// One compiled kernel variant.
struct KernelVariant {
    int alg, model, prec;   // ode_alg, ode_model, ode_precision
    int n;                  // state count handled (lanes * comps)
    int lanes;              // lanes per trajectory
    int smem_per_group;     // dynamic shared memory per lane group (bytes)
    const void* fn;         // __global__ function
    void (*launch)(const EnsembleArgs&, int grid, int block, size_t smem, cudaStream_t);
    const char* name;
    // the same kernel for forward spans only (no direction in its step loop), or null
    const void* fwd_fn;
    void (*fwd_launch)(const EnsembleArgs&, int grid, int block, size_t smem, cudaStream_t);
};

// One launch integrating every size class of an uneven ensemble.
struct FusedVariant {
    int alg, model, prec;
    const void* fn;
    void (*launch)(const EnsembleArgs&, int grid, int block, size_t smem, cudaStream_t);
    const char* name;
    const void* fwd_fn;   // forward spans only, or null
    void (*fwd_launch)(const EnsembleArgs&, int grid, int block, size_t smem, cudaStream_t);
};

// Dense-output evaluation sol(t) at query times (device pointers):
//   ts[s*N + j], us[(s*n + i)*N + j], ks[((s*nk + q)*n + i)*N + j], nsaved[j],
//   tq[r] (shared) or tq[r*N + j] (per trajectory), out[(r*n + i)*N + j].
struct DenseArgs {
    long long N;
    int n, nq, tq_per_traj;
    int cap;                // save slots per trajectory (nsaved is clamped to it)
    const double* p;
    const double* ts;
    const double* us;
    const double* ks;
    const int32_t* nsaved;
    const double* tq;
    double* out;
    int deriv;              // 0: sol(t); 1-3: sol(t, Val{deriv})
    int right;              // continuity = :right (a query at a time saved twice takes the later save)
};

// Dense vectors stored per step, by ode_alg (Tsit5, Vern7, Rodas5P, Rosenbrock23,
// AutoTsit5(Rosenbrock23())): NDENSE of each method, 0 without dense output.
constexpr int kNumAlgs = 5;
constexpr int kDenseVectors[kNumAlgs] = {7, 7, 3, 2, 0};

// One compiled evaluation kernel: model -1 for the model-free (componentwise)
// interpolants, else the model whose right-hand side the interpolant needs.
struct DenseVariant {
    int alg, model, n, lanes;
    void (*launch)(const DenseArgs&, int grid, int block, cudaStream_t);
    const char* name;
};
const DenseVariant* dense_variants(int* count);

// Registries filled by each translation unit (static arrays).
const KernelVariant* tsit5_variants(int* count);
const KernelVariant* vern7_variants(int* count);
const KernelVariant* rodas_variants(int* count);
const KernelVariant* rodas_group_variants(int* count);
const KernelVariant* ros23_variants(int* count);
const KernelVariant* ros23_group_variants(int* count);
const KernelVariant* auto_variants(int* count);
const FusedVariant* fused_tsit5_variants(int* count);
const FusedVariant* fused_vern7_variants(int* count);

template <class K>
void launch_kernel(K kernel, const EnsembleArgs& a, int grid, int block, size_t smem, cudaStream_t s) {
    kernel<<<grid, block, smem, s>>>(a);
}

}  // namespace odegb
