// Kernel-side parameter block and the launcher table shared by the CUDA
// translation units and the host runtime (ode_capi.cu).  Plain C++ types only.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

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
};

// One launch integrating every size class of an uneven ensemble.
struct FusedVariant {
    int alg, model, prec;
    const void* fn;
    void (*launch)(const EnsembleArgs&, int grid, int block, size_t smem, cudaStream_t);
    const char* name;
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
