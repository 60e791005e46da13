// Rodas5P kernel variants for 16 to 64 states: one lane group per trajectory,
// W and its LU in shared memory (lu_group.cuh).
#include "rodas.cuh"
#include "ode_kernels.h"
#include "models.cuh"

namespace odegb {

#define VAR(MODEL, MID, R, PREC, L, C)                                                                  \
    {2, MID, PREC, (L) * (C), L, Rodas5PGroupAlg::smem_bytes<R, L, C>(),                                \
     (const void*)ensemble_kernel<Rodas5PGroupAlg, MODEL, R, L, C>,                                     \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                               \
         launch_kernel(ensemble_kernel<Rodas5PGroupAlg, MODEL, R, L, C>, a, g, b, s, st);                \
     },                                                                                                 \
     "rodas5p-smem/" #MODEL "/" #R "/L" #L "C" #C}
#define BOTH(MODEL, MID, L, C) VAR(MODEL, MID, double, 0, L, C), VAR(MODEL, MID, float, 1, L, C)
// with the forward-only form (benchmarked workloads: a second copy of the step loop)
#define VARF(MODEL, MID, R, PREC, L, C)                                                                 \
    {2, MID, PREC, (L) * (C), L, Rodas5PGroupAlg::smem_bytes<R, L, C>(),                                \
     (const void*)ensemble_kernel<Rodas5PGroupAlg, MODEL, R, L, C>,                                     \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                               \
         launch_kernel(ensemble_kernel<Rodas5PGroupAlg, MODEL, R, L, C>, a, g, b, s, st);                \
     },                                                                                                 \
     "rodas5p-smem/" #MODEL "/" #R "/L" #L "C" #C,                                                      \
     (const void*)ensemble_kernel<Rodas5PGroupAlg, MODEL, R, L, C, true>,                               \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                               \
         launch_kernel(ensemble_kernel<Rodas5PGroupAlg, MODEL, R, L, C, true>, a, g, b, s, st);          \
     }}

static const KernelVariant kVariants[] = {
    BOTH(Brusselator, M_BRUSSELATOR, 8, 2),  BOTH(Brusselator, M_BRUSSELATOR, 16, 2),
    VARF(Brusselator, M_BRUSSELATOR, double, 0, 32, 2), VARF(Brusselator, M_BRUSSELATOR, float, 1, 32, 2),
    BOTH(Brusselator, M_BRUSSELATOR, 16, 4),
};

const KernelVariant* rodas_group_variants(int* count) {
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace odegb
