// Rosenbrock23 kernel variants for 16 to 64 states: one lane group per
// trajectory, W and its LU in shared memory (lu_group.cuh).
#include "ros23.cuh"
#include "ode_kernels.h"
#include "models.cuh"

namespace odegb {

#define VAR(MODEL, MID, R, PREC, L, C)                                                                  \
    {3, MID, PREC, (L) * (C), L, Rosenbrock23GroupAlg::smem_bytes<R, L, C>(),                           \
     (const void*)ensemble_kernel<Rosenbrock23GroupAlg, MODEL, R, L, C>,                                \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                               \
         launch_kernel(ensemble_kernel<Rosenbrock23GroupAlg, MODEL, R, L, C>, a, g, b, s, st);           \
     },                                                                                                 \
     "rosenbrock23-smem/" #MODEL "/" #R "/L" #L "C" #C}
#define BOTH(MODEL, MID, L, C) VAR(MODEL, MID, double, 0, L, C), VAR(MODEL, MID, float, 1, L, C)

static const KernelVariant kVariants[] = {
    BOTH(Brusselator, M_BRUSSELATOR, 8, 2),  BOTH(Brusselator, M_BRUSSELATOR, 16, 2),
    BOTH(Brusselator, M_BRUSSELATOR, 32, 2), BOTH(Brusselator, M_BRUSSELATOR, 16, 4),
};

const KernelVariant* ros23_group_variants(int* count) {
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace odegb
