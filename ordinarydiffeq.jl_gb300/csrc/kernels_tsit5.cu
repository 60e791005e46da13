// Tsit5 kernel variants (FP64 and mixed, one lane or a lane group per trajectory).
#include "erk.cuh"
#include "ode_kernels.h"
#include "models.cuh"

namespace odegb {

#define VAR(MODEL, MID, R, PREC, L, C)                                                              \
    {0, MID, PREC, (L) * (C), L, 0, (const void*)ensemble_kernel<Tsit5Alg, MODEL, R, L, C>,          \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                           \
         launch_kernel(ensemble_kernel<Tsit5Alg, MODEL, R, L, C>, a, g, b, s, st);                   \
     },                                                                                             \
     "tsit5/" #MODEL "/" #R "/L" #L "C" #C}
#define BOTH(MODEL, MID, L, C) VAR(MODEL, MID, double, 0, L, C), VAR(MODEL, MID, float, 1, L, C)
// with the forward-only form (benchmarked workloads: a second copy of the step loop)
#define VARF(MODEL, MID, R, PREC, L, C)                                                             \
    {0, MID, PREC, (L) * (C), L, 0, (const void*)ensemble_kernel<Tsit5Alg, MODEL, R, L, C>,          \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                           \
         launch_kernel(ensemble_kernel<Tsit5Alg, MODEL, R, L, C>, a, g, b, s, st);                   \
     },                                                                                             \
     "tsit5/" #MODEL "/" #R "/L" #L "C" #C,                                                         \
     (const void*)ensemble_kernel<Tsit5Alg, MODEL, R, L, C, true>,                                  \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                           \
         launch_kernel(ensemble_kernel<Tsit5Alg, MODEL, R, L, C, true>, a, g, b, s, st);             \
     }}

static const KernelVariant kVariants[] = {
    BOTH(BouncingBall, M_BOUNCING_BALL, 1, 2),
    BOTH(VanDerPol, M_VANDERPOL, 1, 2),
    BOTH(PKOneCompartment, M_PK1, 1, 2),
    BOTH(ForcedDuffing, M_FORCED_DUFFING, 1, 2),
    BOTH(Linear, M_LINEAR, 1, 1),   BOTH(Linear, M_LINEAR, 1, 2),   BOTH(Linear, M_LINEAR, 1, 8),
    VARF(Lorenz, M_LORENZ, double, 0, 1, 3), VAR(Lorenz, M_LORENZ, float, 1, 1, 3),
    BOTH(Duffing, M_DUFFING, 1, 4), BOTH(Duffing, M_DUFFING, 1, 8), BOTH(Duffing, M_DUFFING, 2, 4),
    BOTH(Duffing, M_DUFFING, 4, 4), BOTH(Duffing, M_DUFFING, 8, 4), BOTH(Duffing, M_DUFFING, 16, 4),
};

const KernelVariant* tsit5_variants(int* count) {
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace odegb
