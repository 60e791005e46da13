// AutoTsit5(Rosenbrock23()) kernel variants (one lane per trajectory; FP64 and mixed).
#include "autoswitch.cuh"
#include "ode_kernels.h"
#include "models.cuh"

namespace odegb {

#define VAR(MODEL, MID, R, PREC, L, C)                                                                   \
    {4, MID, PREC, (L) * (C), L, 0, (const void*)ensemble_kernel<AutoTsit5Rosenbrock23Alg, MODEL, R, L, C>, \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                                \
         launch_kernel(ensemble_kernel<AutoTsit5Rosenbrock23Alg, MODEL, R, L, C>, a, g, b, s, st);         \
     },                                                                                                  \
     "autotsit5-rosenbrock23/" #MODEL "/" #R "/L" #L "C" #C}
#define BOTH(MODEL, MID, L, C) VAR(MODEL, MID, double, 0, L, C), VAR(MODEL, MID, float, 1, L, C)

static const KernelVariant kVariants[] = {
    BOTH(VanDerPol, M_VANDERPOL, 1, 2), BOTH(Robertson, M_ROBERTSON, 1, 3), BOTH(Lorenz, M_LORENZ, 1, 3),
    BOTH(PKOneCompartment, M_PK1, 1, 2),
    BOTH(ForcedDuffing, M_FORCED_DUFFING, 1, 2),
    BOTH(Linear, M_LINEAR, 1, 1),       BOTH(Linear, M_LINEAR, 1, 2),       BOTH(BouncingBall, M_BOUNCING_BALL, 1, 2),
};

const KernelVariant* auto_variants(int* count) {
    *count = (int)(sizeof(kVariants) / sizeof(kVariants[0]));
    return kVariants;
}

}  // namespace odegb
