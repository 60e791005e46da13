// Tsit5 over every size class of an uneven ensemble in one persistent
// launch (fused_class_kernel in integrator.cuh).
#include "erk.cuh"
#include "ode_kernels.h"
#include "models.cuh"

namespace odegb {

#define FUSED(MODEL, MID, R, PREC, C)                                                              \
    {0, MID, PREC, (const void*)fused_class_kernel<Tsit5Alg, MODEL, R, C>,                            \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                          \
         launch_kernel(fused_class_kernel<Tsit5Alg, MODEL, R, C>, a, g, b, s, st);                     \
     },                                                                                            \
     "tsit5-classes/" #MODEL "/" #R "/C" #C}

static const FusedVariant kFused[] = {
    FUSED(Duffing, M_DUFFING, double, 0, 4),
    FUSED(Duffing, M_DUFFING, float, 1, 4),
};

const FusedVariant* fused_tsit5_variants(int* count) {
    *count = (int)(sizeof(kFused) / sizeof(kFused[0]));
    return kFused;
}

}  // namespace odegb
