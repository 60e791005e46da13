// Vern7 over every size class of an uneven ensemble in one persistent
// launch (fused_class_kernel in integrator.cuh).
#include "erk.cuh"
#include "models.cuh"

namespace odegb {

#define FUSED(MODEL, MID, R, PREC)                                                                  \
    {1, MID, PREC, (const void*)fused_class_kernel<Vern7Alg, MODEL, R>,                                \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                           \
         launch_kernel(fused_class_kernel<Vern7Alg, MODEL, R>, a, g, b, s, st);                         \
     },                                                                                             \
     "vern7-classes/" #MODEL "/" #R}

static const FusedVariant kFused[] = {
    FUSED(Duffing, M_DUFFING, double, 0),
    FUSED(Duffing, M_DUFFING, float, 1),
};

const FusedVariant* fused_vern7_variants(int* count) {
    *count = (int)(sizeof(kFused) / sizeof(kFused[0]));
    return kFused;
}

}  // namespace odegb
