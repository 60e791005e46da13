// Vern7 over every size class of an uneven ensemble in one persistent
// launch (fused_class_kernel in integrator.cuh).  The mixed form runs 2 states
// per lane (measured 1.2-1.5x faster per class than 4: a smaller per-lane step
// and more lanes per trajectory); the FP64 form 4, where the FP64 control path
// is shared by more trajectories per warp.
#include "erk.cuh"
#include "ode_kernels.h"
#include "models.cuh"

namespace odegb {

#define FUSED(MODEL, MID, R, PREC, C)                                                              \
    {1, MID, PREC, (const void*)fused_class_kernel<Vern7Alg, MODEL, R, C>,                            \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                          \
         launch_kernel(fused_class_kernel<Vern7Alg, MODEL, R, C>, a, g, b, s, st);                     \
     },                                                                                            \
     "vern7-classes/" #MODEL "/" #R "/C" #C,                                                        \
     (const void*)fused_class_kernel<Vern7Alg, MODEL, R, C, true>,                                   \
     [](const EnsembleArgs& a, int g, int b, size_t s, cudaStream_t st) {                          \
         launch_kernel(fused_class_kernel<Vern7Alg, MODEL, R, C, true>, a, g, b, s, st);              \
     }}

static const FusedVariant kFused[] = {
    FUSED(Duffing, M_DUFFING, double, 0, 4),
    FUSED(Duffing, M_DUFFING, float, 1, 2),
};

const FusedVariant* fused_vern7_variants(int* count) {
    *count = (int)(sizeof(kFused) / sizeof(kFused[0]));
    return kFused;
}

}  // namespace odegb
