// Host interface of models registered at run time (rtc_models.cu).
#pragma once
#include <string>

#include "ode_kernels.h"

namespace odegb {

constexpr int kRtcMaxStates = 32;            // explicit methods: the state and stages in registers
constexpr int kRtcMaxStatesRosenbrock = 8;   // Rosenbrock methods: J, W and its LU in registers too
constexpr int kRtcMaxParams = 32;

// Register source for a model named `name` (a C identifier): returns ODE_OK and
// the new model id, or a status with the reason in *err.
int rtc_register(const char* source, const char* name, int n, int np, int flags, int* id, std::string* err);
// The registered model's state and parameter counts and flags; false if `model` is not one.
bool rtc_lookup(int model, int* n, int* np, int* flags);
// The kernel of a registered model for (alg, precision), compiled on first use;
// nullptr with *status and *err set when it cannot be built.
const KernelVariant* rtc_variant(int alg, int model, int prec, int* status, std::string* err);

}  // namespace odegb
