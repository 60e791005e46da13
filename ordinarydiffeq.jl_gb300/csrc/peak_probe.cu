// Scalar-pipe peak probe: the roofline denominator for the integrator kernels,
// which are bound by the FP64 (plain) or FP32 (mixed) FMA pipe, not by HBM or
// the tensor cores.  Each thread runs 8 independent FMA chains so the pipe,
// not latency, limits the rate; grid = 8 x SM count x 4 blocks of 256.
#include "ode_gb300.h"

#include <cuda_runtime.h>

namespace {

template <class T>
__global__ void fma_chains(T* out, int iters, T a, T b) {
    T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == (T)-1.2345) out[blockIdx.x] = s;  // keeps the chains live; never true for these inputs
}

template <class T>
int run(int device, double* flops) {
    cudaSetDevice(device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * 65536) != cudaSuccess) return ODE_E_NOMEM;
    const int block = 256, grid = sms * 4 * 8;
    const int iters = sizeof(T) == 8 ? 2048 : 65536;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T><<<grid, block>>>(out, iters / 8, (T)0.999999, (T)1e-7);  // warm-up
    cudaEventRecord(e0);
    fma_chains<T><<<grid, block>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0) return ODE_E_CUDA;
    *flops = 2.0 * 8.0 * (double)iters * (double)grid * (double)block / (ms * 1e-3);
    return ODE_OK;
}

}  // namespace

extern "C" int ode_measure_fma_peak(int device, int precision, double* flops_per_s) {
    if (!flops_per_s) return ODE_E_INVALID;
    return precision == ODE_PREC_FP64 ? run<double>(device, flops_per_s) : run<float>(device, flops_per_s);
}
