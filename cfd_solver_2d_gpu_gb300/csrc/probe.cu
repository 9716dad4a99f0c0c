// FP64 arithmetic throughput of the device (fvgb_fp64_peak): the roofline
// denominator for kernels bound by the FP64 pipe, measured rather than quoted.
// No counterpart in the reference.
//
// Each thread runs eight independent FMA chains on registers; the only memory
// access is one store per thread into a buffer of exactly grid * block doubles.
#include <cuda_runtime.h>

#include <string>

#include "internal.h"
#include "physics.cuh"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fma_chain(double* __restrict__ out, int iters, double a, double b) {
    double x[kChains];
#pragma unroll
    for (int j = 0; j < kChains; j++) x[j] = threadIdx.x + j;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < kChains; j++) x[j] = fma(x[j], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < kChains; j++) s += x[j];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// the library's reciprocal on n values
__global__ void k_math_eval(const double* __restrict__ x, double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = fvgb::dev::rcp(x[i]);
}

}  // namespace

#define PK(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            if (buf) cudaFree(buf);                                                                     \
            if (e0) cudaEventDestroy(e0);                                                               \
            if (e1) cudaEventDestroy(e1);                                                               \
            return fvgb::fail(FVGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
        }                                                                                               \
    } while (0)

extern "C" int fvgb_fp64_peak(int device, double* gflops) {
    if (!gflops) return fvgb::fail(FVGB_ERR_ARG, "gflops is NULL");
    double* buf = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PK(cudaSetDevice(device));
    int sms = 0;
    PK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    const int grid = sms * 8, iters = 4096;
    PK(cudaMalloc(&buf, sizeof(double) * (size_t)grid * kThreads));
    PK(cudaEventCreate(&e0));
    PK(cudaEventCreate(&e1));
    k_fma_chain<<<grid, kThreads>>>(buf, 64, 0.999, 1e-3);  // warm-up
    PK(cudaGetLastError());
    float best = 0.0f;
    for (int rep = 0; rep < 3; rep++) {
        PK(cudaEventRecord(e0));
        k_fma_chain<<<grid, kThreads>>>(buf, iters, 0.999, 1e-3);
        PK(cudaEventRecord(e1));
        PK(cudaEventSynchronize(e1));
        float ms = 0.0f;
        PK(cudaEventElapsedTime(&ms, e0, e1));
        if (rep == 0 || ms < best) best = ms;
    }
    PK(cudaGetLastError());
    cudaFree(buf);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flop = 2.0 * kChains * (double)iters * grid * kThreads;  // an FMA is two flops
    *gflops = flop / (best * 1e-3) / 1e9;
    return 0;
}

// No counterpart in the reference: the device reciprocal rcp (physics.cuh) evaluated on
// n host values, for accuracy tests against correctly rounded results.
extern "C" int fvgb_math_eval(int device, int n, const double* x, double* out) {
    if (n < 0 || (n > 0 && (!x || !out))) return fvgb::fail(FVGB_ERR_ARG, "fvgb_math_eval: bad arguments");
    if (n == 0) return 0;
    double* buf = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PK(cudaSetDevice(device));
    PK(cudaMalloc(&buf, sizeof(double) * 2 * (size_t)n));
    PK(cudaMemcpy(buf, x, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
    k_math_eval<<<(n + 255) / 256, 256>>>(buf, buf + n, n);
    PK(cudaGetLastError());
    PK(cudaMemcpy(out, buf + n, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
    cudaFree(buf);
    return 0;
}
