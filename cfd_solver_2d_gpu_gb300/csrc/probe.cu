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
#include "softfp64.cuh"

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

// the library's reciprocal (op 0), reciprocal square root (1) or square root (2) on n values
__global__ void k_math_eval(int op, const double* __restrict__ x, double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = op == 0 ? fvgb::dev::rcp(x[i]) : (op == 1 ? fvgb::dev::rsq(x[i]) : fvgb::dev::sq(x[i]));
}

// Throughput of correctly rounded FP64 multiply (OP 0) or add (OP 1): HW independent chains
// on the FP64 pipe and SW chains through the integer-pipe versions of softfp64.cuh, in the
// same thread, so that a launch with both measures how far the two run side by side.
template <int OP, int HW, int SW>
__global__ void __launch_bounds__(kThreads) k_soft_chain(double* __restrict__ out, int iters, double c) {
    double x[HW + SW > 0 ? HW + SW : 1];
#pragma unroll
    for (int j = 0; j < HW + SW; j++) x[j] = 1.0 + threadIdx.x + j;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < HW; j++) x[j] = OP == 0 ? __dmul_rn(x[j], c) : __dadd_rn(x[j], c);
#pragma unroll
        for (int j = HW; j < HW + SW; j++) x[j] = OP == 0 ? fvgb::soft::dmul(x[j], c) : fvgb::soft::dadd(x[j], c);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < HW + SW; j++) s += x[j];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// a op b on n pairs, by the integer-pipe version and by the hardware instruction
__global__ void k_soft_eval(int op, const double* __restrict__ a, const double* __restrict__ b,
                            double* __restrict__ soft, double* __restrict__ hw, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = a[i], y = b[i];
    soft[i] = op == 0 ? fvgb::soft::dmul(x, y) : fvgb::soft::dadd(x, y);
    hw[i] = op == 0 ? __dmul_rn(x, y) : __dadd_rn(x, y);
}

template <int OP, int HW, int SW>
int time_chain(int grid, int iters, double c, double* buf, cudaEvent_t e0, cudaEvent_t e1, double* gops) {
    k_soft_chain<OP, HW, SW><<<grid, kThreads>>>(buf, 16, c);  // warm-up
    float best = 0.0f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        k_soft_chain<OP, HW, SW><<<grid, kThreads>>>(buf, iters, c);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) return -1;
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep == 0 || ms < best) best = ms;
    }
    if (cudaGetLastError() != cudaSuccess) return -1;
    *gops = (double)(HW + SW) * iters * grid * kThreads / (best * 1e-3) / 1e9;
    return 0;
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

// No counterpart in the reference: the device reciprocal rcp, reciprocal square root rsq or
// square root sq (physics.cuh; op 0, 1, 2) evaluated on n host values, for accuracy tests
// against correctly rounded results.
extern "C" int fvgb_math_eval(int device, int op, int n, const double* x, double* out) {
    if (n < 0 || op < 0 || op > 2 || (n > 0 && (!x || !out)))
        return fvgb::fail(FVGB_ERR_ARG, "fvgb_math_eval: bad arguments");
    if (n == 0) return 0;
    double* buf = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PK(cudaSetDevice(device));
    PK(cudaMalloc(&buf, sizeof(double) * 2 * (size_t)n));
    PK(cudaMemcpy(buf, x, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
    k_math_eval<<<(n + 255) / 256, 256>>>(op, buf, buf + n, n);
    PK(cudaGetLastError());
    PK(cudaMemcpy(out, buf + n, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
    cudaFree(buf);
    return 0;
}

// No counterpart in the reference: the integer-pipe FP64 multiply / add (softfp64.cuh, op 0 /
// 1) and the hardware instruction on the same n pairs, on the given device, for bitwise tests.
extern "C" int fvgb_softfp64_eval(int device, int op, int n, const double* a, const double* b, double* soft,
                                  double* hw) {
    if (n < 0 || (op != 0 && op != 1) || (n > 0 && (!a || !b || !soft || !hw)))
        return fvgb::fail(FVGB_ERR_ARG, "fvgb_softfp64_eval: bad arguments");
    if (n == 0) return 0;
    double* buf = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PK(cudaSetDevice(device));
    PK(cudaMalloc(&buf, sizeof(double) * 4 * (size_t)n));
    PK(cudaMemcpy(buf, a, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
    PK(cudaMemcpy(buf + n, b, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
    k_soft_eval<<<(n + 255) / 256, 256>>>(op, buf, buf + n, buf + 2 * (size_t)n, buf + 3 * (size_t)n, n);
    PK(cudaGetLastError());
    PK(cudaMemcpy(soft, buf + 2 * (size_t)n, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
    PK(cudaMemcpy(hw, buf + 3 * (size_t)n, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
    cudaFree(buf);
    return 0;
}

// No counterpart in the reference: the same functions compiled for the host, for CPU tests.
extern "C" int fvgb_softfp64_host(int op, int n, const double* a, const double* b, double* out) {
    if (n < 0 || (op != 0 && op != 1) || (n > 0 && (!a || !b || !out)))
        return fvgb::fail(FVGB_ERR_ARG, "fvgb_softfp64_host: bad arguments");
    for (int i = 0; i < n; i++) out[i] = op == 0 ? fvgb::soft::dmul(a[i], b[i]) : fvgb::soft::dadd(a[i], b[i]);
    return 0;
}

// No counterpart in the reference: G operations/s of independent FP64 chains (8 per thread):
// out[0..3] multiply on the FP64 pipe alone, on the integer pipes alone, 4 + 4 and 2 + 6 side by
// side; out[4..7] the same for add (the last 6 + 2); out[8] the SM count and out[9] the maximum
// SM clock in MHz, for operations per SM per cycle.
extern "C" int fvgb_softfp64_rate(int device, double out[10]) {
    if (!out) return fvgb::fail(FVGB_ERR_ARG, "out is NULL");
    double* buf = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    PK(cudaSetDevice(device));
    int sms = 0, khz = 0;
    PK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    PK(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, device));
    const int grid = sms * 8, iters = 2048;
    PK(cudaMalloc(&buf, sizeof(double) * (size_t)grid * kThreads));
    PK(cudaEventCreate(&e0));
    PK(cudaEventCreate(&e1));
    int rc = 0;
    rc |= time_chain<0, 8, 0>(grid, iters, 1.0000001, buf, e0, e1, &out[0]);
    rc |= time_chain<0, 0, 8>(grid, iters, 1.0000001, buf, e0, e1, &out[1]);
    rc |= time_chain<0, 4, 4>(grid, iters, 1.0000001, buf, e0, e1, &out[2]);
    rc |= time_chain<0, 2, 6>(grid, iters, 1.0000001, buf, e0, e1, &out[3]);
    rc |= time_chain<1, 8, 0>(grid, iters, 1e-3, buf, e0, e1, &out[4]);
    rc |= time_chain<1, 0, 8>(grid, iters, 1e-3, buf, e0, e1, &out[5]);
    rc |= time_chain<1, 4, 4>(grid, iters, 1e-3, buf, e0, e1, &out[6]);
    rc |= time_chain<1, 6, 2>(grid, iters, 1e-3, buf, e0, e1, &out[7]);
    cudaFree(buf);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return fvgb::fail(FVGB_ERR_CUDA, "fvgb_softfp64_rate: a timed launch failed");
    out[8] = sms;
    out[9] = khz / 1e3;
    return 0;
}
