// FP64 pipe throughput probe: the roofline denominator for the FP64-bound
// RHS kernels (the measured-peaks file of the target machines records HBM
// copy and bf16 GEMM rates only).  Each thread runs 8 independent DFMA
// chains; the result is checked on the host so the work cannot be elided.
#include <cuda_runtime.h>

#include "dgb_internal.h"

namespace dgb {
namespace {

__global__ void __launch_bounds__(256) dfma_kernel(double *out, int iters, double a, double b)
{
    double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
    double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int r = 0; r < 8; r++) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace
}  // namespace dgb

extern "C" dgb_status dgb_measure_fp64_peak(double *gflops, double *ms_out)
{
    using namespace dgb;
    if (!gflops) return DGB_ERR_INVALID;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return DGB_ERR_NOT_INIT;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = nsm * 8, threads = 256, iters = 4096;
    double *d = nullptr;
    if (cudaMalloc(&d, sizeof(double) * blocks * threads) != cudaSuccess) return DGB_ERR_ALLOC;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        cudaEventRecord(e0);
        dfma_kernel<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (err != cudaSuccess) {
        set_error(std::string("fp64 probe: ") + cudaGetErrorString(err));
        return DGB_ERR_CUDA;
    }
    const double flops = 2.0 * 64.0 * iters * (double)blocks * threads;
    *gflops = flops / (best * 1e-3) / 1e9;
    if (ms_out) *ms_out = best;
    return DGB_OK;
}
