// fem_probe.cu -- in-run peak probes used as roofline denominators: an FP64
// FMA-chain kernel (independent dependency chains per thread, enough warps
// per SM to cover the FMA latency) timed with CUDA events.
#include <cuda_runtime.h>

#include "fem_internal.hpp"

namespace {

constexpr int kChains = 8;

__global__ void fma_chain_kernel(double* out, int iters, double a, double b) {
    double x[kChains];
    for (int k = 0; k < kChains; ++k) x[k] = threadIdx.x * 1e-3 + k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
    for (int k = 0; k < kChains; ++k) s += x[k];
    if (s == 12345.678) out[0] = s;  // keeps the chains alive
}

}  // namespace

extern "C" fem_gpu_status fem_gpu_probe_fp64_tflops(int32_t iters, double* tflops) {
    if (!tflops || iters < 1) return FEM_GPU_BAD_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FEM_GPU_NO_DEVICE;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return FEM_GPU_OUT_OF_MEMORY;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    fma_chain_kernel<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);  // warm-up
    cudaEventRecord(e0);
    fma_chain_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    const double flops = 2.0 * kChains * (double)iters * blocks * threads;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return FEM_GPU_OK;
}
