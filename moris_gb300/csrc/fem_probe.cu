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

namespace {

// m8n8k4 FP64 tensor-core MMA (PTX ISA mma.sync.aligned.m8n8k4.row.col.f64):
// 256 FMAs per warp instruction; four independent accumulators per warp.
__device__ __forceinline__ void dmma(double& d0, double& d1, double a, double b) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                 : "+d"(d0), "+d"(d1)
                 : "d"(a), "d"(b));
}

// mixed: warps with (warp & 1) == 0 issue DMMA, odd warps DFMA chains when
// mixed != 0; otherwise every warp issues DMMA
__global__ void dmma_kernel(double* out, int iters, int mixed) {
    const int warp = threadIdx.x >> 5;
    if (mixed && (warp & 1)) {
        double x[kChains];
        for (int k = 0; k < kChains; ++k) x[k] = threadIdx.x * 1e-3 + k;
        for (int i = 0; i < iters * 4; ++i) {
#pragma unroll
            for (int k = 0; k < kChains; ++k) x[k] = fma(x[k], 0.999999, 1e-7);
        }
        double s = 0.0;
        for (int k = 0; k < kChains; ++k) s += x[k];
        if (s == 12345.678) out[0] = s;
        return;
    }
    double c[8];
    for (int k = 0; k < 8; ++k) c[k] = 0.0;
    const double a = 1e-3 * (threadIdx.x & 7), b = 0.5;
    for (int i = 0; i < iters; ++i) {
        dmma(c[0], c[1], a, b);
        dmma(c[2], c[3], a, b);
        dmma(c[4], c[5], a, b);
        dmma(c[6], c[7], a, b);
    }
    double s = 0.0;
    for (int k = 0; k < 8; ++k) s += c[k];
    if (s == 12345.678) out[0] = s;
}

}  // namespace

extern "C" fem_gpu_status fem_gpu_probe_dmma_tflops(int32_t iters, int32_t mixed, double* tflops) {
    if (!tflops || iters < 1) return FEM_GPU_BAD_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return FEM_GPU_NO_DEVICE;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return FEM_GPU_OUT_OF_MEMORY;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 4, threads = 256;
    dmma_kernel<<<blocks, threads>>>(out, 16, mixed);
    cudaEventRecord(e0);
    dmma_kernel<<<blocks, threads>>>(out, iters, mixed);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return FEM_GPU_CUDA_ERROR;
    const double warps = (double)blocks * (threads / 32);
    double flops;
    if (mixed)  // half the warps: 4 DMMA x 256 FMA per iteration; other half: 8 chains x 4 x iters FMA x 32 lanes
        flops = 2.0 * (warps / 2) * iters * 4 * 256 + 2.0 * (warps / 2) * 32 * kChains * 4.0 * iters;
    else
        flops = 2.0 * warps * iters * 4 * 256;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return FEM_GPU_OK;
}
