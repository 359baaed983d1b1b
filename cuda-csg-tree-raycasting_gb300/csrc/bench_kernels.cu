// Measurement helper: the FP32 FMA issue rate of the GPU, the denominator of the FP32
// roofline the ray-casting kernels are reported against.
#include <cuda_runtime.h>

#include "csgrt.h"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) fma_rate_kernel(float* out, int iters, float a, float b)
{
    float x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = (float)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) x[k] = __fmaf_rn(x[k], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += x[k];
    if (s == 1234.5f) out[0] = s;  // keeps the chains alive; never true for these inputs
}

}  // namespace

extern "C" int csg_probe_fp32_peak(float* tflops, float* ms)
{
    if (!tflops) return CSG_E_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return CSG_E_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return CSG_E_CUDA;
    float* d = nullptr;
    if (cudaMalloc(&d, sizeof(float)) != cudaSuccess) return CSG_E_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256, iters = 1 << 14;
    fma_rate_kernel<<<blocks, threads>>>(d, 256, 0.999f, 0.001f);  // warm-up
    cudaEventRecord(e0);
    fma_rate_kernel<<<blocks, threads>>>(d, iters, 0.999f, 0.001f);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float t = 0.f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (err != cudaSuccess || t <= 0.f) return CSG_E_CUDA;
    const double flops = 2.0 * kChains * (double)iters * threads * blocks;
    *tflops = (float)(flops / (t * 1e-3) / 1e12);
    if (ms) *ms = t;
    return CSG_OK;
}
