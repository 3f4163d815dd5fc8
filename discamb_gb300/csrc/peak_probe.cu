// FP32 FMA throughput probe: the denominator of the roofline fraction of
// the FP32-bulk kernel (an FP32 CUDA-core bound kernel; the measured-peaks
// file of the pool lists HBM bandwidth and tensor-core throughput only).
// Each thread runs 8 independent FMA chains; the result is written so the
// chains are not removed.  Host entry returns the best of several runs.
#include <cuda_runtime.h>

__global__ void fma_chains(float *out, int iters, float a, float b)
{
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
    float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 16; k++) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

extern "C" int dsf_probe_fp32_tflops(int device, double *tflops)
{
    if (cudaSetDevice(device) != cudaSuccess) return 1;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int threads = 256, blocks = sms * 8, iters = 4096;
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * threads * blocks) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 6; rep++) {
        cudaEventRecord(e0);
        fma_chains<<<blocks, threads>>>(out, iters, 0.9999f, 1e-4f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
        if (rep > 0 && ms > 0) best = best > flops / (ms * 1e-3) ? best : flops / (ms * 1e-3);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    *tflops = best * 1e-12;
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
