// FP32 FFMA issue-rate probe: the denominator of the mixed walk's roofline.
// Eight independent FMA chains per thread, enough blocks to fill every SM.
#include <cuda_runtime.h>

#include "idwarp_gb300.h"

namespace {

__global__ void k_ffma(float *out, int iters) {
    float a0 = threadIdx.x * 1e-3f, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f;
    float a4 = a0 + 4.f, a5 = a0 + 5.f, a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float b = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a0 = fmaf(a0, b, c);
            a1 = fmaf(a1, b, c);
            a2 = fmaf(a2, b, c);
            a3 = fmaf(a3, b, c);
            a4 = fmaf(a4, b, c);
            a5 = fmaf(a5, b, c);
            a6 = fmaf(a6, b, c);
            a7 = fmaf(a7, b, c);
        }
    }
    float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" int idw_probe_ffma(void *stream, int device, double *tflops) {
    (void)device;
    if (!tflops) return IDW_ERR_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return IDW_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return IDW_ERR_CUDA;
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * 64 * sms) != cudaSuccess) return IDW_ERR_NOMEM;
    const int threads = 256, blocksPerSm = 8, iters = 8192;
    const int grid = blocksPerSm * sms;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_ffma<<<grid, threads, 0, st>>>(out, 64);  // warm-up
    cudaEventRecord(e0, st);
    k_ffma<<<grid, threads, 0, st>>>(out, iters);
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess || ms <= 0.f) return IDW_ERR_CUDA;
    double flops = 2.0 * 8.0 * 4.0 * double(iters) * double(grid) * double(threads);
    *tflops = flops / (double(ms) * 1e-3) / 1e12;
    return IDW_OK;
}
