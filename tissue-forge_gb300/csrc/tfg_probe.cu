// FP32 CUDA-core throughput probe: the roofline denominator for the pair pass, which is
// bound by FP32 issue rather than by HBM or tensor cores.  Each thread runs eight
// independent FMA chains so the pipe stays full; the result is 2 * FMAs / time.
#include <cuda_runtime.h>

#include "tfg.h"

namespace {

constexpr int kIters = 8192;

__global__ void k_ffma(float *out, float a, float b) {
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
          x7 = x0 + 7;
#pragma unroll 16
    for (int k = 0; k < kIters; k++) {
        x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
        x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
    float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 1234.5f) out[blockIdx.x] = s;   // keep the chains live
}

}  // namespace

extern "C" TFG_API int tfg_probe_fp32_tflops(int device, double *tflops) {
    if (!tflops) return TFG_E_INVAL;
    if (cudaSetDevice(device) != cudaSuccess) return TFG_E_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float) * 65536) != cudaSuccess) return TFG_E_OOM;
    const int blocks = sms * 8, threads = 256;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_ffma<<<blocks, threads>>>(out, 0.9999f, 0.0001f);   // warm-up
    float best = 1e30f;
    for (int r = 0; r < 5; r++) {
        cudaEventRecord(e0);
        k_ffma<<<blocks, threads>>>(out, 0.9999f, 0.0001f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (cudaGetLastError() != cudaSuccess) return TFG_E_CUDA;
    const double flops = 2.0 * 8.0 * kIters * (double)blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return TFG_OK;
}
