// Measurement helpers that need no context: the FP32 FMA rate of the GPU, the
// denominator of the neighbour sweeps' secondary (arithmetic) roofline.
#include <cuda_runtime.h>

#include <cstdio>

#include "ctx.h"

namespace tsph {

void set_last_error_text(const char *msg);  // api.cu

constexpr int kFmaChains = 8;     // independent chains per thread (covers the FMA latency)
constexpr int kFmaBlock = 256;
constexpr int kFmaBlocksPerSM = 8;  // 2048 threads per SM

__global__ void __launch_bounds__(kFmaBlock) k_fma_chains(float *sink, int iters, float a, float b) {
    float x[kFmaChains];
#pragma unroll
    for (int i = 0; i < kFmaChains; ++i) x[i] = (float)threadIdx.x * 1e-3f + (float)i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kFmaChains; ++i) x[i] = fmaf(x[i], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < kFmaChains; ++i) s += x[i];
    if (s == -1.f) sink[blockIdx.x] = s;  // never true (the chains stay positive); keeps them live
}

}  // namespace tsph

using namespace tsph;

extern "C" int tsph_fp32_fma_peak(double *tflops_out, void *stream) {
    if (!tflops_out) {
        set_last_error_text("tsph_fp32_fma_peak: null output");
        return TSPH_ERR_INVALID;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *sink = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(float) * (size_t)sms * kFmaBlocksPerSM);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    const int blocks = sms * kFmaBlocksPerSM, iters = 4096;
    double best = 0.0;
    for (int rep = 0; rep < 6 && e == cudaSuccess; ++rep) {
        cudaEventRecord(e0, st);
        k_fma_chains<<<blocks, kFmaBlock, 0, st>>>(sink, iters, 0.999f, 1e-4f);
        cudaEventRecord(e1, st);
        e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e == cudaSuccess && rep > 0 && ms > 0.f) {  // the first launch warms up
            const double flops = 2.0 * kFmaChains * (double)iters * blocks * kFmaBlock;
            const double tf = flops / (ms * 1e-3) / 1e12;
            if (tf > best) best = tf;
        }
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (sink) cudaFree(sink);
    if (e != cudaSuccess) {
        char msg[200];
        std::snprintf(msg, sizeof(msg), "tsph_fp32_fma_peak: %s", cudaGetErrorString(e));
        set_last_error_text(msg);
        return TSPH_ERR_CUDA;
    }
    *tflops_out = best;
    return TSPH_OK;
}
