// Throughput probes for the roofline denominators of the FP32-pipe kernels
// (the measured peaks at hand cover only HBM and BF16 tensor throughput):
// dependent-chain-free FMA loops in FP32 and FP64, timed with CUDA events on
// the context stream.
#include "sg_internal.cuh"

namespace {

template <class T>
__global__ void __launch_bounds__(256) k_fma(T* out, int iters, T b, T c) {
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = (T)(threadIdx.x + k) * (T)1e-3;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = a[k] * b + c;
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == (T)12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the loop alive
}

template <class T>
int run(sg_ctx* ctx, int iters, double* tflops) {
    const int block = 256, grid = ctx->num_sms * 8;
    T* out = nullptr;
    SG_CUDA(ctx, cudaMallocAsync(&out, sizeof(T) * (size_t)grid * block, ctx->stream));
    cudaEvent_t a, b;
    SG_CUDA(ctx, cudaEventCreate(&a));
    SG_CUDA(ctx, cudaEventCreate(&b));
    k_fma<T><<<grid, block, 0, ctx->stream>>>(out, iters / 10, (T)0.999, (T)1e-4);  // warm-up
    SG_CUDA(ctx, cudaEventRecord(a, ctx->stream));
    k_fma<T><<<grid, block, 0, ctx->stream>>>(out, iters, (T)0.999, (T)1e-4);
    SG_CUDA(ctx, cudaEventRecord(b, ctx->stream));
    SG_CUDA(ctx, cudaEventSynchronize(b));
    float ms = 0.f;
    SG_CUDA(ctx, cudaEventElapsedTime(&ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    SG_CUDA(ctx, cudaFreeAsync(out, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const double flops = 2.0 * 8.0 * (double)iters * (double)grid * block;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return SG_OK;
}

}  // namespace

extern "C" int sg_peak_fma(sg_ctx* ctx, int32_t fp64, double* tflops) {
    if (!ctx || !tflops) return SG_EINVAL;
    return fp64 ? run<double>(ctx, 1 << 14, tflops) : run<float>(ctx, 1 << 16, tflops);
}
