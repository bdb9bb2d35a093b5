// Philox4x32-10 entry points: a host copy of the block function and two
// device kernels that fill counters supplied by the caller.
#include "sg_internal.cuh"
#include "philox.cuh"

__global__ void k_philox(int64_t n, const uint4* __restrict__ ctr, uint32_t k0, uint32_t k1, uint4* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint4 c = ctr[i];
        sg_u4 w = sg_philox(c.x, c.y, c.z, c.w, k0, k1);
        out[i] = make_uint4(w.x, w.y, w.z, w.w);
    }
}

__global__ void k_normal3(int64_t n, const int4* __restrict__ ctr, double* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int4 c = ctr[i];
        double a, b, d;
        sg_normal_3seq((uint32_t)c.x, (uint32_t)c.y, (uint32_t)c.z, (uint32_t)c.w, SG_PHILOX_KEY0, SG_PHILOX_KEY1, a, b, d);
        out[3 * i] = a;
        out[3 * i + 1] = b;
        out[3 * i + 2] = d;
    }
}

extern "C" {

void sg_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t k0 = key ? key[0] : SG_PHILOX_KEY0, k1 = key ? key[1] : SG_PHILOX_KEY1;
    sg_u4 w = sg_philox(ctr[0], ctr[1], ctr[2], ctr[3], k0, k1);
    out[0] = w.x; out[1] = w.y; out[2] = w.z; out[3] = w.w;
}

int sg_philox4x32_device(sg_ctx* ctx, int64_t n, const uint32_t* ctr, const uint32_t key[2], uint32_t* out) {
    if (!ctx || n < 0 || (n > 0 && (!ctr || !out))) return SG_EINVAL;
    if (n == 0) return SG_OK;
    uint4 *dc = nullptr, *dout = nullptr;
    SG_CUDA(ctx, cudaMallocAsync(&dc, sizeof(uint4) * n, ctx->stream));
    SG_CUDA(ctx, cudaMallocAsync(&dout, sizeof(uint4) * n, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(dc, ctr, sizeof(uint4) * n, cudaMemcpyHostToDevice, ctx->stream));
    uint32_t k0 = key ? key[0] : SG_PHILOX_KEY0, k1 = key ? key[1] : SG_PHILOX_KEY1;
    int grid = (int)std::min<int64_t>((n + 255) / 256, 8 * (int64_t)ctx->num_sms);
    k_philox<<<grid, 256, 0, ctx->stream>>>(n, dc, k0, k1, dout);
    SG_LAUNCH_CHECK(ctx, "k_philox");
    SG_CUDA(ctx, cudaMemcpyAsync(out, dout, sizeof(uint4) * n, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaFreeAsync(dc, ctx->stream));
    SG_CUDA(ctx, cudaFreeAsync(dout, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_philox_normal_3seq_device(sg_ctx* ctx, int64_t n, const int32_t* ctr, double* out) {
    if (!ctx || n < 0 || (n > 0 && (!ctr || !out))) return SG_EINVAL;
    if (n == 0) return SG_OK;
    int4* dc = nullptr;
    double* dout = nullptr;
    SG_CUDA(ctx, cudaMallocAsync(&dc, sizeof(int4) * n, ctx->stream));
    SG_CUDA(ctx, cudaMallocAsync(&dout, sizeof(double) * 3 * n, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(dc, ctr, sizeof(int4) * n, cudaMemcpyHostToDevice, ctx->stream));
    int grid = (int)std::min<int64_t>((n + 255) / 256, 8 * (int64_t)ctx->num_sms);
    k_normal3<<<grid, 256, 0, ctx->stream>>>(n, dc, dout);
    SG_LAUNCH_CHECK(ctx, "k_normal3");
    SG_CUDA(ctx, cudaMemcpyAsync(out, dout, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaFreeAsync(dc, ctx->stream));
    SG_CUDA(ctx, cudaFreeAsync(dout, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

}  // extern "C"
