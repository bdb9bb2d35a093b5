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

// set_velocity_to_temperature (fortran/system.f90:361-421) in two passes over
// the particles, each drawing particle I's three normals from counter
// (I, int(T*1000), seed, 42) under the default key (1-based I, as the
// reference's loop). Pass 1 sums the normals and their squares in FP64 (the
// finishing block stores the four totals in out); pass 2 draws them again and
// writes (v - v_com) * factor rounded once to FP32, the inverse mass in vel.w
// kept. sum |v - c|^2 is taken as sum |v|^2 - N |c|^2 with c = sum v / N: the
// subtracted term is about 1/N of the sum, so nothing cancels.
__global__ void k_vinit_sums(int n, uint32_t tint, uint32_t seed, double* partials, unsigned int* done, double* out) {
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double a, b, c;
        sg_normal_3seq((uint32_t)(i + 1), tint, seed, 42u, SG_PHILOX_KEY0, SG_PHILOX_KEY1, a, b, c);
        v[0] += a;
        v[1] += b;
        v[2] += c;
        v[3] += a * a + b * b + c * c;
    }
    block_reduce_finish<4>(v, partials, done, out, nullptr, true);
}

// dof_t = n_dof * T * Nrigid (the reference's product order)
__global__ void k_vinit_write(int n, uint32_t tint, uint32_t seed, const double* __restrict__ sums, double dof_t,
                              int remove_com, float4* __restrict__ vel) {
    double cx = 0.0, cy = 0.0, cz = 0.0;
    if (remove_com) {
        cx = sums[0] / (double)n;
        cy = sums[1] / (double)n;
        cz = sums[2] / (double)n;
    }
    const double factor = sqrt(dof_t / (sums[3] - (double)n * (cx * cx + cy * cy + cz * cz)));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double a, b, c;
        sg_normal_3seq((uint32_t)(i + 1), tint, seed, 42u, SG_PHILOX_KEY0, SG_PHILOX_KEY1, a, b, c);
        const float w = vel[i].w;
        vel[i] = make_float4((float)((a - cx) * factor), (float)((b - cy) * factor), (float)((c - cz) * factor), w);
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

int sg_set_velocity_to_temperature(sg_ctx* ctx, double rtemp, int32_t seed, int32_t remove_com, int32_t nrigid) {
    if (!ctx) return SG_EINVAL;
    if (ctx->nrep > 0) return sg_fail(ctx, SG_EINVAL, "sg_set_velocity_to_temperature takes a single system");
    if (ctx->n < 1) return sg_fail(ctx, SG_EINVAL, "the system has no particles");
    if (remove_com && ctx->n < 2) return sg_fail(ctx, SG_EINVAL, "removing the mean velocity needs two particles");
    if (!(rtemp > 0.0 && rtemp * 1000.0 < 2147483647.0) || nrigid < 1)
        return sg_fail(ctx, SG_EINVAL, "rtemp must be in (0, 2147483.647) and nrigid >= 1");
    const int64_t ndof = 6 * (int64_t)ctx->n - ctx->con_n - (remove_com ? 3 : 0);
    if (ndof <= 0) return sg_fail(ctx, SG_EINVAL, "6N - NC%s leaves no degrees of freedom", remove_com ? " - 3" : "");
    const uint32_t tint = (uint32_t)(int32_t)(rtemp * 1000.0), useed = (uint32_t)seed;
    const int grid = std::min(1024, (ctx->n + 255) / 256);
    if (int rc = sg_ensure_partials(ctx, 4 * 1024 + 4)) return rc;
    double* sums = ctx->partials + 4 * 1024;   // after the block partials of pass 1
    k_vinit_sums<<<grid, 256, 0, ctx->stream>>>(ctx->n, tint, useed, ctx->partials, ctx->done_counter, sums);
    SG_LAUNCH_CHECK(ctx, "k_vinit_sums");
    const double dof_t = (double)ndof * rtemp * (double)nrigid;
    k_vinit_write<<<grid, 256, 0, ctx->stream>>>(ctx->n, tint, useed, sums, dof_t, remove_com ? 1 : 0, ctx->vel);
    SG_LAUNCH_CHECK(ctx, "k_vinit_write");
    sg_state_touched(ctx);
    return SG_OK;
}

}  // extern "C"
