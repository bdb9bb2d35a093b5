// Pair-force entry points of the C ABI, and the MLP weight store.
#include <cmath>
#include <vector>

#include <cuda_bf16.h>

#include "sg_internal.cuh"
#include "ecp_mlp.cuh"

namespace {

int launch_forces(sg_ctx* ctx, const sg_pair_params* p) {
    if (!ctx || !p) return SG_EINVAL;
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "pair forces need sg_nlist_init first");
    if (!ctx->step_fused) {   // the fused step's initial half step zeroed them
        SG_CUDA(ctx, cudaMemsetAsync(ctx->acc + 4, 0, sizeof(double) * 2, ctx->stream));
        SG_CUDA(ctx, cudaMemsetAsync(ctx->stats, 0, sizeof(unsigned long long) * 32, ctx->stream));
    }
    ctx->launch_family = p->kind < 10 ? 0 : (p->kind < 20 ? 1 : 2);
    if (ctx->nrep && ctx->fam_pstart[ctx->launch_family] == ctx->fam_pstart[ctx->launch_family + 1])
        return SG_OK;   // no replica of this family
    switch (p->kind) {
        case SG_LJ: case SG_LJ12: case SG_LJW: case SG_WCA: return sg_launch_pair_simple(ctx, p);
        case SG_MORSE: case SG_DH: case SG_COULOMB: case SG_DIPOLE: return sg_launch_pair_elec(ctx, p);
        case SG_GB: case SG_GBR: case SG_GBW: case SG_GBC: case SG_GBWC: return sg_launch_pair_gb(ctx, p);
        case SG_ECP: case SG_ECPR: case SG_ECPW: case SG_ECPC: case SG_ECPWC: return sg_launch_pair_ecp(ctx, p);
        default: return sg_fail(ctx, SG_EINVAL, "unknown pair kind %d", p->kind);
    }
}

__global__ void k_to_bf16(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

}  // namespace

extern "C" {

int sg_pair_forces_async(sg_ctx* ctx, const sg_pair_params* params) { return launch_forces(ctx, params); }

int sg_pair_forces(sg_ctx* ctx, const sg_pair_params* params, double* pot_eng, double* virial, sg_ecp_stats* stats) {
    if (int rc = launch_forces(ctx, params)) return rc;
    double e[2];
    int flags[4];
    unsigned long long st[32];
    SG_CUDA(ctx, cudaMemcpyAsync(e, ctx->acc + 4, sizeof(e), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(flags, ctx->nl.dev_flags, sizeof(flags), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(st, ctx->stats, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (pot_eng) *pot_eng += e[0];
    if (virial) *virial += e[1];
    if (stats) {
        stats->pairs = (int64_t)st[0];
        stats->solver_evals = (int64_t)st[1];
        stats->nonconverged = (int64_t)st[2];
        stats->fallbacks = (int64_t)st[3];
        for (int k = 0; k < 24; ++k) stats->iter_hist[k] = (int64_t)st[4 + k];
        stats->fp64_refined = (int64_t)st[28];
    }
    if (flags[1]) return sg_fail(ctx, SG_ECAPACITY, "neighbour list overflowed (row of %d); call sg_nlist_build", flags[1]);
    if (!std::isfinite(e[0])) return sg_fail(ctx, SG_ENAN, "non-finite potential energy");
    if (st[2]) return sg_fail(ctx, SG_ENOCONV, "%llu pairs did not converge", (unsigned long long)st[2]);
    return SG_OK;
}

int sg_ecp_lambda(sg_ctx* ctx, float* lam, int64_t capacity) {
    if (!ctx || !lam) return SG_EINVAL;
    int64_t k = 0;
    if (int rc = sg_nlist_count(ctx, &k)) return rc;
    if (!ctx->ecp_lambda) return sg_fail(ctx, SG_ENOTREADY, "no ECP call yet");
    if (capacity < k) return sg_fail(ctx, SG_ECAPACITY, "lambda capacity too small");
    return sg_gather_pair_floats(ctx, ctx->ecp_lambda, k, lam);
}

int64_t sg_mlp_weight_count(void) { return SG_MLP_NPARAM; }

int sg_mlp_set_weights(sg_ctx* ctx, const float* w, int64_t count) {
    if (!ctx || !w || count != SG_MLP_NPARAM) return SG_EINVAL;
    if (!ctx->mlp_w) SG_CUDA(ctx, cudaMalloc(&ctx->mlp_w, sizeof(float) * SG_MLP_NPARAM));
    if (!ctx->mlp_wbf16) SG_CUDA(ctx, cudaMalloc(&ctx->mlp_wbf16, sizeof(__nv_bfloat16) * (64 * 16 + 2 * 64 * 64)));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->mlp_w, w, sizeof(float) * SG_MLP_NPARAM, cudaMemcpyHostToDevice, ctx->stream));
    __nv_bfloat16* wb = (__nv_bfloat16*)ctx->mlp_wbf16;
    k_to_bf16<<<(64 * 16 + 255) / 256, 256, 0, ctx->stream>>>(ctx->mlp_w + SG_MLP_OFF_W1, wb, 64 * 16);
    k_to_bf16<<<(64 * 64 + 255) / 256, 256, 0, ctx->stream>>>(ctx->mlp_w + SG_MLP_OFF_W2, wb + 64 * 16, 64 * 64);
    k_to_bf16<<<(64 * 64 + 255) / 256, 256, 0, ctx->stream>>>(ctx->mlp_w + SG_MLP_OFF_W3, wb + 64 * 16 + 64 * 64, 64 * 64);
    SG_LAUNCH_CHECK(ctx, "k_to_bf16");
    MlpDev d;
    d.W1 = wb;
    d.W2 = wb + 64 * 16;
    d.W3 = wb + 64 * 16 + 64 * 64;
    d.b1 = ctx->mlp_w + SG_MLP_OFF_B1;
    d.b2 = ctx->mlp_w + SG_MLP_OFF_B2;
    d.b3 = ctx->mlp_w + SG_MLP_OFF_B3;
    d.w4 = ctx->mlp_w + SG_MLP_OFF_W4;
    d.b4 = w[SG_MLP_OFF_B4];
    static_assert(sizeof(MlpDev) <= sizeof(ctx->mlp_host_desc), "descriptor size");
    memcpy(ctx->mlp_host_desc, &d, sizeof(d));
    ctx->mlp_ready = 1;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_mlp_get_weights(sg_ctx* ctx, float* w, int64_t count) {
    if (!ctx || !w || count != SG_MLP_NPARAM) return SG_EINVAL;
    if (!ctx->mlp_w) return sg_fail(ctx, SG_ENOTREADY, "no MLP weights");
    SG_CUDA(ctx, cudaMemcpyAsync(w, ctx->mlp_w, sizeof(float) * SG_MLP_NPARAM, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

}  // extern "C"
