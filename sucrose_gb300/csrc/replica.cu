// Batched replicas: thousands of independent systems of uneven size in one
// context. Particles of replica r occupy [off[r], off[r+1]) of every state
// array; per-replica tables (box, list radius and grid, temperature, Philox
// key) are read by the same list, pair and integrator kernels as a single
// system, so one captured step advances every replica. Replicas are grouped
// by potential family (LJ, then GB, then ECP) so that each family's pairs are
// one contiguous range of the list.
#include <cmath>
#include <vector>

#include "sg_internal.cuh"

__global__ void k_rep_of(int R, const int* __restrict__ off, int* __restrict__ rep_of) {
    const int r = blockIdx.x;
    if (r >= R) return;
    for (int i = off[r] + threadIdx.x; i < off[r + 1]; i += blockDim.x) rep_of[i] = r;
}

// Per-replica sums over particle ranges: KE (translation) and KE_rot, FP64.
__global__ void k_rep_ke(int R, const int* __restrict__ off, const float4* __restrict__ vel,
                         const float4* __restrict__ shape, const float4* __restrict__ quat,
                         const float4* __restrict__ angm, const float4* __restrict__ inert_inv, double* out) {
    const int r = blockIdx.x;
    if (r >= R) return;
    double ke = 0.0, kr = 0.0;
    for (int i = off[r] + threadIdx.x; i < off[r + 1]; i += blockDim.x) {
        const float4 v = vel[i];
        ke += 0.5 * (double)shape[i].w * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
        const float4 q = quat[i], L = angm[i], Ii = inert_inv[i];
        const float w = q.x, x = q.y, y = q.z, z = q.w;
        const float lb0 = (w * w + x * x - y * y - z * z) * L.x + 2.f * (x * y + w * z) * L.y + 2.f * (x * z - w * y) * L.z;
        const float lb1 = 2.f * (x * y - w * z) * L.x + (w * w - x * x + y * y - z * z) * L.y + 2.f * (y * z + w * x) * L.z;
        const float lb2 = 2.f * (x * z + w * y) * L.x + 2.f * (y * z - w * x) * L.y + (w * w - x * x - y * y + z * z) * L.z;
        kr += 0.5 * ((double)(lb0 * lb0) * Ii.x + (double)(lb1 * lb1) * Ii.y + (double)(lb2 * lb2) * Ii.z);
    }
    __shared__ double s0[256], s1[256];
    s0[threadIdx.x] = ke;
    s1[threadIdx.x] = kr;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s0[threadIdx.x] += s0[threadIdx.x + o];
            s1[threadIdx.x] += s1[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[2 * r] = s0[0];
        out[2 * r + 1] = s1[0];
    }
}

extern "C" {

int sg_create_replicas(sg_ctx** out, int32_t nrep, const int32_t* n_per_rep, const double* boxes,
                       const int32_t* family, const double* temps, const uint32_t* keys, int32_t device) {
    if (!out || nrep < 1 || !n_per_rep || !boxes || !family) return SG_EINVAL;
    int64_t total = 0;
    for (int r = 0; r < nrep; ++r) {
        if (n_per_rep[r] < 1) return SG_EINVAL;
        if (family[r] < 0 || family[r] > 2) return SG_EINVAL;
        if (r && family[r] < family[r - 1]) return SG_EINVAL;   // grouped by family
        total += n_per_rep[r];
    }
    if (total > INT32_MAX / 2) return SG_EINVAL;
    if (int rc = sg_create(out, (int32_t)total, device)) return rc;
    sg_ctx* ctx = *out;
    const int R = nrep, n = (int)total;
    ctx->nrep = R;
    ctx->h_rep_off.assign(R + 1, 0);
    ctx->h_rep_box.assign(boxes, boxes + 3 * R);
    ctx->h_rep_family.assign(family, family + R);
    for (int r = 0; r < R; ++r) ctx->h_rep_off[r + 1] = ctx->h_rep_off[r] + n_per_rep[r];
    for (int f = 0; f < 3; ++f) {
        int first = n, first_r = R;
        for (int r = R - 1; r >= 0; --r)
            if (family[r] >= f) {
                first = ctx->h_rep_off[r];
                first_r = r;
            }
        ctx->fam_pstart[f] = first;
        ctx->fam_rstart[f] = first_r;
    }
    ctx->fam_pstart[3] = n;
    ctx->fam_rstart[3] = R;
    double bmax[3] = {0, 0, 0};
    for (int r = 0; r < R; ++r)
        for (int d = 0; d < 3; ++d) bmax[d] = std::max(bmax[d], boxes[3 * r + d]);
    for (int d = 0; d < 3; ++d) ctx->box[d] = bmax[d];
    ctx->periodic = 1;
    // one allocation for every table, 16-byte aligned sections
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t s_boxd = al(sizeof(double) * 3 * R), s_d = al(sizeof(double) * R), s_f4 = al(sizeof(float4) * R),
                 s_i4 = al(sizeof(int4) * R), s_u2 = al(sizeof(uint2) * R),
                 s_i = al(sizeof(int) * R), s_off = al(sizeof(int) * (R + 1)), s_of = al(sizeof(int) * (size_t)n);
    const size_t s_hs = al(sizeof(float) * R);
    const size_t bytes = s_boxd + 3 * s_d + 3 * s_f4 + s_i4 + s_u2 + s_i + s_off + s_of + s_hs;
    char* base = nullptr;
    SG_CUDA(ctx, cudaMalloc(&base, bytes));
    ctx->rep_alloc = base;
    char* p = base;
    double* boxd = (double*)p; p += s_boxd;
    double* rl2 = (double*)p; p += s_d;
    double* trig = (double*)p; p += s_d;
    float4* box = (float4*)p; p += s_f4;
    float4* inv = (float4*)p; p += s_f4;
    float4* blo = (float4*)p; p += s_f4;
    int4* grid = (int4*)p; p += s_i4;
    uint2* key = (uint2*)p; p += s_u2;
    double* temp = (double*)p; p += s_d;
    int* tint = (int*)p; p += s_i;
    int* off = (int*)p; p += s_off;
    float* half_sq = (float*)p; p += s_hs;
    int* rep_of = (int*)p;
    std::vector<float4> hb(R), hi(R), hl(R);
    std::vector<uint2> hk(R);
    std::vector<double> ht(R);
    std::vector<int> hti(R);
    std::vector<float> hhs(R);
    for (int r = 0; r < R; ++r) {
        const double hm = 0.4998 * std::min(boxes[3 * r], std::min(boxes[3 * r + 1], boxes[3 * r + 2]));
        hhs[r] = (float)(hm * hm * (1.0 - 1e-5));
        hb[r] = make_float4((float)boxes[3 * r], (float)boxes[3 * r + 1], (float)boxes[3 * r + 2], 0.f);
        hi[r] = make_float4((float)(1.0 / boxes[3 * r]), (float)(1.0 / boxes[3 * r + 1]), (float)(1.0 / boxes[3 * r + 2]), 0.f);
        hl[r] = make_float4((float)(boxes[3 * r] - (double)hb[r].x), (float)(boxes[3 * r + 1] - (double)hb[r].y),
                            (float)(boxes[3 * r + 2] - (double)hb[r].z), 0.f);
        hk[r] = keys ? make_uint2(keys[2 * r], keys[2 * r + 1]) : make_uint2(0x6D2B79F5u, 0x1B873593u);
        const double T = temps ? temps[r] : 1.0;
        ht[r] = T;
        hti[r] = (int)(T * 1000.0);   // int(T*1000) as Fortran does it on the host
    }
    SG_CUDA(ctx, cudaMemcpy(boxd, boxes, sizeof(double) * 3 * R, cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy(box, hb.data(), sizeof(float4) * R, cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy(inv, hi.data(), sizeof(float4) * R, cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy(blo, hl.data(), sizeof(float4) * R, cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy(key, hk.data(), sizeof(uint2) * R, cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy(temp, ht.data(), sizeof(double) * R, cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy(tint, hti.data(), sizeof(int) * R, cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy(off, ctx->h_rep_off.data(), sizeof(int) * (R + 1), cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy(half_sq, hhs.data(), sizeof(float) * R, cudaMemcpyHostToDevice));
    k_rep_of<<<R, 128, 0, ctx->stream>>>(R, off, rep_of);
    SG_LAUNCH_CHECK(ctx, "k_rep_of");
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->rep.rep_of = rep_of;
    ctx->rep.off = off;
    ctx->rep.box = box;
    ctx->rep.inv_box = inv;
    ctx->rep.box_lo = blo;
    ctx->rep.boxd = boxd;
    ctx->rep.rl2 = rl2;
    ctx->rep.trig = trig;
    ctx->rep.grid = grid;
    ctx->rep.temp = temp;
    ctx->rep.temp_int = tint;
    ctx->rep.key = key;
    ctx->rep.half_sq = half_sq;
    return SG_OK;
}

int sg_rep_kinetic(sg_ctx* ctx, double* ke2) {
    if (!ctx || !ke2) return SG_EINVAL;
    if (!ctx->nrep) return sg_fail(ctx, SG_EINVAL, "not a replica context");
    const int R = ctx->nrep;
    if (int rc = sg_ensure_partials(ctx, 2 * R)) return rc;
    k_rep_ke<<<R, 256, 0, ctx->stream>>>(R, ctx->rep.off, ctx->vel, ctx->shape, ctx->quat, ctx->angm, ctx->inert_inv,
                                        ctx->partials);
    SG_LAUNCH_CHECK(ctx, "k_rep_ke");
    SG_CUDA(ctx, cudaMemcpyAsync(ke2, ctx->partials, sizeof(double) * 2 * R, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

}  // extern "C"
