// Bonded terms (module bonded, fortran/force.f90:2238-2581): bend_, dih_,
// cosine_bend_, cosine_dih_, angle_bend_ and angle_dih_. The reference's user
// loop calls one routine per term and adds FXI..FXL to the four atoms; here a
// registered term list is evaluated one thread per term in FP32, the forces
// scattered with one float4 atomic per atom and the energy summed in FP64.
#include <cmath>
#include <vector>

#include "sg_internal.cuh"

namespace {

struct BGeo {
    float3 box, inv_box;
    int periodic;
};

// r_b - r_a with the minimum image (the reference's VI, VJ, VK)
SG_DEV float3 bvec(const float4* __restrict__ pos, int a, int b, const BGeo& g) {
    const float4 pa = pos[a], pb = pos[b];
    return min_image(make_float3(pb.x - pa.x, pb.y - pa.y, pb.z - pa.z), g.box, g.inv_box, g.periodic);
}

// angle_dih_calculate_forces (force.f90:2508-2579) in FP64; returns PE and
// the forces on I, J, K, L.
SG_DEV float angle_dih_fp64(float3 vi, float3 vj, float3 vk, float coeff, float c0f, float s0f, float3 (&F)[4]) {
    const double VI[3] = {vi.x, vi.y, vi.z}, VJ[3] = {vj.x, vj.y, vj.z}, VK[3] = {vk.x, vk.y, vk.z};
    auto dot = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    const double C11 = dot(VI, VI), C12 = dot(VI, VJ), C13 = dot(VI, VK);
    const double C22 = dot(VJ, VJ), C23 = dot(VJ, VK), C33 = dot(VK, VK);
    const double D12 = C11 * C22 - C12 * C12, D23 = C22 * C33 - C23 * C23;
    const double prefac = 1.0 / sqrt(D23 * D12);
    const double fac = C23 * C12 - C13 * C22, fac1 = fac / D23, fac2 = fac / D12;
    const double fs = (VI[1] * VJ[2] - VI[2] * VJ[1]) * VK[0] + (VI[2] * VJ[0] - VI[0] * VJ[2]) * VK[1] +
                      (VI[0] * VJ[1] - VI[1] * VJ[0]) * VK[2];
    const double c0 = c0f, s0 = s0f, cf = coeff;
    const double cph = -prefac * fac, sph = prefac * fs * sqrt(C22);
    const double a = -(cf * (c0 - s0 * (cph / sph))) * prefac;
    for (int d = 0; d < 3; ++d) {
        const double fl = a * (C12 * VJ[d] - C22 * VI[d] - fac1 * (C22 * VK[d] - C23 * VJ[d]));
        const double fk = a * (C12 * VK[d] - C12 * VJ[d] + C23 * VI[d] + C22 * VI[d] - 2.0 * C13 * VJ[d] -
                               fac2 * (C11 * VJ[d] - C12 * VI[d]) -
                               fac1 * (C33 * VJ[d] - C22 * VK[d] - C23 * VK[d] + C23 * VJ[d]));
        const double fj = a * (-C12 * VK[d] + C23 * VJ[d] - C23 * VI[d] - C22 * VK[d] + 2.0 * C13 * VJ[d] -
                               fac2 * (C22 * VI[d] - C11 * VJ[d] - C12 * VJ[d] + C12 * VI[d]) -
                               fac1 * (-C33 * VJ[d] + C23 * VK[d]));
        const double fi = a * (-C23 * VJ[d] + C22 * VK[d] - fac2 * (-C22 * VI[d] + C12 * VJ[d]));
        (&F[0].x)[d] = (float)fi;
        (&F[1].x)[d] = (float)fj;
        (&F[2].x)[d] = (float)fk;
        (&F[3].x)[d] = (float)fl;
    }
    return (float)(cf * (1.0 - cph * c0 - sph * s0));
}

template <int KIND>
__global__ void k_bonded(int n, const int4* __restrict__ atoms, const float4* __restrict__ par, BGeo g,
                         const float4* __restrict__ pos, float4* force, double* partials, unsigned int* done,
                         double* acc_call, double* acc_total) {
    constexpr bool kBend = KIND == SG_BEND || KIND == SG_COSINE_BEND || KIND == SG_ANGLE_BEND;
    float e[1] = {0.f};
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const int4 at = atoms[t];
        const float4 p = par[t];   // coeff, cos theta0, sin theta0, theta0
        const float coeff = p.x;
        const float3 VI = bvec(pos, at.x, at.y, g);
        const float3 VJ = bvec(pos, at.y, at.z, g);
        if constexpr (kBend) {   // :2244-2284, :2345-2390, :2464-2506
            const float C11 = dot3(VI, VI), C12 = dot3(VI, VJ), C22 = dot3(VJ, VJ);
            const float prefac = rsqrtf(C11 * C22);
            const float fac1 = C12 / C22, fac2 = C12 / C11;
            float strength = coeff;
            if constexpr (KIND == SG_BEND) {
                e[0] += coeff * (1.f - prefac * C12);
            } else if constexpr (KIND == SG_COSINE_BEND) {
                const float c = prefac * C12;
                strength = coeff * (c - p.y);
                e[0] += 0.5f * coeff * (c - p.y) * (c - p.y);
            } else {
                // theta and sin(theta) from the cross product: acos of the
                // FP32 cosine is exactly 0 (and sin 0 divides) for bonds within
                // ~3e-4 rad of parallel, where |VI x VJ| still resolves the angle
                const float3 nb = cross3(VI, VJ);
                const float sn = sqrtf(dot3(nb, nb));
                const float th = atan2f(sn, C12);
                strength = coeff * (th - p.w) / (sn * prefac);
                e[0] += 0.5f * coeff * (th - p.w) * (th - p.w);
            }
            const float s = strength * prefac;
            const float3 FK = -s * (fac1 * VJ - VI);
            const float3 FJ = s * (fac1 * VJ - fac2 * VI + VJ - VI);
            const float3 FI = s * (fac2 * VI - VJ);
            atomicAdd(&force[at.x], make_float4(FI.x, FI.y, FI.z, 0.f));
            atomicAdd(&force[at.y], make_float4(FJ.x, FJ.y, FJ.z, 0.f));
            atomicAdd(&force[at.z], make_float4(FK.x, FK.y, FK.z, 0.f));
        } else {                 // :2286-2343, :2392-2462, :2508-2579
            const float3 VK = bvec(pos, at.z, at.w, g);
            float C11 = dot3(VI, VI), C12 = dot3(VI, VJ), C13 = dot3(VI, VK);
            float C22 = dot3(VJ, VJ), C23 = dot3(VJ, VK), C33 = dot3(VK, VK);
            float prefac = 0.f, fac = 0.f, fac1 = 0.f, fac2 = 0.f;
            float strength = coeff;
            if constexpr (KIND == SG_ANGLE_DIH) {
                // strength carries cos(phi) / sin(phi), which diverges at planar
                // dihedrals, where the force brackets below also cancel to
                // O(sin phi): the whole term runs in FP64 from the FP32 bond vectors
                float3 F[4];
                e[0] += angle_dih_fp64(VI, VJ, VK, coeff, p.y, p.z, F);
                atomicAdd(&force[at.x], make_float4(F[0].x, F[0].y, F[0].z, 0.f));
                atomicAdd(&force[at.y], make_float4(F[1].x, F[1].y, F[1].z, 0.f));
                atomicAdd(&force[at.z], make_float4(F[2].x, F[2].y, F[2].z, 0.f));
                atomicAdd(&force[at.w], make_float4(F[3].x, F[3].y, F[3].z, 0.f));
                continue;
            } else {
                // D12 = C11 C22 - C12^2 = |VI x VJ|^2, D23 = |VJ x VK|^2 and
                // fac = C23 C12 - C13 C22 = (VI x VJ).(VJ x VK) (Lagrange and
                // Binet-Cauchy identities), formed from the cross products: in
                // FP32 the differences cancel to zero or below for bends within
                // ~3e-4 rad of straight, which occur every few thousand steps in
                // a chain melt, and the dihedral then turns NaN
                const float3 n1 = cross3(VI, VJ), n2 = cross3(VJ, VK);
                const float D12 = dot3(n1, n1), D23 = dot3(n2, n2);
                prefac = rsqrtf(D23 * D12);
                fac = dot3(n1, n2);
                fac1 = fac / D23;
                fac2 = fac / D12;
                if constexpr (KIND == SG_DIH) {
                    e[0] += coeff * (1.f + prefac * fac);
                } else {
                    const float fac_sin = dot3(cross3(VI, VJ), VK);
                    const float cph = -prefac * fac;
                    const float sph = prefac * fac_sin * sqrtf(C22);
                    const float cs = cosf(atan2f(sph, cph));
                    strength = coeff * (cs - p.y);
                    e[0] += 0.5f * coeff * (cs - p.y) * (cs - p.y);
                }
            }
            const float a = -strength * prefac;
            const float3 FL = a * (C12 * VJ - C22 * VI - fac1 * (C22 * VK - C23 * VJ));
            const float3 FK = a * (C12 * VK - C12 * VJ + C23 * VI + C22 * VI - 2.f * C13 * VJ -
                                   fac2 * (C11 * VJ - C12 * VI) - fac1 * (C33 * VJ - C22 * VK - C23 * VK + C23 * VJ));
            const float3 FJ = a * (-C12 * VK + C23 * VJ - C23 * VI - C22 * VK + 2.f * C13 * VJ -
                                   fac2 * (C22 * VI - C11 * VJ - C12 * VJ + C12 * VI) - fac1 * (-C33 * VJ + C23 * VK));
            const float3 FI = a * (-C23 * VJ + C22 * VK - fac2 * (-C22 * VI + C12 * VJ));
            atomicAdd(&force[at.x], make_float4(FI.x, FI.y, FI.z, 0.f));
            atomicAdd(&force[at.y], make_float4(FJ.x, FJ.y, FJ.z, 0.f));
            atomicAdd(&force[at.z], make_float4(FK.x, FK.y, FK.z, 0.f));
            atomicAdd(&force[at.w], make_float4(FL.x, FL.y, FL.z, 0.f));
        }
    }
    block_reduce_finish_f<1>(e, partials, done, acc_call, acc_total);
}

int nat_of(int kind) { return (kind == SG_DIH || kind == SG_COSINE_DIH || kind == SG_ANGLE_DIH) ? 4 : 3; }

}  // namespace

void sg_bonded_free(sg_ctx* ctx) {
    for (int k = 0; k < 6; ++k) {
        if (ctx->bonded_atoms[k]) cudaFree(ctx->bonded_atoms[k]);
        if (ctx->bonded_par[k]) cudaFree(ctx->bonded_par[k]);
        ctx->bonded_atoms[k] = nullptr;
        ctx->bonded_par[k] = nullptr;
        ctx->bonded_n[k] = 0;
    }
}

extern "C" {

int sg_bonded_set(sg_ctx* ctx, int32_t kind, int32_t nterms, const int32_t* atoms, const double* coeff,
                  const double* angle, int32_t one_based) {
    if (!ctx || kind < 0 || kind > 5 || nterms < 0) return SG_EINVAL;
    if (nterms > 0 && (!atoms || !coeff)) return SG_EINVAL;
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "bonded terms are per system: no replica contexts");
    const bool needs_angle = kind >= SG_COSINE_BEND;
    if (nterms > 0 && needs_angle && !angle) return sg_fail(ctx, SG_EINVAL, "bonded kind %d needs angles", kind);
    const int nat = nat_of(kind), off = one_based ? 1 : 0;
    std::vector<int4> at(nterms);
    std::vector<float4> par(nterms);
    const double pi = 3.1415926535897932384626433832795;
    for (int t = 0; t < nterms; ++t) {
        int a[4] = {-1, -1, -1, -1};
        for (int k = 0; k < nat; ++k) {
            a[k] = atoms[(size_t)nat * t + k] - off;
            if (a[k] < 0 || a[k] >= ctx->n) return sg_fail(ctx, SG_EINVAL, "bonded term %d: atom out of range", t);
        }
        at[t] = make_int4(a[0], a[1], a[2], a[3]);
        // theta0 = PI - (PI / 180) * angle (force.f90:2380, :2443, :2497, :2559)
        const double th0 = needs_angle ? pi - (pi / 180.0) * angle[t] : 0.0;
        par[t] = make_float4((float)coeff[t], (float)std::cos(th0), (float)std::sin(th0), (float)th0);
    }
    if (ctx->bonded_atoms[kind]) cudaFree(ctx->bonded_atoms[kind]);
    if (ctx->bonded_par[kind]) cudaFree(ctx->bonded_par[kind]);
    ctx->bonded_atoms[kind] = nullptr;
    ctx->bonded_par[kind] = nullptr;
    ctx->bonded_n[kind] = 0;
    ctx->graph_epoch++;
    if (nterms == 0) return SG_OK;
    SG_CUDA(ctx, cudaMalloc(&ctx->bonded_atoms[kind], sizeof(int4) * nterms));
    SG_CUDA(ctx, cudaMalloc(&ctx->bonded_par[kind], sizeof(float4) * nterms));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->bonded_atoms[kind], at.data(), sizeof(int4) * nterms, cudaMemcpyHostToDevice,
                                 ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->bonded_par[kind], par.data(), sizeof(float4) * nterms, cudaMemcpyHostToDevice,
                                 ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->bonded_n[kind] = nterms;
    return SG_OK;
}

int sg_bonded_forces_async(sg_ctx* ctx, int32_t kind) {
    if (!ctx || kind < 0 || kind > 5) return SG_EINVAL;
    SG_CUDA(ctx, cudaMemsetAsync(ctx->acc + 4, 0, sizeof(double), ctx->stream));
    const int n = ctx->bonded_n[kind];
    if (n == 0) return SG_OK;
    BGeo g;
    g.box = make_float3((float)ctx->box[0], (float)ctx->box[1], (float)ctx->box[2]);
    g.inv_box = make_float3((float)(1.0 / ctx->box[0]), (float)(1.0 / ctx->box[1]), (float)(1.0 / ctx->box[2]));
    g.periodic = ctx->periodic;
    const int grid = std::max(1, std::min((n + 255) / 256, 8 * ctx->num_sms));
    if (int rc = sg_ensure_partials(ctx, grid)) return rc;
    const int4* at = ctx->bonded_atoms[kind];
    const float4* par = ctx->bonded_par[kind];
#define SG_BONDED_LAUNCH(K)                                                                                  \
    k_bonded<K><<<grid, 256, 0, ctx->stream>>>(n, at, par, g, ctx->pos, ctx->force, ctx->partials,           \
                                               ctx->done_counter, ctx->acc + 4, ctx->acc)
    switch (kind) {
        case SG_BEND: SG_BONDED_LAUNCH(SG_BEND); break;
        case SG_DIH: SG_BONDED_LAUNCH(SG_DIH); break;
        case SG_COSINE_BEND: SG_BONDED_LAUNCH(SG_COSINE_BEND); break;
        case SG_COSINE_DIH: SG_BONDED_LAUNCH(SG_COSINE_DIH); break;
        case SG_ANGLE_BEND: SG_BONDED_LAUNCH(SG_ANGLE_BEND); break;
        default: SG_BONDED_LAUNCH(SG_ANGLE_DIH); break;
    }
#undef SG_BONDED_LAUNCH
    SG_LAUNCH_CHECK(ctx, "k_bonded");
    return SG_OK;
}

int sg_bonded_forces(sg_ctx* ctx, int32_t kind, double* pot_eng) {
    if (int rc = sg_bonded_forces_async(ctx, kind)) return rc;
    double e = 0.0;
    SG_CUDA(ctx, cudaMemcpyAsync(&e, ctx->acc + 4, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (pot_eng) *pot_eng += e;
    if (!std::isfinite(e)) return sg_fail(ctx, SG_ENAN, "non-finite bonded energy");
    return SG_OK;
}

}  // extern "C"
