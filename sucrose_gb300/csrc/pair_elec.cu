// Morse and charged point-particle pair potentials: morse_ (fortran/force.f90:
// 199-233), dh_ (:2589-2617), coulombic_ (:2627-2665) and dipole_ with its
// reaction field (:2669-2767). FP32 per pair, FP64 energy sums.
//
// Charges live in pos.w (set by sg_set_charges), so a charge pair reads the
// two position float4 it needs for r_ij anyway and nothing else; the dipole
// also reads the two quaternions.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pair_common.cuh"

namespace {

// body z axis of the quaternion (w, x, y, z) held as float4 (x=w, y=x, z=y, w=z):
// the reference's U = (2(qx qz + qw qy), 2(qy qz - qw qx), qw^2 - qx^2 - qy^2 + qz^2)
SG_DEV float3 body_z(float4 q) {
    return make_float3(2.f * (q.y * q.w + q.x * q.z), 2.f * (q.z * q.w - q.x * q.y),
                       q.x * q.x - q.y * q.y - q.z * q.z + q.w * q.w);
}

struct PotElec {
    static constexpr bool kTorque = false;
    static constexpr bool kStats = false;
    static constexpr bool kCountActive = true;
    static constexpr bool kFilterable = true;
    static constexpr int kMinBlocks = 1;
    static constexpr int kMinBlocksFiltered = 4;
    const float4* __restrict__ pos;
    BoxF b;
    int kind;
    float rc;
    float dissoc, width, rmin, pot_cut;   // Morse
    float inv_db;                         // Debye-Hueckel 1 / db_len
    float kq;                             // 1 / (4 pi dielectric)
    float sw, factor;                     // Coulomb switch start (cutoff - 2) and 1 / (cutoff - switch)
    int prefiltered;

    SG_DEV bool in_range(int i, int j) const {
        const float3 r = pair_rij(pos, i, j, b);
        return sqrtf(r.x * r.x + r.y * r.y + r.z * r.z) < rc;
    }

    SG_DEV void eval(bool valid, int i, int j, int, PairOut& o, unsigned long long*) const {
        if (!valid) return;
        float qq;
        const float3 r = pair_rij_q(pos, i, j, b, qq);
        const float rsq = r.x * r.x + r.y * r.y + r.z * r.z;
        const float rmag = sqrtf(rsq);
        if (!prefiltered && !(rmag < rc)) return;
        o.act = 1;
        if (kind == SG_MORSE) {                      // force.f90:218-231
            const float e = expf(-width * (rmag - rmin));
            const float om = 1.f - e;
            o.pe = dissoc * (om * om - 1.f) - pot_cut;
            const float c = -2.f * width * dissoc * om * e * fast_rcp(rmag);
            o.f = c * r;
            o.vir = c * rsq;
        } else if (kind == SG_DH) {                  // force.f90:2609-2615
            const float pe = qq * kq * expf(-rmag * inv_db) * fast_rcp(rmag);
            const float c = pe * (1.f + rmag * inv_db) * fast_rcp(rsq);
            o.pe = pe;
            o.f = c * r;
            o.vir = c * rsq;
        } else {                                     // SG_COULOMB, force.f90:2643-2663
            float pe = qq * kq * fast_rcp(rmag);
            float3 f = (pe * fast_rcp(rsq)) * r;
            if (rmag >= sw) {
                // the reference's quintic switch S(x) = 1 - 10x^3 + 15x^4 - 6x^5 and
                // its derivative, in the factored forms (1-x)^3 (1 + 3x + 6x^2) and
                // -30 x^2 (1-x)^2, which keep FP32 accuracy as x -> 1
                const float x = (rmag - sw) * factor;
                const float om = 1.f - x;
                const float sx = om * om * om * (1.f + 3.f * x + 6.f * x * x);
                const float sdx = -30.f * x * x * om * om;
                pe = sx * pe;
                // FXIJ = sx FXIJ - sdx PE factor: the scalar term is subtracted
                // from each Cartesian component, as the reference does (:2661)
                const float s = sdx * pe * factor;
                f = make_float3(sx * f.x - s, sx * f.y - s, sx * f.z - s);
            }
            o.pe = pe;
            o.f = f;
            o.vir = dot3(r, f);
        }
    }
};

struct PotDipole {
    static constexpr bool kTorque = true;
    static constexpr bool kStats = false;
    static constexpr bool kCountActive = true;
    static constexpr bool kFilterable = true;
    static constexpr int kMinBlocks = 1;
    static constexpr int kMinBlocksFiltered = 4;
    const float4* __restrict__ pos;
    const float4* __restrict__ quat;
    BoxF b;
    float rc;
    int* __restrict__ mark;   // I side of a pair in range: DIP(I) = U1 after the call
    int* __restrict__ cnt;    // J side: how many in-range pairs add U2(J) dip_coeff to RFL
    int prefiltered;

    SG_DEV bool in_range(int i, int j) const {
        const float3 r = pair_rij(pos, i, j, b);
        return sqrtf(r.x * r.x + r.y * r.y + r.z * r.z) < rc;
    }

    // dipole_calculate_forces (force.f90:2687-2751)
    SG_DEV void eval(bool valid, int i, int j, int, PairOut& o, unsigned long long*) const {
        if (!valid) return;
        const float4 a = pos[i], c = pos[j];
        const float3 r = pair_rij(pos, i, j, b);
        const float rsq = r.x * r.x + r.y * r.y + r.z * r.z;
        const float rmag = sqrtf(rsq);
        if (!prefiltered && !(rmag < rc)) return;
        o.act = 1;
        const float3 u1 = a.w * body_z(quat[i]);
        const float3 u2 = c.w * body_z(quat[j]);
        const float ci = dot3(u1, r), cj = dot3(u2, r), cij = dot3(u1, u2);
        const float inv2 = fast_rcp(rsq);
        const float inv3 = inv2 * fast_rcp(rmag);
        const float inv5 = inv3 * inv2;
        const float3 term1 = (cij - 5.f * ci * cj * inv2) * r + cj * u1 + ci * u2;
        const float3 term2 = (3.f * cj * inv2) * r - u2;
        const float3 term3 = (3.f * ci * inv2) * r - u1;
        o.pe = cij * inv3 - 3.f * ci * cj * inv5;
        o.f = (3.f * inv5) * term1;
        o.ti = inv3 * cross3(u1, term2);
        o.tj = inv3 * cross3(u2, term3);
        o.vir = dot3(r, o.f);
        mark[i] = 1;
        atomicAdd(&cnt[j], 1);
    }
};

// The dipole call's side effects on the reaction field (force.f90:2739-2745):
// DIP(I) = U1 for every marked I, and RFL += dip_coeff * sum over in-range
// pairs of U2(J) = dip_coeff * sum_j cnt_j U2(j), summed in FP64 and finished
// by the last block. Marks and counts are cleared for the next call.
__global__ void k_rf_fold(int n, const float4* __restrict__ pos, const float4* __restrict__ quat, int* mark,
                          int* cnt, float4* dip, double dip_coeff, double* partials, unsigned int* done,
                          double* rfl) {
    double v[3] = {0.0, 0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int m = mark[i], k = cnt[i];
        if (!m && !k) continue;
        const float3 u = pos[i].w * body_z(quat[i]);
        if (m) {
            dip[i] = make_float4(u.x, u.y, u.z, 0.f);
            mark[i] = 0;
        }
        if (k) {
            v[0] += (double)k * (double)u.x;
            v[1] += (double)k * (double)u.y;
            v[2] += (double)k * (double)u.z;
            cnt[i] = 0;
        }
    }
    for (int d = 0; d < 3; ++d) v[d] *= dip_coeff;
    block_reduce_finish<3>(v, partials, done, rfl);
}

// eval_reaction_field (force.f90:2753-2766), in FP64 against the FP64 RFL.
__global__ void k_rf_apply(int n, const float4* __restrict__ pos, const float4* __restrict__ dip,
                           const double* __restrict__ rfl, float4* torque, double* partials, unsigned int* done,
                           double* acc_call, double* acc_total) {
    const double Rx = rfl[0], Ry = rfl[1], Rz = rfl[2];
    double e[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (pos[i].w == 0.f) continue;
        const float4 d = dip[i];
        const double dx = d.x, dy = d.y, dz = d.z;
        e[0] += 0.5 * (dx * Rx + dy * Ry + dz * Rz);
        float4 t = torque[i];
        t.x = (float)((double)t.x - (dy * Rz - dz * Ry));
        t.y = (float)((double)t.y - (dz * Rx - dx * Rz));
        t.z = (float)((double)t.z - (dx * Ry - dy * Rx));
        torque[i] = t;
    }
    block_reduce_finish<1>(e, partials, done, acc_call, acc_total);
}

int rf_grid(sg_ctx* ctx) {
    const int g = (ctx->n + 255) / 256;
    return std::max(1, std::min(g, 4 * ctx->num_sms));
}

}  // namespace

int sg_launch_pair_elec(sg_ctx* ctx, const sg_pair_params* p) {
    const double rc = p->cutoff;
    if (p->kind == SG_DIPOLE) {
        if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "the dipole reaction field is per system: no replica contexts");
        if (!ctx->rf_field) return sg_fail(ctx, SG_ENOTREADY, "SG_DIPOLE needs sg_reaction_field_init first");
        if (!(rc > 0.0)) return sg_fail(ctx, SG_EINVAL, "dipole cutoff must be positive");
        PotDipole pot;
        pot.pos = ctx->pos;
        pot.quat = ctx->quat;
        pot.b = make_boxf(ctx);
        pot.rc = (float)rc;
        pot.mark = ctx->rf_mark;
        pot.cnt = ctx->rf_cnt;
        if (int r = launch_pair(ctx, pot, p->kind)) return r;
        // dip_coeff = 2 (eps - 1) / (2 eps + 1) / rc^3 (force.f90:2701-2702)
        const double eps = p->dielectric;
        const double dip_coeff = (2.0 * (eps - 1.0)) / (2.0 * eps + 1.0) / (rc * rc * rc);
        const int grid = rf_grid(ctx);
        if (int r = sg_ensure_partials(ctx, grid * 3)) return r;
        k_rf_fold<<<grid, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->quat, ctx->rf_mark, ctx->rf_cnt, ctx->rf_dip,
                                                 dip_coeff, ctx->partials, ctx->done_counter, ctx->rf_field);
        SG_LAUNCH_CHECK(ctx, "k_rf_fold");
        return SG_OK;
    }
    PotElec pot;
    pot.pos = ctx->pos;
    pot.b = make_boxf(ctx);
    pot.kind = p->kind;
    pot.rc = (float)rc;
    pot.dissoc = (float)p->dissoc;
    pot.width = (float)p->width;
    pot.rmin = (float)p->rmin;
    // pot_cut (force.f90:224-227) from the FP64 host values
    const double ec = std::exp(-p->width * (rc - p->rmin));
    pot.pot_cut = (float)(p->dissoc * ((1.0 - ec) * (1.0 - ec) - 1.0));
    if (p->kind == SG_DH && !(p->db_len > 0.0)) return sg_fail(ctx, SG_EINVAL, "Debye length must be positive");
    if ((p->kind == SG_DH || p->kind == SG_COULOMB) && p->dielectric == 0.0)
        return sg_fail(ctx, SG_EINVAL, "dielectric must be non-zero");
    pot.inv_db = p->kind == SG_DH ? (float)(1.0 / p->db_len) : 0.f;
    pot.kq = p->dielectric != 0.0 ? (float)(1.0 / (4.0 * M_PI * p->dielectric)) : 0.f;
    const double sw = rc - 2.0;   // switch 2 sigma_0 inside the cutoff (force.f90:2644-2645)
    pot.sw = (float)sw;
    pot.factor = (float)(1.0 / (rc - sw));
    return launch_pair(ctx, pot, p->kind);
}

int sg_reaction_field_eval_async(sg_ctx* ctx) {
    if (!ctx->rf_field) return sg_fail(ctx, SG_ENOTREADY, "sg_reaction_field_init must come first");
    SG_CUDA(ctx, cudaMemsetAsync(ctx->acc + 4, 0, sizeof(double), ctx->stream));
    const int grid = rf_grid(ctx);
    if (int r = sg_ensure_partials(ctx, grid)) return r;
    k_rf_apply<<<grid, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->rf_dip, ctx->rf_field, ctx->torque,
                                              ctx->partials, ctx->done_counter, ctx->acc + 4, ctx->acc);
    SG_LAUNCH_CHECK(ctx, "k_rf_apply");
    return SG_OK;
}

extern "C" {

int sg_reaction_field_init(sg_ctx* ctx) {
    if (!ctx) return SG_EINVAL;
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "the dipole reaction field is per system: no replica contexts");
    const size_t n = (size_t)ctx->n;
    if (!ctx->rf_field) {
        SG_CUDA(ctx, cudaMalloc(&ctx->rf_dip, sizeof(float4) * n));
        SG_CUDA(ctx, cudaMalloc(&ctx->rf_mark, sizeof(int) * n));
        SG_CUDA(ctx, cudaMalloc(&ctx->rf_cnt, sizeof(int) * n));
        SG_CUDA(ctx, cudaMalloc(&ctx->rf_field, sizeof(double) * 4));
        ctx->graph_epoch++;
    }
    SG_CUDA(ctx, cudaMemsetAsync(ctx->rf_dip, 0, sizeof(float4) * n, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->rf_mark, 0, sizeof(int) * n, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->rf_cnt, 0, sizeof(int) * n, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->rf_field, 0, sizeof(double) * 4, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_reaction_field_eval(sg_ctx* ctx, double* pot_eng) {
    if (!ctx) return SG_EINVAL;
    if (int r = sg_reaction_field_eval_async(ctx)) return r;
    double e = 0.0;
    SG_CUDA(ctx, cudaMemcpyAsync(&e, ctx->acc + 4, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (pot_eng) *pot_eng += e;
    if (!std::isfinite(e)) return sg_fail(ctx, SG_ENAN, "non-finite reaction-field energy");
    return SG_OK;
}

int sg_reaction_field_read(sg_ctx* ctx, double rfl[3], double* dipx, double* dipy, double* dipz) {
    if (!ctx || !rfl) return SG_EINVAL;
    if (!ctx->rf_field) return sg_fail(ctx, SG_ENOTREADY, "sg_reaction_field_init must come first");
    SG_CUDA(ctx, cudaMemcpyAsync(rfl, ctx->rf_field, sizeof(double) * 3, cudaMemcpyDeviceToHost, ctx->stream));
    if (dipx || dipy || dipz) {
        std::vector<float4> d(ctx->n);
        SG_CUDA(ctx, cudaMemcpyAsync(d.data(), ctx->rf_dip, sizeof(float4) * ctx->n, cudaMemcpyDeviceToHost,
                                     ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int i = 0; i < ctx->n; ++i) {
            if (dipx) dipx[i] = d[i].x;
            if (dipy) dipy[i] = d[i].y;
            if (dipz) dipz[i] = d[i].z;
        }
    }
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

}  // extern "C"
