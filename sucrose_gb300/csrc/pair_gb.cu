// Gay-Berne family: gb_, gbr_, gbw_, gbc_, gbwc_ (fortran/force.f90:237-1030),
// FP32 per pair with (mu, nu) as parameters (the reference fixes (1,2) at :240).
//
// As in the reference, the shape (sig_x, sig_z) and energy (eps_x, eps_z)
// anisotropies are those of particle I. A per-particle prep pass hoists what
// depends on one particle only: the body z axis u (first column of the
// reference's U1 formula, :343-349), chi, chi' and 1/eps_z.
//
// Prep layout (one allocation of 4 float4 per particle):
//   rec[2p]     = (x, y, z, sig_x)   the position, copied, and the width
//   rec[2p + 1] = (u_x, u_y, u_z, chi)
//   aux[p]      = (chi', 1/eps_z, 0, 0)   with aux = rec + 2n
// so the range test reads each particle's position and axis in one 32-byte
// load.
#include <cmath>

// resident 256-thread blocks per SM for the filtered kernel (64 registers);
// measured on the Gay-Berne workload: 3 blocks 99 µs, 4 blocks 93 µs, and 5
// or 6 slower again (register spills)
#ifndef SG_GB_FILTER_MIN_BLOCKS
#define SG_GB_FILTER_MIN_BLOCKS 4
#endif
#include "pair_common.cuh"

namespace {

__global__ void k_gb_prep(int n, const float4* __restrict__ pos, const float4* __restrict__ quat,
                          const float4* __restrict__ shape, const float4* __restrict__ eshape, float muinv,
                          float4* prep) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float4 at = pos[p];
    float4 q = quat[p];  // w x y z
    float w = q.x, x = q.y, y = q.z, z = q.w;
    float3 u = make_float3(2.f * (x * z + w * y), 2.f * (y * z - w * x), w * w - x * x - y * y + z * z);
    float4 s = shape[p], e = eshape[p];
    float lpar = s.z, lprp = s.x;
    float chi = (lpar * lpar - lprp * lprp) / (lpar * lpar + lprp * lprp);
    float ep = powf(e.x, muinv), ez = powf(e.z, muinv);
    float xhi = (ep - ez) / (ep + ez);
    prep[2 * p] = make_float4(at.x, at.y, at.z, lprp);
    prep[2 * p + 1] = make_float4(u.x, u.y, u.z, chi);
    prep[2 * (size_t)n + p] = make_float4(xhi, 1.f / e.z, 0.f, 0.f);
}

struct GTerms {
    float a, b, g;   // (ru1+ru2)/(1+c uu), (ru1-ru2)/(1-c uu), g_func
};

// inv_rsq = 1 / r^2: the divisions by r^2 of the reference become products
SG_DEV GTerms gterms(float c, float ru1, float ru2, float uu, float inv_rsq) {
    GTerms t;
    float sp = ru1 + ru2, sm = ru1 - ru2;
    float dp = fast_rcp(1.f + c * uu), dm = fast_rcp(1.f - c * uu);
    t.a = sp * dp;
    t.b = sm * dm;
    t.g = 1.f - (c * 0.5f * inv_rsq) * (sp * t.a + sm * t.b);
    return t;
}

template <int KIND>
struct PotGB {
    static constexpr bool kTorque = true;
    static constexpr bool kStats = false;
    static constexpr bool kCountActive = true;
    static constexpr bool kWeld = (KIND == SG_GBW || KIND == SG_GBWC);
    static constexpr bool kTaper = (KIND != SG_GBR);
    static constexpr bool kChiral = (KIND == SG_GBC || KIND == SG_GBWC);
    static constexpr bool kFilterable = true;
    static constexpr bool kQueueR = true;        // the range test's r_ij is queued for eval_r
    static constexpr bool kExactFilter = false;  // in_range_r is a superset; eval_r decides
    static constexpr int kMinBlocks = 1;
    static constexpr int kMinBlocksFiltered = SG_GB_FILTER_MIN_BLOCKS;
    const float4* __restrict__ pos;
    const float4* __restrict__ prep;   // rec: 2 per particle
    const float4* __restrict__ aux;    // 1 per particle
    BoxF b;
    float cutoff, wf, chirality;
    int mu, nu;
    int prefiltered;   // eval only sees pairs that passed an exact range test

    // A superset of eval's range test (r against the orientation-dependent
    // contact distance sigma of I's shape plus the cut-off), without its
    // correctly rounded square roots and division: approximate 1/sqrt for r
    // and sigma (a few ulp each), and a slack of 1e-5 (r + sigma), some 80
    // ulp of the larger, which also covers the rounding of sigma + shift. A
    // NaN anywhere keeps the pair: eval_r decides. r_ij is handed on to
    // eval_r.
    SG_DEV bool in_range_r(int i, int j, float3& r) const {
        float4 pi0, pi1, pj0, pj1;
        ld_f4x2(prep + 2 * i, pi0, pi1);
        ld_f4x2(prep + 2 * j, pj0, pj1);
        r = pair_rij_of(make_float3(pi0.x, pi0.y, pi0.z), make_float3(pj0.x, pj0.y, pj0.z), i, b);
        const float rsq = r.x * r.x + r.y * r.y + r.z * r.z;
        const float3 U1 = make_float3(pi1.x, pi1.y, pi1.z), U2 = make_float3(pj1.x, pj1.y, pj1.z);
        const GTerms gc = gterms(pi1.w, dot3(r, U1), dot3(r, U2), dot3(U1, U2), fast_rcp(rsq));
        const float sigma = pi0.w * fast_rsqrt(gc.g);
        const float rmag = rsq * fast_rsqrt(rsq);
        const float shift = (KIND == SG_GBR) ? 0.f : kWeld ? (cutoff + wf - 1.f) : (cutoff - 1.f);
        return !(0.99999f * rmag >= 1.00001f * sigma + shift);
    }
    SG_DEV bool in_range(int i, int j) const {
        float3 r;
        return in_range_r(i, j, r);
    }

    SG_DEV void eval(bool valid, int i, int j, int, PairOut& o, unsigned long long*) const {
        if (!valid) return;
        eval_r(valid, i, j, pair_rij(pos, i, j, b), o);
    }

    SG_DEV void eval_r(bool valid, int i, int j, float3 r, PairOut& o) const {
        if (!valid) return;
        const float rsq = r.x * r.x + r.y * r.y + r.z * r.z;
        const float rmag = sqrtf(rsq);
        const float rinv = fast_rcp(rmag);
        const float inv_rsq = fast_rcp(rsq);
        const float3 rhat = rinv * r;
        const float4 pi1 = prep[2 * i + 1], pj1 = prep[2 * j + 1], ai = aux[i];
        const float3 U1 = make_float3(pi1.x, pi1.y, pi1.z), U2 = make_float3(pj1.x, pj1.y, pj1.z);
        const float lprp = prep[2 * i].w, chi = pi1.w, xhi = ai.x, inv_ez = ai.y;
        const float ru1 = dot3(r, U1), ru2 = dot3(r, U2), uu = dot3(U1, U2);
        const GTerms gc = gterms(chi, ru1, ru2, uu, inv_rsq);
        const GTerms gx = gterms(xhi, ru1, ru2, uu, inv_rsq);
        const float eps1 = rsqrtf(1.f - (chi * uu) * (chi * uu));
        const float eps2 = gx.g * inv_ez;
        const float sigma = lprp / sqrtf(gc.g);   // correctly rounded: r - sigma sets the envelope
        const float ginv = sigma * fast_rcp(gc.g);
        const float reach = kWeld ? (sigma + cutoff + wf - 1.f) : (sigma + cutoff - 1.f);
        const bool active = prefiltered || ((KIND == SG_GBR) ? (rmag <= sigma) : (rmag < reach));
        if (!active) return;
        o.act = 1;
        float sr;
        if (kWeld) {
            if (rmag < sigma) sr = fast_rcp(rmag - sigma + 1.f);
            else if (rmag <= sigma + wf) sr = 1.f;
            else sr = fast_rcp(rmag - sigma + 1.f - wf);
        } else {
            sr = fast_rcp(rmag - sigma + 1.f);
        }
        const float sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        float srx = sr12 - 2.f * sr6;
        if (KIND == SG_GBR) srx += 1.f;
        float srd = 12.f * (sr6 - sr12) * sr;
        const float e1n = ipowf(eps1, nu), e2m = ipowf(eps2, mu);
        const float ee = e1n * e2m;
        const float pe_fac = e1n * ((float)mu * ipowf(eps2, mu - 1));
        const float e1_fac = e2m * ((float)nu * ipowf(eps1, nu + 2));
        // dG/dr, dG/du1, dG/du2 for chi (shape) and chi' (energy), force.f90:266-306
        const float cr = chi * inv_rsq, xr = xhi * inv_rsq;
        const float3 Up = U1 + U2, Um = U1 - U2;
        const float3 dGr_c = (-cr) * (gc.a * Up + gc.b * Um) + ((2.f * inv_rsq) * (1.f - gc.g)) * r;
        const float3 dGr_x = (-xr) * (gx.a * Up + gx.b * Um) + ((2.f * inv_rsq) * (1.f - gx.g)) * r;
        const float qc = chi * chi * 0.5f * inv_rsq * (gc.a * gc.a - gc.b * gc.b);
        const float qx = xhi * xhi * 0.5f * inv_rsq * (gx.a * gx.a - gx.b * gx.b);
        const float3 dGu1_c = (-cr * (gc.a + gc.b)) * r + qc * U2;
        const float3 dGu1_x = (-xr * (gx.a + gx.b)) * r + qx * U2;
        const float3 dGu2_c = (-cr * (gc.a - gc.b)) * r + qc * U1;
        const float3 dGu2_x = (-xr * (gx.a - gx.b)) * r + qx * U1;
        const float c2uu = chi * chi * uu;
        float3 dR_dr = rhat + (0.5f * ginv) * dGr_c;
        float3 de2_dr = pe_fac * dGr_x;
        float3 de1_du1 = (e1_fac * c2uu) * U2;
        float3 de2_du1 = pe_fac * dGu1_x;
        float3 de1_du2 = (e1_fac * c2uu) * U1;
        float3 de2_du2 = pe_fac * dGu2_x;
        float pot = ee * srx;
        float3 F, TQ1, TQ2;
        if (!kChiral) {
            const float3 dR_du1 = (srd * 0.5f * ginv) * dGu1_c;
            const float3 dR_du2 = (srd * 0.5f * ginv) * dGu2_c;
            F = -1.f * ((ee * srd) * dR_dr + srx * de2_dr);
            const float3 TI = -1.f * (srx * (de1_du1 + de2_du1) + ee * dR_du1);
            const float3 TJ = -1.f * (srx * (de1_du2 + de2_du2) + ee * dR_du2);
            TQ1 = cross3(U1, TI);
            TQ2 = cross3(U2, TJ);
        } else {
            // gbc_ / gbwc_ (force.f90:755-827): e1^nu e2^mu folded into dR terms
            float3 dRdr = ee * dR_dr;
            float3 dR_du1 = (ee * 0.5f * ginv) * dGu1_c;
            float3 dR_du2 = (ee * 0.5f * ginv) * dGu2_c;
            F = -1.f * (srx * de2_dr + srd * dRdr);
            float3 TI = -1.f * (srx * (de1_du1 + de2_du1) + srd * dR_du1);
            float3 TJ = -1.f * (srx * (de1_du2 + de2_du2) + srd * dR_du2);
            TQ1 = cross3(U1, TI);
            TQ2 = cross3(U2, TJ);
            if (KIND == SG_GBC) { srx = sr6 * sr; srd = -7.f * sr6 * sr2; }
            else { srx = sr12 - (12.f / 7.f) * sr6 * sr; srd = 12.f * (sr6 * sr2 - sr12 * sr); }
            const float3 u1xu2 = cross3(U1, U2), u2xr = cross3(U2, rhat), rxu1 = cross3(rhat, U1);
            const float uur = dot3(u1xu2, rhat);
            const float su = srx * uur * uu, du = srd * uur * uu;
            float3 Fc = -1.f * (su * de2_dr + du * dRdr + ((ee * srx * uu) * rinv) * (u1xu2 - uur * rhat));
            float3 TIc = -1.f * (su * (de1_du1 + de2_du1) + du * dR_du1 + (ee * srx * uu) * u2xr + (ee * srx * uur) * U2);
            float3 TJc = -1.f * (su * (de1_du2 + de2_du2) + du * dR_du2 + (ee * srx * uu) * rxu1 + (ee * srx * uur) * U1);
            pot += chirality * (ee * srx * uur * uu);
            F = F + chirality * Fc;
            TQ1 = TQ1 + chirality * cross3(U1, TIc);
            TQ2 = TQ2 + chirality * cross3(U2, TJc);
        }
        if (kTaper) {
            const float sw = 0.9f * reach;
            if (rmag >= sw && rmag <= reach) {
                const float factor = fast_rcp(reach - sw);
                const float xx = (rmag - sw) * factor;
                const float x2 = xx * xx, x3 = x2 * xx;
                const float sx = 1.f - 6.f * x3 * x2 + 15.f * x2 * x2 - 10.f * x3;
                const float sdx = -30.f * x2 * x2 + 60.f * x3 - 30.f * x2;
                const float sub = sdx * pot * factor;   // scalar subtracted from each component (reference quirk)
                F = make_float3(sx * F.x - sub, sx * F.y - sub, sx * F.z - sub);
                TQ1 = make_float3(sx * TQ1.x - sub, sx * TQ1.y - sub, sx * TQ1.z - sub);
                TQ2 = make_float3(sx * TQ2.x - sub, sx * TQ2.y - sub, sx * TQ2.z - sub);
                pot = sx * pot;
            }
        }
        o.pe = pot;
        o.f = F;
        o.ti = TQ1;
        o.tj = TQ2;
        o.vir = dot3(r, F);
    }
};

template <int KIND>
int launch_gb(sg_ctx* ctx, const sg_pair_params* p, float4* prep, int mu, int nu) {
    PotGB<KIND> pot;
    pot.pos = ctx->pos;
    pot.prep = prep;
    pot.aux = prep + 2 * (size_t)ctx->n;
    pot.b = make_boxf(ctx);
    pot.cutoff = (float)p->cutoff;
    pot.wf = (float)p->wf;
    pot.chirality = (float)p->chirality;
    pot.mu = mu;
    pot.nu = nu;
    return launch_pair(ctx, pot, KIND);
}

}  // namespace

int sg_launch_pair_gb(sg_ctx* ctx, const sg_pair_params* p) {
    int mu = p->mu, nu = p->nu;
    if (mu == 0 && nu == 0) { mu = 1; nu = 2; }
    if (mu < 1 || nu < 1 || mu > 8 || nu > 8) return sg_fail(ctx, SG_EINVAL, "GB exponents must be in 1..8");
    // prep buffer: reuse the ECP prep allocation (large enough: 4 float4 per particle)
    if (!ctx->ecp_prep) SG_CUDA(ctx, cudaMalloc(&ctx->ecp_prep, sizeof(float4) * 4 * (size_t)ctx->n));
    k_gb_prep<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->quat, ctx->shape,
                                                            ctx->eshape, 1.f / (float)mu, ctx->ecp_prep);
    SG_LAUNCH_CHECK(ctx, "k_gb_prep");
    switch (p->kind) {
        case SG_GB: return launch_gb<SG_GB>(ctx, p, ctx->ecp_prep, mu, nu);
        case SG_GBR: return launch_gb<SG_GBR>(ctx, p, ctx->ecp_prep, mu, nu);
        case SG_GBW: return launch_gb<SG_GBW>(ctx, p, ctx->ecp_prep, mu, nu);
        case SG_GBC: return launch_gb<SG_GBC>(ctx, p, ctx->ecp_prep, mu, nu);
        case SG_GBWC: return launch_gb<SG_GBWC>(ctx, p, ctx->ecp_prep, mu, nu);
        default: return sg_fail(ctx, SG_EINVAL, "unknown GB kind %d", p->kind);
    }
}
