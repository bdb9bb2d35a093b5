// Point-particle pair potentials: lj_, lj12_, ljw_ and wca_
// (fortran/force.f90:6-190), FP32 per pair, FP64 energy sums.
#include <cmath>

#include "pair_common.cuh"

namespace {

struct PotLJ {
    static constexpr bool kTorque = false;
    static constexpr bool kStats = false;
    static constexpr bool kCountActive = true;
    static constexpr bool kFilterable = true;
    static constexpr int kMinBlocks = 1;
    static constexpr int kMinBlocksFiltered = 4;
    const float4* __restrict__ pos;
    BoxF b;
    int kind;
    float sigma, eps, rc, rc2, wf, sig2;
    float pot_cut;    // shift at the cutoff, from the FP64 host value
    int prefiltered;  // eval only sees pairs that passed in_range

    // The range test of eval, alone.
    SG_DEV bool in_range(int i, int j) const {
        const float3 r = pair_rij(pos, i, j, b);
        const float rsq = r.x * r.x + r.y * r.y + r.z * r.z;
        if (kind == SG_LJ || kind == SG_LJ12) return rsq < rc2;
        if (kind == SG_LJW) return sqrtf(rsq) < rc + wf;
        return rsq <= sig2;
    }

    SG_DEV void eval(bool valid, int i, int j, int, PairOut& o, unsigned long long*) const {
        if (!valid) return;
        float3 r = pair_rij(pos, i, j, b);
        float rsq = r.x * r.x + r.y * r.y + r.z * r.z;
        if (kind == SG_LJ) {                         // force.f90:26-47
            if (prefiltered || rsq < rc2) {
                float inv = fast_rcp(rsq);
                float sr2 = sig2 * inv, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
                o.pe = 4.f * eps * (sr12 - sr6) - pot_cut;
                float coeff = 24.f * eps * (2.f * sr12 - sr6) * inv;
                o.f = coeff * r;
                o.vir = coeff * rsq;
                o.act = 1;
            }
        } else if (kind == SG_LJ12) {                // force.f90:72-91
            if (prefiltered || rsq < rc2) {
                float inv = fast_rcp(rsq);
                float sr2 = sig2 * inv, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
                o.pe = eps * (sr12 - 2.f * sr6) - pot_cut;
                float coeff = 12.f * eps * (sr12 - sr6) * inv;
                o.f = coeff * r;
                o.vir = coeff * rsq;
                o.act = 1;
            }
        } else if (kind == SG_LJW) {                 // force.f90:116-144
            float rmag = sqrtf(rsq);
            if (prefiltered || rmag < rc + wf) {
                float sr;
                if (rmag < sigma) sr = sigma / rmag;
                else if (rmag < sigma + wf) sr = 1.f;
                else sr = sigma / (rmag - wf);
                float sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
                o.pe = eps * (sr12 - 2.f * sr6) - pot_cut;
                float coeff = 12.f * eps * (sr12 - sr6) * (sr / sigma) / rmag;
                o.f = coeff * r;
                o.vir = coeff * rsq;
                o.act = 1;
            }
        } else {                                      // SG_WCA, force.f90:175-188
            if (prefiltered || rsq <= sig2) {
                float inv = fast_rcp(rsq);
                float sr2 = sig2 * inv, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
                o.pe = eps * (sr12 - 2.f * sr6) + eps;
                float coeff = 12.f * eps * (sr12 - sr6) * inv;
                o.f = coeff * r;
                o.vir = coeff * rsq;
                o.act = 1;
            }
        }
    }
};

}  // namespace

int sg_launch_pair_simple(sg_ctx* ctx, const sg_pair_params* p) {
    PotLJ pot;
    pot.pos = ctx->pos;
    pot.b = make_boxf(ctx);
    pot.kind = p->kind;
    pot.sigma = (float)p->sigma;
    pot.eps = (float)p->epsilon;
    pot.rc = (float)p->cutoff;
    pot.rc2 = (float)(p->cutoff * p->cutoff);
    pot.wf = (float)p->wf;
    pot.sig2 = (float)(p->sigma * p->sigma);
    double s = p->sigma, e = p->epsilon, rc = p->cutoff;
    double cut = 0.0;
    if (p->kind == SG_LJ) {
        double c2 = (s * s) / (rc * rc), c6 = c2 * c2 * c2;
        cut = 4.0 * e * (c6 * c6 - c6);
    } else if (p->kind == SG_LJ12) {
        double c2 = (s * s) / (rc * rc), c6 = c2 * c2 * c2;
        cut = e * (c6 * c6 - 2.0 * c6);
    } else if (p->kind == SG_LJW) {
        double c = s / rc, c2 = c * c, c6 = c2 * c2 * c2;
        cut = e * (c6 * c6 - 2.0 * c6);
    }
    pot.pot_cut = (float)cut;
    return launch_pair(ctx, pot, p->kind);
}
