// Gay-Berne family: gb_, gbr_, gbw_, gbc_, gbwc_ (fortran/force.f90:237-1030),
// FP32 per pair with (mu, nu) as parameters (the reference fixes (1,2) at :240).
//
// As in the reference, the shape (sig_x, sig_z) and energy (eps_x, eps_z)
// anisotropies are those of particle I. A per-particle prep pass hoists what
// depends on one particle only: the body z axis u (first column of the
// reference's U1 formula, :343-349), chi, chi' and 1/eps_z.
//
// The per-particle prep (gb_prep_one, step_epi.cuh) puts each particle's
// position and axis in one 32-byte record, so the range test reads them in
// one load.
//
// Near contact the envelope (r - sigma + 1)^-13 amplifies the rounding of the
// contact distance sigma = sig_x / sqrt(g) thirteenfold, and g = 1 - h cancels
// down to (1 - chi) / (1 + chi) for end-to-end pairs, so FP32 rounding of h
// reaches the 1e-5 force tolerance there. The range test therefore sorts the
// pairs it keeps into two classes: pairs within SG_GB_NEAR of contact are queued
// separately and evaluated with g, sigma and r - sigma in double-float
// arithmetic (from u and chi to 48 bits); the others in FP32.
// stats[3] (the fallbacks field of sg_ecp_stats) counts the precise class.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

// The precise class: pairs with r below the approximate contact distance plus
// this margin (r - sigma + 1 < 1.02: overlapping pairs, where the envelope's
// amplification of the contact distance's rounding is largest).
#ifndef SG_GB_NEAR
#define SG_GB_NEAR 0.02f
#endif

// resident 256-thread blocks per SM for the filtered kernel (64 registers);
// measured on the Gay-Berne workload: 3 blocks 99 µs, 4 blocks 93 µs, and 5
// or 6 slower again (register spills)
#ifndef SG_GB_FILTER_MIN_BLOCKS
#define SG_GB_FILTER_MIN_BLOCKS 4
#endif
#include "pair_common.cuh"
#include "dfloat.cuh"
#include "step_epi.cuh"

namespace {

__global__ void k_gb_prep(int n, const float4* __restrict__ pos, const float4* __restrict__ quat,
                          const float4* __restrict__ shape, const float4* __restrict__ eshape, float muinv,
                          float4* prep) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    gb_prep_one(n, p, pos[p], quat[p], shape[p], eshape[p], muinv, prep);
}

// Shape term g = 1 - (chi/2) [sp^2 / (1 + chi uu) + sm^2 / (1 - chi uu)] / r^2
// (force.f90:266-306) in double-float, as
// 1 - (chi/2) [sp^2 (1 - chi uu) + sm^2 (1 + chi uu)] / [(1 - (chi uu)^2) r^2],
// from u and chi as hi + lo; rsq (r^2) is returned too.
SG_DEV dfl gb_shape_g_df(float3 r, float3 U1, float3 U1l, float3 U2, float3 U2l, dfl chi, dfl& rsq) {
    const dfl ru1 = df_dot3_lo(r, U1, U1l), ru2 = df_dot3_lo(r, U2, U2l), uu = df_dot3_dd(U1, U1l, U2, U2l);
    rsq = df_dot3(r, r);
    const dfl sp = df_add(ru1, ru2), sm = df_sub(ru1, ru2);
    const dfl cuu = df_mul(chi, uu);
    const dfl omc = df_sub(df_of(1.f), cuu), opc = df_add(df_of(1.f), cuu);
    const dfl num = df_add(df_mul(df_mul(sp, sp), omc), df_mul(df_mul(sm, sm), opc));
    const dfl den = df_mul(df_mul(opc, omc), rsq);
    const dfl h = df_div(df_mul_f(df_mul(chi, num), 0.5f), den);
    return df_sub(df_of(1.f), h);
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

// Records of the replica being evaluated by k_pair_gb_tile (2 float4 per
// particle, dynamic shared memory).
extern __shared__ float4 sg_gb_tile[];

// TILE: the position/axis records come from the replica tile in shared
// memory (index i - rec_base) instead of global memory.
template <int KIND, bool TILE = false>
struct PotGB {
    static constexpr bool kTorque = true;
    static constexpr bool kStats = false;
    static constexpr bool kCountActive = true;
    static constexpr bool kWeld = (KIND == SG_GBW || KIND == SG_GBWC);
    static constexpr bool kTaper = (KIND != SG_GBR);
    static constexpr bool kChiral = (KIND == SG_GBC || KIND == SG_GBWC);
    static constexpr bool kFilterable = true;
    static constexpr bool kQueueR = true;        // the range test's r_ij is queued for eval_r
    static constexpr bool kTwoClass = true;      // near-contact pairs: eval_r<true> (double-float contact)
    static constexpr bool kExactFilter = false;  // in_range_r is a superset; eval_r decides
    static constexpr int kMinBlocks = 1;
    static constexpr int kMinBlocksFiltered = SG_GB_FILTER_MIN_BLOCKS;
    const float4* __restrict__ pos;
    const float4* __restrict__ prep;   // rec: 2 per particle
    const float4* __restrict__ aux;    // 1 per particle
    const float4* __restrict__ lo;     // 1 per particle: low parts of u and chi
    int rec_base;                      // TILE: first particle of the tile
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
    // eval_r. Returns 0 (out of range), 1 (in range) or 2 (in range and
    // within SG_GB_NEAR of the approximate contact distance: the precise class).
    SG_DEV int in_range_r(int i, int j, float3& r) const {
        float4 pi0, pi1, pj0, pj1;
        if (TILE) {
            pi0 = sg_gb_tile[2 * (i - rec_base)];
            pi1 = sg_gb_tile[2 * (i - rec_base) + 1];
            pj0 = sg_gb_tile[2 * (j - rec_base)];
            pj1 = sg_gb_tile[2 * (j - rec_base) + 1];
        } else {
            ld_f4x2(prep + 2 * i, pi0, pi1);
            ld_f4x2(prep + 2 * j, pj0, pj1);
        }
        // (the precise class recomputes r_ij to ~1e-12: across the periodic
        // boundary this FP32 difference carries ulp(box)/2)
        r = pair_rij_of(make_float3(pi0.x, pi0.y, pi0.z), make_float3(pj0.x, pj0.y, pj0.z), i, b);
        const float rsq = r.x * r.x + r.y * r.y + r.z * r.z;
        const float3 U1 = make_float3(pi1.x, pi1.y, pi1.z), U2 = make_float3(pj1.x, pj1.y, pj1.z);
        const GTerms gc = gterms(pi1.w, dot3(r, U1), dot3(r, U2), dot3(U1, U2), fast_rcp(rsq));
        const float sigma = pi0.w * fast_rsqrt(gc.g);
        const float rmag = rsq * fast_rsqrt(rsq);
        const float shift = (KIND == SG_GBR) ? 0.f : kWeld ? (cutoff + wf - 1.f) : (cutoff - 1.f);
        if (0.99999f * rmag >= 1.00001f * sigma + shift) return 0;
        return rmag < sigma + SG_GB_NEAR ? 2 : 1;
    }
    SG_DEV bool in_range(int i, int j) const {
        float3 r;
        return in_range_r(i, j, r) != 0;
    }

    // unfiltered launch: the range test's class picks the evaluation, as the
    // queues of the filtered launch do
    SG_DEV void eval(bool valid, int i, int j, int, PairOut& o, unsigned long long*) const {
        if (!valid) return;
        float3 r;
        if (in_range_r(i, j, r) == 2)
            eval_r<true>(valid, i, j, r, o);
        else
            eval_r<false>(valid, i, j, r, o);
    }

    template <bool PRECISE>
    SG_DEV void eval_r(bool valid, int i, int j, float3 r, PairOut& o) const {
        if (!valid) return;
        const float4* rec = TILE ? sg_gb_tile - 2 * rec_base : prep;
        if (PRECISE) {
            // the minimum image to ~1e-12: across the periodic boundary the
            // FP32 difference carries ulp(box)/2, which the envelope amplifies
            const float4 a = rec[2 * i], c = rec[2 * j];
            r = pair_rij_of_precise(make_float3(a.x, a.y, a.z), make_float3(c.x, c.y, c.z), i, b);
        }
        const float rsq = r.x * r.x + r.y * r.y + r.z * r.z;
        const float rmag = sqrtf(rsq);
        const float rinv = fast_rcp(rmag);
        const float inv_rsq = fast_rcp(rsq);
        const float3 rhat = rinv * r;
        const float4 pi1 = rec[2 * i + 1], pj1 = rec[2 * j + 1], ai = aux[i];
        const float3 U1 = make_float3(pi1.x, pi1.y, pi1.z), U2 = make_float3(pj1.x, pj1.y, pj1.z);
        const float lprp = rec[2 * i].w, chi = pi1.w, xhi = ai.x, inv_ez = ai.y;
        const float ru1 = dot3(r, U1), ru2 = dot3(r, U2), uu = dot3(U1, U2);
        GTerms gc = gterms(chi, ru1, ru2, uu, inv_rsq);
        const GTerms gx = gterms(xhi, ru1, ru2, uu, inv_rsq);
        const float eps1 = rsqrtf(1.f - (chi * uu) * (chi * uu));
        const float eps2 = gx.g * inv_ez;
        float sigma = lprp / sqrtf(gc.g);   // correctly rounded: r - sigma sets the envelope
        float rms = rmag - sigma;          // r - sigma
        if (PRECISE) {
            const float4 li = lo[i], lj = lo[j];
            dfl rsq_d;
            const dfl g = gb_shape_g_df(r, U1, make_float3(li.x, li.y, li.z), U2, make_float3(lj.x, lj.y, lj.z),
                                        dfl{chi, li.w}, rsq_d);
            const dfl sig_d = df_div(df_of(lprp), df_sqrt(g));
            const dfl d = df_sub(df_sqrt(rsq_d), sig_d);
            gc.g = g.hi + g.lo;
            sigma = sig_d.hi + sig_d.lo;
            rms = d.hi + d.lo;
        }
        const float ginv = sigma * fast_rcp(gc.g);
        const float reach = kWeld ? (sigma + cutoff + wf - 1.f) : (sigma + cutoff - 1.f);
        const bool active = prefiltered || ((KIND == SG_GBR) ? (rms <= 0.f) : (rmag < reach));
        if (!active) return;
        o.act = 1;
        // 1 / (r - sigma + 1); correctly rounded in the precise class (sr^12
        // carries twelve times its error)
        auto rcp = [](float x) { return PRECISE ? __frcp_rn(x) : fast_rcp(x); };
        float sr;
        if (kWeld) {
            if (rms < 0.f) sr = rcp(rms + 1.f);
            else if (rms <= wf) sr = 1.f;
            else sr = rcp(rms + 1.f - wf);
        } else {
            sr = rcp(rms + 1.f);
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

// ------------------------------------------------------ replica tiles ----
// Gay-Berne replicas, one at a time per block: the replica's position/axis
// records (32 B per particle, at most SG_GB_TILE_MAXN particles) are staged
// in shared memory once, and the range test and evaluation of every listed
// pair of the replica read them from there instead of gathering them from L2
// per pair. The replica's pairs are one contiguous section of the list; the
// block's warps walk it 32 pairs at a time through the same in-range queues
// as k_pair. Blocks take replicas from a work counter, largest first; the
// last block to finish resets the counter for the next launch.
#define SG_GB_TILE_MAXN 2048

struct GbTile {
    const int* order;   // GB replicas, largest first
    int count;
    int* ctr;           // [0] next replica to take, [1] blocks finished
};

template <int KIND>
__global__ void __launch_bounds__(SG_PAIR_MAX_BLOCK, 2) k_pair_gb_tile(PairLaunch L, PotGB<KIND, true> pot, GbTile T) {
    using Pot = PotGB<KIND, true>;
    using Q = PairQueues<Pot>;
    static_assert(Pot::kFilterable && !Pot::kStats && Pot::kMinBlocks == 1 && Pot::kMinBlocksFiltered > 0,
                  "a filtered potential without solver stats");
    __shared__ unsigned long long sh_stats[SG_NSTATS];
    __shared__ int sh_queue[(SG_PAIR_MAX_BLOCK / 32) * Q::kWords];
    __shared__ int sh_r;
    for (int k = threadIdx.x; k < SG_NSTATS; k += blockDim.x) sh_stats[k] = 0ull;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    EnergySums es;
    Q q;
    q.init(sh_queue + warp * Q::kWords);
    for (;;) {
        __syncthreads();   // every warp is done with the previous tile
        if (threadIdx.x == 0) sh_r = atomicAdd(&T.ctr[0], 1);
        __syncthreads();
        const int k = sh_r;
        if (k >= T.count) break;
        const int r = T.order[k];
        const int o = L.rep_off[r], nr = L.rep_off[r + 1] - o;
        for (int p = threadIdx.x; p < 2 * nr; p += blockDim.x) sg_gb_tile[p] = pot.prep[2 * (size_t)o + p];
        __syncthreads();
        Pot pr = pot;
        pr.rec_base = o;
        const float4 bx = pot.b.rbox[r], ib = pot.b.rinv[r], bl = pot.b.rbox_lo[r];
        pr.b.rep_of = nullptr;
        pr.b.box = make_float3(bx.x, bx.y, bx.z);
        pr.b.inv_box = make_float3(ib.x, ib.y, ib.z);
        pr.b.box_lo = make_float3(bl.x, bl.y, bl.z);
        pr.b.periodic = 1;
        const int v0 = L.row_off[o], cnt = L.row_off[o + nr] - v0;
        const long long s0 = L.sec[r];
        // the pair indices stream from DRAM: the next chunk's are loaded before
        // this chunk is tested
        auto fetch = [&](int base, int& t, int& i, int& j, bool& valid) {
            valid = base + lane < cnt;
            t = (int)(s0 + base + lane);
            i = valid ? __ldcs(L.pair_i + t) : -1;
            j = valid ? __ldcs(L.pair_j + t) : 0;
        };
        int tn, in_, jn;
        bool vn;
        fetch(warp * 32, tn, in_, jn, vn);
        for (int base = warp * 32; base < cnt; base += nw * 32) {
            const int t = tn, i = in_, j = jn;
            const bool valid = vn;
            if (base + nw * 32 < cnt) fetch(base + nw * 32, tn, in_, jn, vn);
            q.feed(L, pr, t, i, j, valid, es, sh_stats);
        }
        q.flush(L, pr, es, sh_stats);
    }
    pdl_trigger();   // the final half step may start loading (see k_pair)
    if (threadIdx.x == 0 && atomicAdd(&T.ctr[1], 1) == (int)gridDim.x - 1) {
        T.ctr[0] = 0;   // every block has left the loop
        T.ctr[1] = 0;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < SG_NSTATS; k += blockDim.x)
        if (sh_stats[k]) atomicAdd(&L.stats[k], sh_stats[k]);
    const float e[2] = {es.pe, es.vir}, elo[2] = {es.pe_lo, es.vir_lo};
    block_reduce_finish_f<2>(e, L.partials, L.done, L.acc, L.acc_total, elo);
}

// The GB family's replicas in launch order (largest first) and the counters,
// built once per context; 0 replicas when the largest does not fit a tile.
int gb_tile_setup(sg_ctx* ctx) {
    if (ctx->gb_tile_order) return SG_OK;
    std::vector<int> order;
    int maxn = 0;
    for (int r = ctx->fam_rstart[1]; r < ctx->fam_rstart[2]; ++r) {
        order.push_back(r);
        maxn = std::max(maxn, ctx->h_rep_off[r + 1] - ctx->h_rep_off[r]);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return ctx->h_rep_off[a + 1] - ctx->h_rep_off[a] > ctx->h_rep_off[b + 1] - ctx->h_rep_off[b];
    });
    const size_t words = order.size() + 2;
    SG_CUDA(ctx, cudaMalloc(&ctx->gb_tile_order, sizeof(int) * words));
    std::vector<int> h(order);
    h.push_back(0);
    h.push_back(0);
    SG_CUDA(ctx, cudaMemcpy(ctx->gb_tile_order, h.data(), sizeof(int) * words, cudaMemcpyHostToDevice));
    ctx->gb_tile_count = maxn <= SG_GB_TILE_MAXN ? (int)order.size() : 0;
    ctx->gb_tile_maxn = maxn;
    ctx->graph_epoch++;
    return SG_OK;
}

template <int KIND>
int launch_gb_tile(sg_ctx* ctx, PotGB<KIND> base) {
    PotGB<KIND, true> pot;
    static_assert(sizeof(pot) == sizeof(base), "same layout");
    memcpy((void*)&pot, (const void*)&base, sizeof(pot));
    pot.prefiltered = 0;   // the range test is a superset: eval_r decides
    PairLaunch L = make_pair_launch(ctx);
    GbTile T;
    T.order = ctx->gb_tile_order;
    T.count = ctx->gb_tile_count;
    T.ctr = ctx->gb_tile_order + ctx->gb_tile_count;
    const size_t smem = sizeof(float4) * 2 * (size_t)ctx->gb_tile_maxn;
    const void* fn = (const void*)k_pair_gb_tile<KIND>;
    SG_CUDA(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int grid = sg_grid_for(ctx, fn, SG_PAIR_MAX_BLOCK, smem);
    grid = std::max(1, std::min(grid, T.count));
    if (int rc = sg_ensure_partials(ctx, grid * 2)) return rc;
    L.partials = ctx->partials;
    k_pair_gb_tile<KIND><<<grid, SG_PAIR_MAX_BLOCK, smem, ctx->stream>>>(L, pot, T);
    SG_LAUNCH_CHECK(ctx, "k_pair_gb_tile");
    return SG_OK;
}

template <int KIND>
int launch_gb(sg_ctx* ctx, const sg_pair_params* p, float4* prep, int mu, int nu) {
    PotGB<KIND> pot;
    pot.prefiltered = 0;
    pot.pos = ctx->pos;
    pot.prep = prep;
    pot.aux = prep + 2 * (size_t)ctx->n;
    pot.lo = prep + 3 * (size_t)ctx->n;
    pot.rec_base = 0;
    pot.b = make_boxf(ctx);
    pot.cutoff = (float)p->cutoff;
    pot.wf = (float)p->wf;
    pot.chirality = (float)p->chirality;
    pot.mu = mu;
    pot.nu = nu;
    if (ctx->nrep && sg_pair_tune_for(ctx, KIND, true).filter == 2) {
        if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "pair forces need sg_nlist_init first");
        if (int rc = gb_tile_setup(ctx)) return rc;
        if (ctx->gb_tile_count > 0) return launch_gb_tile<KIND>(ctx, pot);
    }
    return launch_pair(ctx, pot, KIND);
}

}  // namespace

int sg_launch_pair_gb(sg_ctx* ctx, const sg_pair_params* p) {
    int mu = p->mu, nu = p->nu;
    if (mu == 0 && nu == 0) { mu = 1; nu = 2; }
    if (mu < 1 || nu < 1 || mu > 8 || nu > 8) return sg_fail(ctx, SG_EINVAL, "GB exponents must be in 1..8");
    // prep buffer: reuse the ECP prep allocation (large enough: 4 float4 per particle)
    if (!ctx->ecp_prep) SG_CUDA(ctx, cudaMalloc(&ctx->ecp_prep, sizeof(float4) * SG_PREP_F4 * (size_t)ctx->n));
    if (ctx->step_prep_kind != SG_PREP_GB) {   // else written by the step's initial half step
        k_gb_prep<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->quat, ctx->shape,
                                                                ctx->eshape, 1.f / (float)mu, ctx->ecp_prep);
        SG_LAUNCH_CHECK(ctx, "k_gb_prep");
    }
    switch (p->kind) {
        case SG_GB: return launch_gb<SG_GB>(ctx, p, ctx->ecp_prep, mu, nu);
        case SG_GBR: return launch_gb<SG_GBR>(ctx, p, ctx->ecp_prep, mu, nu);
        case SG_GBW: return launch_gb<SG_GBW>(ctx, p, ctx->ecp_prep, mu, nu);
        case SG_GBC: return launch_gb<SG_GBC>(ctx, p, ctx->ecp_prep, mu, nu);
        case SG_GBWC: return launch_gb<SG_GBWC>(ctx, p, ctx->ecp_prep, mu, nu);
        default: return sg_fail(ctx, SG_EINVAL, "unknown GB kind %d", p->kind);
    }
}
