// Ellipsoid Contact Potential family: ecp_, ecpr_, ecpw_, ecpc_, ecpwc_
// (fortran/force.f90:1034-2236), with three contact-parameter solvers.
//
// Per particle (k_ecp_prep, once per call) the reference's per-pair setup is
// hoisted: A_R = U^T S^2 U and A_E = U^T E U (matmul_atba, :1294-1297), the
// body z axis and the sigma_t factor (:1299). Per pair, in FP32:
//   EAB = A_R + B_R, eps1 = sigma_t sqrt(det EAB^-1)            (:1303-1305)
//   lambda maximising S(l) = l(1-l) r^T [(1-l)A_R + l B_R]^-1 r    (:1307)
//   K_E, K_R by 3x3 Cholesky, eps2, phi, sigma = phi^-1/2        (:1310-1321)
//   envelope, forces and torques, taper                          (:1325-1376)
// d eps1/d u is summed over the three body axes in the reference (:1346-1352);
// sum_k m_k x (EM m_k) with m_k = s_k u_k equals the axial vector of
// EM A_R, which is what is evaluated here (same value, 18 instead of 45 FMAs).
//
// Solvers:
//   BRENT_COMPAT  the reference's Brent (:1046-1172) in FP64 with every
//                 operation rounded once, in the reference's order: the same
//                 lambda bits as the FP64 reference on the same input.
//   NEWTON        Newton on S'(l) = (1-2l) r.K - l(1-l) K.D.K (D = B_R - A_R)
//                 in FP32 with bracketing, from l = 1/2, then an FP64 check
//                 of |S'| (one step of FP64 iterative refinement of K).
//   NEWTON_SUPPORT the same Newton from l = h_A / (h_A + h_B), where
//                 h_A = sqrt(r.A_R r) and h_B = sqrt(r.B_R r) are |r| times
//                 the support functions of the two ellipsoids along r: the
//                 maximiser of S for two spheres, and on random orientations
//                 2.9 instead of 3.5 evaluations per pair, 4 instead of 6 for
//                 the slowest pair of 32.
//   MLP_NEWTON    the same Newton from the learned guess, at most three
//                 steps, else the plain Newton (counted as a fallback).
#include <cmath>

// Minimum resident blocks of 256 threads the Newton ECP pair kernels are
// compiled for, which caps their registers: 4 -> 64 registers (~300 B
// spilled to L1-resident local memory), 32 resident warps instead of 16. The
// FP64 residual check's latency wants the extra warps: 79.8 -> 72.3 us on the
// N = 65 536 benchmark (3 -> 80 registers: 75.6 us). The Brent and inline-MLP
// kernels keep every register they use.
#ifndef SG_ECP_MIN_BLOCKS
#define SG_ECP_MIN_BLOCKS 4
#endif
#include "pair_common.cuh"
#include "ecp_mlp.cuh"
#include "step_epi.cuh"

// Internal solver ids. SOLVER_MLP_PRE: Newton from a guess already stored in
// the per-pair lambda array (the tensor-core guess pass of mlp_tc.cu).
// SOLVER_GIVEN: the force kernel of the split Newton path, which starts from
// the lambda that k_ecp_solve stored (negative: that solve hit its cap).
#define SOLVER_MLP_PRE 10
#define SOLVER_GIVEN 11

// Minimum resident blocks of 256 threads the force kernel of the split path
// (SOLVER_GIVEN) is compiled for.
#ifndef SG_ECP_FORCE_MIN_BLOCKS
#define SG_ECP_FORCE_MIN_BLOCKS 3
#endif

namespace {

// ------------------------------------------------------------------ prep ---
__global__ void k_ecp_prep(int n, const float4* __restrict__ pos, const float4* __restrict__ quat,
                           const float4* __restrict__ shape, const float4* __restrict__ eshape, float muinv,
                           float4* __restrict__ prep, double* __restrict__ prep64) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    ecp_prep_one(p, pos[p], quat[p], shape[p], eshape[p], muinv, prep, prep + 4 * (size_t)n, prep64);
}

// ------------------------------------------------------------- 3x3 SPD ----
// symmetric storage: 0 xx, 1 xy, 2 xz, 3 yy, 4 yz, 5 zz
struct Chol { float i11, l21, l31, i22, l32, i33; };

SG_DEV Chol chol(const float* g) {
    Chol c;
    c.i11 = rsqrtf(g[0]);
    c.l21 = g[1] * c.i11;
    c.l31 = g[2] * c.i11;
    c.i22 = rsqrtf(g[3] - c.l21 * c.l21);
    c.l32 = (g[4] - c.l31 * c.l21) * c.i22;
    c.i33 = rsqrtf(g[5] - c.l31 * c.l31 - c.l32 * c.l32);
    return c;
}

SG_DEV float3 chol_solve(const Chol& c, float3 b) {
    float y1 = b.x * c.i11;
    float y2 = (b.y - c.l21 * y1) * c.i22;
    float y3 = (b.z - c.l31 * y1 - c.l32 * y2) * c.i33;
    float x3 = y3 * c.i33;
    float x2 = (y2 - c.l32 * x3) * c.i22;
    float x1 = (y1 - c.l21 * x2 - c.l31 * x3) * c.i11;
    return make_float3(x1, x2, x3);
}

SG_DEV float3 symv(const float* m, float3 v) {
    return make_float3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[1] * v.x + m[3] * v.y + m[4] * v.z,
                       m[2] * v.x + m[4] * v.y + m[5] * v.z);
}

// Axial vector of M = S1 * S2 (both symmetric): v_a = eps_abc M_cb.
SG_DEV float3 axial_prod(const float* s1, const float* s2) {
    // M_cb = sum_k s1[c][k] s2[k][b]
    auto e = [](const float* s, int r, int c) {
        const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
        return s[idx[r][c]];
    };
    auto M = [&](int c, int b) { return e(s1, c, 0) * e(s2, 0, b) + e(s1, c, 1) * e(s2, 1, b) + e(s1, c, 2) * e(s2, 2, b); };
    return make_float3(M(2, 1) - M(1, 2), M(0, 2) - M(2, 0), M(1, 0) - M(0, 1));
}

// --------------------------------------------------- FP64 reference Brent --
struct DPair { double ar[6], br[6]; double r[3]; };

__device__ __forceinline__ double ref_optim_dist(double L, const DPair& p) {
    // G = (1-L)*AR + L*BR elementwise (force.f90:1195)
    const double oml = __dsub_rn(1.0, L);
    double g[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) g[m] = __dadd_rn(__dmul_rn(oml, p.ar[m]), __dmul_rn(L, p.br[m]));
    // cholesky_solve (xmath.f90:281-304)
    const double inv_l11 = __ddiv_rn(1.0, __dsqrt_rn(g[0]));
    const double l21 = __dmul_rn(g[1], inv_l11);
    const double l31 = __dmul_rn(g[2], inv_l11);
    const double inv_l22 = __ddiv_rn(1.0, __dsqrt_rn(__dsub_rn(g[3], __dmul_rn(l21, l21))));
    const double l32 = __dmul_rn(__dsub_rn(g[4], __dmul_rn(l31, l21)), inv_l22);
    const double inv_l33 = __ddiv_rn(1.0, __dsqrt_rn(__dsub_rn(__dsub_rn(g[5], __dmul_rn(l31, l31)), __dmul_rn(l32, l32))));
    const double y1 = __dmul_rn(p.r[0], inv_l11);
    const double y2 = __dmul_rn(__dsub_rn(p.r[1], __dmul_rn(l21, y1)), inv_l22);
    const double y3 = __dmul_rn(__dsub_rn(__dsub_rn(p.r[2], __dmul_rn(l31, y1)), __dmul_rn(l32, y2)), inv_l33);
    const double k3 = __dmul_rn(y3, inv_l33);
    const double k2 = __dmul_rn(__dsub_rn(y2, __dmul_rn(l32, k3)), inv_l22);
    const double k1 = __dmul_rn(__dsub_rn(__dsub_rn(y1, __dmul_rn(l21, k2)), __dmul_rn(l31, k3)), inv_l11);
    const double dot = __dadd_rn(__dadd_rn(__dmul_rn(p.r[0], k1), __dmul_rn(p.r[1], k2)), __dmul_rn(p.r[2], k3));
    return -__dmul_rn(__dmul_rn(L, oml), dot);
}

// brent (force.f90:1046-1172): atol 1e-3, rtol 1e-2, <= 10000 iterations,
// including the two evaluations at a and b that the reference discards.
__device__ double ref_brent(const DPair& pair, int& nevals) {
    const int max_iter = 10000;
    const double psi = __dmul_rn(0.5, __dsub_rn(3.0, __dsqrt_rn(5.0)));
    const double atol = 1e-3, rtol = 1e-2;
    double a = 0.0, b = 1.0;
    double c = __dadd_rn(__dmul_rn(__dsub_rn(1.0, psi), a), __dmul_rn(psi, b));
    volatile double fa = ref_optim_dist(a, pair);
    volatile double fb = ref_optim_dist(b, pair);
    (void)fa; (void)fb;
    double fc = ref_optim_dist(c, pair);
    nevals = 3;
    double v = c, w = v, x = w;
    double fv = fc, fw = fv, ft = fw;
    double deltax = 0.0, rat = 0.0;
    for (int iter = 0; iter < max_iter; ++iter) {
        const double tol1 = __dadd_rn(__dmul_rn(rtol, fabs(x)), atol);
        const double tol2 = __dmul_rn(2.0, tol1);
        const double xmid = __dmul_rn(0.5, __dadd_rn(a, b));
        if (fabs(__dsub_rn(x, xmid)) < __dsub_rn(tol2, __dmul_rn(0.5, __dsub_rn(b, a)))) break;
        if (fabs(deltax) <= tol1) {
            deltax = (x >= xmid) ? __dsub_rn(a, x) : __dsub_rn(b, x);
            rat = __dmul_rn(psi, deltax);
        } else {
            double tmp1 = __dmul_rn(__dsub_rn(x, w), __dsub_rn(ft, fv));
            double tmp2 = __dmul_rn(__dsub_rn(x, v), __dsub_rn(ft, fw));
            double pp = __dsub_rn(__dmul_rn(__dsub_rn(x, v), tmp2), __dmul_rn(__dsub_rn(x, w), tmp1));
            tmp2 = __dmul_rn(2.0, __dsub_rn(tmp2, tmp1));
            if (tmp2 > 0.0) pp = -pp;
            tmp2 = fabs(tmp2);
            const double dx_temp = deltax;
            deltax = rat;
            if ((pp > __dmul_rn(tmp2, __dsub_rn(a, x))) && (pp < __dmul_rn(tmp2, __dsub_rn(b, x))) &&
                (fabs(pp) < fabs(__dmul_rn(__dmul_rn(0.5, tmp2), dx_temp)))) {
                rat = __ddiv_rn(__dmul_rn(pp, 1.0), tmp2);
                const double u = __dadd_rn(x, rat);
                if (__dsub_rn(u, a) < tol2 || __dsub_rn(b, u) < tol2) rat = (__dsub_rn(xmid, x) >= 0) ? tol1 : -tol1;
            } else {
                deltax = (x >= xmid) ? __dsub_rn(a, x) : __dsub_rn(b, x);
                rat = __dmul_rn(psi, deltax);
            }
        }
        double u;
        if (fabs(rat) < tol1) u = (rat >= 0) ? __dadd_rn(x, tol1) : __dsub_rn(x, tol1);
        else u = __dadd_rn(x, rat);
        const double fu = ref_optim_dist(u, pair);
        ++nevals;
        if (fu > ft) {
            if (u < x) a = u; else b = u;
            if ((fu <= fw) || (w == x)) { v = w; w = u; fv = fw; fw = fu; }
            else if ((fu <= fv) || (v == x) || (v == w)) { v = u; fv = fu; }
        } else {
            if (u >= x) a = x; else b = x;
            v = w; w = x; x = u;
            fv = fw; fw = ft; ft = fu;
        }
    }
    return x;
}

// -------------------------------------------------------- Newton (FP32) ----
// Start of the support-function Newton: h_A / (h_A + h_B) with h_X = sqrt(r.X r).
SG_DEV float support_guess(const float* A, const float* B, float3 r) {
    const float ha = sqrtf(dot3(r, symv(A, r))), hb = sqrtf(dot3(r, symv(B, r)));
    return ha / (ha + hb);
}

// Bracketed Newton on S'(l) in FP32. Quadratic convergence makes the step
// after one of size < step_tol land at the FP32 noise floor, so that step is
// taken, K is recomputed at the new lambda, and the loop ends.
struct NewtonResult { float lam; int iters; bool converged; Chol c; float3 K; };

SG_DEV NewtonResult newton_solve(const float* A, const float* D, float3 r, float lam0, int max_iter, float step_tol) {
    NewtonResult res;
    float lam = lam0, lo = 0.f, hi = 1.f;
    res.converged = false;
    res.iters = 0;
    float g[6];
    for (int it = 0; it < max_iter; ++it) {
#pragma unroll
        for (int m = 0; m < 6; ++m) g[m] = fmaf(lam, D[m], A[m]);
        res.c = chol(g);
        res.K = chol_solve(res.c, r);
        res.lam = lam;
        res.iters = it + 1;
        const float3 DK = symv(D, res.K);
        const float3 Z = chol_solve(res.c, DK);
        const float rK = dot3(r, res.K), KDK = dot3(res.K, DK), DKZ = dot3(DK, Z);
        const float l1 = lam * (1.f - lam);
        const float s1 = (1.f - 2.f * lam) * rK - l1 * KDK;
        const float s2 = -2.f * rK - 2.f * (1.f - 2.f * lam) * KDK + 2.f * l1 * DKZ;
        if (s1 == 0.f) { res.converged = true; break; }
        const float dl = (s2 < 0.f) ? -s1 / s2 : 1.f;
        // a Newton step below step_tol lands at the FP32 noise floor: take it
        // unbracketed (it may be below the resolution of lambda) and stop
        const bool last = fabsf(dl) < step_tol;
        float ln;
        if (last) {
            ln = fminf(fmaxf(lam + dl, 1e-6f), 1.f - 1e-6f);
        } else {
            if (s1 > 0.f) lo = lam; else hi = lam;
            ln = (s2 < 0.f) ? lam + dl : 0.5f * (lo + hi);
            if (!(ln > lo && ln < hi)) ln = 0.5f * (lo + hi);
        }
        lam = ln;
        if (last) {
#pragma unroll
            for (int m = 0; m < 6; ++m) g[m] = fmaf(lam, D[m], A[m]);
            res.c = chol(g);
            res.K = chol_solve(res.c, r);
            res.lam = lam;
            res.converged = true;
            break;
        }
    }
    return res;
}

// Residual check of the contact solve. The linear-system residual
// e = r - G K of the FP32 solution K, with G = A + lambda D formed exactly, is
// evaluated in extended precision, the correction G^-1 e is solved with the
// FP32 factor, and S'(lambda) = (1-2l) r.K - l(1-l) K.D.K is formed from the
// refined K. With K accurate to ~1e-13 the FP32 dot products contribute
// ~1e-7 of r.K to S' (ten times under the 1e-6 bound); without the refinement
// the FP32 solve alone leaves an error of the order of the bound.
//   mode 1: e in FP64 (nine FP64 FMAs; operands widened on the integer pipe);
//   mode 2: e in double-float arithmetic on the FP32 pipe (error-free
//           products and sums, ~48-bit significand), no FP64 instruction.
// Returns s1 = S' and rK = r.K (the check is |s1| <= tol rK) and S'' (FP32).
SG_DEV void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// e = r - G K in FP64 arithmetic. G = A + lam D is formed exactly as gh + gl
// on the FP32 pipe (gh = fl(A + lam D); gl its rounding error, to 2^-48 |G|);
// r, gh and K are widened exactly, so every product gh_ij K_j is exact in FP64
// and the row sums r_i - sum_j gh_ij K_j carry one FP64 rounding per term:
// nine FP64 FMAs per pair. The small part gl K (~2^-24 |r|) is added in FP32.
SG_DEV float3 lin_residual_fp64(const float* A, const float* D, float3 r, float lam, float3 K) {
    double G[6];
    float gl[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
        const float p = lam * D[m];
        const float pe = fmaf(lam, D[m], -p);
        float sh, se;
        two_sum(A[m], p, sh, se);
        G[m] = widen(sh);
        gl[m] = se + pe;
    }
    const double kx = widen(K.x), ky = widen(K.y), kz = widen(K.z);
    double ex = fma(-G[0], kx, widen(r.x));
    double ey = fma(-G[1], kx, widen(r.y));
    double ez = fma(-G[2], kx, widen(r.z));
    ex = fma(-G[1], ky, ex); ey = fma(-G[3], ky, ey); ez = fma(-G[4], ky, ez);
    ex = fma(-G[2], kz, ex); ey = fma(-G[4], kz, ey); ez = fma(-G[5], kz, ez);
    const float cx = gl[0] * K.x + gl[1] * K.y + gl[2] * K.z;
    const float cy = gl[1] * K.x + gl[3] * K.y + gl[4] * K.z;
    const float cz = gl[2] * K.x + gl[4] * K.y + gl[5] * K.z;
    return make_float3(narrow_trunc(ex) - cx, narrow_trunc(ey) - cy, narrow_trunc(ez) - cz);
}

SG_DEV float3 lin_residual_df(const float* A, const float* D, float3 r, float lam, float3 K) {
    // G = A + lam D as hi + lo (exact up to the lo rounding)
    float gh[6], gl[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) {
        const float p = lam * D[m];
        const float pe = fmaf(lam, D[m], -p);
        float sh, se;
        two_sum(A[m], p, sh, se);
        gh[m] = sh;
        gl[m] = se + pe;
    }
    const float kv[3] = {K.x, K.y, K.z};
    const float rv[3] = {r.x, r.y, r.z};
    const int row[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    float out[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        // e_i = r_i - sum_j G_ij K_j, accumulated as hi + lo
        float hi = rv[i], lo = 0.f;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int m = row[i][j];
            const float t = gh[m] * kv[j];
            const float te = fmaf(gh[m], kv[j], -t);
            float sh, se;
            two_sum(hi, -t, sh, se);
            hi = sh;
            lo += se - te - gl[m] * kv[j];
        }
        out[i] = hi + lo;
    }
    return make_float3(out[0], out[1], out[2]);
}

// K + dk as a float pair: hi = fl(K + dk) and the exact rounding error.
SG_DEV void add_refinement(float3 K, float3 dk, float3& hi, float3& lo) {
    float s, e;
    two_sum(K.x, dk.x, s, e); hi.x = s; lo.x = e;
    two_sum(K.y, dk.y, s, e); hi.y = s; lo.y = e;
    two_sum(K.z, dk.z, s, e); hi.z = s; lo.z = e;
}

SG_DEV float residual_check(int mode, const float* A, const float* D, float3 r, float lam, const Chol& c, float3 K,
                            float& rK_out, float& s2, float3& Kr, float3& Krlo) {
    const float3 e = mode == 2 ? lin_residual_df(A, D, r, lam, K) : lin_residual_fp64(A, D, r, lam, K);
    const float3 dk = chol_solve(c, e);
    add_refinement(K, dk, Kr, Krlo);
    const float3 DK = symv(D, Kr);
    const float rK = dot3(r, Kr), KDK = dot3(Kr, DK);
    const float3 Z = chol_solve(c, DK);
    const float l1 = lam * (1.f - lam);
    s2 = -2.f * rK - 2.f * (1.f - 2.f * lam) * KDK + 2.f * l1 * dot3(DK, Z);
    rK_out = rK;
    return (1.f - 2.f * lam) * rK - l1 * KDK;
}

template <int SOLVER>
struct PotECP {
    static constexpr bool kTorque = true;
    static constexpr bool kStats = true;
    static constexpr bool kCountActive = false;
    // the Newton solvers take the support-function range test (in_range)
    static constexpr bool kFilterable = SOLVER == SG_SOLVER_NEWTON || SOLVER == SG_SOLVER_NEWTON_SUPPORT;
    static constexpr bool kExactFilter = false;
    static constexpr int kMinBlocks =
        (SOLVER == SG_SOLVER_NEWTON || SOLVER == SG_SOLVER_NEWTON_SUPPORT || SOLVER == SOLVER_MLP_PRE)
            ? SG_ECP_MIN_BLOCKS
        : SOLVER == SOLVER_GIVEN                                ? SG_ECP_FORCE_MIN_BLOCKS
                                                                : 1;
    static constexpr int kMinBlocksFiltered = SG_ECP_MIN_BLOCKS;
    int prefiltered;
    // Range test of the filtered launch, a superset of the pairs eval keeps,
    // from two upper bounds on the Perram-Wertheim contact distance sigma:
    //  (1) sigma <= h_A + h_B, the two ellipsoids' support functions along r
    //      (h_X = sqrt(r.X r) / |r|, X = U^T S^2 U): at that separation a plane
    //      normal to r separates them;
    //  (2) sigma <= |r| / sqrt(F(l0)) for any l, F(l) = l(1-l) r.(A + l(B-A))^-1 r
    //      the contact function whose maximum over l gives sigma = |r| / sqrt(F*);
    //      taken at the support start l0 = h_A / (h_A + h_B), one evaluation.
    // A pair with |r| >= bound + (reach - sigma) is inactive in eval and skips
    // the contact solve. The bounds are widened (2e-4 and 1e-3 relative, 1e-4)
    // for the FP32 rounding of r, h, F and sigma; NaN keeps the pair. Each
    // particle's position and A_R come from its 32-byte range record (one
    // load), A_R as the FP16 matrix plus d I, which bounds A_R from above
    // (ecp_range_one), so both bounds stay upper bounds.
    SG_DEV bool in_range(int i, int j) const {
        float4 a0, a1, b0, b1;
        ld_f4x2(range + 2 * i, a0, a1);
        ld_f4x2(range + 2 * j, b0, b1);
        float A[6], B[6];
        range_matrix(a0.w, a1, A);
        range_matrix(b0.w, b1, B);
        return range_test(make_float3(a0.x, a0.y, a0.z), make_float3(b0.x, b0.y, b0.z), A, B, i);
    }
    static SG_DEV void range_matrix(float d, float4 w, float (&A)[6]) {
        const unsigned u[3] = {__float_as_uint(w.x), __float_as_uint(w.y), __float_as_uint(w.z)};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            A[2 * k] = __half2float(__ushort_as_half((unsigned short)(u[k] & 0xffffu)));
            A[2 * k + 1] = __half2float(__ushort_as_half((unsigned short)(u[k] >> 16)));
        }
        A[0] += d;
        A[3] += d;
        A[5] += d;
    }
    SG_DEV bool range_test(float3 pi, float3 pj, const float (&A)[6], const float (&B)[6], int i) const {
        const float3 r = pair_rij_of(pi, pj, i, b);
        const float rsq = dot3(r, r), rinv = rsqrtf(rsq), rm = rsq * rinv;
        const float ha = sqrtf(dot3(r, symv(A, r))), hb = sqrtf(dot3(r, symv(B, r)));   // |r| h_A, |r| h_B
        if (rm >= ((ha + hb) * rinv + reach_extra) * 1.0002f + 1e-4f) return false;
        const float l0 = ha / (ha + hb);
        float g[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) g[m] = fmaf(l0, B[m] - A[m], A[m]);
        const float F = l0 * (1.f - l0) * dot3(r, chol_solve(chol(g), r));
        return !(rm >= (rm * rsqrtf(F) + reach_extra) * 1.001f + 1e-4f);
    }
    // a listed pair that in_range turned away: its lambda reads NaN (not solved)
    SG_DEV void filtered_out(int t) const {
        if (lam_out) lam_out[t] = __int_as_float(0x7fc00000);
    }
    const float4* __restrict__ pos;
    const float4* __restrict__ quat;
    const float4* __restrict__ shape;
    const float4* __restrict__ prep;
    const float4* __restrict__ range;   // the range records (prep + 4n)
    const double* __restrict__ prep64;
    float* __restrict__ lam_out;
    MlpDev mlp;
    BoxF b;
    double bx, by, bz;
    int kind, mu, nu, max_iter, fp64_check;
    float cutoff, wf, chirality, tol, step_tol;
    float reach_extra;   // reach - sigma: cutoff - 1 (+ wf welded), 0 for the repulsive kind
    bool weld, chiral, rep;

    SG_DEV void eval(bool valid, int i, int j, int t, PairOut& o, unsigned long long* sh) const;
    SG_DEV float solve_lambda(int i, int j, float3 r, const float* A, const float* Bm, float lam0, Chol& cR,
                              float3& KR, float3& KRlo, unsigned& evals, unsigned& iters, bool& nonconv, bool& fallback,
                              bool& refined) const;
};

template <int SOLVER>
SG_DEV float PotECP<SOLVER>::solve_lambda(int i, int j, float3 r, const float* A, const float* Bm, float lam0,
                                          Chol& cR, float3& KR, float3& KRlo, unsigned& evals, unsigned& iters,
                                          bool& nonconv,
                                          bool& fallback, bool& refined) const {
    float D[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) D[m] = Bm[m] - A[m];
    float lam;
    if (SOLVER == SG_SOLVER_BRENT_COMPAT) {
        DPair dp;
        const float4 a = pos[i], c = pos[j];
        double dx = __dsub_rn((double)a.x, (double)c.x), dy = __dsub_rn((double)a.y, (double)c.y),
               dz = __dsub_rn((double)a.z, (double)c.z);
        if (b.periodic) {
            dx = __dsub_rn(dx, __dmul_rn(round(__ddiv_rn(dx, bx)), bx));
            dy = __dsub_rn(dy, __dmul_rn(round(__ddiv_rn(dy, by)), by));
            dz = __dsub_rn(dz, __dmul_rn(round(__ddiv_rn(dz, bz)), bz));
        }
        dp.r[0] = dx; dp.r[1] = dy; dp.r[2] = dz;
#pragma unroll
        for (int m = 0; m < 6; ++m) { dp.ar[m] = prep64[6 * (size_t)i + m]; dp.br[m] = prep64[6 * (size_t)j + m]; }
        int nev = 0;
        lam = (float)ref_brent(dp, nev);
        evals = nev;
        iters = nev;
        float g[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) g[m] = fmaf(lam, D[m], A[m]);
        cR = chol(g);
        KR = chol_solve(cR, r);
        KRlo = make_float3(0.f, 0.f, 0.f);
        if (fp64_check) {
            // refine K_R against the exact G(lambda): it sets the contact distance
            const float3 e = fp64_check == 2 ? lin_residual_df(A, D, r, lam, KR) : lin_residual_fp64(A, D, r, lam, KR);
            const float3 dk = chol_solve(cR, e);
            add_refinement(KR, dk, KR, KRlo);
        }
        return lam;
    }
    NewtonResult nr;
    if constexpr (SOLVER == SOLVER_GIVEN) {
        // lambda from k_ecp_solve (negative: its solve hit the iteration cap);
        // the factor and K at that lambda are those of its last evaluation
        lam = fabsf(lam0);
        nonconv = lam0 < 0.f;
        float g[6];
#pragma unroll
        for (int m = 0; m < 6; ++m) g[m] = fmaf(lam, D[m], A[m]);
        nr.c = chol(g);
        nr.K = chol_solve(nr.c, r);
        nr.lam = lam;
    } else {
        constexpr bool kGuess = (SOLVER == SG_SOLVER_MLP_NEWTON || SOLVER == SOLVER_MLP_PRE);
        const int budget = kGuess ? 3 : max_iter;
        if (SOLVER == SG_SOLVER_NEWTON_SUPPORT) lam0 = support_guess(A, Bm, r);
        nr = newton_solve(A, D, r, lam0, budget, step_tol);
        evals = nr.iters;
        if (kGuess && !nr.converged) {
            fallback = true;
            nr = newton_solve(A, D, r, 0.5f, max_iter, step_tol);
            evals += nr.iters;
        }
        iters = nr.iters;
        lam = nr.lam;
        nonconv = !nr.converged;
    }
    KRlo = make_float3(0.f, 0.f, 0.f);
    if (fp64_check) {
        float s2, rK;
        float3 Kr;
        const float s1 = residual_check(fp64_check, A, D, r, lam, nr.c, nr.K, rK, s2, Kr, KRlo);
        if (!(fabsf(s1) <= tol * rK)) {
            // one Newton step driven by the extended-precision residual
            refined = true;
            evals += 1;
            if (s2 < 0.f) {
                const float ln = lam - s1 / s2;
                if (ln > 0.f && ln < 1.f) {
                    lam = ln;
                    float g[6];
#pragma unroll
                    for (int m = 0; m < 6; ++m) g[m] = fmaf(lam, D[m], A[m]);
                    nr.c = chol(g);
                    nr.K = chol_solve(nr.c, r);
                }
            }
            const float s1b = residual_check(fp64_check, A, D, r, lam, nr.c, nr.K, rK, s2, Kr, KRlo);
            if (!(fabsf(s1b) <= tol * rK)) nonconv = true;
        }
        nr.K = Kr;   // the refined K feeds the force terms
    }
    cR = nr.c;
    KR = nr.K;
    return lam;
}

template <int SOLVER>
SG_DEV void PotECP<SOLVER>::eval(bool valid, int i, int j, int t, PairOut& o, unsigned long long* sh) const {
    const float3 r = pair_rij_precise(pos, i, j, b);   // invalid lanes evaluate (0,0): never used
    float lam0 = 0.5f;
    if (SOLVER == SOLVER_MLP_PRE || SOLVER == SOLVER_GIVEN) {
        // the guess of the tensor-core pass, or the solved lambda, stored where
        // this pair's lambda goes
        lam0 = valid ? lam_out[t] : 0.5f;
    }
    if (SOLVER == SG_SOLVER_MLP_NEWTON) {
        float f[16];
        mlp_features(valid ? r : make_float3(1.f, 0.f, 0.f), quat[i], quat[j], shape[i], shape[j], f);
        lam0 = mlp_warp_guess(mlp, f);   // all 32 lanes
    }
    const float rsq = dot3(r, r);
    const float rinv = rsqrtf(rsq);
    const float rmag = rsq * rinv;
    const float3 rhat = rinv * r;
    const float4 pi0 = prep[4 * i], pi1 = prep[4 * i + 1], pi2 = prep[4 * i + 2], pi3 = prep[4 * i + 3];
    const float4 pj0 = prep[4 * j], pj1 = prep[4 * j + 1], pj2 = prep[4 * j + 2], pj3 = prep[4 * j + 3];
    const float A[6] = {pi0.x, pi0.y, pi0.z, pi0.w, pi1.x, pi1.y};
    const float Bm[6] = {pj0.x, pj0.y, pj0.z, pj0.w, pj1.x, pj1.y};
    const float AE[6] = {pi1.z, pi1.w, pi2.x, pi2.y, pi2.z, pi2.w};
    const float BE[6] = {pj1.z, pj1.w, pj2.x, pj2.y, pj2.z, pj2.w};

    unsigned evals = 0, iters = 0;
    bool nonconv = false, fallback = false, refined = false;
    Chol cR;
    float3 KR = make_float3(0.f, 0.f, 0.f), KRlo = KR;
    float lam = 0.5f;
    if (valid) {
        lam = solve_lambda(i, j, r, A, Bm, lam0, cR, KR, KRlo, evals, iters, nonconv, fallback, refined);
        if (lam_out && (SOLVER != SOLVER_GIVEN || refined || nonconv)) lam_out[t] = lam;
    }
    {
        // warp-aggregated solver statistics into the block's shared counters
        const unsigned full = 0xffffffffu;
        const int lane = threadIdx.x & 31;
        const unsigned ev = __reduce_add_sync(full, valid ? evals : 0u);
        const unsigned np = __popc(__ballot_sync(full, valid));
        const unsigned nc = __popc(__ballot_sync(full, valid && nonconv));
        const unsigned fb = __popc(__ballot_sync(full, valid && fallback));
        const unsigned rf = __popc(__ballot_sync(full, valid && refined));
        if (SOLVER != SOLVER_GIVEN) {   // the split path's solve kernel keeps the histogram
            const unsigned key = valid ? min(iters, 23u) : 255u;
            const unsigned peers = __match_any_sync(full, key);
            if (key != 255u && lane == __ffs(peers) - 1) atomicAdd(&sh[4 + key], (unsigned long long)__popc(peers));
        }
        if (lane == 0) {
            atomicAdd(&sh[0], (unsigned long long)np);
            if (ev) atomicAdd(&sh[1], (unsigned long long)ev);
            if (nc) atomicAdd(&sh[2], (unsigned long long)nc);
            if (fb) atomicAdd(&sh[3], (unsigned long long)fb);
            if (rf) atomicAdd(&sh[28], (unsigned long long)rf);
        }
    }
    if (!valid) return;
    // eps1 = sigma_t sqrt(det (A+B)^-1); EM = (A+B)^-1 (symmetric)
    float S[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) S[m] = A[m] + Bm[m];
    const float c00 = S[3] * S[5] - S[4] * S[4], c01 = S[2] * S[4] - S[1] * S[5], c02 = S[1] * S[4] - S[2] * S[3];
    const float c11 = S[0] * S[5] - S[2] * S[2], c12 = S[1] * S[2] - S[0] * S[4], c22 = S[0] * S[3] - S[1] * S[1];
    const float det = S[0] * c00 + S[1] * c01 + S[2] * c02;
    const float idet = 1.f / det;
    const float EM[6] = {c00 * idet, c01 * idet, c02 * idet, c11 * idet, c12 * idet, c22 * idet};
    const float eps1 = sqrtf(pi3.w * pj3.w * idet);
    const float oml = 1.f - lam;
    float GE[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) GE[m] = oml * AE[m] + lam * BE[m];
    const Chol cE = chol(GE);
    const float3 KE = chol_solve(cE, r);   // enters eps2^mu only: FP32 suffices
    const float l1 = lam * oml;
    const float rKE = dot3(r, KE), rKR = dot3(r, KR);
    const float inv_rsq = 1.f / rsq;
    const float eps2 = l1 * rKE * inv_rsq;
    // contact distance sigma = r / sqrt(S), S = l(1-l) r.K_R (force.f90:1316-1317); the
    // envelope needs r - sigma, formed without cancellation as r (S-1) / (sqrt S (sqrt S + 1)).
    // S - 1 is what sets the repulsion near contact, so it is formed in double-float:
    // r.K_R from the refined K_R (hi + lo) with exact products, l(1-l) exactly.
    const float Sc = l1 * rKR;
    float Sm1;
    {
        float omh, oml_e;
        two_sum(1.f, -lam, omh, oml_e);                     // 1 - lambda = omh + oml_e
        const float l1h = lam * omh, l1e = fmaf(lam, omh, -l1h) + lam * oml_e;
        float rkh = r.x * KR.x, rke = fmaf(r.x, KR.x, -rkh);
        float p = r.y * KR.y, pe = fmaf(r.y, KR.y, -p), s, e;
        two_sum(rkh, p, s, e); rkh = s; rke += e + pe;
        p = r.z * KR.z; pe = fmaf(r.z, KR.z, -p);
        two_sum(rkh, p, s, e); rkh = s; rke += e + pe;
        rke += r.x * KRlo.x + r.y * KRlo.y + r.z * KRlo.z;
        const float Sh = l1h * rkh, Se = fmaf(l1h, rkh, -Sh) + l1h * rke + l1e * rkh;
        two_sum(Sh, -1.f, s, e);
        Sm1 = s + (e + Se);
    }
    const float sqS = sqrtf(Sc);
    const float rexact = sqrtf(rsq);
    const float rms = rexact * Sm1 / (sqS * (sqS + 1.f));   // r - sigma
    const float sigma = rexact / sqS;
    const float fac = 2.f * l1 * inv_rsq;   // efac = rfac (lambda_E = lambda_R, force.f90:1308)
    const float pi32 = sigma * sigma * sigma;
    const float reach = weld ? (sigma + cutoff + wf - 1.f) : (sigma + cutoff - 1.f);
    const bool active = rep ? (rms <= 0.f) : (rmag < reach);
    if (!active) return;
    float sr;
    if (weld) {
        if (rms < 0.f) sr = 1.f / (rms + 1.f);
        else if (rms <= wf) sr = 1.f;
        else sr = 1.f / (rms + 1.f - wf);
    } else {
        sr = 1.f / (rms + 1.f);
    }
    const float sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
    float srx = sr12 - 2.f * sr6;
    if (rep) srx += 1.f;
    float srd = 12.f * (sr6 - sr12) * sr;
    const float e1n = ipowf(eps1, nu), e2m = ipowf(eps2, mu);
    const float ee = e1n * e2m;
    const float e2fac = e1n * ((float)mu * ipowf(eps2, mu - 1));
    const float e1fac = e2m * ((float)nu * ipowf(eps1, nu));
    const float rhKR = rKR * rinv, rhKE = rKE * rinv;
    const float3 dR_dr = rhat + (0.5f * fac * pi32) * (KR - rhKR * rhat);
    const float3 de2_dr = (e2fac * fac) * (KE - rhKE * rhat);
    const float3 ax1 = axial_prod(EM, A), ax2 = axial_prod(EM, Bm);
    const float3 xa = cross3(symv(AE, KE), KE), xb = cross3(symv(A, KR), KR);
    const float3 xc = cross3(symv(BE, KE), KE), xd = cross3(symv(Bm, KR), KR);
    // terms without the envelope factors srx / srd
    const float3 de1_du1 = e1fac * ax1, de1_du2 = e1fac * ax2;
    const float3 de2_du1 = (e2fac * oml * fac) * xa, de2_du2 = (e2fac * lam * fac) * xc;
    const float3 dR_du1 = (ee * 0.5f * oml * fac * pi32) * xb, dR_du2 = (ee * 0.5f * lam * fac * pi32) * xd;
    float pot = ee * srx;
    float3 F = -1.f * ((ee * srd) * dR_dr + srx * de2_dr);
    float3 TQ1 = srx * (de1_du1 + de2_du1) + srd * dR_du1;
    float3 TQ2 = srx * (de1_du2 + de2_du2) + srd * dR_du2;
    if (chiral) {
        // ecpc_ (force.f90:1774-1826) / ecpwc_ (:2021-2073)
        if (kind == SG_ECPC) { srx = sr6 * sr; srd = -7.f * sr6 * sr2; }
        else { srx = sr12 - (12.f / 7.f) * sr6 * sr; srd = 12.f * (sr6 * sr2 - sr12 * sr); }
        const float3 u1z = make_float3(pi3.x, pi3.y, pi3.z), u2z = make_float3(pj3.x, pj3.y, pj3.z);
        const float3 u1xu2 = cross3(u1z, u2z), u2xr = cross3(u2z, rhat), rxu1 = cross3(rhat, u1z);
        const float uur = dot3(u1xu2, rhat), uu = dot3(u1z, u2z);
        const float su = srx * uur * uu, du = srd * uur * uu;
        const float3 Fc = -1.f * (su * de2_dr + (du * ee) * dR_dr + ((ee * srx * uu) * rinv) * (u1xu2 - uur * rhat));
        const float3 t1 = (ee * srx * uu) * u2xr + (ee * srx * uur) * u2z;
        const float3 t2 = (ee * srx * uu) * rxu1 + (ee * srx * uur) * u1z;
        const float3 T1c = su * (de1_du1 + de2_du1) + du * dR_du1 - cross3(u1z, t1);
        const float3 T2c = su * (de1_du2 + de2_du2) + du * dR_du2 - cross3(u2z, t2);
        pot += chirality * (ee * srx * uur * uu);
        F = F + chirality * Fc;
        TQ1 = TQ1 + chirality * T1c;
        TQ2 = TQ2 + chirality * T2c;
    }
    if (!rep) {
        const float sw = 0.9f * reach;
        if (rmag >= sw && rmag <= reach) {
            const float factor = 1.f / (reach - sw);
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

// ------------------------------------------------- split Newton: solve ----
// The Newton solve of the split path: lambda for every listed pair and the
// solver statistics, nothing else. Its registers are those of the Newton loop
// alone, so it keeps many more warps resident than a kernel that also holds
// the force terms; the force kernel (PotECP<SOLVER_GIVEN>) then starts from
// the stored lambda with the same work for every pair, the residual check
// included. lambda is stored negated when the solve hit its iteration cap.
struct EcpSolveArgs {
    const float4* __restrict__ pos;
    const float4* __restrict__ prep;
    float* __restrict__ lam;   // in: the learned guess (SOLVER_MLP_PRE); out: lambda
    BoxF b;
    int max_iter;
    float step_tol;
};

template <int SOLVER>
__global__ void __launch_bounds__(SG_PAIR_MAX_BLOCK) k_ecp_solve(PairLaunch L, EcpSolveArgs a) {
    constexpr bool kGuess = SOLVER == SOLVER_MLP_PRE;
    __shared__ unsigned long long sh[SG_NSTATS];
    for (int k = threadIdx.x; k < SG_NSTATS; k += blockDim.x) sh[k] = 0ull;
    __syncthreads();
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int np = *L.npairs;
    const int b0 = L.begin ? *L.begin : 0;
    const int bstart = L.sec ? (b0 & ~31) : b0;
    for (int base = bstart + gwarp * 32; base < np; base += nwarps * 32) {
        int t, i, j;
        bool valid;
        pair_fetch(L, base, lane, np, b0, t, i, j, valid);
        unsigned evals = 0, iters = 0;
        bool fallback = false;
        if (valid) {
            const float3 r = pair_rij_precise(a.pos, i, j, a.b);
            const float4 pi0 = a.prep[4 * i], pi1 = a.prep[4 * i + 1];
            const float4 pj0 = a.prep[4 * j], pj1 = a.prep[4 * j + 1];
            const float A[6] = {pi0.x, pi0.y, pi0.z, pi0.w, pi1.x, pi1.y};
            const float D[6] = {pj0.x - A[0], pj0.y - A[1], pj0.z - A[2], pj0.w - A[3], pj1.x - A[4], pj1.y - A[5]};
            const float B[6] = {pj0.x, pj0.y, pj0.z, pj0.w, pj1.x, pj1.y};
            const float lam0 = kGuess                                 ? a.lam[t]
                               : SOLVER == SG_SOLVER_NEWTON_SUPPORT ? support_guess(A, B, r)
                                                                      : 0.5f;
            NewtonResult nr = newton_solve(A, D, r, lam0, kGuess ? 3 : a.max_iter, a.step_tol);
            evals = nr.iters;
            if (kGuess && !nr.converged) {
                fallback = true;
                nr = newton_solve(A, D, r, 0.5f, a.max_iter, a.step_tol);
                evals += nr.iters;
            }
            iters = nr.iters;
            a.lam[t] = nr.converged ? nr.lam : -nr.lam;
        }
        // warp-aggregated: evaluations, fallbacks, iteration histogram
        const unsigned ev = __reduce_add_sync(full, evals);
        const unsigned fb = __popc(__ballot_sync(full, fallback));
        const unsigned key = valid ? min(iters, 23u) : 255u;
        const unsigned peers = __match_any_sync(full, key);
        if (key != 255u && lane == __ffs(peers) - 1) atomicAdd(&sh[4 + key], (unsigned long long)__popc(peers));
        if (lane == 0) {
            if (ev) atomicAdd(&sh[1], (unsigned long long)ev);
            if (fb) atomicAdd(&sh[3], (unsigned long long)fb);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < SG_NSTATS; k += blockDim.x)
        if (sh[k]) atomicAdd(&L.stats[k], sh[k]);
}

template <int SOLVER>
int launch_ecp_solve(sg_ctx* ctx, const sg_pair_params* p) {
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "pair forces need sg_nlist_init first");
    PairLaunch L = make_pair_launch(ctx);
    EcpSolveArgs a;
    a.pos = ctx->pos;
    a.prep = ctx->ecp_prep;
    a.lam = ctx->ecp_lambda;
    a.b = make_boxf(ctx);
    a.max_iter = p->newton_max_iter > 0 ? p->newton_max_iter : 20;
    a.step_tol = 1e-4f;
    const int block = SG_PAIR_MAX_BLOCK;
    int grid = sg_grid_for(ctx, (const void*)k_ecp_solve<SOLVER>, block, 0);
    const int64_t max_useful = (ctx->nl.pair_capacity + block - 1) / block;
    if (grid > max_useful) grid = (int)std::max<int64_t>(1, max_useful);
    k_ecp_solve<SOLVER><<<grid, block, 0, ctx->stream>>>(L, a);
    SG_LAUNCH_CHECK(ctx, "k_ecp_solve");
    return SG_OK;
}

template <int SOLVER>
int launch_ecp(sg_ctx* ctx, const sg_pair_params* p, int mu, int nu) {
    PotECP<SOLVER> pot;
    pot.pos = ctx->pos;
    pot.quat = ctx->quat;
    pot.shape = ctx->shape;
    pot.prep = ctx->ecp_prep;
    pot.range = ctx->ecp_prep + 4 * (size_t)ctx->n;
    pot.prep64 = ctx->ecp_prep64;
    pot.lam_out = ctx->ecp_lambda;
    if (ctx->mlp_ready) pot.mlp = *(const MlpDev*)ctx->mlp_host_desc;
    else pot.mlp = MlpDev{};
    pot.b = make_boxf(ctx);
    pot.bx = ctx->box[0]; pot.by = ctx->box[1]; pot.bz = ctx->box[2];
    pot.kind = p->kind;
    pot.mu = mu;
    pot.nu = nu;
    pot.max_iter = p->newton_max_iter > 0 ? p->newton_max_iter : 20;
    pot.fp64_check = p->fp64_check;
    pot.cutoff = (float)p->cutoff;
    pot.wf = (float)p->wf;
    pot.chirality = (float)p->chirality;
    pot.tol = (float)(p->newton_tol > 0.0 ? p->newton_tol : 1e-6);
    pot.step_tol = 1e-4f;
    pot.weld = (p->kind == SG_ECPW || p->kind == SG_ECPWC);
    pot.chiral = (p->kind == SG_ECPC || p->kind == SG_ECPWC);
    pot.rep = (p->kind == SG_ECPR);
    pot.reach_extra = pot.rep ? 0.f : pot.cutoff - 1.f + (pot.weld ? pot.wf : 0.f);
    const PairTune tune = sg_pair_tune_for(ctx, p->kind, false);
    // the support-filtered launch (tune.filter 2) leaves lambda unset (NaN)
    // for the pairs it does not solve
    ctx->ecp_lambda_partial = PotECP<SOLVER>::kFilterable && tune.filter == 2;
    // single systems: the range test in a pass of its own, then the contact
    // solve over the compacted pairs; replica contexts: per-warp queues
    if constexpr (PotECP<SOLVER>::kFilterable)
        if (tune.filter == 2 && !ctx->nrep) return launch_pair_two_pass(ctx, pot, tune.block);
    return launch_pair(ctx, pot, p->kind);
}

}  // namespace

int sg_ecp_prepare(sg_ctx* ctx, const sg_pair_params* p, int need64) {
    int mu = p->mu > 0 ? p->mu : 2;
    if (!ctx->ecp_prep) SG_CUDA(ctx, cudaMalloc(&ctx->ecp_prep, sizeof(float4) * SG_PREP_F4 * (size_t)ctx->n));
    if (need64 && !ctx->ecp_prep64) SG_CUDA(ctx, cudaMalloc(&ctx->ecp_prep64, sizeof(double) * 6 * (size_t)ctx->n));
    k_ecp_prep<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->quat, ctx->shape, ctx->eshape,
                                                             1.f / (float)mu, ctx->ecp_prep,
                                                             need64 ? ctx->ecp_prep64 : nullptr);
    SG_LAUNCH_CHECK(ctx, "k_ecp_prep");
    return SG_OK;
}

int sg_launch_pair_ecp(sg_ctx* ctx, const sg_pair_params* p) {
    int mu = p->mu, nu = p->nu;
    if (mu == 0 && nu == 0) { mu = 2; nu = 1; }
    if (mu < 1 || nu < 1 || mu > 8 || nu > 8) return sg_fail(ctx, SG_EINVAL, "ECP exponents must be in 1..8");
    const int brent = p->solver == SG_SOLVER_BRENT_COMPAT;
    if (p->solver == SG_SOLVER_MLP_NEWTON && !ctx->mlp_ready)
        return sg_fail(ctx, SG_ENOTREADY, "MLP solver selected but no weights were set (sg_mlp_set_weights)");
    if (!(ctx->step_prep_kind == SG_PREP_ECP && !brent))   // else written by the step's initial half step
        if (int rc = sg_ecp_prepare(ctx, p, brent)) return rc;
    if (ctx->ecp_lambda_cap < ctx->nl.pair_capacity) {
        ctx->graph_epoch++;
        if (ctx->ecp_lambda) cudaFree(ctx->ecp_lambda);
        ctx->ecp_lambda = nullptr;
        SG_CUDA(ctx, cudaMalloc(&ctx->ecp_lambda, sizeof(float) * (size_t)ctx->nl.pair_capacity));
        ctx->ecp_lambda_cap = ctx->nl.pair_capacity;
    }
    // launch shape, second axis: 0 one kernel, 1 split (solve, then forces),
    // 2 one kernel behind the support-function range test (Newton solvers)
    const bool split = sg_pair_tune_for(ctx, p->kind, false).filter == 1;
    switch (p->solver) {
        case SG_SOLVER_BRENT_COMPAT: return launch_ecp<SG_SOLVER_BRENT_COMPAT>(ctx, p, mu, nu);
        case SG_SOLVER_NEWTON:
            if (!split) return launch_ecp<SG_SOLVER_NEWTON>(ctx, p, mu, nu);
            // split path: the Newton solve, then the forces from its lambda
            if (int rc = launch_ecp_solve<SG_SOLVER_NEWTON>(ctx, p)) return rc;
            return launch_ecp<SOLVER_GIVEN>(ctx, p, mu, nu);
        case SG_SOLVER_NEWTON_SUPPORT:
            if (!split) return launch_ecp<SG_SOLVER_NEWTON_SUPPORT>(ctx, p, mu, nu);
            if (int rc = launch_ecp_solve<SG_SOLVER_NEWTON_SUPPORT>(ctx, p)) return rc;
            return launch_ecp<SOLVER_GIVEN>(ctx, p, mu, nu);
        case SG_SOLVER_MLP_NEWTON:
            if (ctx->mlp_inline) return launch_ecp<SG_SOLVER_MLP_NEWTON>(ctx, p, mu, nu);
            // tensor-core guess pass, then Newton from it
            if (int rc = sg_mlp_guess_tc_launch(ctx, ctx->ecp_lambda)) return rc;
            if (!split) return launch_ecp<SOLVER_MLP_PRE>(ctx, p, mu, nu);
            if (int rc = launch_ecp_solve<SOLVER_MLP_PRE>(ctx, p)) return rc;
            return launch_ecp<SOLVER_GIVEN>(ctx, p, mu, nu);
        default: return sg_fail(ctx, SG_EINVAL, "unknown ECP solver %d", p->solver);
    }
}
