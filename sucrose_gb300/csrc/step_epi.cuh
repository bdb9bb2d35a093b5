// Per-particle work that the captured step folds into the initial half step,
// and the per-particle set-up of the ellipsoid pair kernels.
//
// The step's initial half step is the last reader of the previous forces and
// the last writer of positions and orientations before the pair stage, so its
// kernel also (a) runs the Verlet-list displacement test on the new position
// (needs_rebuild, fortran/system.f90:1005-1039), (b) zeroes the particle's
// force and torque (initialize_forces, :423-436), and (c) writes the pair
// potential's per-particle set-up (ECP or Gay-Berne) from the new state. The
// step then launches four kernels instead of a dozen nodes; each of these
// helpers is also the body of the stand-alone kernel it replaces, so both
// forms compute the same bits.
#pragma once

#include <cmath>

#include <cuda_fp16.h>

#include "dfloat.cuh"
#include "sg_internal.cuh"

// ------------------------------------------------------------ list trigger --
// needs_rebuild on the FP32 state: 4 |r - r_last|^2 (minimum image) against
// the trigger bound, decided in FP32 when clear of it by 1e-3 relative and
// otherwise with the reference's FP64 operations.
struct CheckArgs {
    const float4* last;     // positions at the last build
    float3 box, inv_box;
    double bx, by, bz;
    int periodic;
    double trigger_sq;
    int* flags;             // flags[0]: rebuild request
    int* rep_flag;          // replica contexts: per-replica request
    RepDev rp;
};

inline CheckArgs check_args(const sg_ctx* ctx) {
    CheckArgs c;
    c.last = ctx->nl.pos_last;
    c.box = make_float3((float)ctx->box[0], (float)ctx->box[1], (float)ctx->box[2]);
    c.inv_box = make_float3((float)(1.0 / ctx->box[0]), (float)(1.0 / ctx->box[1]), (float)(1.0 / ctx->box[2]));
    c.bx = ctx->box[0];
    c.by = ctx->box[1];
    c.bz = ctx->box[2];
    c.periodic = ctx->periodic;
    c.trigger_sq = ctx->nl.trigger_sq;
    c.flags = ctx->nl.dev_flags;
    c.rep_flag = ctx->nl.rep_flag;
    c.rp = ctx->rep;
    return c;
}

SG_DEV void check_displacement(int i, float4 a, const CheckArgs& c) {
    float3 box = c.box, ib = c.inv_box;
    double bx = c.bx, by = c.by, bz = c.bz, trig = c.trigger_sq;
    int per = c.periodic, r = 0;
    if (c.rp.rep_of) {
        r = c.rp.rep_of[i];
        const float4 b4 = c.rp.box[r], i4 = c.rp.inv_box[r];
        box = make_float3(b4.x, b4.y, b4.z);
        ib = make_float3(i4.x, i4.y, i4.z);
        bx = c.rp.boxd[3 * r];
        by = c.rp.boxd[3 * r + 1];
        bz = c.rp.boxd[3 * r + 2];
        trig = c.rp.trig[r];
        per = 1;
    }
    const float4 b = c.last[i];
    {
        float fx = a.x - b.x, fy = a.y - b.y, fz = a.z - b.z;
        if (per) {
            fx -= roundf(fx * ib.x) * box.x;
            fy -= roundf(fy * ib.y) * box.y;
            fz -= roundf(fz * ib.z) * box.z;
        }
        const float f4 = 4.f * (fx * fx + fy * fy + fz * fz);
        if (f4 < (float)trig * 0.999f && fabsf(fx) < 0.25f * box.x && fabsf(fy) < 0.25f * box.y &&
            fabsf(fz) < 0.25f * box.z)
            return;
    }
    double dx = __dsub_rn((double)a.x, (double)b.x), dy = __dsub_rn((double)a.y, (double)b.y),
           dz = __dsub_rn((double)a.z, (double)b.z);
    if (per) {
        dx = __dsub_rn(dx, __dmul_rn(round(__ddiv_rn(dx, bx)), bx));
        dy = __dsub_rn(dy, __dmul_rn(round(__ddiv_rn(dy, by)), by));
        dz = __dsub_rn(dz, __dmul_rn(round(__ddiv_rn(dz, bz)), bz));
    }
    const double rr = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (__dmul_rn(4.0, rr) > trig) {
        // a replica context rebuilds only the replicas whose particles moved
        if (c.rp.rep_of) c.rep_flag[r] = 1;
        c.flags[0] = 1;
    }
}

// ------------------------------------------------------- ECP particle prep --
// The range record of the filtered ECP launch, 32 bytes that the range test
// reads with one 256-bit load per particle: (x, y, z, d) and A_R rounded to
// FP16, packed two to a word (xx|xy, xz|yy, yz|zz, 0). d >= ||A_R - A16||_F
// >= ||A_R - A16||_2, so A16 + d I - A_R is positive semi-definite: the
// support function sqrt(r.X r) and the contact function's 1 / F(l) taken with
// X = A16 + d I bound those of A_R from above, and the test stays a superset.
// An entry beyond the FP16 range gives d = inf, and the test keeps the pair.
SG_DEV void ecp_range_one(int p, float4 a, const float (&A)[6], float4* __restrict__ range) {
    unsigned h[6];
    float s = 0.f;
#pragma unroll
    for (int m = 0; m < 6; ++m) {
        const __half hv = __float2half_rn(A[m]);
        h[m] = __half_as_ushort(hv);
        const float e = A[m] - __half2float(hv);
        s += (m == 1 || m == 2 || m == 4) ? 2.f * e * e : e * e;   // off-diagonal entries count twice
    }
    range[2 * p] = make_float4(a.x, a.y, a.z, sqrtf(s) * 1.001f);
    reinterpret_cast<uint4*>(range)[2 * p + 1] = make_uint4(h[0] | h[1] << 16, h[2] | h[3] << 16, h[4] | h[5] << 16, 0u);
}

// A_R = U^T S^2 U and A_E = U^T E U (fortran/force.f90:1294-1297), the body z
// axis and the sigma_t factor (:1299), as 4 float4: (A_R 0-3), (A_R 4-5,
// A_E 0-1), (A_E 2-5), (u_z, sigma_t); the range record of position a
// (ecp_range_one) into range. prep64 (optional): A_R in FP64 in the
// reference's operation order (xmath.f90:194-208, :262-279), for the Brent
// compat solver.
SG_DEV void ecp_prep_one(int p, float4 a, float4 q, float4 s4, float4 e4, float muinv, float4* __restrict__ prep,
                         float4* __restrict__ range, double* __restrict__ prep64) {
    const float w = q.x, x = q.y, y = q.z, z = q.w;
    // rows of the reference's U (rotation_matrix form, :1244-1252): body axes in the lab frame
    float u[3][3];
    u[0][0] = w * w + x * x - y * y - z * z; u[0][1] = 2.f * (x * y + w * z); u[0][2] = 2.f * (x * z - w * y);
    u[1][0] = 2.f * (x * y - w * z); u[1][1] = w * w - x * x + y * y - z * z; u[1][2] = 2.f * (y * z + w * x);
    u[2][0] = 2.f * (x * z + w * y); u[2][1] = 2.f * (y * z - w * x); u[2][2] = w * w - x * x - y * y + z * z;
    const float sg[3] = {s4.x, s4.y, s4.z};
    const float ep[3] = {e4.x, e4.y, e4.z};
    const float e0 = fmaxf(fmaxf(ep[0], ep[1]), ep[2]);
    float s2[3], E[3];
    for (int k = 0; k < 3; ++k) {
        float h = 0.5f * sg[k];
        s2[k] = h * h;
        E[k] = powf(e0 / ep[k], muinv) * 0.25f;
    }
    float A[6], B[6];
    const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
    for (int m = 0; m < 6; ++m) {
        float a = 0.f, b = 0.f;
        for (int k = 0; k < 3; ++k) {
            float uu = u[k][ia[m]] * u[k][ib[m]];
            a += s2[k] * uu;
            b += E[k] * uu;
        }
        A[m] = a;
        B[m] = b;
    }
    const float st = (sg[0] * sg[1] + sg[2] * sg[2]) * sqrtf(2.f * sg[0] * sg[1]) * 0.125f;
    prep[4 * p + 0] = make_float4(A[0], A[1], A[2], A[3]);
    prep[4 * p + 1] = make_float4(A[4], A[5], B[0], B[1]);
    prep[4 * p + 2] = make_float4(B[2], B[3], B[4], B[5]);
    prep[4 * p + 3] = make_float4(u[2][0], u[2][1], u[2][2], st);
    ecp_range_one(p, a, A, range);
    if (prep64) {
        const double W = w, X = x, Y = y, Z = z;
        double r[3][3];
        r[0][0] = __dsub_rn(__dsub_rn(__dadd_rn(__dmul_rn(W, W), __dmul_rn(X, X)), __dmul_rn(Y, Y)), __dmul_rn(Z, Z));
        r[0][1] = __dmul_rn(2.0, __dadd_rn(__dmul_rn(X, Y), __dmul_rn(W, Z)));
        r[0][2] = __dmul_rn(2.0, __dsub_rn(__dmul_rn(X, Z), __dmul_rn(W, Y)));
        r[1][0] = __dmul_rn(2.0, __dsub_rn(__dmul_rn(X, Y), __dmul_rn(W, Z)));
        r[1][1] = __dsub_rn(__dadd_rn(__dsub_rn(__dmul_rn(W, W), __dmul_rn(X, X)), __dmul_rn(Y, Y)), __dmul_rn(Z, Z));
        r[1][2] = __dmul_rn(2.0, __dadd_rn(__dmul_rn(Y, Z), __dmul_rn(W, X)));
        r[2][0] = __dmul_rn(2.0, __dadd_rn(__dmul_rn(X, Z), __dmul_rn(W, Y)));
        r[2][1] = __dmul_rn(2.0, __dsub_rn(__dmul_rn(Y, Z), __dmul_rn(W, X)));
        r[2][2] = __dadd_rn(__dsub_rn(__dsub_rn(__dmul_rn(W, W), __dmul_rn(X, X)), __dmul_rn(Y, Y)), __dmul_rn(Z, Z));
        double b[3];
        for (int k = 0; k < 3; ++k) {
            double h = __ddiv_rn((double)sg[k], 2.0);
            b[k] = __dmul_rn(h, h);
        }
        for (int m = 0; m < 6; ++m) {
            const int c1 = ia[m], c2 = ib[m];
            double t0 = __dmul_rn(__dmul_rn(r[0][c1], b[0]), r[0][c2]);
            double t1 = __dmul_rn(__dmul_rn(r[1][c1], b[1]), r[1][c2]);
            double t2 = __dmul_rn(__dmul_rn(r[2][c1], b[2]), r[2][c2]);
            prep64[6 * (size_t)p + m] = __dadd_rn(__dadd_rn(t0, t1), t2);
        }
    }
}

// -------------------------------------------------- Gay-Berne particle prep --
// Layout (4 float4 per particle, n particles):
//   rec[2p]     = (x, y, z, sig_x)   the position, copied, and the width
//   rec[2p + 1] = (u_x, u_y, u_z, chi)
//   aux[p]      = (chi', 1/eps_z, 0, 0)   with aux = rec + 2n
//   lo[p]       = the low parts of u and chi (u, chi from FP64 = hi + lo),
//                 with lo = rec + 3n
// u is the body z axis (the first column of the reference's U1 formula,
// fortran/force.f90:343-349), chi and chi' the shape and energy anisotropies.
SG_DEV void gb_prep_one(int n, int p, float4 at, float4 q, float4 s, float4 e, float muinv, float4* prep) {
    const float w = q.x, x = q.y, y = q.z, z = q.w;
    const float lpar = s.z, lprp = s.x;
    const float ep = powf(e.x, muinv), ez = powf(e.z, muinv);
    const float xhi = (ep - ez) / (ep + ez);
    // u and chi as hi + lo to ~48 bits (the precise class of near-contact
    // pairs), in double-float arithmetic on the FP32 pipe: the products of the
    // FP32 quaternion and shape components are exact there
    const dfl ux = df_mul_f(df_add(df_two_prod(x, z), df_two_prod(w, y)), 2.f);
    const dfl uy = df_mul_f(df_sub(df_two_prod(y, z), df_two_prod(w, x)), 2.f);
    const dfl uz = df_add(df_sub(df_two_prod(w, w), df_two_prod(x, x)), df_sub(df_two_prod(z, z), df_two_prod(y, y)));
    const dfl pp = df_two_prod(lpar, lpar), qq = df_two_prod(lprp, lprp);
    const dfl chi = df_div(df_sub(pp, qq), df_add(pp, qq));
    prep[2 * p] = make_float4(at.x, at.y, at.z, lprp);
    prep[2 * p + 1] = make_float4(ux.hi, uy.hi, uz.hi, chi.hi);
    prep[2 * (size_t)n + p] = make_float4(xhi, 1.f / e.z, 0.f, 0.f);
    prep[3 * (size_t)n + p] = make_float4(ux.lo, uy.lo, uz.lo, chi.lo);
}

// ------------------------------------------------------- step epilogue ----
enum { SG_PREP_NONE = 0, SG_PREP_ECP = 1, SG_PREP_GB = 2 };

struct StepEpi {
    int on;                       // 0: a plain half step (the stand-alone entry points)
    int check;                    // run the displacement test
    CheckArgs chk;
    float4* force;                // zeroed after the half step has read them
    float4* torque;
    int prep_kind;                // SG_PREP_*
    float4* prep;
    const float4* shape;
    const float4* eshape;
    float muinv;
    int n;
    double* acc;                  // acc[0..6] zeroed: pot_eng, virial, kin_eng, kin_rot (initialize_forces),
                                  // the per-call sums [4], [5] and virial_bonded [6]
    unsigned long long* stats;    // the pair kernels' 32 counters, zeroed
};

// The epilogue of the captured step's initial half step (on = 0 outside it).
// The prep buffer is allocated here on the step's first, eager, run.
inline int make_step_epi(sg_ctx* ctx, StepEpi& e) {
    e = StepEpi{};
    if (!ctx->step_fused) return SG_OK;
    e.on = 1;
    e.check = 1;
    e.chk = check_args(ctx);
    e.force = ctx->force;
    e.torque = ctx->torque;
    e.prep_kind = ctx->step_prep_kind;
    if (e.prep_kind != SG_PREP_NONE && !ctx->ecp_prep) {
        ctx->graph_epoch++;
        SG_CUDA(ctx, cudaMalloc(&ctx->ecp_prep, sizeof(float4) * SG_PREP_F4 * (size_t)ctx->n));
    }
    e.prep = ctx->ecp_prep;
    e.shape = ctx->shape;
    e.eshape = ctx->eshape;
    e.muinv = ctx->step_prep_muinv;
    e.n = ctx->n;
    e.acc = ctx->acc;
    e.stats = ctx->stats;
    return SG_OK;
}

// Particle i after its initial half step: new position a, orientation q.
SG_DEV void step_epilogue(const StepEpi& e, int i, float4 a, float4 q) {
    if (e.check) check_displacement(i, a, e.chk);
    e.force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    e.torque[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (e.prep_kind == SG_PREP_ECP)
        ecp_prep_one(i, a, q, e.shape[i], e.eshape[i], e.muinv, e.prep, e.prep + 4 * (size_t)e.n, nullptr);
    else if (e.prep_kind == SG_PREP_GB) gb_prep_one(e.n, i, a, q, e.shape[i], e.eshape[i], e.muinv, e.prep);
    if (i == 0) {
        for (int k = 0; k < 7; ++k) e.acc[k] = 0.0;
        for (int k = 0; k < 32; ++k) e.stats[k] = 0ull;
    }
}
