// Integrators of the reference's verlet, quaternion, langevin and nose_hoover
// modules (fortran/integrators.f90:1-392, :494-676) on FP32 state, one thread
// per particle. Kinetic-energy terms and their sums in double-float on the
// FP32 pipe (block partials finished by the last block, FP64 for the result);
// quaternion renormalisation beyond FP32 precision in double-float.
#include <cmath>

#include "sg_internal.cuh"
#include "philox.cuh"
#include "step_epi.cuh"

namespace {

struct Geo {
    float3 box, inv_box;
    int periodic;
    RepDev rp;
};

Geo make_geo(const sg_ctx* ctx) {
    Geo g;
    g.rp = ctx->rep;
    g.box = make_float3((float)ctx->box[0], (float)ctx->box[1], (float)ctx->box[2]);
    g.inv_box = make_float3((float)(1.0 / ctx->box[0]), (float)(1.0 / ctx->box[1]), (float)(1.0 / ctx->box[2]));
    g.periodic = ctx->periodic;
    return g;
}

SG_DEV float3 wrap_pos(float3 r, const Geo& g, int i) {
    if (g.rp.rep_of) {
        const int k = g.rp.rep_of[i];
        const float4 b = g.rp.box[k], ib = g.rp.inv_box[k];
        r.x -= roundf(r.x * ib.x) * b.x;
        r.y -= roundf(r.y * ib.y) * b.y;
        r.z -= roundf(r.z * ib.z) * b.z;
        return r;
    }
    if (g.periodic) {
        r.x -= roundf(r.x * g.inv_box.x) * g.box.x;
        r.y -= roundf(r.y * g.inv_box.y) * g.box.y;
        r.z -= roundf(r.z * g.inv_box.z) * g.box.z;
    }
    return r;
}

// Rotation matrix rows (body axes in the lab frame), integrators.f90:144-152.
struct Rot { float m[3][3]; };
SG_DEV Rot rot_of(float w, float x, float y, float z) {
    Rot r;
    r.m[0][0] = w * w + x * x - y * y - z * z; r.m[0][1] = 2.f * (x * y + w * z); r.m[0][2] = 2.f * (x * z - w * y);
    r.m[1][0] = 2.f * (x * y - w * z); r.m[1][1] = w * w - x * x + y * y - z * z; r.m[1][2] = 2.f * (y * z + w * x);
    r.m[2][0] = 2.f * (x * z + w * y); r.m[2][1] = 2.f * (y * z - w * x); r.m[2][2] = w * w - x * x - y * y + z * z;
    return r;
}
SG_DEV float3 rot_apply(const Rot& r, float3 v) {   // R v (lab -> body)
    return make_float3(r.m[0][0] * v.x + r.m[0][1] * v.y + r.m[0][2] * v.z,
                       r.m[1][0] * v.x + r.m[1][1] * v.y + r.m[1][2] * v.z,
                       r.m[2][0] * v.x + r.m[2][1] * v.y + r.m[2][2] * v.z);
}
SG_DEV float3 rot_apply_t(const Rot& r, float3 v) { // R^T v (body -> lab)
    return make_float3(r.m[0][0] * v.x + r.m[1][0] * v.y + r.m[2][0] * v.z,
                       r.m[0][1] * v.x + r.m[1][1] * v.y + r.m[2][1] * v.z,
                       r.m[0][2] * v.x + r.m[1][2] * v.y + r.m[2][2] * v.z);
}

// Two fixed-point passes for the mid-step quaternion derivative
// (integrators.f90:140-168, :572-604). Returns qdot of the last pass, the
// rotation and body-frame angular momentum of that pass.
SG_DEV float4 q_midpoint(float4 q, float3 L, float3 Iinv, float dt, Rot& rm, float3& Lb) {
    float4 qn = q;
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const float4 qo = qn;
        rm = rot_of(qo.x, qo.y, qo.z, qo.w);
        Lb = rot_apply(rm, L);
        const float wx = Lb.x * Iinv.x, wy = Lb.y * Iinv.y, wz = Lb.z * Iinv.z;
        float4 qd;
        qd.x = 0.5f * (-qo.y * wx - qo.z * wy - qo.w * wz);
        qd.y = 0.5f * (qo.x * wx + qo.z * wz - qo.w * wy);
        qd.z = 0.5f * (qo.x * wy - qo.y * wz + qo.w * wx);
        qd.w = 0.5f * (qo.x * wz + qo.y * wy - qo.z * wx);
        qn = make_float4(q.x + 0.5f * dt * qd.x, q.y + 0.5f * dt * qd.y, q.z + 0.5f * dt * qd.z, q.w + 0.5f * dt * qd.w);
        if (it == 1) return qd;
    }
    return make_float4(0.f, 0.f, 0.f, 0.f);
}

// Renormalisation to beyond FP32 precision, on the FP32 pipe (FP64 runs at
// 1/64 of its rate on GB300): s = |q|^2 in double-float (squares exact by FMA
// two-products), 1 / sqrt(s) = r0 (1 + e/2) by one Newton step from the FP32
// estimate r0 with e = 1 - s r0^2 formed from the double-float s (about 44
// correct bits), each component rounded once, w r0 + w r0 e/2 in one FMA.
SG_DEV float4 q_advance(float4 q, float4 qd, float dt) {
    const float w = q.x + dt * qd.x, x = q.y + dt * qd.y, y = q.z + dt * qd.z, z = q.w + dt * qd.w;
    const dfl s = df_add(df_dot3(make_float3(w, x, y), make_float3(w, x, y)), df_two_prod(z, z));
    const float r0 = rsqrtf(s.hi);
    const dfl sr2 = df_mul(s, df_two_prod(r0, r0));
    const float c = 0.5f * ((1.f - sr2.hi) - sr2.lo) * r0;
    return make_float4(fmaf(w, r0, w * c), fmaf(x, r0, x * c), fmaf(y, r0, y * c), fmaf(z, r0, z * c));
}

// Kinetic terms in double-float on the FP32 pipe; the sums take them through
// block_reduce_finish_df, so FP64 appears once per reduction, not per particle.
// m |v|^2: the squares exact, their sum and the product with m to ~48 bits.
SG_DEV dfl mv2_df(float m, float4 v) {
    const float3 u = make_float3(v.x, v.y, v.z);
    return df_mul_f(df_dot3(u, u), m);
}
SG_DEV dfl df_half(dfl a) { return {0.5f * a.hi, 0.5f * a.lo}; }
// 2 KE_rot = sum_k L_b,k^2 / I_k with L_b = R L the body-frame angular
// momentum (integrators.f90:190-215): the squares rounded to FP32, their
// products with 1/I_k exact, the sum in double-float.
SG_DEV dfl kin_rot2_df(float4 q, float3 L, float3 Iinv) {
    Rot r = rot_of(q.x, q.y, q.z, q.w);
    float3 Lb = rot_apply(r, L);
    return df_dot3(make_float3(Lb.x * Lb.x, Lb.y * Lb.y, Lb.z * Lb.z), Iinv);
}

// ------------------------------------------------------------------- VV ----
__global__ void k_vv_initial(int n, float dt, Geo g, float4* __restrict__ pos, float4* __restrict__ vel,
                             const float4* __restrict__ force) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = vel[i], f = force[i], r = pos[i];
    const float h = 0.5f * dt, im = v.w;
    v.x += h * (f.x * im); v.y += h * (f.y * im); v.z += h * (f.z * im);
    float3 p = wrap_pos(make_float3(r.x + dt * v.x, r.y + dt * v.y, r.z + dt * v.z), g, i);
    vel[i] = v;
    pos[i] = make_float4(p.x, p.y, p.z, r.w);
}

// final half kick; KE = sum 0.5 m v^2 (mass from shape.w)
__global__ void k_vv_final(int n, float dt, float4* __restrict__ vel, const float4* __restrict__ force,
                           const float4* __restrict__ shape, double* partials, unsigned int* done, double* acc) {
    dfl e[1] = {{0.f, 0.f}};
    const float h = 0.5f * dt;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 v = vel[i], f = force[i];
        const float im = v.w;
        v.x += h * (f.x * im); v.y += h * (f.y * im); v.z += h * (f.z * im);
        vel[i] = v;
        e[0] = df_add(e[0], df_half(mv2_df(shape[i].w, v)));
    }
    block_reduce_finish_df<1>(e, partials, done, acc, false);
}

// --------------------------------------------------------------- rotation --
__global__ void k_qq_initial(int n, float dt, float4* __restrict__ quat, float4* __restrict__ angm,
                             const float4* __restrict__ torque, const float4* __restrict__ inert_inv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 L4 = angm[i], T = torque[i], Ii = inert_inv[i];
    const float h = 0.5f * dt;
    float3 L = make_float3(L4.x + h * T.x, L4.y + h * T.y, L4.z + h * T.z);
    Rot rm;
    float3 Lb;
    float4 qd = q_midpoint(quat[i], L, make_float3(Ii.x, Ii.y, Ii.z), dt, rm, Lb);
    quat[i] = q_advance(quat[i], qd, dt);
    angm[i] = make_float4(L.x, L.y, L.z, 0.f);
}

__global__ void k_qq_final(int n, float dt, const float4* __restrict__ quat, float4* __restrict__ angm,
                           const float4* __restrict__ torque, const float4* __restrict__ inert_inv, double* partials,
                           unsigned int* done, double* acc) {
    dfl e[1] = {{0.f, 0.f}};
    const float h = 0.5f * dt;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 L4 = angm[i], T = torque[i], Ii = inert_inv[i];
        float3 L = make_float3(L4.x + h * T.x, L4.y + h * T.y, L4.z + h * T.z);
        angm[i] = make_float4(L.x, L.y, L.z, 0.f);
        e[0] = df_add(e[0], df_half(kin_rot2_df(quat[i], L, make_float3(Ii.x, Ii.y, Ii.z))));
    }
    block_reduce_finish_df<1>(e, partials, done, acc, false);
}

// --------------------------------------------------------------- Langevin --
struct LgvConst {
    const int* step_dev;   // when set, the step counter is read from the device (captured graphs)
    float dt, ed, kk12, T;
    double c2;          // 1 - exp(-2 gamma dt)
    double rot_amp;     // 2 gamma T dt
    float Tc2;          // T (1 - exp(-2 gamma dt))
    float rot_ampf;
    double g2, dtd;     // 2 gamma and dt: per-replica 2 gamma T dt, evaluated in the host's order
    float kk2;
    uint32_t step, temp_int, k0, k1;
};

__global__ void k_lgv_initial(int n, LgvConst c, Geo g, float4* __restrict__ pos, float4* __restrict__ vel,
                              const float4* __restrict__ force, float4* __restrict__ quat, float4* __restrict__ angm,
                              const float4* __restrict__ torque, const float4* __restrict__ inert,
                              const float4* __restrict__ inert_inv, int rotations, StepEpi epi) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float h = 0.5f * c.dt;
    float4 v = vel[i], f = force[i], r = pos[i];
    const float im = v.w;
    v.x += h * (f.x * im); v.y += h * (f.y * im); v.z += h * (f.z * im);
    float3 p = make_float3(r.x + h * v.x, r.y + h * v.y, r.z + h * v.z);
    float n1a, n1b, n1c, n2a = 0.f, n2b = 0.f, n2c = 0.f;
    // counters (I, step, int(T*1000), stream) with I 1-based (integrators.f90:546-547)
    const uint32_t step = c.step_dev ? (uint32_t)*c.step_dev : c.step;
    // counter index, temperature and key: the replica's own in a batched context,
    // so a replica draws exactly the numbers of its single-system run
    uint32_t idx = (uint32_t)(i + 1), tint = c.temp_int, k0 = c.k0, k1 = c.k1;
    float Tc2 = c.Tc2, rot_ampf = c.rot_ampf;
    if (g.rp.rep_of) {
        const int k = g.rp.rep_of[i];
        idx = (uint32_t)(i - g.rp.off[k] + 1);
        tint = (uint32_t)g.rp.temp_int[k];
        k0 = g.rp.key[k].x;
        k1 = g.rp.key[k].y;
        const double T = g.rp.temp[k];
        Tc2 = (float)(T * c.c2);
        rot_ampf = (float)(c.g2 * T * c.dtd);
    }
    sg_normal_3seq_f32(idx, step, tint, 0u, k0, k1, n1a, n1b, n1c);
    if (rotations) sg_normal_3seq_f32(idx, step, tint, 1u, k0, k1, n2a, n2b, n2c);
    const float amp = sqrtf(Tc2 * im);
    v.x = c.ed * v.x + amp * n1a;
    v.y = c.ed * v.y + amp * n1b;
    v.z = c.ed * v.z + amp * n1c;
    p = wrap_pos(make_float3(p.x + h * v.x, p.y + h * v.y, p.z + h * v.z), g, i);
    vel[i] = v;
    const float4 pn = make_float4(p.x, p.y, p.z, r.w);
    pos[i] = pn;
    if (!rotations) {
        if (epi.on) step_epilogue(epi, i, pn, quat[i]);
        return;
    }
    float4 L4 = angm[i], T = torque[i], I4 = inert[i], Ii = inert_inv[i];
    float3 L = make_float3(L4.x + h * T.x, L4.y + h * T.y, L4.z + h * T.z);
    Rot rm;
    float3 Lb;
    const float4 q = quat[i];
    float4 qd = q_midpoint(q, L, make_float3(Ii.x, Ii.y, Ii.z), c.dt, rm, Lb);
    Lb.x = c.kk12 * Lb.x + c.kk2 * sqrtf(rot_ampf * I4.x) * n2a;
    Lb.y = c.kk12 * Lb.y + c.kk2 * sqrtf(rot_ampf * I4.y) * n2b;
    Lb.z = c.kk12 * Lb.z + c.kk2 * sqrtf(rot_ampf * I4.z) * n2c;
    L = rot_apply_t(rm, Lb);
    angm[i] = make_float4(L.x, L.y, L.z, 0.f);
    const float4 qn = q_advance(q, qd, c.dt);
    quat[i] = qn;
    if (epi.on) step_epilogue(epi, i, pn, qn);
}

__global__ void k_lgv_final(int n, float dt, float4* __restrict__ vel, const float4* __restrict__ force,
                            const float4* __restrict__ shape, const float4* __restrict__ quat,
                            float4* __restrict__ angm, const float4* __restrict__ torque,
                            const float4* __restrict__ inert_inv, int rotations, double* partials, unsigned int* done,
                            double* acc, int* step_inc) {
    dfl e[2] = {{0.f, 0.f}, {0.f, 0.f}};
    const float h = 0.5f * dt;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    // the first particle's inputs that the pair stage before does not write
    float4 v0{}, s0{}, L0{}, I0{}, q0{};
    if (i0 < n) {
        v0 = vel[i0];
        s0 = shape[i0];
        if (rotations) {
            L0 = angm[i0];
            I0 = inert_inv[i0];
            q0 = quat[i0];
        }
    }
    pdl_wait();
    for (int i = i0; i < n; i += stride) {
        const bool first = i == i0;
        float4 v = first ? v0 : vel[i];
        const float4 f = force[i];
        const float im = v.w;
        v.x += h * (f.x * im); v.y += h * (f.y * im); v.z += h * (f.z * im);
        vel[i] = v;
        e[0] = df_add(e[0], df_half(mv2_df((first ? s0 : shape[i]).w, v)));
        if (rotations) {
            const float4 L4 = first ? L0 : angm[i], T = torque[i], Ii = first ? I0 : inert_inv[i];
            const float4 q = first ? q0 : quat[i];
            float3 L = make_float3(L4.x + h * T.x, L4.y + h * T.y, L4.z + h * T.z);
            angm[i] = make_float4(L.x, L.y, L.z, 0.f);
            e[1] = df_add(e[1], df_half(kin_rot2_df(q, L, make_float3(Ii.x, Ii.y, Ii.z))));
        }
    }
    // step_inc (captured step): the sums are stored, and the step counter advances
    if (block_reduce_finish_df<2>(e, partials, done, acc, step_inc != nullptr) && step_inc && threadIdx.x == 0)
        *step_inc += 1;
}

// ------------------------------------------------------------ Nose-Hoover --
// integrators.f90:233-301; chain length 3. nh layout: [0..2] eta, [3..5] p_eta,
// [6..8] eta_r, [9..11] p_eta_r, [12] translational scale, [13] rotational
// scale, [14] sum m v^2 scratch, [15] sum L_b^2/I scratch, [16] the scaled
// sum m v^2, [17] the compat sweep's KE, [18] the two scales rounded to FP32
// (a float pair: the particle kernels read them without an FP64 conversion),
// [22], [23] 2 KE and 2 KE_rot of the last fused final half step.
// The standard chain's constants in double-float (hi + lo split on the host).
struct NhDf {
    dfl t4, hdt, T, ndofT, nrotT;   // dt/4, dt/2, T, ndof T, nrot T
    dfl iHB[3], iHBr[3];
};
struct NhConst {
    double dt, T, ndof, nrot;
    double HB[3], HBr[3];
    double iHB[3], iHBr[3];   // 1 / HB: the chains multiply (an FP64 division is a long serial sequence)
    NhDf d;
};


// exp(x) in FP64. The chain's arguments are dt/4 p/Q-sized, |x| << 0.03, where
// the Taylor polynomial of degree 9 is below half an ulp (x^10/10! < 2e-22 at
// |x| = 0.03); a short dependent chain of FMAs instead of the library's range
// reduction, which matters because the chains run in one thread each.
__device__ __forceinline__ double exp_chain(double x) {
    if (fabs(x) >= 0.03) return exp(x);
    double f = 1.0 / 362880.0;
    f = fma(f, x, 1.0 / 40320.0);
    f = fma(f, x, 1.0 / 5040.0);
    f = fma(f, x, 1.0 / 720.0);
    f = fma(f, x, 1.0 / 120.0);
    f = fma(f, x, 1.0 / 24.0);
    f = fma(f, x, 1.0 / 6.0);
    f = fma(f, x, 0.5);
    f = fma(f, x, 1.0);
    return fma(f, x, 1.0);
}

// The standard chain in double-float arithmetic on the FP32 pipe (~48-bit
// significands): one thread runs each chain, and a dependent FP64 operation
// costs it several hundred cycles on GB300, a double-float one a few dozen.
// u4_propagator (integrators.f90:233-301): G_1 from the supplied sum (m v^2
// or L_b^2/I), G_j = p_(j-1)^2 / Q_(j-1) - T, with exprel(y) = (e^y - 1)/y; G_j,
// the products and the sums in double-float, the two factors e^-x and
// exprel(-x) in FP32 (their relative precision enters once per half step).
SG_DEV void u4_df(dfl t, int j_start, int j_stop, int stride, dfl (&p)[3], const dfl (&iq)[3], dfl K, dfl dofT,
                  dfl T) {
#pragma unroll
    for (int j = j_start; stride > 0 ? j <= j_stop : j >= j_stop; j += stride) {
        const dfl gj = (j == 1) ? df_sub(K, dofT) : df_sub(df_mul(df_mul(p[j - 2], p[j - 2]), iq[j - 2]), T);
        if (j == 3) {
            p[2] = df_add(p[2], df_mul(t, gj));
        } else {
            const float x = t.hi * p[j].hi * iq[j].hi;
            float ex, c;
            if (fabsf(x) < 1.f) {
                const float u = 0.5f * x, y = u * u;
                const float h = expf(-u);
                // sinh(u)/u = 1 + y/6 + y^2/120 + y^3/5040 + y^4/362880 (|u| < 0.5: < 1e-9 left)
                const float sh = fmaf(fmaf(fmaf(fmaf(y, 1.f / 362880.f, 1.f / 5040.f), y, 1.f / 120.f), y, 1.f / 6.f), y,
                                      1.f);
                ex = h * h;
                c = h * sh;
            } else {
                ex = expf(-x);
                c = (1.f - ex) / x;
            }
            p[j - 1] = df_add(df_mul_f(p[j - 1], ex), df_mul_f(df_mul(t, gj), c));
        }
    }
}

// e^x in double-float: for |x| <= 1e-3, 1 + x + x^2/2 in double-float and
// x^3 (1/6 + x/24 + x^2/120) in FP32 (the rest of the series is below 2e-21);
// larger |x| through the FP64 series.
SG_DEV dfl exp_df(dfl x) {
    if (!(fabsf(x.hi) <= 1e-3f)) return df_from_double(exp_chain(df_to_double(x)));
    const float r = fmaf(fmaf(x.hi, 1.f / 120.f, 1.f / 24.f), x.hi, 1.f / 6.f);
    const float x3r = x.hi * x.hi * x.hi * r;
    const dfl x2 = df_mul(x, x);
    return df_add(df_add(df_of(1.f), x), df_add(dfl{0.5f * x2.hi, 0.5f * x2.lo}, df_of(x3r)));
}

__global__ void k_sum_mv2(int n, const float4* __restrict__ vel, const float4* __restrict__ shape,
                          const float4* __restrict__ quat, const float4* __restrict__ angm,
                          const float4* __restrict__ inert_inv, int rot, double* partials, unsigned int* done,
                          double* dst) {
    dfl e[2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 v = vel[i];
        e[0] = df_add(e[0], mv2_df(shape[i].w, v));
        if (rot) {
            float4 L = angm[i], Ii = inert_inv[i];
            e[1] = df_add(e[1], kin_rot2_df(quat[i], make_float3(L.x, L.y, L.z), make_float3(Ii.x, Ii.y, Ii.z)));
        }
    }
    block_reduce_finish_df<2>(e, partials, done, dst, false);
}

// Standard NHC half step on the chain(s): nh[14], nh[15] hold the sums on
// entry (zeroed by the host before the reduction). Writes the scale factors.
// The translational chain (which = 0) and the rotational chain (which = 1)
// are independent, and the caller runs them in two different warps.
// The chain state (FP64 in nh) is read once into double-float registers and
// written back at the end; the sequence runs in double-float (u4_df).
// K: the sum (m v^2 or L_b^2/I) for this chain.
__device__ void nhc_chain_one(const NhConst& c, double* nh, int which, double Kd) {
    double* eta = nh + 6 * which;
    dfl e[3], p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        e[k] = df_from_double(eta[k]);
        p[k] = df_from_double(eta[3 + k]);
    }
    const dfl(&iq)[3] = which ? c.d.iHBr : c.d.iHB;
    const dfl dofT = which ? c.d.nrotT : c.d.ndofT;
    const dfl K = df_from_double(Kd);
    u4_df(c.d.t4, 3, 1, -1, p, iq, K, dofT, c.d.T);
    const dfl sc = exp_df(df_neg(df_mul(c.d.hdt, df_mul(p[0], iq[0]))));
#pragma unroll
    for (int k = 0; k < 3; ++k) e[k] = df_add(e[k], df_mul(c.d.hdt, df_mul(p[k], iq[k])));
    const dfl K2 = df_mul(K, df_mul(sc, sc));
    u4_df(c.d.t4, 1, 3, 1, p, iq, K2, dofT, c.d.T);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        eta[k] = df_to_double(e[k]);
        eta[3 + k] = df_to_double(p[k]);
    }
    nh[12 + which] = df_to_double(sc);
    reinterpret_cast<float*>(nh + 18)[which] = sc.hi + sc.lo;
    if (!which) nh[16] = df_to_double(K2);
}

// threads 0 (translation) and 32 (rotation, or the unit scale without it).
// tot: the two sums (shared memory), else nh[14], nh[15].
__device__ void nhc_chain_threads(const NhConst& c, double* nh, int rot, const double* tot) {
    if (threadIdx.x == 0) nhc_chain_one(c, nh, 0, tot ? tot[0] : nh[14]);
    if (threadIdx.x == 32) {
        if (rot) {
            nhc_chain_one(c, nh, 1, tot ? tot[1] : nh[15]);
        } else {
            nh[13] = 1.0;
            reinterpret_cast<float*>(nh + 18)[1] = 1.f;
        }
    }
}

__global__ void k_nhc_chain(NhConst c, double* nh, int rot) {
    if (blockIdx.x != 0) return;
    nhc_chain_threads(c, nh, rot, nullptr);
}

// The initial chain from the sums the previous step's final half stored in
// nh[22], nh[23]: sum m v^2 = 2 KE and sum L_b^2/I = 2 KE_rot. Both sums run
// the same grid partition in double-float, where halving is exact, so these
// are the bits k_nhc_sum_chain would compute from the unchanged state.
__global__ void k_nhc_chain_acc(NhConst c, double* nh, int rot) {
    pdl_trigger();   // the particle pass may start loading: this kernel writes only nh
    __shared__ double tot[2];
    if (threadIdx.x == 0) {
        tot[0] = nh[22];
        tot[1] = nh[23];
        nh[14] = tot[0];
        nh[15] = tot[1];
    }
    __syncthreads();
    nhc_chain_threads(c, nh, rot, tot);
}

// the translational and rotational scales as FP32 (nh[18])
SG_DEV float2 nh_scale_f(const double* nh) { return *reinterpret_cast<const float2*>(nh + 18); }

// ---- fused Nose-Hoover step (the captured step's form) -----------------------
// The same arithmetic as the separate entry points, in fewer passes:
//   initial: [sum m v^2, L_b^2/I -> chain in the finishing block] [scale, kick, drift, rotate]
//   final:   [kick, sums -> chain in the finishing block] [scale, rotational kick, KE, KE_rot]

// Sums of m v^2 and 2 KE_rot (after an optional half kick of v), then the
// chain update in the block that finishes the sums.
__global__ void k_nhc_sum_chain(int n, float dt, int kick, float4* __restrict__ vel, const float4* __restrict__ force,
                                const float4* __restrict__ shape, const float4* __restrict__ quat,
                                const float4* __restrict__ angm, const float4* __restrict__ inert_inv, int rot,
                                NhConst c, double* partials, unsigned int* done, double* nh) {
    dfl e[2] = {{0.f, 0.f}, {0.f, 0.f}};
    const float h = 0.5f * dt;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    // the first particle's inputs, none of which the pair stage before writes
    float4 v0{}, s0{}, q0{}, L0{}, I0{};
    if (i0 < n) {
        v0 = vel[i0];
        s0 = shape[i0];
        if (rot) {
            q0 = quat[i0];
            L0 = angm[i0];
            I0 = inert_inv[i0];
        }
    }
    pdl_wait();
    pdl_trigger();
    for (int i = i0; i < n; i += stride) {
        const bool first = i == i0;
        float4 v = first ? v0 : vel[i];
        if (kick) {
            const float4 f = force[i];
            const float im = v.w;
            v.x += h * (f.x * im); v.y += h * (f.y * im); v.z += h * (f.z * im);
            vel[i] = v;
        }
        e[0] = df_add(e[0], mv2_df((first ? s0 : shape[i]).w, v));
        if (rot) {
            const float4 L = first ? L0 : angm[i], Ii = first ? I0 : inert_inv[i], q = first ? q0 : quat[i];
            e[1] = df_add(e[1], kin_rot2_df(q, make_float3(L.x, L.y, L.z), make_float3(Ii.x, Ii.y, Ii.z)));
        }
    }
    __shared__ double tot[2];
    if (block_reduce_finish_df<2>(e, partials, done, nh + 14, true, tot)) {
        __syncthreads();
        nhc_chain_threads(c, nh, rot, tot);
    }
}

// Chain scaling, half kick and drift, then the quaternion update with the
// rotational half kick (k_nhc_apply(do_vv = 1) followed by k_qq_initial).
__global__ void k_nhc_initial_fused(int n, const double* nh, float dt, Geo g, float4* __restrict__ pos,
                                    float4* __restrict__ vel, const float4* __restrict__ force,
                                    float4* __restrict__ quat, float4* __restrict__ angm,
                                    const float4* __restrict__ torque, const float4* __restrict__ inert_inv,
                                    int rot_chain, int rotations, StepEpi epi) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // the particle's state, which the sums and chain before do not write
    float4 v = vel[i], L4 = angm[i];
    const float4 f = force[i], r = pos[i], q = quat[i];
    float4 T{}, Ii{};
    if (rotations) {
        T = torque[i];
        Ii = inert_inv[i];
    }
    pdl_wait();
    const float2 scf = nh_scale_f(nh);
    const float sc = scf.x;
    v.x *= sc; v.y *= sc; v.z *= sc;
    if (rot_chain) {
        const float sr = scf.y;
        L4 = make_float4(L4.x * sr, L4.y * sr, L4.z * sr, L4.w);
    }
    const float h = 0.5f * dt, im = v.w;
    v.x += h * (f.x * im); v.y += h * (f.y * im); v.z += h * (f.z * im);
    float3 p = wrap_pos(make_float3(r.x + dt * v.x, r.y + dt * v.y, r.z + dt * v.z), g, i);
    const float4 pn = make_float4(p.x, p.y, p.z, r.w);
    pos[i] = pn;
    vel[i] = v;
    float4 qn = q;
    if (rotations) {
        float3 L = make_float3(L4.x + h * T.x, L4.y + h * T.y, L4.z + h * T.z);
        Rot rm;
        float3 Lb;
        float4 qd = q_midpoint(q, L, make_float3(Ii.x, Ii.y, Ii.z), dt, rm, Lb);
        qn = q_advance(q, qd, dt);
        quat[i] = qn;
        angm[i] = make_float4(L.x, L.y, L.z, 0.f);
    } else if (rot_chain) {
        angm[i] = L4;
    }
    if (epi.on) step_epilogue(epi, i, pn, qn);
}

// Chain scaling, then the rotational half kick; KE = sum 0.5 m v^2 and KE_rot
// into acc[0], acc[1] (k_nhc_apply(do_vv = 0), the KE sum and k_qq_final).
__global__ void k_nhc_final_fused(int n, const double* nh, float dt, float4* __restrict__ vel,
                                  const float4* __restrict__ shape, const float4* __restrict__ quat,
                                  float4* __restrict__ angm, const float4* __restrict__ torque,
                                  const float4* __restrict__ inert_inv, int rot_chain, int rotations, double* partials,
                                  unsigned int* done, double* acc, int* step_inc, double* sums) {
    dfl e[2] = {{0.f, 0.f}, {0.f, 0.f}};
    const float h = 0.5f * dt;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    // the first particle's inputs that the sums and chain before do not write
    float4 s0{}, L0{}, T0{}, I0{}, q0{};
    if (i0 < n) {
        s0 = shape[i0];
        if (rot_chain || rotations) L0 = angm[i0];
        if (rotations) {
            T0 = torque[i0];
            I0 = inert_inv[i0];
            q0 = quat[i0];
        }
    }
    pdl_wait();
    const float2 scf = nh_scale_f(nh);
    const float sc = scf.x;
    const float sr = rot_chain ? scf.y : 1.f;
    for (int i = i0; i < n; i += stride) {
        const bool first = i == i0;
        float4 v = vel[i];
        v.x *= sc; v.y *= sc; v.z *= sc;
        vel[i] = v;
        e[0] = df_add(e[0], df_half(mv2_df((first ? s0 : shape[i]).w, v)));
        if (rot_chain || rotations) {
            float4 L4 = first ? L0 : angm[i];
            if (rot_chain) L4 = make_float4(L4.x * sr, L4.y * sr, L4.z * sr, L4.w);
            if (rotations) {
                const float4 T = first ? T0 : torque[i], Ii = first ? I0 : inert_inv[i], q = first ? q0 : quat[i];
                const float3 L = make_float3(L4.x + h * T.x, L4.y + h * T.y, L4.z + h * T.z);
                angm[i] = make_float4(L.x, L.y, L.z, 0.f);
                e[1] = df_add(e[1], df_half(kin_rot2_df(q, L, make_float3(Ii.x, Ii.y, Ii.z))));
            } else {
                angm[i] = L4;
            }
        }
    }
    // the sums are stored; step_inc (captured step): the step counter advances;
    // sums: 2 KE and 2 KE_rot, the next initial chain's sums (k_nhc_chain_acc)
    __shared__ double tot[2];
    if (block_reduce_finish_df<2>(e, partials, done, acc, true, tot) && threadIdx.x == 0) {
        if (step_inc) *step_inc += 1;
        sums[0] = 2.0 * tot[0];
        sums[1] = 2.0 * tot[1];
    }
}

// scale v (and L), then optionally the VV kick + drift (initial step)
__global__ void k_nhc_apply(int n, const double* nh, int do_vv, float dt, Geo g, float4* __restrict__ pos,
                            float4* __restrict__ vel, const float4* __restrict__ force, float4* __restrict__ angm,
                            int rot) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 scf = nh_scale_f(nh);
    const float sc = scf.x;
    float4 v = vel[i];
    v.x *= sc; v.y *= sc; v.z *= sc;
    if (rot) {
        const float sr = scf.y;
        float4 L = angm[i];
        angm[i] = make_float4(L.x * sr, L.y * sr, L.z * sr, L.w);
    }
    if (do_vv) {
        const float4 f = force[i], r = pos[i];
        const float h = 0.5f * dt, im = v.w;
        v.x += h * (f.x * im); v.y += h * (f.y * im); v.z += h * (f.z * im);
        float3 p = wrap_pos(make_float3(r.x + dt * v.x, r.y + dt * v.y, r.z + dt * v.z), g, i);
        pos[i] = make_float4(p.x, p.y, p.z, r.w);
    }
    vel[i] = v;
}

__global__ void k_kick(int n, float dt, float4* __restrict__ vel, const float4* __restrict__ force) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = vel[i];
    const float4 f = force[i];
    const float h = 0.5f * dt, im = v.w;
    v.x += h * (f.x * im); v.y += h * (f.y * im); v.z += h * (f.z * im);
    vel[i] = v;
}

// The reference's per-particle chain (integrators.f90:324-352, :372-390): a
// serial recurrence over particles in index order, one thread. The O(N) SUM
// that the reference repeats at every particle is carried as a running sum,
// updated by each particle's change. The recurrence runs in double-float on
// the FP32 pipe (a dependent FP64 operation costs one thread several hundred
// cycles on GB300, a double-float one a few dozen): the chain state, the
// running sum, the per-particle terms (squares exact) and both factors of u4
// (e^-x and exprel(-x) to ~48 bits, since N applications would accumulate an
// FP32 factor's rounding) and the scale. The chain masses enter through their
// reciprocals. The next particle's state is loaded while this one's chain runs.

// e^-x and exprel(-x) = (1 - e^-x)/x in double-float: for |x| <= 1e-3, e^-x
// by exp_df and 1 - x/2 + x^2/6 in double-float with -x^3/24 + x^4/120 in
// FP32 (the rest below 1e-20 relative); larger |x| by the FP64 forms of u4.
SG_DEV void u4_factors_df(dfl x, dfl& ex, dfl& c) {
    if (!(fabsf(x.hi) <= 1e-3f)) {
        const double xd = df_to_double(x);
        const double hh = exp_chain(-0.5 * xd);
        const double e = hh * hh;
        double cd;
        if (fabs(xd) > 0.01) {
            cd = (e - 1.0) / (-xd);
        } else {
            const double y = (0.5 * xd) * (0.5 * xd);
            cd = hh * (1.0 + y * (1.0 / 6 + y * (1.0 / 120 + y * (1.0 / 5040 + y / 362880))));
        }
        ex = df_from_double(e);
        c = df_from_double(cd);
        return;
    }
    ex = exp_df(df_neg(x));
    constexpr float kSixthHi = 1.f / 6.f;
    constexpr float kSixthLo = (float)(1.0 / 6.0 - (double)kSixthHi);
    const float tail = x.hi * x.hi * x.hi * fmaf(x.hi, 1.f / 120.f, -1.f / 24.f);
    c = df_add(df_add(df_of(1.f), dfl{-0.5f * x.hi, -0.5f * x.lo}),
               df_add(df_mul(df_mul(x, x), dfl{kSixthHi, kSixthLo}), df_of(tail)));
}

// u4 of the reference, all in double-float (u4_factors_df for the factors).
SG_DEV void u4_compat_df(dfl t, int j_start, int j_stop, int stride, dfl (&p)[3], const dfl (&iq)[3], dfl K,
                         dfl dofT, dfl T) {
#pragma unroll
    for (int j = j_start; stride > 0 ? j <= j_stop : j >= j_stop; j += stride) {
        const dfl gj = (j == 1) ? df_sub(K, dofT) : df_sub(df_mul(df_mul(p[j - 2], p[j - 2]), iq[j - 2]), T);
        if (j == 3) {
            p[2] = df_add(p[2], df_mul(t, gj));
        } else {
            dfl ex, c;
            u4_factors_df(df_mul(t, df_mul(p[j], iq[j])), ex, c);
            p[j - 1] = df_add(df_mul(p[j - 1], ex), df_mul(df_mul(t, gj), c));
        }
    }
}

// m (|b|^2 - |a|^2) in double-float (squares exact)
SG_DEV dfl dmv2_df(float m, float3 b, float3 a) {
    return df_mul_f(df_sub(df_dot3(b, b), df_dot3(a, a)), m);
}

__global__ void k_nh_compat(int n, NhConst c, int initial, Geo g, double* nh, float4* __restrict__ pos,
                            float4* __restrict__ vel, const float4* __restrict__ force,
                            const float4* __restrict__ shape) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    dfl eta[3], p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        eta[k] = df_from_double(nh[k]);
        p[k] = df_from_double(nh[3 + k]);
    }
    dfl K = df_from_double(nh[14]);
    dfl ke = df_of(0.f);
    const float h = 0.5f * (float)c.dt, dtf = (float)c.dt;
    float4 v_n{}, f_n{}, s_n{};
    if (n > 0) {
        v_n = vel[0];
        f_n = force[0];
        s_n = shape[0];
    }
    for (int i = 0; i < n; ++i) {
        const float4 v = v_n, f = f_n;
        const float m = s_n.w, im = v.w;
        if (i + 1 < n) {   // the next particle's state, in flight during this one's chain
            v_n = vel[i + 1];
            f_n = force[i + 1];
            s_n = shape[i + 1];
        }
        float3 u = make_float3(v.x, v.y, v.z);
        if (!initial) {
            const float3 o = u;
            u = make_float3(u.x + h * (f.x * im), u.y + h * (f.y * im), u.z + h * (f.z * im));
            K = df_add(K, dmv2_df(m, u, o));
        }
        u4_compat_df(c.d.t4, 3, 1, -1, p, c.d.iHB, K, c.d.ndofT, c.d.T);
        const dfl sc = exp_df(df_neg(df_mul(c.d.hdt, df_mul(p[0], c.d.iHB[0]))));
        {
            const float3 o = u;
            u = make_float3(fmaf(u.x, sc.hi, u.x * sc.lo), fmaf(u.y, sc.hi, u.y * sc.lo),
                            fmaf(u.z, sc.hi, u.z * sc.lo));
            K = df_add(K, dmv2_df(m, u, o));
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) eta[k] = df_add(eta[k], df_mul(c.d.hdt, df_mul(p[k], c.d.iHB[k])));
        u4_compat_df(c.d.t4, 1, 3, 1, p, c.d.iHB, K, c.d.ndofT, c.d.T);
        if (initial) {
            const float3 o = u;
            u = make_float3(u.x + h * (f.x * im), u.y + h * (f.y * im), u.z + h * (f.z * im));
            K = df_add(K, dmv2_df(m, u, o));
            const float4 r = pos[i];
            const float3 q = wrap_pos(make_float3(r.x + dtf * u.x, r.y + dtf * u.y, r.z + dtf * u.z), g, i);
            pos[i] = make_float4(q.x, q.y, q.z, r.w);
        } else {
            ke = df_add(ke, df_half(mv2_df(m, make_float4(u.x, u.y, u.z, 0.f))));
        }
        vel[i] = make_float4(u.x, u.y, u.z, v.w);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        nh[k] = df_to_double(eta[k]);
        nh[3 + k] = df_to_double(p[k]);
    }
    nh[14] = df_to_double(K);
    nh[17] = df_to_double(ke);
}

__global__ void k_half_into(const double* src, double* dst) { *dst = 0.5 * *src; }

int reduce_grid(const sg_ctx* ctx) { return std::max(1, std::min(2 * ctx->num_sms, (ctx->n + 255) / 256)); }

NhConst nh_const(const sg_ctx* ctx, double dt, double T, double coupling) {
    NhConst c;
    c.dt = dt;
    c.T = T;
    c.ndof = 3.0 * ctx->n - 3.0;            // 3 (N / Nrigid) - 3, Nrigid = 1
    c.nrot = 3.0 * ctx->n;
    const double tau = 2.0;
    for (int k = 0; k < 3; ++k) {
        c.HB[k] = coupling > 0.0 ? coupling : T * tau * tau;
        c.HBr[k] = coupling > 0.0 ? coupling : T * tau * tau;
    }
    if (!(coupling > 0.0)) {
        c.HB[0] = c.ndof * T * tau * tau;
        c.HBr[0] = c.nrot * T * tau * tau;
    }
    for (int k = 0; k < 3; ++k) {
        c.iHB[k] = 1.0 / c.HB[k];
        c.iHBr[k] = 1.0 / c.HBr[k];
    }
    auto split = [](double x) {
        const float h = (float)x;
        return dfl{h, (float)(x - (double)h)};
    };
    c.d.t4 = split(dt / 4.0);
    c.d.hdt = split(0.5 * dt);
    c.d.T = split(T);
    c.d.ndofT = split(c.ndof * T);
    c.d.nrotT = split(c.nrot * T);
    for (int k = 0; k < 3; ++k) {
        c.d.iHB[k] = split(c.iHB[k]);
        c.d.iHBr[k] = split(c.iHBr[k]);
    }
    return c;
}

int sum_mv2(sg_ctx* ctx, int rot) {
    SG_CUDA(ctx, cudaMemsetAsync(ctx->nh + 14, 0, sizeof(double) * 2, ctx->stream));
    int grid = reduce_grid(ctx);
    if (int rc = sg_ensure_partials(ctx, grid * 2)) return rc;
    k_sum_mv2<<<grid, 256, 0, ctx->stream>>>(ctx->n, ctx->vel, ctx->shape, ctx->quat, ctx->angm, ctx->inert_inv, rot,
                                            ctx->partials, ctx->done_counter, ctx->nh + 14);
    SG_LAUNCH_CHECK(ctx, "k_sum_mv2");
    return SG_OK;
}

int read_acc(sg_ctx* ctx, int idx, double* out) {
    if (!out) return SG_OK;
    SG_CUDA(ctx, cudaMemcpyAsync(out, ctx->acc + idx, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

}  // namespace

extern "C" {

int sg_vv_initial(sg_ctx* ctx, double dt) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    k_vv_initial<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, (float)dt, make_geo(ctx), ctx->pos, ctx->vel,
                                                                ctx->force);
    SG_LAUNCH_CHECK(ctx, "k_vv_initial");
    return SG_OK;
}

int sg_vv_final(sg_ctx* ctx, double dt, double* kin_eng) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    SG_CUDA(ctx, cudaMemsetAsync(ctx->acc + 2, 0, sizeof(double), ctx->stream));
    int grid = reduce_grid(ctx);
    if (int rc = sg_ensure_partials(ctx, grid)) return rc;
    k_vv_final<<<grid, 256, 0, ctx->stream>>>(ctx->n, (float)dt, ctx->vel, ctx->force, ctx->shape, ctx->partials,
                                             ctx->done_counter, ctx->acc + 2);
    SG_LAUNCH_CHECK(ctx, "k_vv_final");
    return read_acc(ctx, 2, kin_eng);
}

int sg_qq_initial(sg_ctx* ctx, double dt) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    k_qq_initial<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, (float)dt, ctx->quat, ctx->angm, ctx->torque,
                                                                ctx->inert_inv);
    SG_LAUNCH_CHECK(ctx, "k_qq_initial");
    return SG_OK;
}

int sg_qq_final(sg_ctx* ctx, double dt, double* kin_rot) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    SG_CUDA(ctx, cudaMemsetAsync(ctx->acc + 3, 0, sizeof(double), ctx->stream));
    int grid = reduce_grid(ctx);
    if (int rc = sg_ensure_partials(ctx, grid)) return rc;
    k_qq_final<<<grid, 256, 0, ctx->stream>>>(ctx->n, (float)dt, ctx->quat, ctx->angm, ctx->torque, ctx->inert_inv,
                                             ctx->partials, ctx->done_counter, ctx->acc + 3);
    SG_LAUNCH_CHECK(ctx, "k_qq_final");
    return read_acc(ctx, 3, kin_rot);
}

int sg_lgv_initial(sg_ctx* ctx, double dt, int32_t step, double damping, double target_temp, const uint32_t* key) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    LgvConst c;
    c.step_dev = ctx->lgv_step_dev;
    c.dt = (float)dt;
    c.ed = (float)std::exp(-damping * dt);
    c.c2 = 1.0 - std::exp(-2.0 * damping * dt);
    const double kk1 = 1.0 - (damping * dt) / 2.0, kk2 = 1.0 / (1.0 + (damping * dt) / 2.0);
    c.kk12 = (float)(kk2 * kk1);
    c.kk2 = (float)kk2;
    c.rot_amp = 2.0 * damping * target_temp * dt;
    c.Tc2 = (float)(target_temp * c.c2);
    c.g2 = 2.0 * damping;
    c.dtd = dt;
    c.rot_ampf = (float)c.rot_amp;
    c.T = (float)target_temp;
    c.step = (uint32_t)step;
    c.temp_int = (uint32_t)(int32_t)(target_temp * 1000.0);
    c.k0 = key ? key[0] : SG_PHILOX_KEY0;
    c.k1 = key ? key[1] : SG_PHILOX_KEY1;
    StepEpi epi;
    if (int rc = make_step_epi(ctx, epi)) return rc;
    k_lgv_initial<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, c, make_geo(ctx), ctx->pos, ctx->vel,
                                                                 ctx->force, ctx->quat, ctx->angm, ctx->torque,
                                                                 ctx->inert, ctx->inert_inv, ctx->lgv_rotations, epi);
    SG_LAUNCH_CHECK(ctx, "k_lgv_initial");
    return SG_OK;
}

int sg_lgv_final(sg_ctx* ctx, double dt, double damping, double* kin_eng, double* kin_rot) {
    (void)damping;
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    if (!ctx->step_fused) SG_CUDA(ctx, cudaMemsetAsync(ctx->acc + 2, 0, sizeof(double) * 2, ctx->stream));
    int grid = reduce_grid(ctx);
    if (int rc = sg_ensure_partials(ctx, grid * 2)) return rc;
    // in the fused step the pair stage's kernels come directly before: this
    // kernel's loads of the particle state overlap their tail
    const bool pdl = ctx->step_fused && !ctx->step_events;
    SG_CUDA(ctx, launch_pdl(pdl, k_lgv_final, grid, 256, 0, ctx->stream, ctx->n, (float)dt, ctx->vel, ctx->force,
                            ctx->shape, ctx->quat, ctx->angm, ctx->torque, ctx->inert_inv, ctx->lgv_rotations,
                            ctx->partials, ctx->done_counter, ctx->acc + 2,
                            ctx->step_fused ? ctx->step_dev : nullptr));
    if (int rc = read_acc(ctx, 2, kin_eng)) return rc;
    return read_acc(ctx, 3, kin_rot);
}

int sg_nht_initial(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t mode, int32_t rot_chain) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "Nose-Hoover chains are per system: not available on a replica context");
    if (!(target_temp > 0.0)) return sg_fail(ctx, SG_EINVAL, "Target temperature not set.");
    NhConst c = nh_const(ctx, dt, target_temp, coupling);
    const int nb = (ctx->n + 255) / 256;
    if (mode == 0) {
        if (rot_chain) return sg_fail(ctx, SG_EINVAL, "the reference chain (mode 0) thermostats translation only");
        if (int rc = sum_mv2(ctx, 0)) return rc;
        k_nh_compat<<<1, 32, 0, ctx->stream>>>(ctx->n, c, 1, make_geo(ctx), ctx->nh, ctx->pos, ctx->vel, ctx->force,
                                               ctx->shape);
        SG_LAUNCH_CHECK(ctx, "k_nh_compat");
        return SG_OK;
    }
    if (int rc = sum_mv2(ctx, rot_chain)) return rc;
    k_nhc_chain<<<1, 64, 0, ctx->stream>>>(c, ctx->nh, rot_chain);
    k_nhc_apply<<<nb, 256, 0, ctx->stream>>>(ctx->n, ctx->nh, 1, (float)dt, make_geo(ctx), ctx->pos, ctx->vel,
                                             ctx->force, ctx->angm, rot_chain);
    SG_LAUNCH_CHECK(ctx, "k_nhc_apply");
    return SG_OK;
}

int sg_nht_final(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t mode, int32_t rot_chain,
                 double* kin_eng) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "Nose-Hoover chains are per system: not available on a replica context");
    if (!(target_temp > 0.0)) return sg_fail(ctx, SG_EINVAL, "Target temperature not set.");
    NhConst c = nh_const(ctx, dt, target_temp, coupling);
    const int nb = (ctx->n + 255) / 256;
    if (mode == 0) {
        if (rot_chain) return sg_fail(ctx, SG_EINVAL, "the reference chain (mode 0) thermostats translation only");
        if (int rc = sum_mv2(ctx, 0)) return rc;
        k_nh_compat<<<1, 32, 0, ctx->stream>>>(ctx->n, c, 0, make_geo(ctx), ctx->nh, ctx->pos, ctx->vel, ctx->force,
                                               ctx->shape);
        SG_LAUNCH_CHECK(ctx, "k_nh_compat");
        SG_CUDA(ctx, cudaMemcpyAsync(ctx->acc + 2, ctx->nh + 17, sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        return read_acc(ctx, 2, kin_eng);
    }
    k_kick<<<nb, 256, 0, ctx->stream>>>(ctx->n, (float)dt, ctx->vel, ctx->force);
    if (int rc = sum_mv2(ctx, rot_chain)) return rc;
    k_nhc_chain<<<1, 64, 0, ctx->stream>>>(c, ctx->nh, rot_chain);
    k_nhc_apply<<<nb, 256, 0, ctx->stream>>>(ctx->n, ctx->nh, 0, (float)dt, make_geo(ctx), ctx->pos, ctx->vel,
                                             ctx->force, ctx->angm, rot_chain);
    SG_LAUNCH_CHECK(ctx, "k_nhc_apply");
    // kinetic energy after scaling, summed again in FP64: acc[2] = 0.5 sum m v^2
    if (int rc = sum_mv2(ctx, 0)) return rc;
    k_half_into<<<1, 1, 0, ctx->stream>>>(ctx->nh + 14, ctx->acc + 2);
    SG_LAUNCH_CHECK(ctx, "k_half_into");
    return read_acc(ctx, 2, kin_eng);
}

}  // extern "C"

// Nose-Hoover (standard chain) halves of the captured step, fused kernels.
int sg_nhc_step_initial(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t rot_chain,
                        int32_t rotations) {
    if (!ctx) return SG_EINVAL;
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "Nose-Hoover chains are per system: not available on a replica context");
    if (!(target_temp > 0.0)) return sg_fail(ctx, SG_EINVAL, "Target temperature not set.");
    NhConst c = nh_const(ctx, dt, target_temp, coupling);
    int grid = reduce_grid(ctx);
    if (int rc = sg_ensure_partials(ctx, grid * 2)) return rc;
    if (ctx->step_sums_from_acc)
        k_nhc_chain_acc<<<1, 64, 0, ctx->stream>>>(c, ctx->nh, rot_chain);
    else
        k_nhc_sum_chain<<<grid, 256, 0, ctx->stream>>>(ctx->n, (float)dt, 0, ctx->vel, ctx->force, ctx->shape,
                                                      ctx->quat, ctx->angm, ctx->inert_inv, rot_chain, c,
                                                      ctx->partials, ctx->done_counter, ctx->nh);
    StepEpi epi;
    if (int rc = make_step_epi(ctx, epi)) return rc;
    // programmatic dependent launch: the particle loads overlap the chain
    SG_CUDA(ctx, launch_pdl(true, k_nhc_initial_fused, (ctx->n + 255) / 256, 256, 0, ctx->stream, ctx->n,
                            (const double*)ctx->nh, (float)dt, make_geo(ctx), ctx->pos, ctx->vel,
                            (const float4*)ctx->force, ctx->quat, ctx->angm, (const float4*)ctx->torque,
                            (const float4*)ctx->inert_inv, (int)rot_chain, (int)rotations, epi));
    return SG_OK;
}

int sg_nhc_step_final(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t rot_chain,
                      int32_t rotations) {
    if (!ctx) return SG_EINVAL;
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "Nose-Hoover chains are per system: not available on a replica context");
    if (!(target_temp > 0.0)) return sg_fail(ctx, SG_EINVAL, "Target temperature not set.");
    NhConst c = nh_const(ctx, dt, target_temp, coupling);
    int grid = reduce_grid(ctx);
    if (int rc = sg_ensure_partials(ctx, grid * 2)) return rc;
    // programmatic dependent launches: the sums' particle loads overlap the
    // pair stage's tail, the final half's loads the sums and chain
    SG_CUDA(ctx, launch_pdl(!ctx->step_events, k_nhc_sum_chain, grid, 256, 0, ctx->stream, ctx->n, (float)dt, 1,
                            ctx->vel, (const float4*)ctx->force, (const float4*)ctx->shape,
                            (const float4*)ctx->quat, (const float4*)ctx->angm, (const float4*)ctx->inert_inv,
                            (int)rot_chain, c, ctx->partials, ctx->done_counter, ctx->nh));
    SG_CUDA(ctx, launch_pdl(true, k_nhc_final_fused, grid, 256, 0, ctx->stream, ctx->n, (const double*)ctx->nh,
                            (float)dt, ctx->vel, (const float4*)ctx->shape, (const float4*)ctx->quat, ctx->angm,
                            (const float4*)ctx->torque, (const float4*)ctx->inert_inv, (int)rot_chain,
                            (int)rotations, ctx->partials, ctx->done_counter, ctx->acc + 2,
                            ctx->step_fused ? ctx->step_dev : nullptr, ctx->nh + 22));
    return SG_OK;
}

extern "C" {

int sg_nht_state(sg_ctx* ctx, double* get12, const double* set12) {
    if (!ctx) return SG_EINVAL;
    if (set12) SG_CUDA(ctx, cudaMemcpyAsync(ctx->nh, set12, sizeof(double) * 12, cudaMemcpyHostToDevice, ctx->stream));
    if (get12) SG_CUDA(ctx, cudaMemcpyAsync(get12, ctx->nh, sizeof(double) * 12, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

}  // extern "C"
