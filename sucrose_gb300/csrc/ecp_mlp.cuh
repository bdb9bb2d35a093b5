// Learned initial guess for the ECP contact parameter (no counterpart in the
// reference): a 16 -> 64 -> 64 -> 64 -> 1 perceptron, ReLU hidden layers and a
// sigmoid output, BF16 operands with FP32 accumulation on the tensor cores.
//
// Features of pair (i, j), 14 used, padded to 16 with zeros:
//   0-2   direction of r_j - r_i in the body frame of i (unit vector; the
//         contact parameter does not depend on |r|)
//   3-6   relative orientation q_i^* q_j, sign fixed so that w >= 0
//   7-9   semi-axes of i, 10-12 semi-axes of j
//   13    |r_ij| / 4
// One warp evaluates the 32 pairs of its lanes at once: 2 row tiles of 16
// pairs, each layer an m16n8k16 BF16 MMA chain whose FP32 accumulators are
// re-packed in registers as the next layer's A operand.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#define SG_MLP_IN 16
#define SG_MLP_H 64

struct MlpDev {
    const __nv_bfloat16* W1;   // [64][16] row-major (out, in)
    const __nv_bfloat16* W2;   // [64][64]
    const __nv_bfloat16* W3;   // [64][64]
    const float* b1;           // [64]
    const float* b2;
    const float* b3;
    const float* w4;           // [64]
    float b4;
};

// FP32 master layout shared with the host API and the trainer:
// W1[64*16] b1[64] W2[64*64] b2[64] W3[64*64] b3[64] w4[64] b4[1]
#define SG_MLP_OFF_W1 0
#define SG_MLP_OFF_B1 (SG_MLP_OFF_W1 + 64 * 16)
#define SG_MLP_OFF_W2 (SG_MLP_OFF_B1 + 64)
#define SG_MLP_OFF_B2 (SG_MLP_OFF_W2 + 64 * 64)
#define SG_MLP_OFF_W3 (SG_MLP_OFF_B2 + 64)
#define SG_MLP_OFF_B3 (SG_MLP_OFF_W3 + 64 * 64)
#define SG_MLP_OFF_W4 (SG_MLP_OFF_B3 + 64)
#define SG_MLP_OFF_B4 (SG_MLP_OFF_W4 + 64)
#define SG_MLP_NPARAM (SG_MLP_OFF_B4 + 1)

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// B fragment of W (row-major [N][K] bf16) for n-tile nt, k-tile kt:
// b0 = W[n][k0+2t .. +1], b1 = W[n][k0+8+2t .. +1], n = 8 nt + lane/4.
__device__ __forceinline__ void load_b(const __nv_bfloat16* W, int K, int nt, int kt, int lane, uint32_t& b0,
                                       uint32_t& b1) {
    const int n = nt * 8 + (lane >> 2);
    const int k = kt * 16 + (lane & 3) * 2;
    const uint32_t* row = reinterpret_cast<const uint32_t*>(W + (size_t)n * K);
    b0 = __ldg(row + (k >> 1));
    b1 = __ldg(row + ((k + 8) >> 1));
}

// Features of one pair; r = r_i - r_j (minimum image).
__device__ __forceinline__ void mlp_features(float3 r, float4 qi, float4 qj, float4 si, float4 sj, float (&f)[16]) {
    const float w = qi.x, x = qi.y, y = qi.z, z = qi.w;
    // rows of the rotation (lab -> body of i)
    const float u00 = w * w + x * x - y * y - z * z, u01 = 2.f * (x * y + w * z), u02 = 2.f * (x * z - w * y);
    const float u10 = 2.f * (x * y - w * z), u11 = w * w - x * x + y * y - z * z, u12 = 2.f * (y * z + w * x);
    const float u20 = 2.f * (x * z + w * y), u21 = 2.f * (y * z - w * x), u22 = w * w - x * x - y * y + z * z;
    const float rr = sqrtf(r.x * r.x + r.y * r.y + r.z * r.z);
    const float inv = rr > 0.f ? 1.f / rr : 0.f;
    const float dx = -r.x * inv, dy = -r.y * inv, dz = -r.z * inv;
    f[0] = u00 * dx + u01 * dy + u02 * dz;
    f[1] = u10 * dx + u11 * dy + u12 * dz;
    f[2] = u20 * dx + u21 * dy + u22 * dz;
    // q_i^* (x) q_j
    float rw = w * qj.x + x * qj.y + y * qj.z + z * qj.w;
    float rx = w * qj.y - x * qj.x - y * qj.w + z * qj.z;
    float ry = w * qj.z + x * qj.w - y * qj.x - z * qj.y;
    float rz = w * qj.w - x * qj.z + y * qj.y - z * qj.x;
    const float sgn = rw < 0.f ? -1.f : 1.f;
    f[3] = sgn * rw; f[4] = sgn * rx; f[5] = sgn * ry; f[6] = sgn * rz;
    f[7] = 0.5f * si.x; f[8] = 0.5f * si.y; f[9] = 0.5f * si.z;
    f[10] = 0.5f * sj.x; f[11] = 0.5f * sj.y; f[12] = 0.5f * sj.z;
    f[13] = 0.25f * rr;
    f[14] = 0.f; f[15] = 0.f;
}

// Hidden layer on the accumulators of 8 n-tiles (64 outputs) -> A fragments
// of the next layer (4 k-tiles), with bias and ReLU.
__device__ __forceinline__ void acc_to_a(const float (&acc)[8][4], const float* bias, int lane, uint32_t (&a)[4][4]) {
    const int c = (lane & 3) * 2;
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        const int n0 = 16 * kt + c, n1 = 16 * kt + 8 + c;
        const float b00 = __ldg(bias + n0), b01 = __ldg(bias + n0 + 1);
        const float b10 = __ldg(bias + n1), b11 = __ldg(bias + n1 + 1);
        const float(&lo)[4] = acc[2 * kt];
        const float(&hi)[4] = acc[2 * kt + 1];
        a[kt][0] = pack_bf16(fmaxf(lo[0] + b00, 0.f), fmaxf(lo[1] + b01, 0.f));
        a[kt][1] = pack_bf16(fmaxf(lo[2] + b00, 0.f), fmaxf(lo[3] + b01, 0.f));
        a[kt][2] = pack_bf16(fmaxf(hi[0] + b10, 0.f), fmaxf(hi[1] + b11, 0.f));
        a[kt][3] = pack_bf16(fmaxf(hi[2] + b10, 0.f), fmaxf(hi[3] + b11, 0.f));
    }
}

// Whole warp: every lane passes its 16 features, every lane gets its guess.
// Must be called by all 32 lanes.
__device__ __forceinline__ float mlp_warp_guess(const MlpDev& m, const float (&f)[16]) {
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, c = (lane & 3) * 2;
    float out_rows[2][2];  // [m-tile][row g / g+8]
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
        // A fragment of layer 1 (16 pairs x 16 features): rows g and g+8 of
        // this m-tile live in lanes ra and rb. A shuffle delivers the source
        // lane's register, so every feature index is shuffled uniformly and
        // each lane keeps the columns (c, c+1, 8+c, 9+c) it needs.
        uint32_t a1[4];
        {
            const int ra = mt * 16 + g, rb = mt * 16 + g + 8;
            float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                const float xa = __shfl_sync(0xffffffffu, f[k], ra);
                const float xb = __shfl_sync(0xffffffffu, f[k], rb);
                if (k == c) { v[0] = xa; v[2] = xb; }
                if (k == c + 1) { v[1] = xa; v[3] = xb; }
                if (k == 8 + c) { v[4] = xa; v[6] = xb; }
                if (k == 9 + c) { v[5] = xa; v[7] = xb; }
            }
            a1[0] = pack_bf16(v[0], v[1]);
            a1[1] = pack_bf16(v[2], v[3]);
            a1[2] = pack_bf16(v[4], v[5]);
            a1[3] = pack_bf16(v[6], v[7]);
        }
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
            uint32_t b0, b1;
            load_b(m.W1, 16, nt, 0, lane, b0, b1);
            mma_bf16_16816(acc[nt], a1, b0, b1);
        }
        uint32_t a[4][4];
        acc_to_a(acc, m.b1, lane, a);
#pragma unroll
        for (int layer = 0; layer < 2; ++layer) {
            const __nv_bfloat16* W = layer == 0 ? m.W2 : m.W3;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
                for (int kt = 0; kt < 4; ++kt) {
                    uint32_t b0, b1;
                    load_b(W, 64, nt, kt, lane, b0, b1);
                    mma_bf16_16816(acc[nt], a[kt], b0, b1);
                }
            }
            if (layer == 0) acc_to_a(acc, m.b2, lane, a);
        }
        // output layer on FP32 accumulators: rows g (c0,c1) and g+8 (c2,c3)
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const int n = nt * 8 + c;
            const float b0 = __ldg(m.b3 + n), b1 = __ldg(m.b3 + n + 1);
            const float w0 = __ldg(m.w4 + n), w1 = __ldg(m.w4 + n + 1);
            s0 += fmaxf(acc[nt][0] + b0, 0.f) * w0 + fmaxf(acc[nt][1] + b1, 0.f) * w1;
            s1 += fmaxf(acc[nt][2] + b0, 0.f) * w0 + fmaxf(acc[nt][3] + b1, 0.f) * w1;
        }
        s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
        s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
        s1 += __shfl_xor_sync(0xffffffffu, s1, 1);
        s1 += __shfl_xor_sync(0xffffffffu, s1, 2);
        out_rows[mt][0] = s0;
        out_rows[mt][1] = s1;
    }
    // lane L needs row L: m-tile L/16, row (L%16) -> held by lanes 4*(L%8) .. , slot (L%16)/8
    const int mt = lane >> 4, rr = lane & 15;
    const int src = (rr & 7) * 4;
    const float z0 = __shfl_sync(0xffffffffu, out_rows[0][0], src);
    const float z1 = __shfl_sync(0xffffffffu, out_rows[0][1], src);
    const float z2 = __shfl_sync(0xffffffffu, out_rows[1][0], src);
    const float z3 = __shfl_sync(0xffffffffu, out_rows[1][1], src);
    const float zsel = mt == 0 ? (rr < 8 ? z0 : z1) : (rr < 8 ? z2 : z3);
    const float z = zsel + m.b4;
    float lam = 1.f / (1.f + __expf(-z));
    return fminf(fmaxf(lam, 0.02f), 0.98f);
}
