// Philox4x32-10 on the device, the generator of the reference's philox_rng
// module (fortran/xmath.f90:5-113): multipliers 0xD2511F53 / 0xCD9E8D57, Weyl
// key increments 0x9E3779B9 / 0xBB67AE85 after rounds 1-9, default key
// (0x6D2B79F5, 0x1B873593). Outputs are the four 32-bit words; uniforms are
// word * 2^-32 (exact in FP64).
#pragma once
#include <cstdint>

struct sg_u4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ sg_u4 sg_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                                     uint32_t k1) {
#pragma unroll
    for (int round = 0; round < 10; ++round) {
#ifdef __CUDA_ARCH__
        uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        if (round < 9) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    }
    return sg_u4{c0, c1, c2, c3};
}

#define SG_PHILOX_KEY0 0x6D2B79F5u
#define SG_PHILOX_KEY1 0x1B873593u

// Three N(0,1) variates from one counter by two Box-Muller pairs, the fourth
// dropped, u1 and u3 clamped to 1e-35 (fortran/xmath.f90:78-113). FP64.
__device__ __forceinline__ void sg_normal_3seq(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                               uint32_t k1, double& n1, double& n2, double& n3) {
    sg_u4 w = sg_philox(c0, c1, c2, c3, k0, k1);
    const double s = 1.0 / 4294967296.0;
    double u1 = fmax((double)w.x * s, 1.0e-35);
    double u2 = (double)w.y * s;
    double u3 = fmax((double)w.z * s, 1.0e-35);
    double u4 = (double)w.w * s;
    const double TWOPI = 6.283185307179586;
    double r1 = sqrt(-2.0 * log(u1));
    double r2 = sqrt(-2.0 * log(u3));
    double s1, c1v;
    sincos(TWOPI * u2, &s1, &c1v);
    n1 = r1 * c1v;
    n2 = r1 * s1;
    n3 = r2 * cos(TWOPI * u4);
}

// The same three variates evaluated in FP32 from the same Philox words, for
// kernels whose state is FP32: the words are the reference's bit for bit; the
// variates agree with the FP64 ones to FP32 rounding (~1e-7 relative).
__device__ __forceinline__ void sg_normal_3seq_f32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                                   uint32_t k1, float& n1, float& n2, float& n3) {
    sg_u4 w = sg_philox(c0, c1, c2, c3, k0, k1);
    const float s = 2.3283064365386963e-10f;   // 2^-32
    const float u1 = fmaxf((float)w.x * s, 1.0e-35f);
    const float u2 = (float)w.y * s;
    const float u3 = fmaxf((float)w.z * s, 1.0e-35f);
    const float u4 = (float)w.w * s;
    const float r1 = sqrtf(-2.0f * logf(u1));
    const float r2 = sqrtf(-2.0f * logf(u3));
    float s1, c1v;
    sincospif(2.0f * u2, &s1, &c1v);
    n1 = r1 * c1v;
    n2 = r1 * s1;
    n3 = r2 * cospif(2.0f * u4);
}
