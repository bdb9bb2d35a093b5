// Double-float arithmetic on the FP32 pipe: a value is hi + lo with
// |lo| <= ulp(hi) / 2, about 48 significant bits. Error-free transformations
// (Knuth's two-sum, the FMA two-product) carry each rounding error into lo.
// Used where FP32 cancellation would be amplified past the force tolerance
// and FP64 (1/64 of the FP32 rate on GB300) would be too slow.
#pragma once

#include "sg_internal.cuh"

struct dfl {
    float hi, lo;
};

SG_DEV dfl df_of(float a) { return {a, 0.f}; }
// a + b exactly (any magnitudes)
SG_DEV dfl df_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
// a + b exactly, when |a| >= |b|
SG_DEV dfl df_fast_two_sum(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}
// a * b exactly
SG_DEV dfl df_two_prod(float a, float b) {
    const float p = a * b;
    return {p, fmaf(a, b, -p)};
}
SG_DEV dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }
SG_DEV dfl df_add(dfl a, dfl b) {
    const dfl s = df_two_sum(a.hi, b.hi);
    return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
SG_DEV dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }
SG_DEV dfl df_mul(dfl a, dfl b) {
    const dfl p = df_two_prod(a.hi, b.hi);
    return df_fast_two_sum(p.hi, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo)));
}
SG_DEV dfl df_mul_f(dfl a, float b) {
    const dfl p = df_two_prod(a.hi, b);
    return df_fast_two_sum(p.hi, fmaf(a.lo, b, p.lo));
}
// a / b: the FP32 quotient, then one correction from the double-float residual
SG_DEV dfl df_div(dfl a, dfl b) {
    const float rb = __frcp_rn(b.hi);
    const float q1 = a.hi * rb;
    const dfl r = df_sub(a, df_mul_f(b, q1));
    return df_fast_two_sum(q1, r.hi * rb);
}
SG_DEV dfl df_sqrt(dfl a) {
    const float s = sqrtf(a.hi);
    const dfl p = df_two_prod(s, s);
    return df_fast_two_sum(s, (((a.hi - p.hi) - p.lo) + a.lo) * (0.5f / s));
}
// a . b of two FP32 vectors
SG_DEV dfl df_dot3(float3 a, float3 b) {
    const dfl x = df_two_prod(a.x, b.x), y = df_two_prod(a.y, b.y), z = df_two_prod(a.z, b.z);
    const dfl s = df_two_sum(x.hi, y.hi);
    const dfl t = df_two_sum(s.hi, z.hi);
    return df_fast_two_sum(t.hi, ((x.lo + y.lo) + z.lo) + (s.lo + t.lo));
}
// a . (b + bl) with bl the low parts of a double-float vector
SG_DEV dfl df_dot3_lo(float3 a, float3 b, float3 bl) {
    dfl d = df_dot3(a, b);
    return df_fast_two_sum(d.hi, d.lo + fmaf(a.x, bl.x, fmaf(a.y, bl.y, a.z * bl.z)));
}
// (a + al) . (b + bl), both double-float vectors
SG_DEV dfl df_dot3_dd(float3 a, float3 al, float3 b, float3 bl) {
    dfl d = df_dot3(a, b);
    const float c = fmaf(a.x, bl.x, fmaf(a.y, bl.y, fmaf(a.z, bl.z, fmaf(al.x, b.x, fmaf(al.y, b.y, al.z * b.z)))));
    return df_fast_two_sum(d.hi, d.lo + c);
}

// Exact FP32 -> FP64 widening on the integer pipe: the exponent is rebiased
// and the significand shifted into place, the same bits the conversion
// instruction gives for every normal number, infinity and NaN (zero and
// subnormals give a signed zero). On GB300 the conversion instructions share
// the FP64 pipe, which runs at 1/64 of the FP32 rate.
SG_DEV double widen(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned e = u & 0x7f800000u, sgn = u & 0x80000000u, m = (u >> 3) & 0x000fffffu;
    unsigned hi = sgn | ((e >> 3) + (896u << 20)) | m, lo = u << 29;
    if (e == 0u) { hi = sgn; lo = 0u; }
    if (e == 0x7f800000u) hi = sgn | 0x7ff00000u | m;
    return __hiloint2double((int)hi, (int)lo);
}

// FP64 -> FP32 on the integer pipe, truncating the significand (relative
// error below 2^-23); magnitudes under the FP32 normal range give a signed
// zero, over it a NaN. For residuals that enter only as small corrections.
SG_DEV float narrow_trunc(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned sgn = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu) - 896;
    unsigned u = sgn | ((unsigned)e << 23) | ((hi & 0x000fffffu) << 3) | (lo >> 29);
    if (e <= 0) u = sgn;
    if (e >= 255) u = sgn | 0x7fc00000u;
    return __uint_as_float(u);
}

// FP64 <-> double-float with one FP64 addition each way (the conversions on
// the integer pipe): hi the truncated double, lo the truncated remainder
// (about 47 bits together).
SG_DEV dfl df_from_double(double d) {
    const float h = narrow_trunc(d);
    return {h, narrow_trunc(d - widen(h))};
}
SG_DEV double df_to_double(dfl a) { return widen(a.hi) + widen(a.lo); }

// ------------------------------------------------ double-float grid sums --
// Warp sum of K double-float values by shuffles (lane 0 holds the result).
template <int K>
SG_DEV void df_warp_sum(dfl (&v)[K]) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const dfl w = {__shfl_down_sync(0xffffffffu, v[k].hi, o), __shfl_down_sync(0xffffffffu, v[k].lo, o)};
            v[k] = df_add(v[k], w);
        }
    }
}

// Grid sum of K per-thread double-float values, every level in double-float
// on the FP32 pipe: warps by shuffles, the block from one value per warp, the
// block partials (hi, lo pairs in the slots of partials, gridDim.x * K of
// them) in the block that finishes last, in a fixed order. FP64 appears once,
// for the result: out[k] = total (store) or out[k] += total. tot (optional,
// shared memory): the totals for the finishing block's own threads after a
// __syncthreads. Every thread of the block calls it; returns true in the
// finishing block (block-uniform).
template <int K>
__device__ bool block_reduce_finish_df(dfl (&v)[K], double* partials, unsigned int* done, double* out, bool store,
                                       double* tot = nullptr) {
    __shared__ float2 sh[32][K];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    float2* part = reinterpret_cast<float2*>(partials);
    df_warp_sum<K>(v);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) sh[warp][k] = make_float2(v[k].hi, v[k].lo);
    }
    __syncthreads();
    if (warp == 0) {
        dfl t[K];
#pragma unroll
        for (int k = 0; k < K; ++k) t[k] = lane < nw ? dfl{sh[lane][k].x, sh[lane][k].y} : dfl{0.f, 0.f};
        df_warp_sum<K>(t);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < K; ++k) part[(size_t)blockIdx.x * K + k] = make_float2(t[k].hi, t[k].lo);
        }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return false;
    __threadfence();
    dfl s[K];
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] = dfl{0.f, 0.f};
    for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float2 p = __ldcg(part + (size_t)b * K + k);   // L2: written by other blocks
            s[k] = df_add(s[k], dfl{p.x, p.y});
        }
    }
    df_warp_sum<K>(s);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) sh[warp][k] = make_float2(s[k].hi, s[k].lo);
    }
    __syncthreads();
    if (warp == 0) {
        dfl t[K];
#pragma unroll
        for (int k = 0; k < K; ++k) t[k] = lane < nw ? dfl{sh[lane][k].x, sh[lane][k].y} : dfl{0.f, 0.f};
        df_warp_sum<K>(t);
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const double d = (double)t[k].hi + (double)t[k].lo;
                if (store) out[k] = d;
                else out[k] += d;
                if (tot) tot[k] = d;
            }
            *done = 0u;
        }
    }
    return true;
}
