// Training of the contact-parameter MLP on the tensor cores (no counterpart in
// the reference): BF16 operands, FP32 accumulation, FP32 master weights and
// Adam state.
//
// One training step on a minibatch X (B x 16, BF16), y (B, FP32):
//   forward   Z1 = X W1^T, H1 = relu(Z1 + b1) (BF16), Z2, H2 likewise,
//             Z3 = H2 W3^T, H3 = relu(Z3 + b3) (FP32), z4 = H3 w4 + b4,
//             yhat = sigmoid(z4), loss = mean (yhat - y)^2
//   backward  d4 = 2 (yhat - y) yhat (1 - yhat) / B
//             dw4 = H3^T d4, db4 = sum d4
//             D3 = (d4 w4^T) . [H3 > 0]         dW3 = D3^T H2, db3 = colsum D3
//             D2 = (D3 W3) . [H2 > 0]           dW2 = D2^T H1, db2 = colsum D2
//             D1 = (D2 W2) . [H1 > 0]           dW1 = D1^T X,  db1 = colsum D1
//   update    Adam on the FP32 master copy, then the BF16 copies of W1..W3
// Every product is one launch of k_gemm, a 64x64-tile mma.sync m16n8k16 BF16
// GEMM with arbitrary operand strides; the weight gradients (K = B) are
// split over K and summed with FP32 atomics. The forward pass rounds
// operands at the same points as the inference path in ecp_mlp.cuh.
#include <cmath>
#include <cstdint>
#include <vector>

#include <cuda_bf16.h>

#include "sg_internal.cuh"
#include "ecp_mlp.cuh"

namespace {

constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;

// C[m][n] (+)= sum_k A(m,k) B(k,n); A(m,k) = A[m*sam + k*sak], B(k,n) = B[k*sbk + n*sbn].
// Grid: (ceil(N/64), ceil(M/64), splitk). With splitk > 1 (or accumulate), C
// is updated with atomicAdd and must be initialised by the caller.
__global__ void __launch_bounds__(128) k_gemm(int M, int N, int K, const __nv_bfloat16* __restrict__ A, long long sam,
                                              long long sak, const __nv_bfloat16* __restrict__ B, long long sbk,
                                              long long sbn, float* __restrict__ C, int ldc, int atomic_out) {
    __shared__ __align__(16) __nv_bfloat16 As[BM][BK + PAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[BN][BK + PAD];   // transposed: [n][k]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = warp >> 1, wn = warp & 1;
    const int m_blk = blockIdx.y * BM, n_blk = blockIdx.x * BN;
    const int ksplit = gridDim.z;
    const int kchunk = ((K + ksplit - 1) / ksplit + BK - 1) / BK * BK;
    const int k_lo = blockIdx.z * kchunk, k_hi = min(K, k_lo + kchunk);
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
    const __nv_bfloat16 zero = __float2bfloat16(0.f);
    for (int k0 = k_lo; k0 < k_hi; k0 += BK) {
        // stage A (BM x BK) and B^T (BN x BK); the contiguous operand dimension
        // varies fastest across threads
        if (sak == 1) {
            for (int e = tid; e < BM * BK; e += 128) {
                const int r = e / BK, c = e % BK, m = m_blk + r, k = k0 + c;
                As[r][c] = (m < M && k < k_hi) ? A[m * sam + k] : zero;
            }
        } else {
            for (int e = tid; e < BM * BK; e += 128) {
                const int r = e % BM, c = e / BM, m = m_blk + r, k = k0 + c;
                As[r][c] = (m < M && k < k_hi) ? A[m * sam + k * sak] : zero;
            }
        }
        if (sbn == 1) {
            for (int e = tid; e < BN * BK; e += 128) {
                const int r = e % BN, c = e / BN, n = n_blk + r, k = k0 + c;
                Bs[r][c] = (n < N && k < k_hi) ? B[k * sbk + n] : zero;
            }
        } else {
            for (int e = tid; e < BN * BK; e += 128) {
                const int r = e / BK, c = e % BK, n = n_blk + r, k = k0 + c;
                Bs[r][c] = (n < N && k < k_hi) ? B[k * sbk + n * sbn] : zero;
            }
        }
        __syncthreads();
        const int g = lane >> 2, t = lane & 3;
#pragma unroll
        for (int kk = 0; kk < BK; kk += 16) {
            uint32_t af[2][4];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int r0 = wm * 32 + mt * 16 + g;
                af[mt][0] = *reinterpret_cast<const uint32_t*>(&As[r0][kk + 2 * t]);
                af[mt][1] = *reinterpret_cast<const uint32_t*>(&As[r0 + 8][kk + 2 * t]);
                af[mt][2] = *reinterpret_cast<const uint32_t*>(&As[r0][kk + 8 + 2 * t]);
                af[mt][3] = *reinterpret_cast<const uint32_t*>(&As[r0 + 8][kk + 8 + 2 * t]);
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int c0 = wn * 32 + nt * 8 + g;
                const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&Bs[c0][kk + 2 * t]);
                const uint32_t b1 = *reinterpret_cast<const uint32_t*>(&Bs[c0][kk + 8 + 2 * t]);
#pragma unroll
                for (int mt = 0; mt < 2; ++mt) mma_bf16_16816(acc[mt][nt], af[mt], b0, b1);
            }
        }
        __syncthreads();
    }
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int m = m_blk + wm * 32 + mt * 16 + g + (c >= 2 ? 8 : 0);
                const int n = n_blk + wn * 32 + nt * 8 + 2 * t + (c & 1);
                if (m < M && n < N) {
                    if (atomic_out) atomicAdd(&C[(size_t)m * ldc + n], acc[mt][nt][c]);
                    else C[(size_t)m * ldc + n] = acc[mt][nt][c];
                }
            }
}

// H = relu(Z + b) as BF16 (and FP32 when h32 is given)
__global__ void k_bias_relu(long long rows, const float* __restrict__ Z, const float* __restrict__ b,
                            __nv_bfloat16* __restrict__ H, float* __restrict__ h32) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= rows * 64) return;
    const float v = fmaxf(Z[e] + b[e & 63], 0.f);
    if (H) H[e] = __float2bfloat16_rn(v);
    if (h32) h32[e] = v;
}

// output layer, loss, d4, dw4 / db4 partial sums (one warp per row group)
__global__ void k_out(long long rows, const float* __restrict__ H3, const float* __restrict__ w4, float b4,
                      const float* __restrict__ y, float* __restrict__ yhat, float* __restrict__ d4, float inv_rows,
                      float* __restrict__ grad, float* __restrict__ loss) {
    __shared__ float sw[64];
    __shared__ float sdw[64];
    __shared__ float sdb, sloss;
    if (threadIdx.x < 64) { sw[threadIdx.x] = w4[threadIdx.x]; sdw[threadIdx.x] = 0.f; }
    if (threadIdx.x == 0) { sdb = 0.f; sloss = 0.f; }
    __syncthreads();
    const long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const bool valid = s < rows;
    const float* h = H3 + (valid ? s : 0) * 64;
    float d = 0.f;
    if (valid) {
        float z = b4;
        for (int k = 0; k < 64; ++k) z += h[k] * sw[k];
        const float p = 1.f / (1.f + expf(-z));
        if (yhat) yhat[s] = p;
        if (y) {
            const float err = p - y[s];
            d = 2.f * err * p * (1.f - p) * inv_rows;
            d4[s] = d;
            atomicAdd(&sloss, err * err * inv_rows);
            atomicAdd(&sdb, d);
        }
    }
    if (y) {
        // every lane takes part in the reductions (invalid rows contribute 0)
        for (int k = 0; k < 64; ++k) {
            float v = valid ? d * h[k] : 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0) atomicAdd(&sdw[k], v);
        }
    }
    __syncthreads();
    if (y) {
        if (threadIdx.x < 64) atomicAdd(&grad[SG_MLP_OFF_W4 + threadIdx.x], sdw[threadIdx.x]);
        if (threadIdx.x == 0) {
            atomicAdd(&grad[SG_MLP_OFF_B4], sdb);
            atomicAdd(loss, sloss);
        }
    }
}

// D3 = d4 w4 . [H3 > 0]
__global__ void k_delta3(long long rows, const float* __restrict__ d4, const float* __restrict__ w4,
                         const float* __restrict__ H3, __nv_bfloat16* __restrict__ D) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= rows * 64) return;
    D[e] = __float2bfloat16_rn(H3[e] > 0.f ? d4[e >> 6] * w4[e & 63] : 0.f);
}

// D = G . [H > 0] (H as BF16)
__global__ void k_mask(long long rows, const float* __restrict__ G, const __nv_bfloat16* __restrict__ H,
                       __nv_bfloat16* __restrict__ D) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= rows * 64) return;
    D[e] = __float2bfloat16_rn(__bfloat162float(H[e]) > 0.f ? G[e] : 0.f);
}

// db[c] += sum over rows of D[r][c]
__global__ void k_colsum(long long rows, const __nv_bfloat16* __restrict__ D, float* __restrict__ db) {
    __shared__ float s[64];
    if (threadIdx.x < 64) s[threadIdx.x] = 0.f;
    __syncthreads();
    const int c = threadIdx.x & 63;
    float a = 0.f;
    for (long long r = blockIdx.x * (long long)(blockDim.x / 64) + threadIdx.x / 64; r < rows;
         r += (long long)gridDim.x * (blockDim.x / 64))
        a += __bfloat162float(D[r * 64 + c]);
    atomicAdd(&s[c], a);
    __syncthreads();
    if (threadIdx.x < 64) atomicAdd(&db[threadIdx.x], s[threadIdx.x]);
}

__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_bf16(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

// features + labels of the current list from the last ECP call's lambda
__global__ void k_features(const int* __restrict__ pair_i, const int* __restrict__ pair_j, const int* npairs,
                           const float4* __restrict__ pos, const float4* __restrict__ quat,
                           const float4* __restrict__ shape, const float* __restrict__ lam, float3 box,
                           float3 inv_box, int periodic, long long cap, __nv_bfloat16* __restrict__ X,
                           float* __restrict__ y) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= *npairs || t >= cap) return;
    const int i = pair_i[t], j = pair_j[t];
    const float4 a = pos[i], b = pos[j];
    const float3 r = min_image(make_float3(a.x - b.x, a.y - b.y, a.z - b.z), box, inv_box, periodic);
    float f[16];
    mlp_features(r, quat[i], quat[j], shape[i], shape[j], f);
#pragma unroll
    for (int k = 0; k < 16; ++k) X[t * 16 + k] = __float2bfloat16_rn(f[k]);
    y[t] = lam[t];
}

// The inference path exactly as the ECP kernel runs it (warp-level MMA on the
// 32 pairs of a warp), for the current list: one guess per listed pair.
__global__ void k_guess(const int* __restrict__ pair_i, const int* __restrict__ pair_j, const int* npairs,
                        const float4* __restrict__ pos, const float4* __restrict__ quat,
                        const float4* __restrict__ shape, float3 box, float3 inv_box, int periodic, MlpDev m,
                        float* __restrict__ out) {
    const int np = *npairs;
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int base = gwarp * 32; base < np; base += nwarps * 32) {
        const int t = base + lane;
        const bool valid = t < np;
        const int i = valid ? pair_i[t] : 0, j = valid ? pair_j[t] : 0;
        const float4 a = pos[i], b = pos[j];
        float3 r = min_image(make_float3(a.x - b.x, a.y - b.y, a.z - b.z), box, inv_box, periodic);
        if (!valid) r = make_float3(1.f, 0.f, 0.f);
        float f[16];
        mlp_features(r, quat[i], quat[j], shape[i], shape[j], f);
        const float g = mlp_warp_guess(m, f);
        if (valid) out[t] = g;
    }
}

struct Work {
    long long cap = 0;
    float *Z = nullptr, *G = nullptr, *H3 = nullptr, *yhat = nullptr, *d4 = nullptr, *grad = nullptr, *m = nullptr,
          *v = nullptr, *loss = nullptr;
    __nv_bfloat16 *H1 = nullptr, *H2 = nullptr, *D = nullptr, *D2 = nullptr;
};

Work& work(sg_ctx* ctx) {
    if (!ctx->mlp_work) ctx->mlp_work = new Work();
    return *static_cast<Work*>(ctx->mlp_work);
}

int ensure_work(sg_ctx* ctx, long long rows) {
    Work& w = work(ctx);
    if (!w.grad) {
        SG_CUDA(ctx, cudaMalloc(&w.grad, sizeof(float) * SG_MLP_NPARAM));
        SG_CUDA(ctx, cudaMalloc(&w.m, sizeof(float) * SG_MLP_NPARAM));
        SG_CUDA(ctx, cudaMalloc(&w.v, sizeof(float) * SG_MLP_NPARAM));
        SG_CUDA(ctx, cudaMalloc(&w.loss, sizeof(float)));
        SG_CUDA(ctx, cudaMemsetAsync(w.m, 0, sizeof(float) * SG_MLP_NPARAM, ctx->stream));
        SG_CUDA(ctx, cudaMemsetAsync(w.v, 0, sizeof(float) * SG_MLP_NPARAM, ctx->stream));
    }
    if (rows > w.cap) {
        float* fb[] = {w.Z, w.G, w.H3, w.yhat, w.d4};
        for (float* p : fb)
            if (p) cudaFree(p);
        __nv_bfloat16* bb[] = {w.H1, w.H2, w.D, w.D2};
        for (auto* p : bb)
            if (p) cudaFree(p);
        const size_t r = (size_t)rows;
        SG_CUDA(ctx, cudaMalloc(&w.Z, sizeof(float) * r * 64));
        SG_CUDA(ctx, cudaMalloc(&w.G, sizeof(float) * r * 64));
        SG_CUDA(ctx, cudaMalloc(&w.H3, sizeof(float) * r * 64));
        SG_CUDA(ctx, cudaMalloc(&w.yhat, sizeof(float) * r));
        SG_CUDA(ctx, cudaMalloc(&w.d4, sizeof(float) * r));
        SG_CUDA(ctx, cudaMalloc(&w.H1, sizeof(__nv_bfloat16) * r * 64));
        SG_CUDA(ctx, cudaMalloc(&w.H2, sizeof(__nv_bfloat16) * r * 64));
        SG_CUDA(ctx, cudaMalloc(&w.D, sizeof(__nv_bfloat16) * r * 64));
        SG_CUDA(ctx, cudaMalloc(&w.D2, sizeof(__nv_bfloat16) * r * 64));
        w.cap = rows;
    }
    return SG_OK;
}

int gemm(sg_ctx* ctx, int M, int N, int K, const __nv_bfloat16* A, long long sam, long long sak,
         const __nv_bfloat16* B, long long sbk, long long sbn, float* C, int ldc, int splitk, int atomic_out) {
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, splitk);
    k_gemm<<<grid, 128, 0, ctx->stream>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, atomic_out);
    SG_LAUNCH_CHECK(ctx, "k_gemm");
    return SG_OK;
}

inline int ew_blocks(long long n) { return (int)((n + 255) / 256); }

// forward (+ backward when y is given) on rows samples; gradients into w.grad
int fwd_bwd(sg_ctx* ctx, const __nv_bfloat16* X, const float* y, long long rows, float* yhat_out) {
    if (!ctx->mlp_ready) return sg_fail(ctx, SG_ENOTREADY, "MLP weights are not set");
    if (int rc = ensure_work(ctx, rows)) return rc;
    Work& w = work(ctx);
    const float* P = ctx->mlp_w;
    const __nv_bfloat16* Wb = (const __nv_bfloat16*)ctx->mlp_wbf16;
    const __nv_bfloat16 *W1 = Wb, *W2 = Wb + 64 * 16, *W3 = Wb + 64 * 16 + 64 * 64;
    const int R = (int)rows;
    // forward: Z = H W^T with W [64][K] row-major: B(k,n) = W[n][k]
    if (int rc = gemm(ctx, R, 64, 16, X, 16, 1, W1, 1, 16, w.Z, 64, 1, 0)) return rc;
    k_bias_relu<<<ew_blocks(rows * 64), 256, 0, ctx->stream>>>(rows, w.Z, P + SG_MLP_OFF_B1, w.H1, nullptr);
    if (int rc = gemm(ctx, R, 64, 64, w.H1, 64, 1, W2, 1, 64, w.Z, 64, 1, 0)) return rc;
    k_bias_relu<<<ew_blocks(rows * 64), 256, 0, ctx->stream>>>(rows, w.Z, P + SG_MLP_OFF_B2, w.H2, nullptr);
    if (int rc = gemm(ctx, R, 64, 64, w.H2, 64, 1, W3, 1, 64, w.Z, 64, 1, 0)) return rc;
    k_bias_relu<<<ew_blocks(rows * 64), 256, 0, ctx->stream>>>(rows, w.Z, P + SG_MLP_OFF_B3, nullptr, w.H3);
    SG_LAUNCH_CHECK(ctx, "forward");
    float b4 = 0.f;
    memcpy(&b4, ctx->mlp_host_desc + offsetof(MlpDev, b4), sizeof(float));
    if (y) {
        SG_CUDA(ctx, cudaMemsetAsync(w.grad, 0, sizeof(float) * SG_MLP_NPARAM, ctx->stream));
        SG_CUDA(ctx, cudaMemsetAsync(w.loss, 0, sizeof(float), ctx->stream));
    }
    k_out<<<ew_blocks(rows), 256, 0, ctx->stream>>>(rows, w.H3, P + SG_MLP_OFF_W4, b4, y,
                                                   yhat_out ? yhat_out : w.yhat, w.d4, 1.f / (float)rows, w.grad,
                                                   w.loss);
    SG_LAUNCH_CHECK(ctx, "k_out");
    if (!y) return SG_OK;
    const int split = std::max(1, std::min(256, R / 256));
    // layer 3
    k_delta3<<<ew_blocks(rows * 64), 256, 0, ctx->stream>>>(rows, w.d4, P + SG_MLP_OFF_W4, w.H3, w.D);
    k_colsum<<<std::min(1024, ew_blocks(rows)), 256, 0, ctx->stream>>>(rows, w.D, w.grad + SG_MLP_OFF_B3);
    // dW3 = D3^T H2: A(m=n_out, k=s) = D[s][m], B(k=s, n) = H2[s][n]
    if (int rc = gemm(ctx, 64, 64, R, w.D, 1, 64, w.H2, 64, 1, w.grad + SG_MLP_OFF_W3, 64, split, 1)) return rc;
    // G2 = D3 W3: A = D3 [s][i], B(k=i, n=j) = W3[i][j]
    if (int rc = gemm(ctx, R, 64, 64, w.D, 64, 1, W3, 64, 1, w.G, 64, 1, 0)) return rc;
    k_mask<<<ew_blocks(rows * 64), 256, 0, ctx->stream>>>(rows, w.G, w.H2, w.D2);
    k_colsum<<<std::min(1024, ew_blocks(rows)), 256, 0, ctx->stream>>>(rows, w.D2, w.grad + SG_MLP_OFF_B2);
    if (int rc = gemm(ctx, 64, 64, R, w.D2, 1, 64, w.H1, 64, 1, w.grad + SG_MLP_OFF_W2, 64, split, 1)) return rc;
    // G1 = D2 W2
    if (int rc = gemm(ctx, R, 64, 64, w.D2, 64, 1, W2, 64, 1, w.G, 64, 1, 0)) return rc;
    k_mask<<<ew_blocks(rows * 64), 256, 0, ctx->stream>>>(rows, w.G, w.H1, w.D);
    k_colsum<<<std::min(1024, ew_blocks(rows)), 256, 0, ctx->stream>>>(rows, w.D, w.grad + SG_MLP_OFF_B1);
    // dW1 = D1^T X: (64 x 16)
    if (int rc = gemm(ctx, 64, 16, R, w.D, 1, 64, X, 16, 1, w.grad + SG_MLP_OFF_W1, 16, split, 1)) return rc;
    SG_LAUNCH_CHECK(ctx, "backward");
    return SG_OK;
}

int refresh_bf16(sg_ctx* ctx) {
    __nv_bfloat16* wb = (__nv_bfloat16*)ctx->mlp_wbf16;
    k_bf16<<<(64 * 16 + 255) / 256, 256, 0, ctx->stream>>>(ctx->mlp_w + SG_MLP_OFF_W1, wb, 64 * 16);
    k_bf16<<<(64 * 64 + 255) / 256, 256, 0, ctx->stream>>>(ctx->mlp_w + SG_MLP_OFF_W2, wb + 64 * 16, 64 * 64);
    k_bf16<<<(64 * 64 + 255) / 256, 256, 0, ctx->stream>>>(ctx->mlp_w + SG_MLP_OFF_W3, wb + 64 * 16 + 64 * 64, 64 * 64);
    SG_LAUNCH_CHECK(ctx, "k_bf16");
    return SG_OK;
}

}  // namespace

extern "C" {

int sg_mlp_init(sg_ctx* ctx, uint64_t seed) {
    if (!ctx) return SG_EINVAL;
    // Kaiming-uniform weights, zero biases, output bias 0 (lambda = 1/2)
    std::vector<float> w(SG_MLP_NPARAM, 0.f);
    uint64_t s = seed * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
    auto uni = [&]() {
        s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
        return (float)((s * 0x2545F4914F6CDD1Dull) >> 40) / (float)(1ull << 24);
    };
    auto fill = [&](int off, int count, int fan_in) {
        const float a = sqrtf(6.f / (float)fan_in);
        for (int k = 0; k < count; ++k) w[off + k] = (2.f * uni() - 1.f) * a;
    };
    fill(SG_MLP_OFF_W1, 64 * 16, 14);
    fill(SG_MLP_OFF_W2, 64 * 64, 64);
    fill(SG_MLP_OFF_W3, 64 * 64, 64);
    fill(SG_MLP_OFF_W4, 64, 64);
    for (int k = 0; k < 64; ++k) w[SG_MLP_OFF_W4 + k] *= 0.1f;
    if (int rc = sg_mlp_set_weights(ctx, w.data(), SG_MLP_NPARAM)) return rc;
    Work& wk = work(ctx);
    if (wk.m) {
        SG_CUDA(ctx, cudaMemsetAsync(wk.m, 0, sizeof(float) * SG_MLP_NPARAM, ctx->stream));
        SG_CUDA(ctx, cudaMemsetAsync(wk.v, 0, sizeof(float) * SG_MLP_NPARAM, ctx->stream));
    }
    ctx->mlp_adam_t = 0;
    return SG_OK;
}

int sg_mlp_features(sg_ctx* ctx, void* x_bf16, float* y, int64_t capacity, int64_t* count) {
    if (ctx && ctx->nrep) return sg_fail(ctx, SG_EINVAL, "learned-guess data comes from single-system contexts");
    if (!ctx || !x_bf16 || !y || !count) return SG_EINVAL;
    int64_t k = 0;
    if (int rc = sg_nlist_count(ctx, &k)) return rc;
    if (!ctx->ecp_lambda) return sg_fail(ctx, SG_ENOTREADY, "no ECP call has produced lambda yet");
    if (ctx->ecp_lambda_partial)
        return sg_fail(ctx, SG_ENOTREADY,
                       "the last ECP call used the support-filtered launch, which leaves lambda of the pairs it "
                       "does not solve unset: select another launch (sg_pair_set_launch filter 0) to collect samples");
    const float3 box = make_float3((float)ctx->box[0], (float)ctx->box[1], (float)ctx->box[2]);
    const float3 ib = make_float3((float)(1.0 / ctx->box[0]), (float)(1.0 / ctx->box[1]), (float)(1.0 / ctx->box[2]));
    const long long n = std::min<long long>(k, capacity);
    if (n > 0)
        k_features<<<(int)((n + 255) / 256), 256, 0, ctx->stream>>>(ctx->nl.pair_i, ctx->nl.pair_j,
                                                                    ctx->nl.dev_flags + 2, ctx->pos, ctx->quat,
                                                                    ctx->shape, ctx->ecp_lambda, box, ib,
                                                                    ctx->periodic, capacity,
                                                                    (__nv_bfloat16*)x_bf16, y);
    SG_LAUNCH_CHECK(ctx, "k_features");
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *count = n;
    return SG_OK;
}

int sg_mlp_guess(sg_ctx* ctx, float* out_dev, int64_t capacity) {
    if (ctx && ctx->nrep) return sg_fail(ctx, SG_EINVAL, "learned-guess data comes from single-system contexts");
    if (!ctx || !out_dev) return SG_EINVAL;
    if (!ctx->mlp_ready) return sg_fail(ctx, SG_ENOTREADY, "MLP weights are not set");
    int64_t k = 0;
    if (int rc = sg_nlist_count(ctx, &k)) return rc;
    if (capacity < k) return sg_fail(ctx, SG_ECAPACITY, "guess capacity too small");
    const float3 box = make_float3((float)ctx->box[0], (float)ctx->box[1], (float)ctx->box[2]);
    const float3 ib = make_float3((float)(1.0 / ctx->box[0]), (float)(1.0 / ctx->box[1]), (float)(1.0 / ctx->box[2]));
    MlpDev m;
    memcpy(&m, ctx->mlp_host_desc, sizeof(m));
    const int grid = std::max(1, std::min(4 * ctx->num_sms, (int)((k + 255) / 256)));
    k_guess<<<grid, 256, 0, ctx->stream>>>(ctx->nl.pair_i, ctx->nl.pair_j, ctx->nl.dev_flags + 2, ctx->pos, ctx->quat,
                                           ctx->shape, box, ib, ctx->periodic, m, out_dev);
    SG_LAUNCH_CHECK(ctx, "k_guess");
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_mlp_grad(sg_ctx* ctx, const void* x_bf16, const float* y, int64_t rows, float* grad_host, float* loss_host) {
    if (!ctx || !x_bf16 || !y || rows < 1) return SG_EINVAL;
    if (int rc = fwd_bwd(ctx, (const __nv_bfloat16*)x_bf16, y, rows, nullptr)) return rc;
    Work& w = work(ctx);
    if (grad_host)
        SG_CUDA(ctx, cudaMemcpyAsync(grad_host, w.grad, sizeof(float) * SG_MLP_NPARAM, cudaMemcpyDeviceToHost, ctx->stream));
    if (loss_host) SG_CUDA(ctx, cudaMemcpyAsync(loss_host, w.loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_mlp_predict(sg_ctx* ctx, const void* x_bf16, int64_t rows, float* yhat_dev) {
    if (!ctx || !x_bf16 || !yhat_dev || rows < 1) return SG_EINVAL;
    return fwd_bwd(ctx, (const __nv_bfloat16*)x_bf16, nullptr, rows, yhat_dev);
}

int sg_mlp_train_step(sg_ctx* ctx, const void* x_bf16, const float* y, int64_t rows, float lr, float* loss_host) {
    if (!ctx || !x_bf16 || !y || rows < 1) return SG_EINVAL;
    if (int rc = fwd_bwd(ctx, (const __nv_bfloat16*)x_bf16, y, rows, nullptr)) return rc;
    Work& w = work(ctx);
    ctx->mlp_adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)ctx->mlp_adam_t), c2 = 1.f - powf(b2, (float)ctx->mlp_adam_t);
    k_adam<<<(SG_MLP_NPARAM + 255) / 256, 256, 0, ctx->stream>>>(SG_MLP_NPARAM, ctx->mlp_w, w.grad, w.m, w.v, lr, b1, b2,
                                                                1e-8f, c1, c2);
    SG_LAUNCH_CHECK(ctx, "k_adam");
    if (int rc = refresh_bf16(ctx)) return rc;
    // keep the host descriptor's output bias current
    float b4 = 0.f;
    SG_CUDA(ctx, cudaMemcpyAsync(&b4, ctx->mlp_w + SG_MLP_OFF_B4, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    if (loss_host) SG_CUDA(ctx, cudaMemcpyAsync(loss_host, w.loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    memcpy(ctx->mlp_host_desc + offsetof(MlpDev, b4), &b4, sizeof(float));
    return SG_OK;
}

}  // extern "C"

void sg_mlp_free(sg_ctx* ctx) {
    if (!ctx->mlp_work) return;
    Work* w = static_cast<Work*>(ctx->mlp_work);
    void* bufs[] = {w->Z, w->G, w->H3, w->yhat, w->d4, w->grad, w->m, w->v, w->loss, w->H1, w->H2, w->D, w->D2};
    for (void* p : bufs)
        if (p) cudaFree(p);
    delete w;
    ctx->mlp_work = nullptr;
}
