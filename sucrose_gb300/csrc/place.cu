// Seeded isotropic placement of hard ellipsoids at a target number density,
// on the device. It makes the initial state of the ellipsoid workloads,
// which the reference has no routine for (its only generator is the FCC
// lattice, fortran/system.f90:438-523).
//
// Positions start uniform in the box and orientations uniform on the unit
// 3-sphere, both from Philox words of the seed. The ellipsoids then grow from
// a fifth of their size to full size while Jacobi sweeps relax every
// overlapping pair. Overlap is the Perram-Wertheim test: with
// A = sum_k a_k^2 e_k e_k^T (e_k the body axes in the lab frame, a_k the
// semi-axes) and G(l) = (1 - l) A + l B, the pair overlaps iff
// F = max_l l (1 - l) r^T G(l)^-1 r < 1 (F = g^2 when the ellipsoids touch
// after scaling by g). At the optimal l, with K = G^-1 r and r = r_j - r_i,
//   dF/dr_j = 2 l (1 - l) K = -dF/dr_i,
//   dF/dtheta_i = -2 l (1 - l)^2 (A_i K x K),  dF/dtheta_j = -2 l^2 (1 - l) (A_j K x K)
// for lab-frame turns theta. Each overlapping pair contributes the
// linearised Newton step that raises F to a target slightly above the
// acceptance gap along this full gradient (orientations measured as arc
// length a_max theta); a particle takes 1.5 times the average of its pairs'
// steps. Each sweep grows the ellipsoids by 2 % while no pair overlaps, by
// 0.5 % while under one particle in a hundred is in an overlapping pair,
// and not at all above that; at full size the sweeps only relax.
//
// Positions, orientations and shape matrices are kept in FP64; the contact
// solve and the steps are FP32 (one warp per particle, lanes over its
// candidates), and a pair is accepted 1e-5 above gap^2 to cover FP32's error
// in F. Deterministic: every pair's step is computed by the same operations
// whatever order the neighbours are visited in, and a particle's steps are
// summed as 64-bit fixed-point integers (2^-40 units), whose sum does not
// depend on order; the overlap count is an integer and the minimum is
// order-free. The same seed gives the same bits on every run of the same
// build on the same GPU model.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "philox.cuh"
#include "sucrose_gpu.h"

namespace {

constexpr double kFix = 1099511627776.0;   // 2^40
constexpr double kRelax = 1.5;
constexpr double kOvershoot = 0.03;
constexpr double kCreep = 0.005;
constexpr int kMaxSweeps = 20000;

struct Sym {
    double xx, xy, xz, yy, yz, zz;
};

// Row k of the rotation matrix of q = (w, x, y, z) is body axis k in the lab
// frame, the convention of the pair kernels (force.f90:1244-1252).
__device__ Sym shape_matrix(const double q[4], const double a[3]) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double e[3][3] = {{w * w + x * x - y * y - z * z, 2.0 * (x * y + w * z), 2.0 * (x * z - w * y)},
                            {2.0 * (x * y - w * z), w * w - x * x + y * y - z * z, 2.0 * (y * z + w * x)},
                            {2.0 * (x * z + w * y), 2.0 * (y * z - w * x), w * w - x * x - y * y + z * z}};
    Sym s{0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 3; ++k) {
        const double a2 = a[k] * a[k];
        s.xx += a2 * e[k][0] * e[k][0];
        s.xy += a2 * e[k][0] * e[k][1];
        s.xz += a2 * e[k][0] * e[k][2];
        s.yy += a2 * e[k][1] * e[k][1];
        s.yz += a2 * e[k][1] * e[k][2];
        s.zz += a2 * e[k][2] * e[k][2];
    }
    return s;
}

__device__ __forceinline__ double wrap(double x, double L) {   // into [-L/2, L/2)
    double y = x - L * floor(x / L + 0.5);
    if (y >= 0.5 * L) y -= L;
    return y;
}

struct Geo {
    double L[3];
    double a[3];
    double amax;
    int nc[3];     // cells per side; 1 x 1 x 1 = all pairs
    int span;      // 1 with a cell stencil, 0 for all pairs
};

__device__ __forceinline__ int cell_of(const double* r, const Geo& g, int ci[3]) {
    for (int d = 0; d < 3; ++d) {
        const double u = (r[d] + 0.5 * g.L[d]) / g.L[d];
        ci[d] = min(max((int)floor(u * g.nc[d]), 0), g.nc[d] - 1);
    }
    return (ci[2] * g.nc[1] + ci[1]) * g.nc[0] + ci[0];
}

// Uniform positions and orientations (Marsaglia's method: two points
// uniform in the unit disk by rejection, no transcendental function).
__global__ void k_place_init(int n, uint32_t slo, uint32_t shi, Geo g, double* r, double* q, Sym* A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s32 = 1.0 / 4294967296.0, s31 = 1.0 / 2147483648.0;
    const sg_u4 w = sg_philox((uint32_t)i, slo, shi, 0x504F5354u, SG_PHILOX_KEY0, SG_PHILOX_KEY1);
    r[3 * i + 0] = ((double)w.x * s32 - 0.5) * g.L[0];
    r[3 * i + 1] = ((double)w.y * s32 - 0.5) * g.L[1];
    r[3 * i + 2] = ((double)w.z * s32 - 0.5) * g.L[2];
    double x1 = 0, y1 = 0, s1 = 2, x2 = 0, y2 = 0, s2 = 2;
    // each attempt succeeds with probability (pi/4)^2 for both disks: the
    // bound is never reached in practice, and a last miss keeps a valid axis
    for (uint32_t att = 0; att < 64 && (s1 >= 1.0 || s2 >= 1.0 || s2 <= 0.0); ++att) {
        const sg_u4 v = sg_philox((uint32_t)i, slo, shi, 0x51554154u + att, SG_PHILOX_KEY0, SG_PHILOX_KEY1);
        if (s1 >= 1.0) {
            x1 = (double)v.x * s31 - 1.0;
            y1 = (double)v.y * s31 - 1.0;
            s1 = x1 * x1 + y1 * y1;
        }
        x2 = (double)v.z * s31 - 1.0;
        y2 = (double)v.w * s31 - 1.0;
        s2 = x2 * x2 + y2 * y2;
    }
    double qq[4];
    if (s1 < 1.0 && s2 < 1.0 && s2 > 0.0) {
        const double f = sqrt((1.0 - s1) / s2);
        qq[0] = x1; qq[1] = y1; qq[2] = x2 * f; qq[3] = y2 * f;
    } else {
        qq[0] = 1.0; qq[1] = qq[2] = qq[3] = 0.0;
    }
    const double nn = sqrt(qq[0] * qq[0] + qq[1] * qq[1] + qq[2] * qq[2] + qq[3] * qq[3]);
    const double sg = qq[0] < 0.0 ? -1.0 : 1.0;
    for (int k = 0; k < 4; ++k) q[4 * i + k] = sg * qq[k] / nn;
    A[i] = shape_matrix(&q[4 * i], g.a);
}

__global__ void k_place_count(int n, Geo g, const double* r, int* cid, int* cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int ci[3];
    const int c = cell_of(&r[3 * i], g, ci);
    cid[i] = c;
    atomicAdd(&cnt[c], 1);
}

// exclusive scan of the cell counts, one block (cells <= 64^3)
__global__ void k_place_scan(int ncell, const int* cnt, int* start, int* fill) {
    __shared__ int part[1024];
    const int t = threadIdx.x, per = (ncell + 1023) / 1024;
    const int b = t * per, e = min(ncell, b + per);
    int s = 0;
    for (int c = b; c < e; ++c) s += cnt[c];
    part[t] = s;
    __syncthreads();
    if (t == 0) {
        int acc = 0;
        for (int k = 0; k < 1024; ++k) {
            const int v = part[k];
            part[k] = acc;
            acc += v;
        }
        start[ncell] = acc;
    }
    __syncthreads();
    int acc = part[t];
    for (int c = b; c < e; ++c) {
        start[c] = acc;
        fill[c] = acc;
        acc += cnt[c];
    }
}

__global__ void k_place_fill(int n, const int* cid, int* fill, int* list) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    list[atomicAdd(&fill[cid[i]], 1)] = i;   // order within a cell does not matter (integer sums)
}

struct SweepCounters {
    unsigned long long overlaps;   // overlapping (i, j) seen from both ends
    unsigned long long fmin_bits;  // bits of the smallest F (non-negative doubles order as integers)
};

// FP32 forms for the sweep: the contact solve only steers the relaxation and
// decides acceptance, where FP32's ~1e-6 relative error in F is covered by
// the acceptance margin below.
struct SymF {
    float xx, xy, xz, yy, yz, zz;
};

__device__ __forceinline__ SymF to_f(const Sym& m) {
    return SymF{(float)m.xx, (float)m.xy, (float)m.xz, (float)m.yy, (float)m.yz, (float)m.zz};
}

__device__ __forceinline__ void mulf(const SymF& m, const float v[3], float o[3]) {
    o[0] = m.xx * v[0] + m.xy * v[1] + m.xz * v[2];
    o[1] = m.xy * v[0] + m.yy * v[1] + m.yz * v[2];
    o[2] = m.xz * v[0] + m.yz * v[1] + m.zz * v[2];
}

__device__ __forceinline__ float dotf(const float a[3], const float b[3]) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

__device__ __forceinline__ void crossf(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// G^-1 v through the adjugate (G symmetric positive definite)
__device__ __forceinline__ void solvef(const SymF& m, const float v[3], float x[3]) {
    const float c00 = m.yy * m.zz - m.yz * m.yz, c01 = m.xz * m.yz - m.xy * m.zz, c02 = m.xy * m.yz - m.xz * m.yy;
    const float c11 = m.xx * m.zz - m.xz * m.xz, c12 = m.xy * m.xz - m.xx * m.yz, c22 = m.xx * m.yy - m.xy * m.xy;
    const float inv = 1.0f / (m.xx * c00 + m.xy * c01 + m.xz * c02);
    x[0] = (c00 * v[0] + c01 * v[1] + c02 * v[2]) * inv;
    x[1] = (c01 * v[0] + c11 * v[1] + c12 * v[2]) * inv;
    x[2] = (c02 * v[0] + c12 * v[1] + c22 * v[2]) * inv;
}

__device__ __forceinline__ SymF lerpf(const SymF& A, const SymF& B, float l) {
    const float u = 1.0f - l;
    return SymF{u * A.xx + l * B.xx, u * A.xy + l * B.xy, u * A.xz + l * B.xz,
                u * A.yy + l * B.yy, u * A.yz + l * B.yz, u * A.zz + l * B.zz};
}

// The Perram-Wertheim contact function in FP32 (safeguarded Newton, at
// most 40 steps); returns F, the optimal l and K = G(l)^-1 r.
__device__ float pw_contact_f(const SymF& A, const SymF& B, const float r[3], float& lam, float K[3]) {
    const SymF D{B.xx - A.xx, B.xy - A.xy, B.xz - A.xz, B.yy - A.yy, B.yz - A.yz, B.zz - A.zz};
    float lo = 0.0f, hi = 1.0f, l = 0.5f;
    for (int it = 0; it < 40; ++it) {
        const SymF G = lerpf(A, B, l);
        const float u = 1.0f - l;
        float DK[3], GDK[3];
        solvef(G, r, K);
        mulf(D, K, DK);
        solvef(G, DK, GDK);
        const float rk = dotf(r, K), kdk = dotf(K, DK), h2 = dotf(DK, GDK);
        const float d1 = (1.0f - 2.0f * l) * rk - l * u * kdk;
        const float d2 = -2.0f * rk - 2.0f * (1.0f - 2.0f * l) * kdk + 2.0f * l * u * h2;
        if (d1 > 0.0f) lo = l;
        else hi = l;
        float ln = (d2 < 0.0f) ? l - d1 / d2 : 0.5f * (lo + hi);
        if (!(ln > lo && ln < hi)) ln = 0.5f * (lo + hi);
        const float step = ln - l;
        l = ln;
        if (fabsf(step) < 1e-6f || hi - lo < 1e-6f) break;
    }
    solvef(lerpf(A, B, l), r, K);
    lam = l;
    return l * (1.0f - l) * dotf(r, K);
}

__device__ __forceinline__ long long fix(float v) { return __double2ll_rn((double)v * kFix); }

// One Jacobi sweep, one warp per particle, lanes over the candidates of its
// cell stencil: every lane sums the projection steps of its overlapping
// pairs in fixed point, the warp adds the integer sums (exact, so the order
// of candidates does not matter) and lane 0 writes them.
__global__ void __launch_bounds__(256) k_place_sweep(int n, Geo g, float s, float accept, float target,
                                                     const double* __restrict__ r, const Sym* __restrict__ A,
                                                     const int* __restrict__ start, const int* __restrict__ list,
                                                     long long* __restrict__ acc, int* __restrict__ contacts,
                                                     SweepCounters* cnt) {
    const int lane = threadIdx.x & 31;
    const int i = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (i >= n) return;   // warp-uniform
    const float s2 = s * s, tgap = sqrtf(target), ia2 = 1.0f / (float)(g.amax * g.amax);
    const float range = 2.0f * s * (float)g.amax * tgap, range2 = range * range;
    const float max_move = 0.5f * s * (float)g.amax;   // cap on one pair's step (near-coincident centres)
    const double ri[3] = {r[3 * i], r[3 * i + 1], r[3 * i + 2]};
    const SymF Ai = to_f(A[i]);
    long long p[6] = {0, 0, 0, 0, 0, 0};
    int nc = 0;
    float fmin_v = 3.0e38f;
    int ci[3];
    cell_of(ri, g, ci);
    for (int dz = -g.span; dz <= g.span; ++dz)
        for (int dy = -g.span; dy <= g.span; ++dy)
            for (int dx = -g.span; dx <= g.span; ++dx) {
                const int kx = (ci[0] + dx + g.nc[0]) % g.nc[0];
                const int ky = (ci[1] + dy + g.nc[1]) % g.nc[1];
                const int kz = (ci[2] + dz + g.nc[2]) % g.nc[2];
                const int cell = (kz * g.nc[1] + ky) * g.nc[0] + kx;
                for (int m = start[cell] + lane; m < start[cell + 1]; m += 32) {
                    const int j = list[m];
                    if (j == i) continue;
                    float d[3];
                    for (int k = 0; k < 3; ++k) d[k] = (float)wrap(r[3 * j + k] - ri[k], g.L[k]);
                    const float dd = dotf(d, d);
                    if (dd >= range2) continue;
                    const SymF Aj = to_f(A[j]);
                    float Ad[3], Bd[3];
                    mulf(Ai, d, Ad);
                    mulf(Aj, d, Bd);
                    // separated along the centre line by more than the two support
                    // distances (h = sqrt(d.A d) / |d|): no overlap at the target gap
                    if (dd >= tgap * s * (sqrtf(dotf(d, Ad)) + sqrtf(dotf(d, Bd)))) continue;
                    float lam, K[3];
                    const float f = pw_contact_f(Ai, Aj, d, lam, K) / s2;
                    fmin_v = fminf(fmin_v, f);
                    if (!(f < accept)) continue;
                    ++nc;
                    const float u = 1.0f - lam;
                    float AK[3], BK[3], gi[3], gj[3], gr[3];
                    mulf(Ai, K, AK);
                    mulf(Aj, K, BK);
                    crossf(AK, K, gi);
                    crossf(BK, K, gj);
                    for (int k = 0; k < 3; ++k) {
                        gr[k] = -2.0f * lam * u * K[k] / s2;   // dF/dr_i of the grown pair
                        gi[k] *= -2.0f * lam * u * u / s2;
                        gj[k] *= -2.0f * lam * lam * u / s2;
                    }
                    const float norm2 = 2.0f * dotf(gr, gr) + (dotf(gi, gi) + dotf(gj, gj)) * ia2;
                    if (!(norm2 > 1e-30f)) continue;
                    float step = (target - f) / norm2;
                    const float move = step * sqrtf(norm2);
                    if (move > max_move) step *= max_move / move;
                    for (int k = 0; k < 3; ++k) {
                        p[k] += fix(step * gr[k]);
                        p[3 + k] += fix(step * gi[k] * ia2);
                    }
                }
            }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 6; ++k) p[k] += __shfl_xor_sync(0xffffffffu, p[k], o);
        nc += __shfl_xor_sync(0xffffffffu, nc, o);
        fmin_v = fminf(fmin_v, __shfl_xor_sync(0xffffffffu, fmin_v, o));
    }
    if (lane == 0) {
        for (int k = 0; k < 6; ++k) acc[6 * (size_t)i + k] = p[k];
        contacts[i] = nc;
        if (nc) atomicAdd(&cnt->overlaps, (unsigned long long)nc);
        if (fmin_v < 3.0e38f)
            atomicMin(&cnt->fmin_bits, (unsigned long long)__double_as_longlong((double)fmin_v));
    }
}

// r += relax * mean step; q <- dq (x) q with dq = (1, theta / 2) normalised
// (the body axes turn by theta in the lab frame, to first order).
__global__ void k_place_apply(int n, Geo g, const long long* __restrict__ acc, const int* __restrict__ contacts,
                              double* r, double* q, Sym* A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nc = contacts[i];
    if (!nc) return;
    const double w = kRelax / (double)nc / kFix;
    for (int k = 0; k < 3; ++k) r[3 * i + k] = wrap(r[3 * i + k] + w * (double)acc[6 * (size_t)i + k], g.L[k]);
    const double x = 0.5 * w * (double)acc[6 * (size_t)i + 3], y = 0.5 * w * (double)acc[6 * (size_t)i + 4],
                 z = 0.5 * w * (double)acc[6 * (size_t)i + 5];
    double* qi = &q[4 * i];
    const double o[4] = {qi[0] - x * qi[1] - y * qi[2] - z * qi[3], qi[1] + x * qi[0] + y * qi[3] - z * qi[2],
                         qi[2] - x * qi[3] + y * qi[0] + z * qi[1], qi[3] + x * qi[2] - y * qi[1] + z * qi[0]};
    const double nn = sqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2] + o[3] * o[3]);
    for (int k = 0; k < 4; ++k) qi[k] = o[k] / nn;
    A[i] = shape_matrix(qi, g.a);
}

struct Buffers {
    double *r = nullptr, *q = nullptr;
    Sym* A = nullptr;
    long long* acc = nullptr;
    int *contacts = nullptr, *cid = nullptr, *cnt = nullptr, *start = nullptr, *fill = nullptr, *list = nullptr;
    SweepCounters* ctr = nullptr;
    SweepCounters* ctr_host = nullptr;
    ~Buffers() {
        cudaFree(r); cudaFree(q); cudaFree(A); cudaFree(acc); cudaFree(contacts); cudaFree(cid);
        cudaFree(cnt); cudaFree(start); cudaFree(fill); cudaFree(list); cudaFree(ctr);
        cudaFreeHost(ctr_host);
    }
};

}  // namespace

extern "C" int sg_place_isotropic(int64_t n, const double semi_axes[3], const double box[3], uint64_t seed,
                                  double gap, double* r_out, double* q_out, sg_place_report* rep) {
    if (n < 2 || n > (1 << 28) || !semi_axes || !box || !r_out || !q_out) return SG_EINVAL;
    Geo g;
    g.amax = 0.0;
    for (int k = 0; k < 3; ++k) {
        if (!(semi_axes[k] > 0.0) || !(box[k] > 0.0)) return SG_EINVAL;
        g.a[k] = semi_axes[k];
        g.L[k] = box[k];
        g.amax = std::max(g.amax, semi_axes[k]);
    }
    if (!(gap >= 1.0 && gap < 2.0)) return SG_EINVAL;
    const double tgap = gap + kOvershoot;
    // the minimum image must see every neighbour within the contact range
    for (int k = 0; k < 3; ++k)
        if (box[k] < 4.0 * g.amax * tgap) return SG_ECUTOFF_GT_HALFBOX;
    const int N = (int)n;
    // cells at the full size serve every stage (the range only grows)
    const double range = 2.0 * g.amax * tgap;
    g.span = 1;
    for (int k = 0; k < 3; ++k) {
        g.nc[k] = std::min(64, (int)std::floor(box[k] / range));
        if (g.nc[k] < 3) g.span = 0;
    }
    if (!g.span) g.nc[0] = g.nc[1] = g.nc[2] = 1;
    const int ncell = g.nc[0] * g.nc[1] * g.nc[2];
    Buffers b;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return SG_ECUDA;
    bool ok = cudaMalloc(&b.r, sizeof(double) * 3 * N) == cudaSuccess &&
              cudaMalloc(&b.q, sizeof(double) * 4 * N) == cudaSuccess &&
              cudaMalloc(&b.A, sizeof(Sym) * N) == cudaSuccess &&
              cudaMalloc(&b.acc, sizeof(long long) * 6 * N) == cudaSuccess &&
              cudaMalloc(&b.contacts, sizeof(int) * N) == cudaSuccess &&
              cudaMalloc(&b.cid, sizeof(int) * N) == cudaSuccess &&
              cudaMalloc(&b.cnt, sizeof(int) * ncell) == cudaSuccess &&
              cudaMalloc(&b.start, sizeof(int) * (ncell + 1)) == cudaSuccess &&
              cudaMalloc(&b.fill, sizeof(int) * ncell) == cudaSuccess &&
              cudaMalloc(&b.list, sizeof(int) * N) == cudaSuccess &&
              cudaMalloc(&b.ctr, sizeof(SweepCounters)) == cudaSuccess &&
              cudaMallocHost(&b.ctr_host, sizeof(SweepCounters)) == cudaSuccess;
    if (!ok) {
        cudaStreamDestroy(st);
        return SG_ECUDA;
    }
    const int T = 128, B = (N + T - 1) / T;
    k_place_init<<<B, T, 0, st>>>(N, (uint32_t)seed, (uint32_t)(seed >> 32), g, b.r, b.q, b.A);
    double s = 0.2;
    int stages = 0, sweeps = 0;
    unsigned long long overlaps = 0;
    double fmin_v = 1e300;
    double big = 1e300;
    unsigned long long big_bits = 0;
    std::memcpy(&big_bits, &big, sizeof(big));
    const SweepCounters zero{0ull, big_bits};
    int rc = SG_OK;
    for (; sweeps < kMaxSweeps;) {
        cudaMemsetAsync(b.cnt, 0, sizeof(int) * ncell, st);
        k_place_count<<<B, T, 0, st>>>(N, g, b.r, b.cid, b.cnt);
        k_place_scan<<<1, 1024, 0, st>>>(ncell, b.cnt, b.start, b.fill);
        k_place_fill<<<B, T, 0, st>>>(N, b.cid, b.fill, b.list);
        cudaMemcpyAsync(b.ctr, &zero, sizeof(zero), cudaMemcpyHostToDevice, st);
        // acceptance 1e-5 above gap^2 covers the FP32 contact solve
        k_place_sweep<<<(int)(((int64_t)N * 32 + 255) / 256), 256, 0, st>>>(
            N, g, (float)s, (float)(gap * gap * (1.0 + 1e-5)), (float)(tgap * tgap), b.r, b.A, b.start, b.list,
            b.acc, b.contacts, b.ctr);
        k_place_apply<<<B, T, 0, st>>>(N, g, b.acc, b.contacts, b.r, b.q, b.A);
        cudaMemcpyAsync(b.ctr_host, b.ctr, sizeof(SweepCounters), cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) {
            rc = SG_ECUDA;
            break;
        }
        ++sweeps;
        overlaps = b.ctr_host->overlaps / 2;   // each pair seen from both ends
        std::memcpy(&fmin_v, &b.ctr_host->fmin_bits, sizeof(fmin_v));
        if (overlaps == 0 && s >= 1.0) break;
        const double grow = overlaps == 0 ? 0.02 : ((int64_t)overlaps * 100 < n ? kCreep : 0.0);
        if (grow > 0.0 && s < 1.0) {
            s = std::min(1.0, s * (1.0 + grow));
            ++stages;
        }
    }
    if (rc == SG_OK) {
        std::vector<double> hr(3 * (size_t)N), hq(4 * (size_t)N);
        if (cudaMemcpy(hr.data(), b.r, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(hq.data(), b.q, sizeof(double) * 4 * N, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = SG_ECUDA;
        std::copy(hr.begin(), hr.end(), r_out);
        std::copy(hq.begin(), hq.end(), q_out);
    }
    cudaStreamDestroy(st);
    if (rep) {
        rep->stages = stages;
        rep->sweeps = sweeps;
        rep->overlaps = (int64_t)overlaps;
        rep->min_contact_ratio = std::sqrt(std::max(fmin_v, 0.0));
        rep->final_scale = s;
    }
    if (rc != SG_OK) return rc;
    return (overlaps == 0 && s >= 1.0) ? SG_OK : SG_ENOCONV;
}
