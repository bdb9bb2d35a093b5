// Verlet half list on the device: the reference's build_nlist / needs_rebuild
// (fortran/system.f90:895-1051) re-designed as integer cell binning.
//
// Pair set contract: a pair (i < j) is listed iff the reference's FP64 test
// accepts it: RIJ = R(I) - R(J); RIJ -= ANINT(RIJ/box)*box when periodic;
// SUM(RIJ*RIJ) < (rc+skin)^2 (:980-989), evaluated on the FP32 state promoted
// to FP64. The FP32 filter decides only pairs clear of the threshold by a
// relative guard band of 1e-4; every other candidate is re-tested with the
// reference's exact FP64 operation sequence (no contraction).
//
// Layout in HBM: per-particle rows of at most max_nb neighbours are written
// column-major into nb_pad (k * n + i), then compacted into the flattened pair
// arrays pair_i / pair_j, rows in particle order, which every pair kernel
// walks 32 pairs per warp.
#include <algorithm>
#include <cmath>
#include <vector>

#include "sg_internal.cuh"

namespace {

constexpr int SCAN_BLOCK = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_BLOCK * SCAN_ITEMS;

// flags layout
enum { F_REBUILD = 0, F_OVERFLOW = 1, F_NPAIRS = 2, F_BUILDS = 3 };

struct ListGeom {
    float3 box, inv_box;
    double bx, by, bz;
    double rl2;       // (rc+skin)^2
    float rl2_lo, rl2_hi;
    int periodic;
    int nc[3];
};

// Reference FP64 acceptance test, operation by operation (system.f90:980-989).
__device__ __forceinline__ bool ref_accept(float4 pi, float4 pj, const ListGeom& g) {
    double dx = __dsub_rn((double)pi.x, (double)pj.x);
    double dy = __dsub_rn((double)pi.y, (double)pj.y);
    double dz = __dsub_rn((double)pi.z, (double)pj.z);
    if (g.periodic) {
        dx = __dsub_rn(dx, __dmul_rn(round(__ddiv_rn(dx, g.bx)), g.bx));
        dy = __dsub_rn(dy, __dmul_rn(round(__ddiv_rn(dy, g.by)), g.by));
        dz = __dsub_rn(dz, __dmul_rn(round(__ddiv_rn(dz, g.bz)), g.bz));
    }
    double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return r2 < g.rl2;
}

__device__ __forceinline__ bool near_half(float d, float inv_b) {
    float f = fabsf(d * inv_b);
    f = f - floorf(f);
    return fabsf(f - 0.5f) < 1e-4f;
}

// FP32 filter, exact FP64 decision inside the guard band.
__device__ __forceinline__ bool accept_pair(float4 pi, float4 pj, const ListGeom& g) {
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    bool halfcase = false;
    if (g.periodic) {
        halfcase = near_half(dx, g.inv_box.x) || near_half(dy, g.inv_box.y) || near_half(dz, g.inv_box.z);
        dx -= roundf(dx * g.inv_box.x) * g.box.x;
        dy -= roundf(dy * g.inv_box.y) * g.box.y;
        dz -= roundf(dz * g.inv_box.z) * g.box.z;
    }
    float r2 = dx * dx + dy * dy + dz * dz;
    if (!halfcase) {
        if (r2 < g.rl2_lo) return true;
        if (r2 > g.rl2_hi) return false;
    }
    return ref_accept(pi, pj, g);
}

__device__ __forceinline__ int wrapc(int c, int n) {
    c %= n;
    return c < 0 ? c + n : c;
}

__device__ __forceinline__ int cell_of(float4 p, const ListGeom& g, int& cx, int& cy, int& cz) {
    cx = wrapc((int)floorf((p.x + 0.5f * g.box.x) * (g.nc[0] * g.inv_box.x)), g.nc[0]);
    cy = wrapc((int)floorf((p.y + 0.5f * g.box.y) * (g.nc[1] * g.inv_box.y)), g.nc[1]);
    cz = wrapc((int)floorf((p.z + 0.5f * g.box.z) * (g.nc[2] * g.inv_box.z)), g.nc[2]);
    return (cz * g.nc[1] + cy) * g.nc[0] + cx;
}

// ---------------------------------------------------------------- trigger --
// needs_rebuild (system.f90:1005-1039) in FP64 on the FP32 state: any
// particle with 4 |dr|^2 > trigger_sq requests a rebuild (the maximum over
// particles exceeds the bound iff some particle does).
__global__ void k_check(int n, const float4* __restrict__ pos, const float4* __restrict__ last, ListGeom g,
                        double trigger_sq, int* flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = pos[i], b = last[i];
    {
        // FP32 screen: decide in FP32 when clear of the bound by 1e-3 relative
        float fx = a.x - b.x, fy = a.y - b.y, fz = a.z - b.z;
        if (g.periodic) {
            fx -= roundf(fx * g.inv_box.x) * g.box.x;
            fy -= roundf(fy * g.inv_box.y) * g.box.y;
            fz -= roundf(fz * g.inv_box.z) * g.box.z;
        }
        const float f4 = 4.f * (fx * fx + fy * fy + fz * fz);
        if (f4 < (float)trigger_sq * 0.999f && fabsf(fx) < 0.25f * g.box.x && fabsf(fy) < 0.25f * g.box.y &&
            fabsf(fz) < 0.25f * g.box.z)
            return;
    }
    double dx = __dsub_rn((double)a.x, (double)b.x), dy = __dsub_rn((double)a.y, (double)b.y),
           dz = __dsub_rn((double)a.z, (double)b.z);
    if (g.periodic) {
        dx = __dsub_rn(dx, __dmul_rn(round(__ddiv_rn(dx, g.bx)), g.bx));
        dy = __dsub_rn(dy, __dmul_rn(round(__ddiv_rn(dy, g.by)), g.by));
        dz = __dsub_rn(dz, __dmul_rn(round(__ddiv_rn(dz, g.bz)), g.bz));
    }
    double r = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    if (__dmul_rn(4.0, r) > trigger_sq) flags[F_REBUILD] = 1;
}

__global__ void k_begin(int* flags, int* cell_count, int* cell_fill, int ncells) {
    if (!flags[F_REBUILD]) return;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    for (int c = t; c < ncells; c += gridDim.x * blockDim.x) {
        cell_count[c] = 0;
        cell_fill[c] = 0;
    }
    if (t == 0) flags[F_OVERFLOW] = 0;
}

__global__ void k_bin(int n, const float4* __restrict__ pos, ListGeom g, int* particle_cell, int* cell_count,
                      const int* flags) {
    if (!flags[F_REBUILD]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int cx, cy, cz;
    int c = cell_of(pos[i], g, cx, cy, cz);
    particle_cell[i] = c;
    atomicAdd(&cell_count[c], 1);
}

__global__ void k_fill(int n, const int* __restrict__ particle_cell, const int* __restrict__ cell_start, int* cell_fill,
                       int* cell_particles, const int* flags) {
    if (!flags[F_REBUILD]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = particle_cell[i];
    int s = atomicAdd(&cell_fill[c], 1);
    cell_particles[cell_start[c] + s] = i;
}

// Order each cell's particles by index so that rows are deterministic.
__global__ void k_sort_cells(int ncells, const int* __restrict__ cell_start, int* cell_particles, const int* flags) {
    if (!flags[F_REBUILD]) return;
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    int b = cell_start[c], e = cell_start[c + 1];
    for (int k = b + 1; k < e; ++k) {
        int v = cell_particles[k];
        int m = k - 1;
        while (m >= b && cell_particles[m] > v) {
            cell_particles[m + 1] = cell_particles[m];
            --m;
        }
        cell_particles[m + 1] = v;
    }
}

__global__ void k_rows_cells(int n, const float4* __restrict__ pos, ListGeom g, const int* __restrict__ cell_start,
                             const int* __restrict__ cell_particles, int max_nb, int* nb_pad, int* nb_count,
                             int* flags) {
    if (!flags[F_REBUILD]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 pi = pos[i];
    int cx, cy, cz;
    cell_of(pi, g, cx, cy, cz);
    int cnt = 0;
    for (int dz = -1; dz <= 1; ++dz) {
        int zz = wrapc(cz + dz, g.nc[2]);
        for (int dy = -1; dy <= 1; ++dy) {
            int yy = wrapc(cy + dy, g.nc[1]);
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = wrapc(cx + dx, g.nc[0]);
                int c = (zz * g.nc[1] + yy) * g.nc[0] + xx;
                int b = cell_start[c], e = cell_start[c + 1];
                for (int k = b; k < e; ++k) {
                    int j = cell_particles[k];
                    if (j <= i) continue;
                    if (accept_pair(pi, pos[j], g)) {
                        if (cnt < max_nb) nb_pad[(size_t)cnt * n + i] = j;
                        ++cnt;
                    }
                }
            }
        }
    }
    nb_count[i] = min(cnt, max_nb);
    if (cnt > max_nb) atomicMax(&flags[F_OVERFLOW], cnt);
}

// All-pairs variant for boxes with fewer than three cells per side and for
// open boundaries: every j > i is tested.
__global__ void k_rows_all(int n, const float4* __restrict__ pos, ListGeom g, int max_nb, int* nb_pad, int* nb_count,
                           int* flags) {
    if (!flags[F_REBUILD]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 pi = pos[i];
    int cnt = 0;
    for (int j = i + 1; j < n; ++j) {
        if (accept_pair(pi, pos[j], g)) {
            if (cnt < max_nb) nb_pad[(size_t)cnt * n + i] = j;
            ++cnt;
        }
    }
    nb_count[i] = min(cnt, max_nb);
    if (cnt > max_nb) atomicMax(&flags[F_OVERFLOW], cnt);
}

// ---- exclusive scan of m ints into out[0..m], out[m] = total -----------------
__global__ void k_scan_tiles(const int* __restrict__ in, int m, int* out, int* tile_sums, const int* flags) {
    if (flags && !flags[F_REBUILD]) return;
    __shared__ int warp_sums[SCAN_BLOCK / 32];
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int v[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        v[k] = (base + k < m) ? in[base + k] : 0;
        s += v[k];
    }
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[w] = x;
    __syncthreads();
    if (w == 0) {
        int ws = warp_sums[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += y;
        }
        warp_sums[lane] = ws;
    }
    __syncthreads();
    int excl = x - s + (w > 0 ? warp_sums[w - 1] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        if (base + k < m) out[base + k] = excl;
        excl += v[k];
    }
    if (threadIdx.x == SCAN_BLOCK - 1) tile_sums[blockIdx.x] = warp_sums[31];
}

// Single block: exclusive scan of the tile sums in place, total at [ntiles].
__global__ void k_scan_sums(int* tile_sums, int ntiles, const int* flags) {
    if (flags && !flags[F_REBUILD]) return;
    __shared__ int sh[SCAN_BLOCK + 1];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < ntiles; base += SCAN_BLOCK) {
        int t = base + threadIdx.x;
        int v = t < ntiles ? tile_sums[t] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < SCAN_BLOCK; o <<= 1) {
            int y = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += y;
            __syncthreads();
        }
        if (t < ntiles) tile_sums[t] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += sh[SCAN_BLOCK - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_sums[ntiles] = carry;
}

__global__ void k_scan_add(int* out, int m, const int* __restrict__ tile_sums, int ntiles, int* total_dst,
                           const int* flags) {
    if (flags && !flags[F_REBUILD]) return;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < m) out[t] += tile_sums[t / SCAN_TILE];
    if (t == 0) {
        out[m] = tile_sums[ntiles];
        if (total_dst) *total_dst = tile_sums[ntiles];
    }
}

__global__ void k_compact(int n, const int* __restrict__ nb_pad, const int* __restrict__ nb_count,
                          const int* __restrict__ row_off, int* pair_i, int* pair_j, const int* flags) {
    if (!flags[F_REBUILD]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int o = row_off[i], c = nb_count[i];
    for (int k = 0; k < c; ++k) {
        pair_i[o + k] = i;
        pair_j[o + k] = nb_pad[(size_t)k * n + i];
    }
}

__global__ void k_finish(int n, const float4* __restrict__ pos, float4* last, int* flags) {
    if (!flags[F_REBUILD]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) last[i] = pos[i];
    __syncthreads();
    // the last block clears the request; blocks only read the flag at entry
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        flags[F_BUILDS] += 1;
    }
}

__global__ void k_clear_request(int* flags) { flags[F_REBUILD] = 0; }
__global__ void k_set_request(int* flags) { flags[F_REBUILD] = 1; }

ListGeom make_geom(const sg_ctx* ctx) {
    ListGeom g;
    g.box = make_float3((float)ctx->box[0], (float)ctx->box[1], (float)ctx->box[2]);
    g.inv_box = make_float3((float)(1.0 / ctx->box[0]), (float)(1.0 / ctx->box[1]), (float)(1.0 / ctx->box[2]));
    g.bx = ctx->box[0]; g.by = ctx->box[1]; g.bz = ctx->box[2];
    g.rl2 = ctx->nl.rl2;
    g.rl2_lo = (float)(ctx->nl.rl2 * (1.0 - 1e-4));
    g.rl2_hi = (float)(ctx->nl.rl2 * (1.0 + 1e-4));
    g.periodic = ctx->periodic;
    for (int d = 0; d < 3; ++d) g.nc[d] = ctx->nl.ncell[d] > 0 ? ctx->nl.ncell[d] : 1;
    return g;
}

int scan(sg_ctx* ctx, const int* in, int m, int* out, int* total_dst, const int* flags) {
    int ntiles = (m + SCAN_TILE - 1) / SCAN_TILE;
    if (ntiles < 1) ntiles = 1;
    k_scan_tiles<<<ntiles, SCAN_BLOCK, 0, ctx->stream>>>(in, m, out, ctx->nl.scan_tmp, flags);
    k_scan_sums<<<1, SCAN_BLOCK, 0, ctx->stream>>>(ctx->nl.scan_tmp, ntiles, flags);
    k_scan_add<<<(m + 255) / 256 + 1, 256, 0, ctx->stream>>>(out, m, ctx->nl.scan_tmp, ntiles, total_dst, flags);
    SG_LAUNCH_CHECK(ctx, "scan");
    return SG_OK;
}

int alloc_rows(sg_ctx* ctx, int max_nb) {
    sg_nlist_state& nl = ctx->nl;
    if (nl.nb_pad) cudaFree(nl.nb_pad);
    if (nl.pair_i) cudaFree(nl.pair_i);
    if (nl.pair_j) cudaFree(nl.pair_j);
    nl.nb_pad = nl.pair_i = nl.pair_j = nullptr;
    ctx->graph_epoch++;
    nl.max_nb = max_nb;
    nl.pair_capacity = (int64_t)max_nb * ctx->n;
    if (nl.pair_capacity > (int64_t)INT32_MAX)
        return sg_fail(ctx, SG_ECAPACITY, "neighbour list capacity %lld exceeds 2^31", (long long)nl.pair_capacity);
    SG_CUDA(ctx, cudaMalloc(&nl.nb_pad, sizeof(int) * (size_t)nl.pair_capacity));
    SG_CUDA(ctx, cudaMalloc(&nl.pair_i, sizeof(int) * (size_t)nl.pair_capacity));
    SG_CUDA(ctx, cudaMalloc(&nl.pair_j, sizeof(int) * (size_t)nl.pair_capacity));
    return SG_OK;
}

// Enqueue the (flag-gated) build kernels.
int enqueue_build(sg_ctx* ctx) {
    sg_nlist_state& nl = ctx->nl;
    const int n = ctx->n;
    ListGeom g = make_geom(ctx);
    const int nb = (n + 255) / 256;
    if (nl.use_cells) {
        k_begin<<<std::max(1, std::min(1024, (nl.ncells + 255) / 256)), 256, 0, ctx->stream>>>(nl.dev_flags, nl.cell_count,
                                                                                                nl.cell_fill, nl.ncells);
        k_bin<<<nb, 256, 0, ctx->stream>>>(n, ctx->pos, g, nl.particle_cell, nl.cell_count, nl.dev_flags);
        if (int rc = scan(ctx, nl.cell_count, nl.ncells, nl.cell_start, nullptr, nl.dev_flags)) return rc;
        k_fill<<<nb, 256, 0, ctx->stream>>>(n, nl.particle_cell, nl.cell_start, nl.cell_fill, nl.cell_particles,
                                            nl.dev_flags);
        k_sort_cells<<<(nl.ncells + 255) / 256, 256, 0, ctx->stream>>>(nl.ncells, nl.cell_start, nl.cell_particles,
                                                                       nl.dev_flags);
        k_rows_cells<<<nb, 256, 0, ctx->stream>>>(n, ctx->pos, g, nl.cell_start, nl.cell_particles, nl.max_nb,
                                                  nl.nb_pad, nl.nb_count, nl.dev_flags);
    } else {
        k_begin<<<1, 32, 0, ctx->stream>>>(nl.dev_flags, nl.cell_count, nl.cell_fill, 0);
        k_rows_all<<<nb, 256, 0, ctx->stream>>>(n, ctx->pos, g, nl.max_nb, nl.nb_pad, nl.nb_count, nl.dev_flags);
    }
    if (int rc = scan(ctx, nl.nb_count, n, nl.row_off, nl.dev_flags + F_NPAIRS, nl.dev_flags)) return rc;
    k_compact<<<nb, 256, 0, ctx->stream>>>(n, nl.nb_pad, nl.nb_count, nl.row_off, nl.pair_i, nl.pair_j, nl.dev_flags);
    k_finish<<<nb, 256, 0, ctx->stream>>>(n, ctx->pos, nl.pos_last, nl.dev_flags);
    k_clear_request<<<1, 1, 0, ctx->stream>>>(nl.dev_flags);
    SG_LAUNCH_CHECK(ctx, "nlist build");
    return SG_OK;
}

// Synchronous build with automatic regrowth on overflow.
int build_sync(sg_ctx* ctx) {
    for (int attempt = 0; attempt < 8; ++attempt) {
        k_set_request<<<1, 1, 0, ctx->stream>>>(ctx->nl.dev_flags);
        if (int rc = enqueue_build(ctx)) return rc;
        int flags[4];
        SG_CUDA(ctx, cudaMemcpyAsync(flags, ctx->nl.dev_flags, sizeof(flags), cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (flags[F_OVERFLOW] == 0) return SG_OK;
        int want = ((flags[F_OVERFLOW] * 5 / 4) + 31) / 32 * 32;
        if (int rc = alloc_rows(ctx, want)) return rc;
    }
    return sg_fail(ctx, SG_ECAPACITY, "neighbour list did not fit after regrowth");
}

}  // namespace

int sg_nlist_free(sg_ctx* ctx) {
    sg_nlist_state& nl = ctx->nl;
    void* bufs[] = {nl.cell_count, nl.cell_start, nl.cell_fill, nl.cell_particles, nl.particle_cell, nl.nb_count,
                    nl.nb_pad, nl.row_off, nl.scan_tmp, nl.pair_i, nl.pair_j, nl.dev_flags, nl.pos_last};
    for (void* b : bufs)
        if (b) cudaFree(b);
    nl = sg_nlist_state();
    return SG_OK;
}

extern "C" {

int sg_nlist_init(sg_ctx* ctx, double skin, double cutoff, int32_t trigger_mode) {
    if (!ctx) return SG_EINVAL;
    if (!(skin >= 0.0) || !(cutoff > 0.0)) return sg_fail(ctx, SG_EINVAL, "skin must be >= 0 and cutoff > 0");
    if (ctx->box[0] <= 0.0) return sg_fail(ctx, SG_ENOTREADY, "sg_set_box must precede sg_nlist_init");
    for (int d = 0; d < 3; ++d)
        if (cutoff > ctx->box[d] / 2.0)
            return sg_fail(ctx, SG_ECUTOFF_GT_HALFBOX, "A cutoff of %.2f is too large for the box dimensions %.2f %.2f %.2f",
                           cutoff, ctx->box[0], ctx->box[1], ctx->box[2]);
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    sg_nlist_free(ctx);
    ctx->graph_epoch++;
    sg_nlist_state& nl = ctx->nl;
    const int n = ctx->n;
    nl.cutoff = cutoff;
    nl.skin = skin;
    nl.trigger_mode = trigger_mode;
    double rskin = cutoff + skin;
    nl.rl2 = rskin * rskin;
    nl.trigger_sq = trigger_mode == 0 ? nl.rl2 : skin * skin;
    nl.use_cells = ctx->periodic ? 1 : 0;
    for (int d = 0; d < 3; ++d) {
        nl.ncell[d] = (int)std::floor(ctx->box[d] / (rskin * (1.0 + 1e-4)));
        if (nl.ncell[d] < 3) nl.use_cells = 0;
    }
    if (!nl.use_cells) nl.ncell[0] = nl.ncell[1] = nl.ncell[2] = 1;
    nl.ncells = nl.ncell[0] * nl.ncell[1] * nl.ncell[2];
    double vol = ctx->box[0] * ctx->box[1] * ctx->box[2];
    double rho = n / vol;
    double expect = 0.5 * (4.0 / 3.0) * M_PI * rskin * rskin * rskin * rho;
    int max_nb = (int)std::ceil(expect * 1.6 + 32.0);
    max_nb = (max_nb + 31) / 32 * 32;
    if (max_nb > n) max_nb = std::max(1, n);
    int ntiles = std::max((n + SCAN_TILE - 1) / SCAN_TILE, (nl.ncells + SCAN_TILE - 1) / SCAN_TILE) + 2;
    SG_CUDA(ctx, cudaMalloc(&nl.cell_count, sizeof(int) * (size_t)nl.ncells));
    SG_CUDA(ctx, cudaMalloc(&nl.cell_start, sizeof(int) * ((size_t)nl.ncells + 1)));
    SG_CUDA(ctx, cudaMalloc(&nl.cell_fill, sizeof(int) * (size_t)nl.ncells));
    SG_CUDA(ctx, cudaMalloc(&nl.cell_particles, sizeof(int) * (size_t)n));
    SG_CUDA(ctx, cudaMalloc(&nl.particle_cell, sizeof(int) * (size_t)n));
    SG_CUDA(ctx, cudaMalloc(&nl.nb_count, sizeof(int) * (size_t)n));
    SG_CUDA(ctx, cudaMalloc(&nl.row_off, sizeof(int) * ((size_t)n + 1)));
    SG_CUDA(ctx, cudaMalloc(&nl.scan_tmp, sizeof(int) * (size_t)(ntiles + 1)));
    SG_CUDA(ctx, cudaMalloc(&nl.dev_flags, sizeof(int) * 8));
    SG_CUDA(ctx, cudaMalloc(&nl.pos_last, sizeof(float4) * (size_t)n));
    SG_CUDA(ctx, cudaMemsetAsync(nl.dev_flags, 0, sizeof(int) * 8, ctx->stream));
    if (int rc = alloc_rows(ctx, max_nb)) return rc;
    nl.initialized = 1;
    return build_sync(ctx);
}

int sg_nlist_build(sg_ctx* ctx) {
    if (!ctx) return SG_EINVAL;
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "sg_nlist_init must precede sg_nlist_build");
    return build_sync(ctx);
}

int sg_nlist_needs_rebuild(sg_ctx* ctx, int32_t* flag) {
    if (!ctx || !flag) return SG_EINVAL;
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "sg_nlist_init must precede sg_nlist_needs_rebuild");
    ListGeom g = make_geom(ctx);
    k_clear_request<<<1, 1, 0, ctx->stream>>>(ctx->nl.dev_flags);
    k_check<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->nl.pos_last, g, ctx->nl.trigger_sq,
                                                           ctx->nl.dev_flags);
    SG_LAUNCH_CHECK(ctx, "k_check");
    int f = 0;
    SG_CUDA(ctx, cudaMemcpyAsync(&f, ctx->nl.dev_flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    k_clear_request<<<1, 1, 0, ctx->stream>>>(ctx->nl.dev_flags);
    *flag = f;
    return SG_OK;
}

int sg_nlist_update(sg_ctx* ctx) {
    if (!ctx) return SG_EINVAL;
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "sg_nlist_init must precede sg_nlist_update");
    ListGeom g = make_geom(ctx);
    k_check<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->nl.pos_last, g, ctx->nl.trigger_sq,
                                                           ctx->nl.dev_flags);
    SG_LAUNCH_CHECK(ctx, "k_check");
    return enqueue_build(ctx);
}

int sg_nlist_count(sg_ctx* ctx, int64_t* npairs) {
    if (!ctx || !npairs) return SG_EINVAL;
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "no neighbour list");
    int flags[4];
    SG_CUDA(ctx, cudaMemcpyAsync(flags, ctx->nl.dev_flags, sizeof(flags), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (flags[F_OVERFLOW]) return sg_fail(ctx, SG_ECAPACITY, "neighbour list overflowed (row of %d)", flags[F_OVERFLOW]);
    *npairs = flags[F_NPAIRS];
    return SG_OK;
}

int sg_nlist_builds(sg_ctx* ctx, int64_t* builds) {
    if (!ctx || !builds) return SG_EINVAL;
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "no neighbour list");
    int flags[4];
    SG_CUDA(ctx, cudaMemcpyAsync(flags, ctx->nl.dev_flags, sizeof(flags), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *builds = flags[F_BUILDS];
    return SG_OK;
}

int sg_nlist_pairs(sg_ctx* ctx, int32_t* pi, int32_t* pj, int64_t capacity, int64_t* npairs) {
    if (!ctx || !npairs) return SG_EINVAL;
    int64_t k = 0;
    if (int rc = sg_nlist_count(ctx, &k)) return rc;
    *npairs = k;
    if (k > capacity || (k > 0 && (!pi || !pj))) return sg_fail(ctx, SG_ECAPACITY, "pair capacity too small");
    if (k > 0) {
        SG_CUDA(ctx, cudaMemcpyAsync(pi, ctx->nl.pair_i, sizeof(int) * k, cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(ctx, cudaMemcpyAsync(pj, ctx->nl.pair_j, sizeof(int) * k, cudaMemcpyDeviceToHost, ctx->stream));
    }
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_nlist_export(sg_ctx* ctx, int32_t* nlist, int64_t capacity, int32_t* offset, int64_t* npairs, int32_t one_based) {
    if (!ctx || !offset || !npairs) return SG_EINVAL;
    int64_t k = 0;
    if (int rc = sg_nlist_count(ctx, &k)) return rc;
    *npairs = k;
    if (k > capacity || (!nlist && k > 0)) return sg_fail(ctx, SG_ECAPACITY, "export capacity %lld < %lld pairs",
                                                          (long long)capacity, (long long)k);
    const int n = ctx->n;
    std::vector<int> off(n + 1), pj(k > 0 ? k : 1);
    SG_CUDA(ctx, cudaMemcpyAsync(off.data(), ctx->nl.row_off, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, ctx->stream));
    if (k > 0)
        SG_CUDA(ctx, cudaMemcpyAsync(pj.data(), ctx->nl.pair_j, sizeof(int) * k, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < n; ++i) std::sort(pj.begin() + off[i], pj.begin() + off[i + 1]);
    for (int64_t t = 0; t < k; ++t) nlist[t] = pj[t] + (one_based ? 1 : 0);
    if (one_based) {
        // offset(I) = start of row I, offset(N) = K+1 (system.f90:977,1000)
        for (int i = 0; i < n - 1; ++i) offset[i] = off[i] + 1;
        offset[n - 1] = (int)k + 1;
    } else {
        for (int i = 0; i <= n; ++i) offset[i] = off[i];
    }
    return SG_OK;
}

}  // extern "C"
