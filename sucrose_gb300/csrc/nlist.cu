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
// into nb_pad (a single system: row-major, i * max_nb + k, by the cooperative
// build; replica contexts: column-major k * n + i in each replica's section),
// then compacted into the flattened pair arrays pair_i / pair_j, rows in
// particle order, which every pair kernel walks 32 pairs per warp.
#include <algorithm>
#include <cmath>
#include <vector>

#include <cooperative_groups.h>

#include "sg_internal.cuh"
#include "step_epi.cuh"

namespace cg = cooperative_groups;

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
    float half_sq;    // (0.4998 min(box))^2, rounded down: a pair with a half-box component is at least this far
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

// FP32 filter, exact FP64 decision inside the guard band.
__device__ __forceinline__ bool accept_pair(float4 pi, float4 pj, const ListGeom& g) {
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    bool halfcase = false;
    if (g.periodic) {
        // a component within 2e-4 of half a box may round the other way in
        // FP64: such pairs take the exact test (the distance to the nearest
        // integer of d / L is read off the rounding the image needs anyway)
        const float tx = dx * g.inv_box.x, ty = dy * g.inv_box.y, tz = dz * g.inv_box.z;
        const float nx = roundf(tx), ny = roundf(ty), nz = roundf(tz);
        halfcase = fabsf(tx - nx) > 0.4998f || fabsf(ty - ny) > 0.4998f || fabsf(tz - nz) > 0.4998f;
        dx -= nx * g.box.x;
        dy -= ny * g.box.y;
        dz -= nz * g.box.z;
    }
    float r2 = dx * dx + dy * dy + dz * dz;
    if (!halfcase) {
        if (r2 < g.rl2_lo) return true;
        if (r2 > g.rl2_hi) return false;
    } else if (g.half_sq > g.rl2_hi) {
        return false;   // beyond the list radius whichever image FP64 picks
    }
    return ref_accept(pi, pj, g);
}

// Relative half-width of the r^2 band where the FP32 test defers to the FP64
// one. The FP32 r^2 of the same FP32 positions is within ~(1.1e-6 L / r_list
// + 3e-7) of the FP64 value (the FP32 box in the image shift dominates), so
// the band is 1e-4, widened for boxes over ~25 list radii.
__host__ __device__ inline double guard_band(double box_max, double rl2) {
    return fmax(1e-4, 4e-6 * box_max / sqrt(rl2));
}

// Geometry of replica r (batched contexts): its box, list radius and grid.
__device__ __forceinline__ ListGeom geom_for(const ListGeom& base, const RepDev& rp, int r) {
    ListGeom g = base;
    const float4 b = rp.box[r], ib = rp.inv_box[r];
    g.box = make_float3(b.x, b.y, b.z);
    g.inv_box = make_float3(ib.x, ib.y, ib.z);
    g.bx = rp.boxd[3 * r];
    g.by = rp.boxd[3 * r + 1];
    g.bz = rp.boxd[3 * r + 2];
    g.rl2 = rp.rl2[r];
    const double band = guard_band(fmax(g.bx, fmax(g.by, g.bz)), g.rl2);
    g.rl2_lo = (float)(g.rl2 * (1.0 - band));
    g.rl2_hi = (float)(g.rl2 * (1.0 + band));
    g.half_sq = rp.half_sq[r];
    const int4 gr = rp.grid[r];
    g.nc[0] = max(gr.x, 1);
    g.nc[1] = max(gr.y, 1);
    g.nc[2] = max(gr.z, 1);
    return g;
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
// particles exceeds the bound iff some particle does). The test itself is
// check_displacement (step_epi.cuh), which the captured step also runs inside
// its initial half step.
__global__ void k_check(int n, const float4* __restrict__ pos, CheckArgs c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    check_displacement(i, pos[i], c);
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

__global__ void k_bin(int n, const float4* __restrict__ pos, ListGeom g0, int* particle_cell, int* cell_count,
                      const int* flags, RepDev rp) {
    if (!flags[F_REBUILD]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int cx, cy, cz;
    int c;
    if (rp.rep_of) {
        const int r = rp.rep_of[i];
        const int4 gr = rp.grid[r];
        if (!gr.x) {
            // a replica under three cells per side is searched all-pairs, not binned
            particle_cell[i] = -1;
            return;
        }
        const ListGeom g = geom_for(g0, rp, r);
        c = gr.w + cell_of(pos[i], g, cx, cy, cz);
    } else {
        c = cell_of(pos[i], g0, cx, cy, cz);
    }
    particle_cell[i] = c;
    atomicAdd(&cell_count[c], 1);
}

// Cell members in arrival order (atomic slots) into the scratch array.
__global__ void k_fill(int n, const int* __restrict__ particle_cell, const int* __restrict__ cell_start, int* cell_fill,
                       int* cell_unsorted, const int* flags) {
    if (!flags[F_REBUILD]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c = particle_cell[i];
    if (c < 0) return;
    int s = atomicAdd(&cell_fill[c], 1);
    cell_unsorted[cell_start[c] + s] = i;
}

// Order each cell's particles by index so that rows are deterministic: one
// warp per cell, each member placed at its rank (the number of smaller
// indices in the cell; indices are distinct).
// pos_cell (optional): the members' positions in the same order, so that the
// row search reads a cell's candidates with contiguous loads.
__global__ void k_sort_cells(int ncells, const int* __restrict__ cell_start, const int* __restrict__ cell_unsorted,
                             int* cell_particles, const int* flags, const float4* __restrict__ pos,
                             float4* __restrict__ pos_cell) {
    if (!flags[F_REBUILD]) return;
    const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= ncells) return;
    const int b = cell_start[c], e = cell_start[c + 1];
    for (int k = b + lane; k < e; k += 32) {
        const int v = cell_unsorted[k];
        int rank = 0;
        for (int t = b; t < e; ++t) rank += cell_unsorted[t] < v;
        cell_particles[b + rank] = v;
        if (pos_cell) pos_cell[b + rank] = pos[v];
    }
}

// Padded-row addressing: slot k of particle i's row is nb_pad[base + k * stride].
struct PadRep {
    const int* max_nb;          // [R] row capacity of each replica
    const long long* pad_off;   // [R] first slot of each replica's section
    int* need;                  // [R] longest row seen on overflow
};

__device__ __forceinline__ void pad_slot(int n, int i, int max_nb, const RepDev& rp, const PadRep& pr, size_t& base,
                                         size_t& stride, int& cap) {
    if (rp.rep_of) {
        const int r = rp.rep_of[i];
        const int o = rp.off[r];
        base = (size_t)pr.pad_off[r] + (size_t)(i - o);
        stride = (size_t)(rp.off[r + 1] - o);
        cap = pr.max_nb[r];
    } else {
        base = (size_t)i;
        stride = (size_t)n;
        cap = max_nb;
    }
}

__device__ __forceinline__ void row_done(int i, int cnt, int cap, int* nb_count, int* flags, const RepDev& rp,
                                         const PadRep& pr) {
    nb_count[i] = min(cnt, cap);
    if (cnt > cap) {
        atomicMax(&flags[F_OVERFLOW], cnt);
        if (rp.rep_of) atomicMax(&pr.need[rp.rep_of[i]], cnt);
    }
}

// Rows of a replica context, a thread per row over the replica's 27 cells
// (or every later particle of a replica under three cells per side).
// block_order: the 256-row block each CTA takes, the blocks with the longest
// rows first, so that no long block starts late and leaves the other SMs idle
// at the end (rows and their contents unchanged)
__global__ void k_rows_cells(int n, const float4* __restrict__ pos, ListGeom g0, const int* __restrict__ cell_start,
                             const int* __restrict__ cell_particles, int max_nb, int* nb_pad, int* nb_count,
                             int* flags, RepDev rp, PadRep pr, const int* rep_flag,
                             const int* __restrict__ block_order) {
    if (!flags[F_REBUILD]) return;
    const int bx = block_order ? block_order[blockIdx.x] : (int)blockIdx.x;
    const int t = bx * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int i = t;
    if (rp.rep_of && !rep_flag[rp.rep_of[i]]) return;   // this replica keeps its rows
    const float4 pi = pos[i];
    ListGeom g = g0;
    int first_cell = 0;
    int cnt = 0;
    size_t base, stride;
    int cap;
    pad_slot(n, i, max_nb, rp, pr, base, stride, cap);
    if (rp.rep_of) {
        const int r = rp.rep_of[i];
        const int4 gr = rp.grid[r];
        g = geom_for(g0, rp, r);
        first_cell = gr.w;
        if (!gr.x) {
            // box under three cells per side: every later particle of the replica
            const int e = rp.off[r + 1];
            for (int j = i + 1; j < e; ++j) {
                if (accept_pair(pi, pos[j], g)) {
                    if (cnt < cap) nb_pad[base + (size_t)cnt * stride] = j;
                    ++cnt;
                }
            }
            row_done(i, cnt, cap, nb_count, flags, rp, pr);
            return;
        }
    }
    int cx, cy, cz;
    cell_of(pi, g, cx, cy, cz);
    for (int dz = -1; dz <= 1; ++dz) {
        int zz = wrapc(cz + dz, g.nc[2]);
        for (int dy = -1; dy <= 1; ++dy) {
            int yy = wrapc(cy + dy, g.nc[1]);
            for (int dx = -1; dx <= 1; ++dx) {
                int xx = wrapc(cx + dx, g.nc[0]);
                int c = first_cell + (zz * g.nc[1] + yy) * g.nc[0] + xx;
                int b = cell_start[c], e = cell_start[c + 1];
                for (int k = b; k < e; ++k) {
                    int j = cell_particles[k];
                    if (j <= i) continue;
                    if (accept_pair(pi, pos[j], g)) {
                        if (cnt < cap) nb_pad[base + (size_t)cnt * stride] = j;
                        ++cnt;
                    }
                }
            }
        }
    }
    row_done(i, cnt, cap, nb_count, flags, rp, pr);
}

// The same rows for one system, G lanes per row (G = 8, 16 or 32; 32 / G rows
// per warp, rows taken in cell order). The three x cells of each (dz, dy) row
// of the 27-cell stencil are consecutive in cell order, so their members are
// one contiguous range of cell_particles (two when the stencil wraps in x,
// listed in the thread-per-row kernel's dx order): nine ranges instead of 27
// cells, tested G members at a time; the accepted ones are appended in member
// order (a ballot over the row's lanes, then each accepting lane's rank), so
// each row holds exactly what the thread-per-particle kernel writes. A chunk
// whose members all have indices <= i is passed over (members are sorted).
// Rows are written row-major (i * max_nb). Launched with G = 32 for dense
// cells (row_lanes_for).
// One row of the x-range search by the G lanes of a group (sub: the lane in
// the group, g0 its first lane, gmask the group's lanes). Row w of the cell
// order, written row-major.
template <int G>
__device__ __forceinline__ void xrange_row(int w, int sub, int g0, unsigned gmask, const ListGeom& g,
                                           const int* cell_start, const int* cell_particles, const float4* pos_cell,
                                           int max_nb, int* nb_pad, int* nb_count, int* flags) {
    const int nx = g.nc[0];
    const int i = cell_particles[w];
    const float4 pi = pos_cell[w];
    const size_t base = (size_t)i * max_nb;
    int cnt = 0;
    int cx, cy, cz;
    cell_of(pi, g, cx, cy, cz);
    for (int dz = -1; dz <= 1; ++dz) {
        const int zz = wrapc(cz + dz, g.nc[2]);
        for (int dy = -1; dy <= 1; ++dy) {
            const int row = (zz * g.nc[1] + wrapc(cy + dy, g.nc[1])) * nx;
            // x cells cx-1 .. cx+1 as ranges of consecutive cells, in dx order
            int lo0 = cx - 1, hi0 = cx + 1, lo1 = 0, hi1 = -1;
            if (cx == 0) { lo0 = nx - 1; hi0 = nx - 1; lo1 = 0; hi1 = 1; }
            else if (cx == nx - 1) { hi0 = nx - 1; lo1 = 0; hi1 = 0; }
            for (int sgm = 0; sgm < 2; ++sgm) {
                const int clo = sgm ? lo1 : lo0, chi = sgm ? hi1 : hi0;
                if (chi < clo) continue;
                const int b = cell_start[row + clo], e = cell_start[row + chi + 1];
                for (int k0 = b; k0 < e; k0 += G) {
                    const int k = k0 + sub;
                    const int j = k < e ? cell_particles[k] : -1;
                    if (!__any_sync(gmask, j > i)) continue;
                    const bool acc = j > i && accept_pair(pi, pos_cell[k], g);
                    const unsigned m = __ballot_sync(gmask, acc) >> g0;
                    if (acc) {
                        const int slot = cnt + __popc(m & ((1u << sub) - 1u));
                        if (slot < max_nb) nb_pad[base + slot] = j;
                    }
                    cnt += __popc(m);
                }
            }
        }
    }
    if (sub == 0) {
        nb_count[i] = min(cnt, max_nb);
        if (cnt > max_nb) atomicMax(&flags[F_OVERFLOW], cnt);
    }
}

// One row of a single system by one thread: row t of the cell order over the
// stencil's nine x ranges (as xrange_row, the same order as a walk over the 27
// cells; cell-ordered candidates, contiguous loads), written row-major.
__device__ __forceinline__ void cells_row(int t, const ListGeom& g, const int* cell_start, const int* cell_particles,
                                          const float4* pos_cell, int max_nb, int* nb_pad, int* nb_count,
                                          int* flags) {
    const int nx = g.nc[0];
    const int i = cell_particles[t];
    const float4 pi = pos_cell[t];
    const size_t base = (size_t)i * max_nb;
    int cnt = 0;
    int cx, cy, cz;
    cell_of(pi, g, cx, cy, cz);
    int lo0 = cx - 1, hi0 = cx + 1, lo1 = 0, hi1 = -1;
    if (cx == 0) { lo0 = nx - 1; hi0 = nx - 1; lo1 = 0; hi1 = 1; }
    else if (cx == nx - 1) { hi0 = nx - 1; lo1 = 0; hi1 = 0; }
    for (int dz = -1; dz <= 1; ++dz) {
        const int zz = wrapc(cz + dz, g.nc[2]);
        for (int dy = -1; dy <= 1; ++dy) {
            const int row = (zz * g.nc[1] + wrapc(cy + dy, g.nc[1])) * nx;
            for (int sgm = 0; sgm < 2; ++sgm) {
                const int clo = sgm ? lo1 : lo0, chi = sgm ? hi1 : hi0;
                if (chi < clo) continue;
                const int b = cell_start[row + clo], e = cell_start[row + chi + 1];
                for (int k = b; k < e; ++k) {
                    const int j = cell_particles[k];
                    if (j <= i) continue;
                    if (accept_pair(pi, pos_cell[k], g)) {
                        if (cnt < max_nb) nb_pad[base + cnt] = j;
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

// Replica of the first pair of every 32-pair chunk of the row order: the
// largest r with row_off[off[r]] <= 32 c (pair kernels start their search there).
// With s_r = row_off[off[r]] the first pair of replica r, the chunks c with
// s_r <= 32 c < s_(r+1) are replica r's: c in [ceil(s_r / 32), ceil(s_(r+1) / 32)).
// A warp per replica writes its range (a replica without pairs has none, and
// its chunk goes to the next replica with pairs, the largest r as required).
__global__ void k_chunk_rep(const int* __restrict__ row_off, const int* __restrict__ rep_off, int R,
                            const int* flags, int* chunk_rep) {
    if (!flags[F_REBUILD]) return;
    const int lane = threadIdx.x & 31;
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int r = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); r < R; r += nwarps) {
        const int c0 = (row_off[rep_off[r]] + 31) >> 5;
        const int c1 = (row_off[rep_off[r + 1]] + 31) >> 5;   // rep_off[R] = n: the total
        for (int c = c0 + lane; c < c1; c += 32) chunk_rep[c] = r;
    }
}

// Rows into the flat pair arrays. A single system stores them in row order
// (pair index = row_off[i] + k). A replica context stores each replica's rows
// in the replica's own section (it starts where the replica's padded rows
// start), so only replicas that rebuilt are rewritten: the pair at row-order
// index v of replica r sits at pad_off[r] + v - row_off[off[r]].
// A warp takes 32 consecutive rows and moves them 32 columns at a time
// through shared memory: slot k of the 32 rows is one coalesced read of the
// column-major padded rows, and each row's 32 entries one coalesced write of
// the flat arrays.
constexpr int COMPACT_BLOCK = 256;
__global__ void __launch_bounds__(COMPACT_BLOCK) k_compact(int n, int max_nb, const int* __restrict__ nb_pad,
                                                           const int* __restrict__ nb_count,
                                                           const int* __restrict__ row_off, int* pair_i, int* pair_j,
                                                           const int* flags, RepDev rp, PadRep pr,
                                                           const int* rep_flag) {
    if (!flags[F_REBUILD]) return;
    __shared__ int tile[COMPACT_BLOCK / 32][32][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool on = i < n;
    size_t base = 0, stride = 0, o = 0;
    int c = 0;
    if (on) {
        int cap;
        pad_slot(n, i, max_nb, rp, pr, base, stride, cap);
        o = (size_t)row_off[i];
        if (rp.rep_of) {
            const int r = rp.rep_of[i];
            on = rep_flag[r] != 0;
            o = (size_t)pr.pad_off[r] + (size_t)(row_off[i] - row_off[rp.off[r]]);
        }
        c = on ? nb_count[i] : 0;
    }
    int cmax = c;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) cmax = max(cmax, __shfl_xor_sync(0xffffffffu, cmax, s));
    int (*t)[33] = tile[w];
    for (int k0 = 0; k0 < cmax; k0 += 32) {
        // read: lane = row, slots k0 .. k0 + 31
        for (int kk = 0; kk < 32; ++kk)
            if (k0 + kk < c) t[kk][lane] = nb_pad[base + (size_t)(k0 + kk) * stride];
        __syncwarp();
        // write: row by row, lane = slot
        for (int rr = 0; rr < 32; ++rr) {
            const int cr = __shfl_sync(0xffffffffu, c, rr);
            const unsigned long long orr = __shfl_sync(0xffffffffu, (unsigned long long)o, rr);
            const int k = k0 + lane;
            if (k < cr) {
                pair_i[orr + k] = blockIdx.x * blockDim.x + (w << 5) + rr;
                pair_j[orr + k] = t[lane][rr];
            }
        }
        __syncwarp();
    }
}

__global__ void k_finish(int n, const float4* __restrict__ pos, float4* last, int* flags, const int* rep_of,
                         const int* rep_flag) {
    if (!flags[F_REBUILD]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && (!rep_of || rep_flag[rep_of[i]])) last[i] = pos[i];
    __syncthreads();
    // the last block clears the request; blocks only read the flag at entry
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        flags[F_BUILDS] += 1;
    }
}

// Request flags: the global one and, in a replica context, one per replica.
// After a build (rep_builds given) each replica that rebuilt is counted.
__global__ void k_clear_request(int* flags, int* rep_flag, int R, int* rep_builds) {
    if (blockIdx.x == 0 && threadIdx.x == 0) flags[F_REBUILD] = 0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x) {
        if (rep_builds && rep_flag[r]) rep_builds[r] += 1;
        rep_flag[r] = 0;
    }
}
__global__ void k_set_request(int* flags, int* rep_flag, int R) {
    if (blockIdx.x == 0 && threadIdx.x == 0) flags[F_REBUILD] = 1;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < R; r += gridDim.x * blockDim.x) rep_flag[r] = 1;
}

// ------------------------------------------------ single-system rebuild --
// The whole rebuild of a single system with cells in one cooperative kernel:
// its phases (bin, scan of the cell counts, fill, sort, row search, scan of
// the row lengths, compaction, finish) are separated by grid-wide barriers
// instead of kernel boundaries. A step without a rebuild then runs one
// launch that exits at its first instruction, where the captured step would
// otherwise evaluate a graph conditional node or a dozen flag-gated
// kernels. Arrays written in one phase and read in a later one are read with
// plain (coherent) loads, never through the read-only path.
struct CoopBuild {
    int n, ncells, ncells_cap, max_nb, row_lanes;
    const float4* pos;
    ListGeom g;
    int* cell_count;
    int* cell_fill;
    int* cell_start;
    int* cell_unsorted;
    int* cell_particles;
    int* particle_cell;
    float4* pos_cell;
    int* nb_pad;
    int* nb_count;
    int* row_off;
    int* pair_i;
    int* pair_j;
    float4* last;
    int* flags;
    int* tmp;   // gridDim.x block totals of the scans
};

// Exclusive scan of in[0, m) into out[0, m] (out[m] = total, also *total_dst)
// by the whole grid: each block scans a contiguous tile, the tiles' totals
// give each block its offset after a grid barrier.
__device__ __forceinline__ void coop_scan(cg::grid_group& grid, const int* in, int m, int* out, int* total_dst, int* tmp) {
    __shared__ int sh[32];
    __shared__ int sh_off;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int T = (m + (int)gridDim.x - 1) / (int)gridDim.x;
    const int lo = min(m, (int)blockIdx.x * T), hi = min(m, lo + T);
    const int per = (T + (int)blockDim.x - 1) / (int)blockDim.x;
    const int tlo = min(hi, lo + (int)threadIdx.x * per), thi = min(hi, tlo + per);
    int s = 0;
    for (int k = tlo; k < thi; ++k) s += in[k];
    int x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int v = lane < nw ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane < nw) sh[lane] = v;
    }
    __syncthreads();
    const int excl = x - s + (w ? sh[w - 1] : 0);
    const int btot = sh[nw - 1];
    if (threadIdx.x == 0) tmp[blockIdx.x] = btot;
    grid.sync();
    int o = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += blockDim.x) o += __ldcg(tmp + b);   // L2: rewritten per scan
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) o += __shfl_xor_sync(0xffffffffu, o, d);
    __syncthreads();
    if (lane == 0) sh[w] = o;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < nw; ++k) t += sh[k];
        sh_off = t;
    }
    __syncthreads();
    int run = sh_off + excl;
    for (int k = tlo; k < thi; ++k) {
        const int v = in[k];
        out[k] = run;
        run += v;
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        const int tot = sh_off + btot;
        out[m] = tot;
        if (total_dst) *total_dst = tot;
    }
    __syncthreads();   // sh is reused by the next scan
}

__global__ void __launch_bounds__(256, 4) k_build_coop(CoopBuild a) {
    if (!a.flags[F_REBUILD]) return;   // grid-uniform: cleared only after the last barrier
    cg::grid_group grid = cg::this_grid();
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int gw = gt >> 5, nwarps = gs >> 5;
    // bin (cell_count is zero: the previous build cleared it after its scan)
    for (int c = gt; c < a.ncells; c += gs) a.cell_fill[c] = 0;
    if (gt == 0) a.flags[F_OVERFLOW] = 0;
    for (int i = gt; i < a.n; i += gs) {
        int cx, cy, cz;
        const int c = cell_of(a.pos[i], a.g, cx, cy, cz);
        a.particle_cell[i] = c;
        atomicAdd(&a.cell_count[c], 1);
    }
    grid.sync();
    coop_scan(grid, a.cell_count, a.ncells, a.cell_start, nullptr, a.tmp);
    grid.sync();
    // members in arrival order; the counts are cleared for the next build
    for (int i = gt; i < a.n; i += gs) {
        const int c = a.particle_cell[i];
        a.cell_unsorted[a.cell_start[c] + atomicAdd(&a.cell_fill[c], 1)] = i;
    }
    for (int c = gt; c < a.ncells_cap; c += gs) a.cell_count[c] = 0;
    grid.sync();
    // each cell's members by index (a warp per cell, each member at its rank),
    // their positions in the same order
    for (int c = gw; c < a.ncells; c += nwarps) {
        const int b = a.cell_start[c], e = a.cell_start[c + 1];
        for (int k = b + lane; k < e; k += 32) {
            const int v = a.cell_unsorted[k];
            int rank = 0;
            for (int t = b; t < e; ++t) rank += a.cell_unsorted[t] < v;
            a.cell_particles[b + rank] = v;
            a.pos_cell[b + rank] = a.pos[v];
        }
    }
    grid.sync();
    // rows, in cell order: a warp per row (dense cells) or a thread per row
    if (a.row_lanes == 32) {
        for (int w = gw; w < a.n; w += nwarps)
            xrange_row<32>(w, lane, 0, 0xffffffffu, a.g, a.cell_start, a.cell_particles, a.pos_cell, a.max_nb, a.nb_pad,
                           a.nb_count, a.flags);
    } else {
        for (int t = gt; t < a.n; t += gs)
            cells_row(t, a.g, a.cell_start, a.cell_particles, a.pos_cell, a.max_nb, a.nb_pad, a.nb_count, a.flags);
    }
    grid.sync();
    coop_scan(grid, a.nb_count, a.n, a.row_off, a.flags + F_NPAIRS, a.tmp);
    grid.sync();
    // rows into the flat pair arrays, contiguous on both sides: a warp per
    // row for dense cells, 8 lanes per row for sparse ones (rows of ~8)
    {
        const int G = a.row_lanes == 32 ? 32 : 8;
        const int sub = lane & (G - 1);
        const int ng = gs / G;
        for (int i = gt / G; i < a.n; i += ng) {
            const int c = a.nb_count[i], o = a.row_off[i];
            for (int k = sub; k < c; k += G) {
                a.pair_i[o + k] = i;
                a.pair_j[o + k] = a.nb_pad[(size_t)i * a.max_nb + k];
            }
        }
    }
    for (int i = gt; i < a.n; i += gs) a.last[i] = a.pos[i];
    if (gt == 0) {
        a.flags[F_BUILDS] += 1;
        a.flags[F_REBUILD] = 0;   // every block read it at entry, before the first barrier
    }
}

int clear_grid(const sg_ctx* ctx) { return std::max(1, std::min(64, (ctx->nrep + 255) / 256)); }

// (0.4998 min(box))^2 with a margin, as a float that never exceeds the true value
float half_sq_of(const double* b) {
    const double h = 0.4998 * std::min(b[0], std::min(b[1], b[2]));
    return (float)(h * h * (1.0 - 1e-5));
}

ListGeom make_geom(const sg_ctx* ctx) {
    ListGeom g;
    g.box = make_float3((float)ctx->box[0], (float)ctx->box[1], (float)ctx->box[2]);
    g.inv_box = make_float3((float)(1.0 / ctx->box[0]), (float)(1.0 / ctx->box[1]), (float)(1.0 / ctx->box[2]));
    g.bx = ctx->box[0]; g.by = ctx->box[1]; g.bz = ctx->box[2];
    g.rl2 = ctx->nl.rl2;
    const double band = guard_band(std::max(ctx->box[0], std::max(ctx->box[1], ctx->box[2])), ctx->nl.rl2);
    g.rl2_lo = (float)(ctx->nl.rl2 * (1.0 - band));
    g.rl2_hi = (float)(ctx->nl.rl2 * (1.0 + band));
    g.half_sq = half_sq_of(ctx->box);
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
    if (nl.chunk_rep) cudaFree(nl.chunk_rep);
    nl.nb_pad = nl.pair_i = nl.pair_j = nl.chunk_rep = nullptr;
    ctx->graph_epoch++;
    nl.max_nb = max_nb;
    nl.pair_capacity = (int64_t)max_nb * ctx->n;
    if (ctx->nrep) {
        // each replica's rows in a section of their own, sized by its own capacity
        const int R = ctx->nrep;
        std::vector<long long> pad(R);
        long long total = 0;
        for (int r = 0; r < R; ++r) {
            pad[r] = total;
            total += (long long)nl.h_rep_max_nb[r] * (ctx->h_rep_off[r + 1] - ctx->h_rep_off[r]);
        }
        nl.pair_capacity = total;
        nl.h_rep_pad_off = pad;
        nl.max_nb = *std::max_element(nl.h_rep_max_nb.begin(), nl.h_rep_max_nb.end());
        if (total <= (long long)INT32_MAX) {
            SG_CUDA(ctx, cudaMemcpy(nl.rep_max_nb, nl.h_rep_max_nb.data(), sizeof(int) * R, cudaMemcpyHostToDevice));
            SG_CUDA(ctx, cudaMemcpy(nl.rep_pad_off, pad.data(), sizeof(long long) * R, cudaMemcpyHostToDevice));
            SG_CUDA(ctx, cudaMemset(nl.rep_need, 0, sizeof(int) * R));
        }
    }
    if (nl.pair_capacity > (int64_t)INT32_MAX)
        return sg_fail(ctx, SG_ECAPACITY, "neighbour list capacity %lld exceeds 2^31", (long long)nl.pair_capacity);
    SG_CUDA(ctx, cudaMalloc(&nl.nb_pad, sizeof(int) * (size_t)nl.pair_capacity));
    SG_CUDA(ctx, cudaMalloc(&nl.pair_i, sizeof(int) * (size_t)nl.pair_capacity));
    SG_CUDA(ctx, cudaMalloc(&nl.pair_j, sizeof(int) * (size_t)nl.pair_capacity));
    if (ctx->nrep) SG_CUDA(ctx, cudaMalloc(&nl.chunk_rep, sizeof(int) * (size_t)(nl.pair_capacity / 32 + 2)));
    return SG_OK;
}

// Grid of the cooperative build (every block resident at once) and its
// scratch, sized once per context.
int coop_setup(sg_ctx* ctx) {
    sg_nlist_state& nl = ctx->nl;
    if (nl.coop_grid) return SG_OK;
    int per_sm = 0;
    SG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_build_coop, 256, 0));
    if (per_sm < 1) return sg_fail(ctx, SG_ECUDA, "the cooperative list build does not fit an SM");
    const int grid = per_sm * ctx->num_sms;
    SG_CUDA(ctx, cudaMalloc(&nl.coop_tmp, sizeof(int) * (size_t)(grid + 1)));
    nl.coop_grid = grid;
    ctx->graph_epoch++;
    return SG_OK;
}

// Lanes per row of a single system's search: 32 (xrange_row) when the
// stencil's x ranges hold 24 members or more on average (8 per cell); sparser
// cells, a thread per row (cells_row over cell-ordered positions; measured
// on the ECP list, 4.2 per cell: 72 us against 91 us for 16 lanes per row).
int row_lanes_for(int use_cells, int n, int ncells) {
    if (!use_cells) return 0;
    return 3.0 * n / std::max(ncells, 1) >= 24.0 ? 32 : 0;
}

// Enqueue the (flag-gated) build kernels.
int enqueue_build(sg_ctx* ctx) {
    sg_nlist_state& nl = ctx->nl;
    const int n = ctx->n;
    ListGeom g = make_geom(ctx);
    const int nb = (n + 255) / 256;
    const PadRep pad{nl.rep_max_nb, nl.rep_pad_off, nl.rep_need};
    if (nl.use_cells && !ctx->nrep) {
        // a single system: the cooperative kernel (rows row-major)
        if (int rc = coop_setup(ctx)) return rc;
        CoopBuild a;
        a.n = n;
        a.ncells = nl.ncells;
        a.ncells_cap = nl.ncells_cap;
        a.max_nb = nl.max_nb;
        a.row_lanes = nl.row_lanes;
        a.pos = ctx->pos;
        a.g = g;
        a.cell_count = nl.cell_count;
        a.cell_fill = nl.cell_fill;
        a.cell_start = nl.cell_start;
        a.cell_unsorted = nl.cell_unsorted;
        a.cell_particles = nl.cell_particles;
        a.particle_cell = nl.particle_cell;
        a.pos_cell = nl.pos_cell;
        a.nb_pad = nl.nb_pad;
        a.nb_count = nl.nb_count;
        a.row_off = nl.row_off;
        a.pair_i = nl.pair_i;
        a.pair_j = nl.pair_j;
        a.last = nl.pos_last;
        a.flags = nl.dev_flags;
        a.tmp = nl.coop_tmp;
        void* args[] = {&a};
        // as many blocks as the row search has rows (a thread per row, or a
        // warp per row for dense cells), up to what is resident at once:
        // blocks without rows would wait at each barrier while the search runs
        const int64_t row_threads = (int64_t)n * (nl.row_lanes ? nl.row_lanes : 1);
        const int grid = (int)std::min<int64_t>(nl.coop_grid, std::max<int64_t>(ctx->num_sms, (row_threads + 255) / 256));
        SG_CUDA(ctx, cudaLaunchCooperativeKernel((const void*)k_build_coop, grid, 256, args, 0, ctx->stream));
        return SG_OK;
    }
    if (nl.use_cells) {
        // replica contexts: flag-gated kernels, a thread per row
        k_begin<<<std::max(1, std::min(1024, (nl.ncells + 255) / 256)), 256, 0, ctx->stream>>>(nl.dev_flags, nl.cell_count,
                                                                                                nl.cell_fill, nl.ncells);
        k_bin<<<nb, 256, 0, ctx->stream>>>(n, ctx->pos, g, nl.particle_cell, nl.cell_count, nl.dev_flags, ctx->rep);
        if (int rc = scan(ctx, nl.cell_count, nl.ncells, nl.cell_start, nullptr, nl.dev_flags)) return rc;
        k_fill<<<nb, 256, 0, ctx->stream>>>(n, nl.particle_cell, nl.cell_start, nl.cell_fill, nl.cell_unsorted,
                                            nl.dev_flags);
        k_sort_cells<<<(nl.ncells + 7) / 8, 256, 0, ctx->stream>>>(nl.ncells, nl.cell_start, nl.cell_unsorted,
                                                                    nl.cell_particles, nl.dev_flags, ctx->pos,
                                                                    nullptr);
        k_rows_cells<<<nb, 256, 0, ctx->stream>>>(n, ctx->pos, g, nl.cell_start, nl.cell_particles, nl.max_nb,
                                                  nl.nb_pad, nl.nb_count, nl.dev_flags, ctx->rep, pad, nl.rep_flag,
                                                  nl.row_block_order);
    } else {
        k_begin<<<1, 32, 0, ctx->stream>>>(nl.dev_flags, nl.cell_count, nl.cell_fill, 0);
        k_rows_all<<<nb, 256, 0, ctx->stream>>>(n, ctx->pos, g, nl.max_nb, nl.nb_pad, nl.nb_count, nl.dev_flags);
    }
    if (int rc = scan(ctx, nl.nb_count, n, nl.row_off, nl.dev_flags + F_NPAIRS, nl.dev_flags)) return rc;
    k_compact<<<(n + COMPACT_BLOCK - 1) / COMPACT_BLOCK, COMPACT_BLOCK, 0, ctx->stream>>>(
            n, nl.max_nb, nl.nb_pad, nl.nb_count, nl.row_off, nl.pair_i, nl.pair_j, nl.dev_flags, ctx->rep, pad,
            nl.rep_flag);
    if (ctx->nrep)
        k_chunk_rep<<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(nl.row_off, ctx->rep.off, ctx->nrep, nl.dev_flags,
                                                              nl.chunk_rep);
    k_finish<<<nb, 256, 0, ctx->stream>>>(n, ctx->pos, nl.pos_last, nl.dev_flags, ctx->rep.rep_of, nl.rep_flag);
    k_clear_request<<<clear_grid(ctx), 256, 0, ctx->stream>>>(nl.dev_flags, nl.rep_flag, ctx->nrep, nl.rep_builds);
    SG_LAUNCH_CHECK(ctx, "nlist build");
    return SG_OK;
}

// Synchronous build with automatic regrowth on overflow.
int build_sync(sg_ctx* ctx) {
    for (int attempt = 0; attempt < 8; ++attempt) {
        k_set_request<<<clear_grid(ctx), 256, 0, ctx->stream>>>(ctx->nl.dev_flags, ctx->nl.rep_flag, ctx->nrep);
        if (int rc = enqueue_build(ctx)) return rc;
        int flags[4];
        SG_CUDA(ctx, cudaMemcpyAsync(flags, ctx->nl.dev_flags, sizeof(flags), cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (flags[F_OVERFLOW] == 0) return SG_OK;
        int want = ((flags[F_OVERFLOW] * 5 / 4) + 31) / 32 * 32;
        if (ctx->nrep) {
            // grow only the replicas whose rows overflowed
            const int R = ctx->nrep;
            std::vector<int> need(R);
            SG_CUDA(ctx, cudaMemcpy(need.data(), ctx->nl.rep_need, sizeof(int) * R, cudaMemcpyDeviceToHost));
            for (int r = 0; r < R; ++r)
                if (need[r] > ctx->nl.h_rep_max_nb[r])
                    ctx->nl.h_rep_max_nb[r] = std::min(((need[r] * 5 / 4) + 31) / 32 * 32,
                                                       ctx->h_rep_off[r + 1] - ctx->h_rep_off[r]);
        }
        if (int rc = alloc_rows(ctx, want)) return rc;
    }
    return sg_fail(ctx, SG_ECAPACITY, "neighbour list did not fit after regrowth");
}

}  // namespace

int sg_nlist_enqueue_check(sg_ctx* ctx) {
    k_check<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, check_args(ctx));
    SG_LAUNCH_CHECK(ctx, "k_check");
    return SG_OK;
}

int sg_nlist_enqueue_build(sg_ctx* ctx) { return enqueue_build(ctx); }

int sg_nlist_free(sg_ctx* ctx) {
    sg_nlist_state& nl = ctx->nl;
    void* bufs[] = {nl.cell_count, nl.cell_start, nl.cell_fill, nl.cell_particles, nl.particle_cell, nl.nb_count,
                    nl.nb_pad, nl.row_off, nl.scan_tmp, nl.pair_i, nl.pair_j, nl.dev_flags, nl.pos_last, nl.pos_cell,
                    nl.rep_max_nb, nl.rep_pad_off, nl.rep_need, nl.rep_flag, nl.rep_builds, nl.cell_unsorted,
                    nl.chunk_rep, nl.row_block_order, nl.coop_tmp};
    for (void* b : bufs)
        if (b) cudaFree(b);
    nl = sg_nlist_state();
    return SG_OK;
}

// The box of a single-system context changed (sg_set_box, the barostat):
// cells must stay at least one list radius wide. A shrinking box gets fewer
// cells (within the allocated count); a growing one keeps its cells, which
// are then wider than needed. Under three cells per side the build falls
// back to the all-pairs rows. The current pair list is left as it is, as
// the reference's list is: the next needs_rebuild decides.
int sg_nlist_box_changed(sg_ctx* ctx) {
    sg_nlist_state& nl = ctx->nl;
    if (!nl.initialized || ctx->nrep) return SG_OK;
    const double rskin = nl.cutoff + nl.skin;
    int want[3];
    bool cells = ctx->periodic != 0 && nl.ncells_cap > 1;
    for (int d = 0; d < 3; ++d) {
        want[d] = (int)std::floor(ctx->box[d] / (rskin * (1.0 + 1e-4)));
        if (want[d] < 3) cells = false;
    }
    if (cells) {
        const long long prod = (long long)want[0] * want[1] * want[2];
        bool fits = prod <= nl.ncells_cap;
        if (!fits) {   // grew: keep the current grid if its cells are still wide enough
            fits = true;
            for (int d = 0; d < 3; ++d) {
                want[d] = nl.use_cells ? nl.ncell[d] : want[d];
                if (ctx->box[d] / want[d] < rskin * (1.0 + 1e-4)) fits = false;
            }
            if (!nl.use_cells) fits = false;
        }
        cells = fits;
    }
    if (cells) {
        for (int d = 0; d < 3; ++d) nl.ncell[d] = want[d];
        nl.use_cells = 1;
    } else {
        nl.ncell[0] = nl.ncell[1] = nl.ncell[2] = 1;
        nl.use_cells = 0;
    }
    nl.ncells = nl.ncell[0] * nl.ncell[1] * nl.ncell[2];
    nl.row_lanes = row_lanes_for(nl.use_cells, ctx->n, nl.ncells);
    ctx->graph_epoch++;
    return SG_OK;
}

extern "C" {

static int alloc_list(sg_ctx* ctx, int max_nb);

int sg_nlist_init(sg_ctx* ctx, double skin, double cutoff, int32_t trigger_mode) {
    if (!ctx) return SG_EINVAL;
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "a replica context takes sg_rep_nlist_init");
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
    nl.row_lanes = row_lanes_for(nl.use_cells, n, nl.ncells);
    double vol = ctx->box[0] * ctx->box[1] * ctx->box[2];
    double rho = n / vol;
    // rows hold the j > i neighbours in index order, so a particle of low
    // index can list nearly all of its neighbours: size for the full count
    double expect = (4.0 / 3.0) * M_PI * rskin * rskin * rskin * rho;
    int max_nb = (int)std::ceil(expect * 1.3 + 32.0);
    max_nb = (max_nb + 31) / 32 * 32;
    if (max_nb > n) max_nb = std::max(1, n);
    return alloc_list(ctx, max_nb);
}

// Buffers of a list with nl.ncells cells and rows of max_nb, then a build.
static int alloc_list(sg_ctx* ctx, int max_nb) {
    sg_nlist_state& nl = ctx->nl;
    const int n = ctx->n;
    int ntiles = std::max((n + SCAN_TILE - 1) / SCAN_TILE, (nl.ncells + SCAN_TILE - 1) / SCAN_TILE) + 2;
    nl.ncells_cap = nl.ncells;
    SG_CUDA(ctx, cudaMalloc(&nl.cell_count, sizeof(int) * (size_t)nl.ncells));
    // zero before the first build: the cooperative build clears the counts after use
    SG_CUDA(ctx, cudaMemsetAsync(nl.cell_count, 0, sizeof(int) * (size_t)nl.ncells, ctx->stream));
    SG_CUDA(ctx, cudaMalloc(&nl.cell_start, sizeof(int) * ((size_t)nl.ncells + 1)));
    SG_CUDA(ctx, cudaMalloc(&nl.cell_fill, sizeof(int) * (size_t)nl.ncells));
    SG_CUDA(ctx, cudaMalloc(&nl.cell_particles, sizeof(int) * (size_t)n));
    SG_CUDA(ctx, cudaMalloc(&nl.cell_unsorted, sizeof(int) * (size_t)n));
    SG_CUDA(ctx, cudaMalloc(&nl.pos_cell, sizeof(float4) * (size_t)n));
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

// Per-replica lists of a batched context: each replica gets its own cell grid
// (or one cell when its box is under three list radii per side), its own list
// radius (cutoff[f] + skin[f] of its potential family f) and its own trigger.
int sg_rep_nlist_init(sg_ctx* ctx, const double* skin, const double* cutoff, int32_t trigger_mode) {
    if (!ctx || !skin || !cutoff) return SG_EINVAL;
    if (!ctx->nrep) return sg_fail(ctx, SG_EINVAL, "not a replica context");
    const int R = ctx->nrep;
    std::vector<double> rl2(R), trig(R);
    std::vector<int4> grid(R);
    std::vector<int> max_nb_r(R);
    int total_cells = 0;
    for (int r = 0; r < R; ++r) {
        const int f = ctx->h_rep_family[r];
        const double* b = &ctx->h_rep_box[3 * r];
        if (!(skin[f] >= 0.0) || !(cutoff[f] > 0.0)) return sg_fail(ctx, SG_EINVAL, "bad skin / cutoff for family %d", f);
        for (int d = 0; d < 3; ++d)
            if (cutoff[f] > b[d] / 2.0)
                return sg_fail(ctx, SG_ECUTOFF_GT_HALFBOX, "replica %d: a cutoff of %.2f is too large for the box %.2f",
                               r, cutoff[f], b[d]);
        const double rs = cutoff[f] + skin[f];
        rl2[r] = rs * rs;
        trig[r] = trigger_mode == 0 ? rl2[r] : skin[f] * skin[f];
        int nc[3];
        bool cells = true;
        for (int d = 0; d < 3; ++d) {
            nc[d] = (int)std::floor(b[d] / (rs * (1.0 + 1e-4)));
            if (nc[d] < 3) cells = false;
        }
        grid[r] = cells ? make_int4(nc[0], nc[1], nc[2], total_cells) : make_int4(0, 0, 0, total_cells);
        total_cells += cells ? nc[0] * nc[1] * nc[2] : 1;
        const int nr = ctx->h_rep_off[r + 1] - ctx->h_rep_off[r];

        const double rho = nr / (b[0] * b[1] * b[2]);
        // full neighbour count: index-ordered half rows of low index reach it
        const double expect = (4.0 / 3.0) * M_PI * rs * rs * rs * rho;
        int mnb = (int)std::ceil(expect * 1.3 + 32.0);
        max_nb_r[r] = std::max(1, std::min((mnb + 31) / 32 * 32, nr));
    }
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    sg_nlist_free(ctx);
    ctx->graph_epoch++;
    SG_CUDA(ctx, cudaMemcpy((void*)ctx->rep.rl2, rl2.data(), sizeof(double) * R, cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy((void*)ctx->rep.trig, trig.data(), sizeof(double) * R, cudaMemcpyHostToDevice));
    SG_CUDA(ctx, cudaMemcpy((void*)ctx->rep.grid, grid.data(), sizeof(int4) * R, cudaMemcpyHostToDevice));
    sg_nlist_state& nl = ctx->nl;
    nl.trigger_mode = trigger_mode;
    nl.use_cells = 1;
    nl.ncell[0] = nl.ncell[1] = nl.ncell[2] = 1;
    nl.ncells = total_cells;
    // many small lists rebuild at once here: a thread per row keeps every lane busy
    nl.row_lanes = 0;
    nl.h_rep_max_nb = max_nb_r;
    SG_CUDA(ctx, cudaMalloc(&nl.rep_max_nb, sizeof(int) * R));
    SG_CUDA(ctx, cudaMalloc(&nl.rep_pad_off, sizeof(long long) * R));
    SG_CUDA(ctx, cudaMalloc(&nl.rep_need, sizeof(int) * R));
    SG_CUDA(ctx, cudaMalloc(&nl.rep_flag, sizeof(int) * R));
    SG_CUDA(ctx, cudaMemset(nl.rep_flag, 0, sizeof(int) * R));
    SG_CUDA(ctx, cudaMalloc(&nl.rep_builds, sizeof(int) * R));
    SG_CUDA(ctx, cudaMemset(nl.rep_builds, 0, sizeof(int) * R));
    {
        // blocks of the row kernel by their longest row: a one-cell replica's
        // row i tests its N - 1 - i later particles, a row of a replica with
        // cells visits 27 cells of about N / cells particles
        const int n = ctx->n, nblk = (n + 255) / 256;
        std::vector<double> work(nblk, 0.0);
        for (int r = 0; r < R; ++r) {
            const int o = ctx->h_rep_off[r], e = ctx->h_rep_off[r + 1], nr = e - o;
            const int4 gr = grid[r];
            const double cells = gr.x ? (double)gr.x * gr.y * gr.z : 1.0;
            for (int i = o; i < e; ++i) {
                const double w = gr.x ? 27.0 * nr / cells : (double)(e - 1 - i);
                double& wb = work[i / 256];
                wb = std::max(wb, w);
            }
        }
        std::vector<int> order(nblk);
        for (int b = 0; b < nblk; ++b) order[b] = b;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
        SG_CUDA(ctx, cudaMalloc(&nl.row_block_order, sizeof(int) * nblk));
        SG_CUDA(ctx, cudaMemcpy(nl.row_block_order, order.data(), sizeof(int) * nblk, cudaMemcpyHostToDevice));
    }
    return alloc_list(ctx, *std::max_element(max_nb_r.begin(), max_nb_r.end()));
}

int sg_nlist_build(sg_ctx* ctx) {
    if (!ctx) return SG_EINVAL;
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "sg_nlist_init must precede sg_nlist_build");
    return build_sync(ctx);
}

int sg_nlist_needs_rebuild(sg_ctx* ctx, int32_t* flag) {
    if (!ctx || !flag) return SG_EINVAL;
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "sg_nlist_init must precede sg_nlist_needs_rebuild");
    k_clear_request<<<clear_grid(ctx), 256, 0, ctx->stream>>>(ctx->nl.dev_flags, ctx->nl.rep_flag, ctx->nrep,
                                                              nullptr);
    k_check<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, check_args(ctx));
    SG_LAUNCH_CHECK(ctx, "k_check");
    int f = 0;
    SG_CUDA(ctx, cudaMemcpyAsync(&f, ctx->nl.dev_flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    k_clear_request<<<clear_grid(ctx), 256, 0, ctx->stream>>>(ctx->nl.dev_flags, ctx->nl.rep_flag, ctx->nrep,
                                                              nullptr);
    *flag = f;
    return SG_OK;
}

int sg_nlist_update(sg_ctx* ctx) {
    if (!ctx) return SG_EINVAL;
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "sg_nlist_init must precede sg_nlist_update");
    k_check<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, check_args(ctx));
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

int sg_nlist_replica_builds(sg_ctx* ctx, int64_t* counts) {
    if (!ctx || !counts) return SG_EINVAL;
    if (!ctx->nl.initialized || !ctx->nl.rep_builds)
        return sg_fail(ctx, SG_ENOTREADY, "no per-replica lists (sg_rep_nlist_init first)");
    std::vector<int> c(ctx->nrep);
    SG_CUDA(ctx, cudaMemcpyAsync(c.data(), ctx->nl.rep_builds, sizeof(int) * c.size(), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int r = 0; r < ctx->nrep; ++r) counts[r] = c[r];
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

}  // extern "C"

// Storage index of every pair in row order (identity for a single system;
// replica sections otherwise), with the row offsets.
int sg_pair_storage_index(sg_ctx* ctx, int64_t k, std::vector<int>& off, std::vector<int64_t>& where) {
    const int n = ctx->n;
    off.assign(n + 1, 0);
    SG_CUDA(ctx, cudaMemcpyAsync(off.data(), ctx->nl.row_off, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    where.resize(k);
    if (!ctx->nrep) {
        for (int64_t v = 0; v < k; ++v) where[v] = v;
        return SG_OK;
    }
    for (int r = 0; r < ctx->nrep; ++r) {
        const int64_t v0 = off[ctx->h_rep_off[r]], v1 = off[ctx->h_rep_off[r + 1]];
        for (int64_t v = v0; v < v1; ++v) where[v] = ctx->nl.h_rep_pad_off[r] + (v - v0);
    }
    return SG_OK;
}

// Row-order copy of a device array of per-pair values.
template <class T>
static int gather_pairs(sg_ctx* ctx, const T* dev, int64_t k, T* out) {
    if (k <= 0) return SG_OK;
    if (!ctx->nrep) {
        SG_CUDA(ctx, cudaMemcpyAsync(out, dev, sizeof(T) * k, cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return SG_OK;
    }
    std::vector<int> off;
    std::vector<int64_t> where;
    if (int rc = sg_pair_storage_index(ctx, k, off, where)) return rc;
    std::vector<T> all((size_t)ctx->nl.pair_capacity);
    SG_CUDA(ctx, cudaMemcpyAsync(all.data(), dev, sizeof(T) * all.size(), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int64_t v = 0; v < k; ++v) out[v] = all[where[v]];
    return SG_OK;
}

int sg_gather_pair_floats(sg_ctx* ctx, const float* dev, int64_t k, float* out) { return gather_pairs(ctx, dev, k, out); }

extern "C" {

int sg_nlist_pairs(sg_ctx* ctx, int32_t* pi, int32_t* pj, int64_t capacity, int64_t* npairs) {
    if (!ctx || !npairs) return SG_EINVAL;
    int64_t k = 0;
    if (int rc = sg_nlist_count(ctx, &k)) return rc;
    *npairs = k;
    if (k > capacity || (k > 0 && (!pi || !pj))) return sg_fail(ctx, SG_ECAPACITY, "pair capacity too small");
    if (int rc = gather_pairs(ctx, ctx->nl.pair_i, k, pi)) return rc;
    return gather_pairs(ctx, ctx->nl.pair_j, k, pj);
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
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (int rc = gather_pairs(ctx, ctx->nl.pair_j, k, pj.data())) return rc;
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
