// RATTLE bond constraints: apply_constraints_a / apply_constraints_b
// (fortran/system.f90:1055-1210) and the constrained integrators vvc_, nhtc_
// and lgvc_ (fortran/integrators.f90:55-108, 394-490, 678-855).
//
// The reference sweeps its whole constraint list in order (Gauss-Seidel) while
// any atom is flagged as moved, at most 100 sweeps; a constraint is visited
// when either atom is flagged, and a visit sets both flags to "corrected" or
// "satisfied". Constraints that share no atom never see each other's updates,
// so the list splits into molecules (connected components of the constraint
// graph). One thread per molecule walks that molecule's constraints in the
// reference's order with the same flags, tests and sweep cap: every molecule
// goes through the updates it gets in the reference's global loop, whose
// extra sweeps leave a settled molecule untouched. FP32 state, r_tol = 1e-5
// as in the reference.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "sg_internal.cuh"

namespace {

constexpr float kRtol = 1.0e-5f;
constexpr int kMaxRattle = 100;

struct ConGeo {
    float3 box, inv_box;
    int periodic;
};

ConGeo con_geo(const sg_ctx* ctx) {
    ConGeo g;
    g.box = make_float3((float)ctx->box[0], (float)ctx->box[1], (float)ctx->box[2]);
    g.inv_box = make_float3((float)(1.0 / ctx->box[0]), (float)(1.0 / ctx->box[1]), (float)(1.0 / ctx->box[2]));
    g.periodic = ctx->periodic;
    return g;
}

struct ConArgs {
    int nmol;                    // molecules this launch walks: ids list[0 .. nmol)
    const int* __restrict__ list;
    const int2* __restrict__ ij;
    const float* __restrict__ len;
    const int* __restrict__ mol;
    const int* __restrict__ atom_off;
    const int* __restrict__ atoms;
    const int2* __restrict__ loc;
    unsigned char* moved;
    int* err;
    unsigned long long* stats;   // [0] max sweeps a, [1] unconverged a, [2] corrections a, [3..5] the same for b
};

constexpr int kSmallAtoms = 16;   // molecules up to this size sweep in shared memory
constexpr int kSmallBlock = 64;
constexpr size_t kSmallSmem = (size_t)kSmallBlock * kSmallAtoms * (3 * sizeof(float4) + 1);

// Per-thread counters summed over the warp, then one atomic per warp and
// counter: tens of thousands of same-address atomics would serialise.
SG_DEV void flush_stats(unsigned long long* st, unsigned sweeps, unsigned unconverged, unsigned corrections) {
    const unsigned mx = __reduce_max_sync(0xffffffffu, sweeps);
    const unsigned un = __reduce_add_sync(0xffffffffu, unconverged);
    const unsigned co = __reduce_add_sync(0xffffffffu, corrections);
    if ((threadIdx.x & 31) == 0) {
        if (mx) atomicMax(&st[0], (unsigned long long)mx);
        if (un) atomicAdd(&st[1], (unsigned long long)un);
        if (co) atomicAdd(&st[2], (unsigned long long)co);
    }
}

SG_DEV void add3(float4& a, float s, float3 d) {
    a.x += s * d.x;
    a.y += s * d.y;
    a.z += s * d.z;
}

// apply_constraints_a (system.f90:1060-1142): positions against the start-of-step
// bond vectors, with the matching velocity correction.
__global__ void k_rattle_a(ConArgs c, ConGeo g, float dt, float4* pos, float4* vel, const float4* __restrict__ pos_old,
                           double* partials, unsigned int* done, double* vir_out) {
    double vir[1] = {0.0};
    const float inv_dt = 1.f / dt;
    const double inv_dt2 = 1.0 / ((double)dt * (double)dt);
    unsigned t_sweeps = 0, t_unconverged = 0, t_corrections = 0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < c.nmol; q += gridDim.x * blockDim.x) {
        const int m = c.list[q];
        const int b = c.mol[m], e = c.mol[m + 1];
        for (int k = b; k < e; ++k) {
            c.moved[c.ij[k].x] = 1;
            c.moved[c.ij[k].y] = 1;
        }
        int sweep = 0;
        bool any = true, failed = false;
        while (any && sweep < kMaxRattle && !failed) {
            for (int k = b; k < e; ++k) {
                const int i = c.ij[k].x, j = c.ij[k].y;
                if (!(c.moved[i] || c.moved[j])) continue;
                const float len2 = c.len[k] * c.len[k];
                const float4 pi = pos[i], pj = pos[j];
                const float3 r = min_image(make_float3(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z), g.box, g.inv_box,
                                           g.periodic);
                const float chi = len2 - dot3(r, r);
                if (fabsf(chi) > 2.f * kRtol * len2) {
                    const float4 oi = pos_old[i], oj = pos_old[j];
                    const float3 ro = min_image(make_float3(oi.x - oj.x, oi.y - oj.y, oi.z - oj.z), g.box,
                                                g.inv_box, g.periodic);
                    const float vdot = dot3(r, ro);
                    if (vdot < kRtol * len2) {
                        // the reference stops the program here (:1102-1106)
                        if (atomicCAS(&c.err[0], 0, k + 1) == 0) {
                            c.err[1] = i;
                            c.err[2] = j;
                        }
                        failed = true;
                        break;
                    }
                    const float4 vi = vel[i], vj = vel[j];
                    const float imi = vi.w, imj = vj.w;
                    const float L = chi / (2.f * vdot * (imi + imj));
                    vir[0] += (double)L * (double)len2 * inv_dt2;
                    float4 qi = pi, qj = pj, wi = vi, wj = vj;
                    add3(qi, L * imi, ro);
                    add3(qj, -(L * imj), ro);
                    add3(wi, L * imi * inv_dt, ro);
                    add3(wj, -(L * imj * inv_dt), ro);
                    pos[i] = qi;
                    pos[j] = qj;
                    vel[i] = wi;
                    vel[j] = wj;
                    c.moved[i] = 1;
                    c.moved[j] = 1;
                    ++t_corrections;
                } else {
                    c.moved[i] = 0;
                    c.moved[j] = 0;
                }
            }
            ++sweep;
            any = false;
            for (int k = b; k < e && !any; ++k) any = c.moved[c.ij[k].x] || c.moved[c.ij[k].y];
        }
        t_sweeps = max(t_sweeps, (unsigned)sweep);
        if (any && !failed) ++t_unconverged;
    }
    flush_stats(c.stats, t_sweeps, t_unconverged, t_corrections);
    block_reduce_finish<1>(vir, partials, done, vir_out);
}

// apply_constraints_b (system.f90:1144-1208): velocities along the bond.
__global__ void k_rattle_b(ConArgs c, ConGeo g, float dt, const float4* __restrict__ pos, float4* vel,
                           double* partials, unsigned int* done, double* vir_out) {
    double vir[1] = {0.0};
    const double inv_dt = 1.0 / (double)dt;
    unsigned t_sweeps = 0, t_unconverged = 0, t_corrections = 0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < c.nmol; q += gridDim.x * blockDim.x) {
        const int m = c.list[q];
        const int b = c.mol[m], e = c.mol[m + 1];
        for (int k = b; k < e; ++k) {
            c.moved[c.ij[k].x] = 1;
            c.moved[c.ij[k].y] = 1;
        }
        int sweep = 0;
        bool any = true;
        while (any && sweep < kMaxRattle) {
            for (int k = b; k < e; ++k) {
                const int i = c.ij[k].x, j = c.ij[k].y;
                if (!(c.moved[i] || c.moved[j])) continue;
                const float len2 = c.len[k] * c.len[k];
                const float4 pi = pos[i], pj = pos[j];
                const float3 r = min_image(make_float3(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z), g.box, g.inv_box,
                                           g.periodic);
                const float4 vi = vel[i], vj = vel[j];
                const float3 v = make_float3(vi.x - vj.x, vi.y - vj.y, vi.z - vj.z);
                const float imi = vi.w, imj = vj.w;
                const float L = -dot3(r, v) / ((imi + imj) * len2);
                if (fabsf(L) > kRtol) {
                    vir[0] += (double)L * (double)len2 * inv_dt;
                    float4 wi = vi, wj = vj;
                    add3(wi, L * imi, r);
                    add3(wj, -(L * imj), r);
                    vel[i] = wi;
                    vel[j] = wj;
                    c.moved[i] = 1;
                    c.moved[j] = 1;
                    ++t_corrections;
                } else {
                    c.moved[i] = 0;
                    c.moved[j] = 0;
                }
            }
            ++sweep;
            any = false;
            for (int k = b; k < e && !any; ++k) any = c.moved[c.ij[k].x] || c.moved[c.ij[k].y];
        }
        t_sweeps = max(t_sweeps, (unsigned)sweep);
        if (any) ++t_unconverged;
    }
    flush_stats(c.stats + 3, t_sweeps, t_unconverged, t_corrections);
    block_reduce_finish<1>(vir, partials, done, vir_out);
}

// The same two passes for molecules of 3 to kSmallAtoms atoms: the
// molecule's positions, start-of-step positions, velocities and moved flags
// are staged in shared memory ([atom][thread], conflict-free), swept there with
// the same visits and tests, and written back once. The sweeps' dependent
// loads become shared-memory latencies instead of L2 round trips.
__global__ void __launch_bounds__(kSmallBlock) k_rattle_a_small(ConArgs c, ConGeo g, float dt, float4* pos,
                                                                 float4* vel, const float4* __restrict__ pos_old,
                                                                 double* partials, unsigned int* done,
                                                                 double* vir_out) {
    extern __shared__ float4 sh[];
    const int T = kSmallBlock, tid = threadIdx.x;
    float4* P = sh;
    float4* O = sh + kSmallAtoms * T;
    float4* V = sh + 2 * kSmallAtoms * T;
    unsigned char* M = reinterpret_cast<unsigned char*>(sh + 3 * kSmallAtoms * T);
    double vir[1] = {0.0};
    const float inv_dt = 1.f / dt;
    const double inv_dt2 = 1.0 / ((double)dt * (double)dt);
    unsigned t_sweeps = 0, t_unconverged = 0, t_corrections = 0;
    for (int q = blockIdx.x * T + tid; q < c.nmol; q += gridDim.x * T) {
        const int m = c.list[q];
        const int a0 = c.atom_off[m], na = c.atom_off[m + 1] - a0;
        for (int a = 0; a < na; ++a) {
            const int id = c.atoms[a0 + a];
            P[a * T + tid] = pos[id];
            O[a * T + tid] = pos_old[id];
            V[a * T + tid] = vel[id];
            M[a * T + tid] = 1;
        }
        const int b = c.mol[m], e = c.mol[m + 1];
        int sweep = 0;
        bool any = true, failed = false;
        while (any && sweep < kMaxRattle && !failed) {
            for (int k = b; k < e; ++k) {
                const int2 l = c.loc[k];
                const int i = l.x * T + tid, j = l.y * T + tid;
                if (!(M[i] || M[j])) continue;
                const float len2 = c.len[k] * c.len[k];
                const float4 pi = P[i], pj = P[j];
                const float3 r = min_image(make_float3(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z), g.box, g.inv_box,
                                           g.periodic);
                const float chi = len2 - dot3(r, r);
                if (fabsf(chi) > 2.f * kRtol * len2) {
                    const float4 oi = O[i], oj = O[j];
                    const float3 ro = min_image(make_float3(oi.x - oj.x, oi.y - oj.y, oi.z - oj.z), g.box,
                                                g.inv_box, g.periodic);
                    const float vdot = dot3(r, ro);
                    if (vdot < kRtol * len2) {
                        if (atomicCAS(&c.err[0], 0, k + 1) == 0) {
                            c.err[1] = c.ij[k].x;
                            c.err[2] = c.ij[k].y;
                        }
                        failed = true;
                        break;
                    }
                    float4 wi = V[i], wj = V[j];
                    const float imi = wi.w, imj = wj.w;
                    const float L = chi / (2.f * vdot * (imi + imj));
                    vir[0] += (double)L * (double)len2 * inv_dt2;
                    float4 qi = pi, qj = pj;
                    add3(qi, L * imi, ro);
                    add3(qj, -(L * imj), ro);
                    add3(wi, L * imi * inv_dt, ro);
                    add3(wj, -(L * imj * inv_dt), ro);
                    P[i] = qi;
                    P[j] = qj;
                    V[i] = wi;
                    V[j] = wj;
                    M[i] = 1;
                    M[j] = 1;
                    ++t_corrections;
                } else {
                    M[i] = 0;
                    M[j] = 0;
                }
            }
            ++sweep;
            any = false;
            for (int a = 0; a < na && !any; ++a) any = M[a * T + tid] != 0;
        }
        for (int a = 0; a < na; ++a) {
            const int id = c.atoms[a0 + a];
            pos[id] = P[a * T + tid];
            vel[id] = V[a * T + tid];
        }
        t_sweeps = max(t_sweeps, (unsigned)sweep);
        if (any && !failed) ++t_unconverged;
    }
    flush_stats(c.stats, t_sweeps, t_unconverged, t_corrections);
    block_reduce_finish<1>(vir, partials, done, vir_out);
}

__global__ void __launch_bounds__(kSmallBlock) k_rattle_b_small(ConArgs c, ConGeo g, float dt,
                                                                 const float4* __restrict__ pos, float4* vel,
                                                                 double* partials, unsigned int* done,
                                                                 double* vir_out) {
    extern __shared__ float4 sh[];
    const int T = kSmallBlock, tid = threadIdx.x;
    float4* P = sh;
    float4* V = sh + 2 * kSmallAtoms * T;
    unsigned char* M = reinterpret_cast<unsigned char*>(sh + 3 * kSmallAtoms * T);
    double vir[1] = {0.0};
    const double inv_dt = 1.0 / (double)dt;
    unsigned t_sweeps = 0, t_unconverged = 0, t_corrections = 0;
    for (int q = blockIdx.x * T + tid; q < c.nmol; q += gridDim.x * T) {
        const int m = c.list[q];
        const int a0 = c.atom_off[m], na = c.atom_off[m + 1] - a0;
        for (int a = 0; a < na; ++a) {
            const int id = c.atoms[a0 + a];
            P[a * T + tid] = pos[id];
            V[a * T + tid] = vel[id];
            M[a * T + tid] = 1;
        }
        const int b = c.mol[m], e = c.mol[m + 1];
        int sweep = 0;
        bool any = true;
        while (any && sweep < kMaxRattle) {
            for (int k = b; k < e; ++k) {
                const int2 l = c.loc[k];
                const int i = l.x * T + tid, j = l.y * T + tid;
                if (!(M[i] || M[j])) continue;
                const float len2 = c.len[k] * c.len[k];
                const float4 pi = P[i], pj = P[j];
                const float3 r = min_image(make_float3(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z), g.box, g.inv_box,
                                           g.periodic);
                float4 wi = V[i], wj = V[j];
                const float3 v = make_float3(wi.x - wj.x, wi.y - wj.y, wi.z - wj.z);
                const float imi = wi.w, imj = wj.w;
                const float L = -dot3(r, v) / ((imi + imj) * len2);
                if (fabsf(L) > kRtol) {
                    vir[0] += (double)L * (double)len2 * inv_dt;
                    add3(wi, L * imi, r);
                    add3(wj, -(L * imj), r);
                    V[i] = wi;
                    V[j] = wj;
                    M[i] = 1;
                    M[j] = 1;
                    ++t_corrections;
                } else {
                    M[i] = 0;
                    M[j] = 0;
                }
            }
            ++sweep;
            any = false;
            for (int a = 0; a < na && !any; ++a) any = M[a * T + tid] != 0;
        }
        for (int a = 0; a < na; ++a) vel[c.atoms[a0 + a]] = V[a * T + tid];
        t_sweeps = max(t_sweeps, (unsigned)sweep);
        if (any) ++t_unconverged;
    }
    flush_stats(c.stats + 3, t_sweeps, t_unconverged, t_corrections);
    block_reduce_finish<1>(vir, partials, done, vir_out);
}

// small = true: the shared-memory molecules, else the large ones
ConArgs con_args(sg_ctx* ctx, bool small) {
    ConArgs c;
    c.nmol = small ? ctx->con_nsmall : ctx->con_nlarge;
    c.list = ctx->con_small + (small ? 0 : ctx->con_nsmall);
    c.atom_off = ctx->con_atom_off;
    c.atoms = ctx->con_atoms;
    c.loc = ctx->con_loc;
    c.ij = ctx->con_ij;
    c.len = ctx->con_len;
    c.mol = ctx->con_mol;
    c.moved = ctx->con_moved;
    c.err = ctx->con_err;
    c.stats = ctx->con_stats;
    return c;
}

int con_grid(sg_ctx* ctx, int nmol, int block) {
    // one thread per molecule
    return std::max(1, std::min((nmol + block - 1) / block, 8 * ctx->num_sms));
}

int need(sg_ctx* ctx) {
    if (!ctx) return SG_EINVAL;
    if (!ctx->con_n) return sg_fail(ctx, SG_ENOTREADY, "no constraints: call sg_set_constraints first");
    return SG_OK;
}

int check_failure(sg_ctx* ctx) {
    int err[3];
    SG_CUDA(ctx, cudaMemcpyAsync(err, ctx->con_err, sizeof(err), cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (err[0])
        return sg_fail(ctx, SG_ENOCONV, "Constraint failure between atoms %d and %d (0-based; constraint %d)", err[1],
                       err[2], err[0] - 1);
    return SG_OK;
}

}  // namespace

int sg_constraints_free(sg_ctx* ctx) {
    void* bufs[] = {ctx->con_ij, ctx->con_len, ctx->con_mol, ctx->con_moved, ctx->pos_old, ctx->con_err,
                    ctx->con_stats, ctx->con_small, ctx->con_atom_off, ctx->con_atoms, ctx->con_loc};
    for (void* b : bufs)
        if (b) cudaFree(b);
    ctx->con_small = nullptr;
    ctx->con_atom_off = nullptr;
    ctx->con_atoms = nullptr;
    ctx->con_loc = nullptr;
    ctx->con_nsmall = ctx->con_nlarge = 0;
    ctx->con_ij = nullptr;
    ctx->con_len = nullptr;
    ctx->con_mol = nullptr;
    ctx->con_moved = nullptr;
    ctx->pos_old = nullptr;
    ctx->con_err = nullptr;
    ctx->con_stats = nullptr;
    ctx->con_n = ctx->con_nmol = ctx->con_max_len = 0;
    return SG_OK;
}

extern "C" {

int sg_set_constraints(sg_ctx* ctx, int32_t nc, const int32_t* bbi, const int32_t* bbj, const double* length,
                       int32_t one_based) {
    if (!ctx || nc < 0 || (nc > 0 && (!bbi || !bbj || !length))) return SG_EINVAL;
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "constraints are per system: no replica contexts");
    const int n = ctx->n, off = one_based ? 1 : 0;
    std::vector<int> I(nc), J(nc);
    for (int k = 0; k < nc; ++k) {
        I[k] = bbi[k] - off;
        J[k] = bbj[k] - off;
        // add_constraint (fortran/system.f90:345-360) checks the constraint index only
        if (I[k] < 0 || I[k] >= n || J[k] < 0 || J[k] >= n || I[k] == J[k])
            return sg_fail(ctx, SG_EINVAL, "constraint %d joins invalid atoms %d, %d", k, bbi[k], bbj[k]);
        if (!(length[k] > 0.0)) return sg_fail(ctx, SG_EINVAL, "constraint %d has a non-positive length", k);
    }
    // molecules: union-find over the atoms
    std::vector<int> parent(n);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int a) {
        while (parent[a] != a) a = parent[a] = parent[parent[a]];
        return a;
    };
    for (int k = 0; k < nc; ++k) {
        const int a = find(I[k]), b = find(J[k]);
        if (a != b) parent[std::max(a, b)] = std::min(a, b);
    }
    // molecules numbered by first appearance in the list; constraints grouped
    // by molecule, keeping the list order inside each group
    std::vector<int> mol_of_root(n, -1), mol(nc), count;
    for (int k = 0; k < nc; ++k) {
        const int r = find(I[k]);
        if (mol_of_root[r] < 0) {
            mol_of_root[r] = (int)count.size();
            count.push_back(0);
        }
        mol[k] = mol_of_root[r];
        ++count[mol[k]];
    }
    const int nmol = (int)count.size();
    std::vector<int> start(nmol + 1, 0);
    for (int m = 0; m < nmol; ++m) start[m + 1] = start[m] + count[m];
    std::vector<int> fill(start.begin(), start.end() - 1);
    std::vector<int2> ij(nc);
    std::vector<float> len(nc);
    for (int k = 0; k < nc; ++k) {
        const int slot = fill[mol[k]]++;
        ij[slot] = make_int2(I[k], J[k]);
        len[slot] = (float)length[k];
    }
    // each molecule's atoms in order of first appearance, the constraints'
    // atoms as indices into that list, and the small / large split
    std::vector<int> atom_off(nmol + 1, 0), atoms, small, large;
    std::vector<int2> loc(nc);
    std::vector<int> local(n, -1);
    atoms.reserve(2 * (size_t)nc);
    for (int m = 0; m < nmol; ++m) {
        atom_off[m] = (int)atoms.size();
        for (int k = start[m]; k < start[m + 1]; ++k) {
            for (int a : {ij[k].x, ij[k].y})
                if (local[a] < 0) {
                    local[a] = (int)atoms.size() - atom_off[m];
                    atoms.push_back(a);
                }
            loc[k] = make_int2(local[ij[k].x], local[ij[k].y]);
        }
        for (int t = atom_off[m]; t < (int)atoms.size(); ++t) local[atoms[t]] = -1;
        // single bonds gain nothing from staging (two visits at most): they
        // stay on the global-memory kernel with its larger blocks
        const int na = (int)atoms.size() - atom_off[m];
        (na >= 3 && na <= kSmallAtoms ? small : large).push_back(m);
    }
    atom_off[nmol] = (int)atoms.size();
    const int nsmall = (int)small.size(), nlarge = (int)large.size();
    small.insert(small.end(), large.begin(), large.end());
    sg_constraints_free(ctx);
    ctx->graph_epoch++;
    ctx->h_bbi = I;
    ctx->h_bbj = J;
    ctx->h_blen.assign(length, length + nc);
    if (nc == 0) return SG_OK;
    SG_CUDA(ctx, cudaMalloc(&ctx->con_ij, sizeof(int2) * nc));
    SG_CUDA(ctx, cudaMalloc(&ctx->con_len, sizeof(float) * nc));
    SG_CUDA(ctx, cudaMalloc(&ctx->con_mol, sizeof(int) * (nmol + 1)));
    SG_CUDA(ctx, cudaMalloc(&ctx->con_moved, (size_t)n));
    SG_CUDA(ctx, cudaMalloc(&ctx->pos_old, sizeof(float4) * (size_t)n));
    SG_CUDA(ctx, cudaMalloc(&ctx->con_err, sizeof(int) * 4));
    SG_CUDA(ctx, cudaMalloc(&ctx->con_stats, sizeof(unsigned long long) * 8));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->con_ij, ij.data(), sizeof(int2) * nc, cudaMemcpyHostToDevice, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->con_len, len.data(), sizeof(float) * nc, cudaMemcpyHostToDevice, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->con_mol, start.data(), sizeof(int) * (nmol + 1), cudaMemcpyHostToDevice,
                                 ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->con_moved, 0, (size_t)n, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->pos_old, ctx->pos, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->con_err, 0, sizeof(int) * 4, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->con_stats, 0, sizeof(unsigned long long) * 8, ctx->stream));
    SG_CUDA(ctx, cudaMalloc(&ctx->con_small, sizeof(int) * nmol));
    SG_CUDA(ctx, cudaMalloc(&ctx->con_atom_off, sizeof(int) * (nmol + 1)));
    SG_CUDA(ctx, cudaMalloc(&ctx->con_atoms, sizeof(int) * atoms.size()));
    SG_CUDA(ctx, cudaMalloc(&ctx->con_loc, sizeof(int2) * nc));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->con_small, small.data(), sizeof(int) * nmol, cudaMemcpyHostToDevice,
                                 ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->con_atom_off, atom_off.data(), sizeof(int) * (nmol + 1),
                                 cudaMemcpyHostToDevice, ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->con_atoms, atoms.data(), sizeof(int) * atoms.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->con_loc, loc.data(), sizeof(int2) * nc, cudaMemcpyHostToDevice, ctx->stream));
    SG_CUDA(ctx, cudaFuncSetAttribute(k_rattle_a_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmem));
    SG_CUDA(ctx, cudaFuncSetAttribute(k_rattle_b_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmem));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->con_nsmall = nsmall;
    ctx->con_nlarge = nlarge;
    ctx->con_n = nc;
    ctx->con_nmol = nmol;
    ctx->con_max_len = *std::max_element(count.begin(), count.end());
    return SG_OK;
}

int sg_constraints_save(sg_ctx* ctx) {
    if (int rc = need(ctx)) return rc;
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->pos_old, ctx->pos, sizeof(float4) * (size_t)ctx->n, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    return SG_OK;
}

int sg_constraints_a(sg_ctx* ctx, double dt) {
    if (int rc = need(ctx)) return rc;
    sg_state_touched(ctx);
    if (ctx->con_nsmall) {
        const int grid = con_grid(ctx, ctx->con_nsmall, kSmallBlock);
        if (int rc = sg_ensure_partials(ctx, grid)) return rc;
        k_rattle_a_small<<<grid, kSmallBlock, kSmallSmem, ctx->stream>>>(
            con_args(ctx, true), con_geo(ctx), (float)dt, ctx->pos, ctx->vel, ctx->pos_old, ctx->partials,
            ctx->done_counter, ctx->acc + 6);
        SG_LAUNCH_CHECK(ctx, "k_rattle_a_small");
    }
    if (ctx->con_nlarge) {
        const int grid = con_grid(ctx, ctx->con_nlarge, 128);
        if (int rc = sg_ensure_partials(ctx, grid)) return rc;
        k_rattle_a<<<grid, 128, 0, ctx->stream>>>(con_args(ctx, false), con_geo(ctx), (float)dt, ctx->pos, ctx->vel,
                                                  ctx->pos_old, ctx->partials, ctx->done_counter, ctx->acc + 6);
        SG_LAUNCH_CHECK(ctx, "k_rattle_a");
    }
    return SG_OK;
}

int sg_constraints_b(sg_ctx* ctx, double dt) {
    if (int rc = need(ctx)) return rc;
    sg_state_touched(ctx);
    if (ctx->con_nsmall) {
        const int grid = con_grid(ctx, ctx->con_nsmall, kSmallBlock);
        if (int rc = sg_ensure_partials(ctx, grid)) return rc;
        k_rattle_b_small<<<grid, kSmallBlock, kSmallSmem, ctx->stream>>>(con_args(ctx, true), con_geo(ctx),
                                                                         (float)dt, ctx->pos, ctx->vel, ctx->partials,
                                                                         ctx->done_counter, ctx->acc + 6);
        SG_LAUNCH_CHECK(ctx, "k_rattle_b_small");
    }
    if (ctx->con_nlarge) {
        const int grid = con_grid(ctx, ctx->con_nlarge, 128);
        if (int rc = sg_ensure_partials(ctx, grid)) return rc;
        k_rattle_b<<<grid, 128, 0, ctx->stream>>>(con_args(ctx, false), con_geo(ctx), (float)dt, ctx->pos, ctx->vel,
                                                  ctx->partials, ctx->done_counter, ctx->acc + 6);
        SG_LAUNCH_CHECK(ctx, "k_rattle_b");
    }
    return SG_OK;
}

int sg_constraints_check(sg_ctx* ctx) {
    if (int rc = need(ctx)) return rc;
    return check_failure(ctx);
}

int sg_constraint_stats(sg_ctx* ctx, int64_t out[6], int32_t reset) {
    if (int rc = need(ctx)) return rc;
    unsigned long long s[8];
    SG_CUDA(ctx, cudaMemcpyAsync(s, ctx->con_stats, sizeof(s), cudaMemcpyDeviceToHost, ctx->stream));
    if (reset) SG_CUDA(ctx, cudaMemsetAsync(ctx->con_stats, 0, sizeof(s), ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (out)
        for (int k = 0; k < 6; ++k) out[k] = (int64_t)s[k];
    return SG_OK;
}

int sg_constraints_clear_error(sg_ctx* ctx) {
    if (int rc = need(ctx)) return rc;
    SG_CUDA(ctx, cudaMemsetAsync(ctx->con_err, 0, sizeof(int) * 4, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

// ---- constrained integrators: the plain half steps with RX_old saved before
// the drift, apply_constraints_a after the initial and apply_constraints_b
// after the final half step (the kinetic energy is summed before b, as in
// the reference)
int sg_vvc_initial(sg_ctx* ctx, double dt) {                   // integrators.f90:55-86
    if (int rc = need(ctx)) return rc;
    if (int rc = sg_constraints_save(ctx)) return rc;
    if (int rc = sg_vv_initial(ctx, dt)) return rc;
    if (int rc = sg_constraints_a(ctx, dt)) return rc;
    return check_failure(ctx);
}

int sg_vvc_final(sg_ctx* ctx, double dt, double* kin_eng) {   // integrators.f90:88-106
    if (int rc = need(ctx)) return rc;
    if (int rc = sg_vv_final(ctx, dt, kin_eng)) return rc;
    if (int rc = sg_constraints_b(ctx, dt)) return rc;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_nhtc_initial(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t mode,
                    int32_t rot_chain) {                          // integrators.f90:394-449
    if (int rc = need(ctx)) return rc;
    if (int rc = sg_constraints_save(ctx)) return rc;
    if (int rc = sg_nht_initial(ctx, dt, target_temp, coupling, mode, rot_chain)) return rc;
    if (int rc = sg_constraints_a(ctx, dt)) return rc;
    return check_failure(ctx);
}

int sg_nhtc_final(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t mode, int32_t rot_chain,
                  double* kin_eng) {                               // integrators.f90:451-490
    if (int rc = need(ctx)) return rc;
    if (int rc = sg_nht_final(ctx, dt, target_temp, coupling, mode, rot_chain, kin_eng)) return rc;
    if (int rc = sg_constraints_b(ctx, dt)) return rc;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_lgvc_initial(sg_ctx* ctx, double dt, int32_t step, double damping, double target_temp,
                    const uint32_t* key) {                          // integrators.f90:678-800
    if (int rc = need(ctx)) return rc;
    if (target_temp <= 1e-3) return sg_fail(ctx, SG_EINVAL, "Target temperature too small.");
    if (int rc = sg_constraints_save(ctx)) return rc;
    if (int rc = sg_lgv_initial(ctx, dt, step, damping, target_temp, key)) return rc;
    if (int rc = sg_constraints_a(ctx, dt)) return rc;
    return check_failure(ctx);
}

int sg_lgvc_final(sg_ctx* ctx, double dt, double damping, double* kin_eng, double* kin_rot) {  // :802-855
    if (int rc = need(ctx)) return rc;
    if (int rc = sg_lgv_final(ctx, dt, damping, kin_eng, kin_rot)) return rc;
    if (int rc = sg_constraints_b(ctx, dt)) return rc;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

}  // extern "C"
