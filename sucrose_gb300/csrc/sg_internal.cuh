// Internal declarations shared by the CUDA translation units of libsucrose_gb300.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <map>
#include <utility>
#include <vector>

#include "../../include/sucrose_gpu.h"

#define SG_DEV __device__ __forceinline__

// ------------------------------------------- programmatic dependent launch --
// A kernel launched by launch_pdl may be scheduled while the kernel before it
// in the stream is still running, once every block of that kernel has called
// pdl_trigger() (or exited). Its blocks then load what the earlier kernel does
// not write, and pdl_wait() (griddepcontrol.wait) returns once the earlier
// grid has completed and its writes are visible; every read of data that grid
// writes, and every write, comes after it. pdl_wait returns at once in a
// kernel launched the ordinary way. A kernel calls pdl_trigger only after its
// own pdl_wait, so that its dependents never overlap the grid before it.
SG_DEV void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
SG_DEV void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// k<<<grid, block, smem, s>>>(args...) with programmatic stream serialisation
// (pdl = true) or as an ordinary launch.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(bool pdl, void (*k)(KArgs...), int grid, int block, size_t smem, cudaStream_t s,
                       Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// ------------------------------------------------------------------ context --
// Per-replica tables of a batched context (sg_create_replicas). A context
// without replicas has rep_of == nullptr and every kernel uses the single
// box of the context.
struct RepDev {
    const int* rep_of = nullptr;      // [n] replica of each particle
    const int* off = nullptr;         // [R+1] first particle of each replica
    const float4* box = nullptr;      // [R] box lengths (x, y, z, 0)
    const float4* inv_box = nullptr;  // [R] 1 / box
    const float4* box_lo = nullptr;   // [R] box - (float)box: the FP64 box as float hi + lo
    const double* boxd = nullptr;     // [3R] box lengths in FP64
    const double* rl2 = nullptr;      // [R] (rc + skin)^2 of the replica's list
    const double* trig = nullptr;     // [R] rebuild bound on 4 |dr|^2
    const int4* grid = nullptr;       // [R] cells per side (x, y, z) and first global cell; x = 0: one cell
    const double* temp = nullptr;     // [R] target temperature
    const int* temp_int = nullptr;    // [R] int(T * 1000) for the Philox counter
    const uint2* key = nullptr;       // [R] Philox key
    const float* half_sq = nullptr;   // [R] (0.4998 min(box))^2, rounded down (list acceptance test)
};

struct sg_nlist_state {
    int initialized = 0;
    int trigger_mode = 0;
    double cutoff = 0.0, skin = 0.0;
    double rl2 = 0.0;                // (rc+skin)^2 in FP64, the reference's r_skin_sq after a build
    double trigger_sq = 0.0;         // compared with 4 * max displacement^2
    int use_cells = 0;
    int coop_grid = 0;               // blocks of the cooperative single-system build (0: not set up)
    int* coop_tmp = nullptr;         // its scans' block totals
    int row_lanes = 0;               // a single system with dense cells: 32 lanes per row in the search; 0: a thread per row
    int ncell[3] = {0, 0, 0};
    int ncells = 0;
    int ncells_cap = 0;              // cells the arrays were sized for
    int max_nb = 0;                  // capacity per particle (half list)
    int64_t pair_capacity = 0;       // capacity of the flattened list
    int* cell_count = nullptr;       // [ncells]
    int* cell_start = nullptr;       // [ncells + 1]
    int* cell_fill = nullptr;        // [ncells]
    int* cell_particles = nullptr;   // [n]
    int* particle_cell = nullptr;    // [n]
    int* nb_count = nullptr;         // [n]
    int* nb_pad = nullptr;           // [max_nb * n], column-major (k * n + i); dense cells: row-major
    float4* pos_cell = nullptr;      // [n] positions in cell order (single systems)
    int* row_off = nullptr;          // [n + 1]
    int* scan_tmp = nullptr;         // block sums of the scan
    int* pair_i = nullptr;           // [pair_capacity]
    int* pair_j = nullptr;           // [pair_capacity]
    int* dev_flags = nullptr;        // [0] rebuild requested, [1] overflow (max row seen), [2] npairs, [3] builds
    float4* pos_last = nullptr;      // positions at the last build
    // replica contexts: rows of replica r have their own capacity max_nb[r] and
    // sit column-major in their own section of nb_pad, starting at pad_off[r]
    int* rep_max_nb = nullptr;       // [R]
    long long* rep_pad_off = nullptr;// [R]
    int* rep_need = nullptr;         // [R] longest row seen when a row overflowed
    int* rep_flag = nullptr;         // [R] rebuild requested for this replica
    int* rep_builds = nullptr;       // [R] rebuilds of each replica's rows since sg_nlist_init
    int* row_block_order = nullptr;  // replica contexts: 256-row blocks of the row kernel, longest rows first
    int* cell_unsorted = nullptr;    // [n] cell members before ordering
    int* chunk_rep = nullptr;        // [capacity / 32 + 2] replica of each 32-pair chunk
    std::vector<int> h_rep_max_nb;
    std::vector<long long> h_rep_pad_off;
};

// Launch shape of a pair kernel (chosen by the autotuner).
struct PairTune {
    int block = 256;   // threads per block (128 or 256)
    int filter = 0;    // range filter + per-warp queue of in-range pairs; ECP kinds: the split Newton path
};

// float4 per particle of the per-particle prep buffer (ecp_prep). ECP: the
// 64-byte record of particle p at 4p and the 32-byte range record at 4n + 2p;
// Gay-Berne: 2 at 2p, 1 at 2n + p, 1 at 3n + p.
#define SG_PREP_F4 6

struct sg_ctx {
    int n = 0;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    double box[3] = {0, 0, 0};
    int periodic = 1;
    char err[512] = {0};

    // FP32 SoA state, float4 each
    float4* pos = nullptr;       // x y z 0
    float4* quat = nullptr;      // w x y z
    float4* vel = nullptr;       // vx vy vz inv_mass
    float4* angm = nullptr;      // lx ly lz 0
    float4* force = nullptr;     // fx fy fz 0
    float4* torque = nullptr;    // tx ty tz 0
    float4* shape = nullptr;     // sig_x sig_y sig_z mass
    float4* eshape = nullptr;    // eps_x eps_y eps_z 0
    float4* inert = nullptr;     // Ixx Iyy Izz 0
    float4* inert_inv = nullptr; // 1/Ixx 1/Iyy 1/Izz 0

    // FP64 accumulators: [0] pot_eng [1] pair virial [2] kin_eng [3] kin_rot
    double* acc = nullptr;
    // FP64 scratch for reductions: per-block partials and completion counter
    double* partials = nullptr;
    unsigned int* done_counter = nullptr;
    int partial_slots = 0;
    // ECP / solver statistics (unsigned long long): [0] pairs [1] evals [2] nonconv [3] fallbacks [4..27] hist
    unsigned long long* stats = nullptr;
    // Nose-Hoover chain state, FP64: eta[3] p_eta[3] eta_r[3] p_eta_r[3] + scratch
    double* nh = nullptr;

    // ECP per-particle prep (FP32) and FP64 copies for the bit-exact Brent
    float4* ecp_prep = nullptr;      // SG_PREP_F4 float4 per particle
    double* ecp_prep64 = nullptr;    // A_R in FP64, 6 doubles per particle
    float* ecp_lambda = nullptr;     // per pair
    int64_t ecp_lambda_cap = 0;

    // MLP weights (FP32 master) and BF16 packed copy
    float* mlp_w = nullptr;
    void* mlp_wbf16 = nullptr;       // device: bf16 W1 W2 W3 then f32 b1 b2 b3 w4
    unsigned char mlp_host_desc[128];  // host copy of the MlpDev descriptor (device pointers)
    int mlp_ready = 0;
    int* mlp_tc_err = nullptr;       // device flag: a tensor-core completion wait ran out
    int mlp_inline = 0;              // 1: the ECP kernel evaluates the guess itself (mma.sync)
    // Captured-step fusion, set while a step is being enqueued: the initial
    // half step also runs the list's displacement test, zeroes forces,
    // torques and the accumulators, and (step_prep_kind) writes the pair
    // potential's per-particle prep; the final half step stores its sums and
    // advances the step counter.
    // Gay-Berne replica tiles (k_pair_gb_tile): the GB family's replicas,
    // largest first, a work counter and a finished-blocks counter, and the
    // largest replica's particle count.
    int* gb_tile_order = nullptr;
    int gb_tile_count = 0;
    int gb_tile_maxn = 0;
    int ecp_lambda_partial = 0;
    int* pair_surv = nullptr;        // two-pass filtered launch: count, then tmap, i, j of the compacted pairs
    int64_t pair_surv_cap = 0;      // the last ECP call left lambda unset (NaN) for unsolved pairs
    int step_fused = 0;
    int step_events = 0;             // the step is captured with event nodes between its stages
    int step_prep_kind = 0;          // SG_PREP_NONE / _ECP / _GB (step_epi.cuh)
    float step_prep_muinv = 1.f;
    int mlp_tc_test_no_mma = 0;      // failure-path test: the next guess pass issues no MMA
    void* mlp_work = nullptr;        // training workspace (mlp_train.cu)
    int mlp_adam_t = 0;

    // dipole reaction field (sg_reaction_field_init): DIP per particle, the
    // pair kernel's marks (I side in range) and counts (J side in range), RFL
    float4* rf_dip = nullptr;
    int* rf_mark = nullptr;
    int* rf_cnt = nullptr;
    double* rf_field = nullptr;      // RFL x, y, z (+ one spare)

    // bonded term lists (sg_bonded_set), one per sg_bonded_kind: atoms
    // (I, J, K, L or -1) and (coeff, cos theta0, sin theta0, theta0)
    int bonded_n[6] = {0, 0, 0, 0, 0, 0};
    int4* bonded_atoms[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    float4* bonded_par[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};

    float4* mc_scratch = nullptr;    // barostat: saved positions, forces, torques (3 n)

    // host copies for the reporters: atom types (set_atom_type) and the
    // constraint list in its given order (0-based)
    std::vector<int> h_types;
    std::vector<int> h_bbi, h_bbj;
    std::vector<double> h_blen;

    // bond constraints (sg_set_constraints): constraints grouped by molecule
    // (connected component), each group in the reference's list order
    int con_n = 0;                   // NC
    int con_nmol = 0;
    int con_max_len = 0;             // constraints in the largest molecule
    int2* con_ij = nullptr;          // (I, J) 0-based
    float* con_len = nullptr;
    int* con_mol = nullptr;          // nmol + 1 offsets into con_ij
    unsigned char* con_moved = nullptr;   // per particle
    // molecules of at most 16 atoms run from shared memory: their atoms
    // (atom_off / atoms) and each constraint's atoms as local indices
    int con_nsmall = 0, con_nlarge = 0;
    int* con_small = nullptr;        // molecule ids, then the large ones (nmol in all)
    int* con_atom_off = nullptr;     // nmol + 1
    int* con_atoms = nullptr;
    int2* con_loc = nullptr;         // per constraint, local atom indices
    float4* pos_old = nullptr;       // RX_old .. RZ_old
    int* con_err = nullptr;          // [0] 1 + first failing constraint, [1] I, [2] J
    unsigned long long* con_stats = nullptr;   // see sg_constraint_stats

    // staging (pinned host) for uploads / downloads
    float4* h_stage = nullptr;
    size_t h_stage_bytes = 0;
    double* d_stage = nullptr;       // device FP64 staging for packing (16 n doubles)
    int sync_transfers = 1;          // uploads wait for completion (the host may free its arrays)

    // captured whole-step graph (sg_step)
    cudaGraphExec_t graph_exec = nullptr;
    // the same step for the launches after the first of an sg_step call: the
    // Nose-Hoover initial chain takes the kinetic sums the previous step's
    // final half stored (nothing can change the state between those launches)
    cudaGraphExec_t graph_exec_cont = nullptr;
    int step_sums_from_acc = 0;      // set while enqueuing that step
    // host calls that write the particle state bump state_version; sg_step
    // records it after its launches, so that the first launch of the next
    // call may take the stored sums only when nothing was written in between
    unsigned state_version = 0;
    unsigned step_clean_version = ~0u;
    int* step_dev = nullptr;         // device step counter used by the captured Langevin kernel
    const int* lgv_step_dev = nullptr;  // set while enqueuing a step: Langevin reads the counter here
    int lgv_rotations = 1;           // Langevin also thermostats rotation
    unsigned graph_epoch = 0;        // bumped whenever a buffer a captured graph uses is reallocated
    unsigned graph_epoch_captured = 0;
    int graph_kernels = 0;
    cudaStream_t aux_stream = nullptr;   // used to capture conditional graph bodies
    unsigned char step_cfg[256];     // copy of the sg_step_config the graph was captured with
    sg_pair_params step_pairs[3];    // pair stage of the step: cfg.pair, or one set per family
    int step_npairs = 1;
    int step_ready = 0;

    sg_nlist_state nl;

    // batched replicas (sg_create_replicas); rep.rep_of == nullptr otherwise
    RepDev rep;
    int nrep = 0;
    int fam_pstart[4] = {0, 0, 0, 0};  // particle ranges of the LJ / GB / ECP families
    int fam_rstart[4] = {0, 0, 0, 0};  // replica ranges of the families
    int launch_family = 0;             // family of the pair launch being enqueued
    std::map<long long, PairTune> tune;   // autotuned pair launch shapes by (kind, size bucket)
    void* rep_alloc = nullptr;         // one device allocation backing the tables
    std::vector<int> h_rep_off;        // host copies
    std::vector<double> h_rep_box;
    std::vector<int> h_rep_family;
};

// --------------------------------------------------------------- errors ----
int sg_fail(sg_ctx* ctx, int code, const char* fmt, ...);
int sg_cuda_check(sg_ctx* ctx, cudaError_t e, const char* what);
#define SG_CUDA(ctx, call)                                              \
    do {                                                                \
        cudaError_t _e = (call);                                        \
        if (_e != cudaSuccess) return sg_cuda_check((ctx), _e, #call);  \
    } while (0)
#define SG_LAUNCH_CHECK(ctx, what) SG_CUDA(ctx, cudaGetLastError())

// A host call wrote velocities, angular momenta, orientations or particle
// constants: the next captured step recomputes its kinetic sums.
inline void sg_state_touched(sg_ctx* ctx) { ctx->state_version++; }
int sg_ensure_partials(sg_ctx* ctx, int slots);
int sg_ensure_stage(sg_ctx* ctx, size_t bytes);
extern "C" int sg_ensure_dstage(sg_ctx* ctx);
int sg_grid_for(sg_ctx* ctx, const void* kernel, int block, size_t smem);

// ------------------------------------------------------- device helpers ----
SG_DEV float3 f3(float4 a) { return make_float3(a.x, a.y, a.z); }
SG_DEV float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
SG_DEV float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
SG_DEV float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
SG_DEV float3 operator*(float3 a, float s) { return make_float3(s * a.x, s * a.y, s * a.z); }
SG_DEV float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SG_DEV float3 cross3(float3 a, float3 b) {
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Minimum image with the reference's ANINT (round half away from zero).
SG_DEV float3 min_image(float3 d, float3 box, float3 inv_box, int periodic) {
    if (periodic) {
        d.x -= roundf(d.x * inv_box.x) * box.x;
        d.y -= roundf(d.y * inv_box.y) * box.y;
        d.z -= roundf(d.z * inv_box.z) * box.z;
    }
    return d;
}

// Shared block reduction of K doubles; the last block to finish adds the
// per-block partials, in block order, into acc[k] (deterministic). Must be
// called by every thread of the block. partials holds gridDim.x * K slots.
// Block sums from one value per warp (held by lane 0), then the grid sum in
// the block that arrives last. Returns true in that block (block-uniform).
// store: acc[k] = total instead of acc[k] += total (no zeroing pass needed).
template <int K>
__device__ bool block_finish_from_warps(const double (&wv)[K], double* partials, unsigned int* done, double* acc,
                                        double* acc_also, bool store = false) {
    __shared__ double sh[32][K];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) sh[warp][k] = wv[k];
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += sh[w][threadIdx.x];
        partials[(size_t)blockIdx.x * K + threadIdx.x] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int t = atomicAdd(done, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (last) {   // block-uniform
        __threadfence();
        // every thread sums a fixed strided subset of the block partials, then
        // a fixed tree: the order of additions does not depend on timing
        double s[K];
#pragma unroll
        for (int k = 0; k < K; ++k) s[k] = 0.0;
        for (unsigned int b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
#pragma unroll
            for (int k = 0; k < K; ++k) s[k] += ((volatile double*)partials)[(size_t)b * K + k];
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double x = s[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) sh[warp][k] = x;
        }
        __syncthreads();
        if (threadIdx.x < K) {
            double t = 0.0;
            for (int w = 0; w < nw; ++w) t += sh[w][threadIdx.x];
            if (store) acc[threadIdx.x] = t;
            else acc[threadIdx.x] += t;
            if (acc_also) acc_also[threadIdx.x] += t;
        }
        if (threadIdx.x == 0) *done = 0u;
    }
    return last;
}

// Per-thread FP64 values: warp sums by shuffles, then block_finish_from_warps.
template <int K>
__device__ bool block_reduce_finish(double (&v)[K], double* partials, unsigned int* done, double* acc,
                                    double* acc_also = nullptr, bool store = false) {
    double wv[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        wv[k] = x;
    }
    return block_finish_from_warps<K>(wv, partials, done, acc, acc_also, store);
}

// The same for per-thread FP32 sums (pair energies and virials): the warp
// level adds in double-float (error-free FP32 two-sums, ~48-bit significand)
// on the FP32 pipe, and FP64 takes over from one value per warp, so the
// result matches an FP64 sum of the FP32 terms to ~1e-14 relative while the
// FP64 pipe sees 1/32 of the additions.
// vlo (optional): low parts of per-thread double-float sums v + vlo.
template <int K>
__device__ bool block_reduce_finish_f(const float (&v)[K], double* partials, unsigned int* done, double* acc,
                                      double* acc_also = nullptr, const float* vlo = nullptr) {
    double w[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        float hi = v[k], lo = vlo ? vlo[k] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ho = __shfl_down_sync(0xffffffffu, hi, o);
            const float lo2 = __shfl_down_sync(0xffffffffu, lo, o);
            const float s = hi + ho;
            const float bb = s - hi;
            const float err = (hi - (s - bb)) + (ho - bb);
            hi = s;
            lo = lo + lo2 + err;
        }
        w[k] = (double)hi + (double)lo;   // used from lane 0
    }
    return block_finish_from_warps<K>(w, partials, done, acc, acc_also);
}

// --------------------------------------------------- internal entry points --
int sg_ecp_prepare(sg_ctx* ctx, const sg_pair_params* p, int need64);
int sg_gather_pair_floats(sg_ctx* ctx, const float* dev, int64_t k, float* out);
int sg_mlp_guess_tc_launch(sg_ctx* ctx, float* out);
int sg_nhc_step_initial(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t rot_chain,
                        int32_t rotations);
int sg_nhc_step_final(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t rot_chain,
                      int32_t rotations);
int sg_launch_pair_simple(sg_ctx* ctx, const sg_pair_params* p);
int sg_launch_pair_elec(sg_ctx* ctx, const sg_pair_params* p);
int sg_reaction_field_eval_async(sg_ctx* ctx);
int sg_constraints_free(sg_ctx* ctx);
int sg_nlist_box_changed(sg_ctx* ctx);   // cell grid for a new box (box scaling, barostat)
void sg_bonded_free(sg_ctx* ctx);
int sg_launch_pair_gb(sg_ctx* ctx, const sg_pair_params* p);
int sg_launch_pair_ecp(sg_ctx* ctx, const sg_pair_params* p);
int sg_nlist_free(sg_ctx* ctx);
int sg_nlist_enqueue_check(sg_ctx* ctx);   // rebuild request flag from the displacement test
int sg_nlist_enqueue_build(sg_ctx* ctx);   // the flag-gated build kernels
void sg_mlp_free(sg_ctx* ctx);
