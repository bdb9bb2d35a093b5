// Pair-parallel driver shared by every pair-potential kernel.
//
// The half list is flattened into (pair_i, pair_j) with rows in particle
// order, so the pairs of one particle i are contiguous. Each warp takes 32
// consecutive pairs; each lane evaluates one pair in the reference's
// orientation (I = pair_i < J = pair_j), then
//   * the J-side force and torque go out as one float4 atomic each,
//   * the I-side terms are summed across lanes with a segmented shuffle scan
//     (segments = runs of equal i), and the last lane of each run issues one
//     float4 atomic,
//   * PE and the pair virial r_ij . F_ij are summed per thread and per warp
//     in double-float (FP32 two-sums), then per block in FP64, and finished
//     deterministically by the last block (block_reduce_finish_f), so the
//     totals do not depend on which pairs a thread happened to evaluate.
// The grid is persistent (a multiple of the SM count); the pair count is read
// from device memory so the launch needs no host synchronisation.
#pragma once
#include <type_traits>

#include "sg_internal.cuh"

// Optional traits of a potential, with their defaults:
//   kQueueR (false): its range test hands r_ij to the in-range queue, and
//     eval_r takes it from there instead of gathering the positions again;
//   kExactFilter (true): in_range decides exactly as eval would. When false,
//     in_range is a superset test and eval makes the decision (and counts it).
template <class P, class = void>
struct QueueR : std::false_type {};
template <class P>
struct QueueR<P, std::void_t<decltype(P::kQueueR)>> : std::integral_constant<bool, P::kQueueR> {};
template <class P, class = void>
struct ExactFilter : std::true_type {};
template <class P>
struct ExactFilter<P, std::void_t<decltype(P::kExactFilter)>> : std::integral_constant<bool, P::kExactFilter> {};

//   kTwoClass (false): its range test returns a class (0 out of range, 1 in
//     range, 2 in range and near contact) and the near-contact pairs queue
//     separately for eval_r<true>, a more precise evaluation.
template <class P, class = void>
struct TwoClass : std::false_type {};
template <class P>
struct TwoClass<P, std::void_t<decltype(P::kTwoClass)>> : std::integral_constant<bool, P::kTwoClass> {};

struct PairOut {
    float3 f;    // force on I (FXIJ)
    float3 ti;   // torque on I (TXI)
    float3 tj;   // torque on J (TXJ)
    float pe;
    float vir;
    int act;     // the pair was inside the potential's range (counted for LJ / GB)
};

struct PairLaunch {
    const int* __restrict__ pair_i;
    const int* __restrict__ pair_j;
    const int* npairs;           // device: end of the (row-order) range
    const int* begin;            // device: start of the range, or nullptr for 0
    // Replica contexts keep each replica's pairs in a section of their own:
    // the pair at row-order index v of replica r sits at
    // sec[r] + v - row_off[rep_off[r]]. sec == nullptr: storage is row order.
    const int* row_off;
    const int* rep_off;
    const long long* sec;
    const int* chunk_rep;        // replica holding pair index 32 c, for every chunk c
    int nrep;
    float4* force;
    float4* torque;
    double* partials;
    unsigned int* done;
    double* acc;                 // per-call sums: acc[0] += PE, acc[1] += virial
    double* acc_total;           // running sums since the last zero_forces
    unsigned long long* stats;   // solver statistics (ECP) or listed / in-range counts (LJ, GB)
    // two-pass filtered launch (k_pair_compact): pair_i / pair_j are the
    // compacted pairs, tmap[v] the list storage index of compacted pair v, and
    // the block that finishes last zeroes *count_reset (the compacted count)
    const int* tmap;
    int* count_reset;
};

// Storage index and particles of lane `lane`'s pair in the 32-pair chunk that
// starts at row-order index `base`; pairs outside [b0, np) are invalid.
SG_DEV void pair_fetch(const PairLaunch& L, int base, int lane, int np, int b0, int& t, int& i, int& j,
                       bool& valid) {
    const int v = base + lane;
    valid = v < np && v >= b0;
    t = v;
    i = -1;
    j = 0;
    if (valid) {
        if (L.sec) {
            int r = L.chunk_rep[base >> 5];
            while (r + 1 < L.nrep && L.row_off[L.rep_off[r + 1]] <= v) ++r;
            t = (int)(L.sec[r] + (long long)(v - L.row_off[L.rep_off[r]]));
        }
        i = L.pair_i[t];
        j = L.pair_j[t];
        if (L.tmap) t = L.tmap[t];
    }
}

SG_DEV void atomic_add_f3(float4* p, float3 v) {
    atomicAdd(p, make_float4(v.x, v.y, v.z, 0.f));
}

template <bool TORQUE>
SG_DEV void segmented_scatter_i(const PairLaunch& L, int i, float3 f, float3 t) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int io = __shfl_up_sync(0xffffffffu, i, o);
        float fx = __shfl_up_sync(0xffffffffu, f.x, o);
        float fy = __shfl_up_sync(0xffffffffu, f.y, o);
        float fz = __shfl_up_sync(0xffffffffu, f.z, o);
        float tx = 0.f, ty = 0.f, tz = 0.f;
        if (TORQUE) {
            tx = __shfl_up_sync(0xffffffffu, t.x, o);
            ty = __shfl_up_sync(0xffffffffu, t.y, o);
            tz = __shfl_up_sync(0xffffffffu, t.z, o);
        }
        if (lane >= o && io == i) {
            f.x += fx; f.y += fy; f.z += fz;
            if (TORQUE) { t.x += tx; t.y += ty; t.z += tz; }
        }
    }
    int inext = __shfl_down_sync(0xffffffffu, i, 1);
    bool last = (lane == 31) || (inext != i);
    // a run of pairs that all lay out of range sums to exact zeros: no atomic
    const bool zero = f.x == 0.f && f.y == 0.f && f.z == 0.f && (!TORQUE || (t.x == 0.f && t.y == 0.f && t.z == 0.f));
    if (last && i >= 0 && !zero) {
        atomic_add_f3(&L.force[i], f);
        if (TORQUE) atomic_add_f3(&L.torque[i], t);
    }
}

#define SG_NSTATS 32
#define SG_PAIR_MAX_BLOCK 256

// Per-thread double-float sums of the pair energy and virial.
struct EnergySums {
    float pe = 0.f, pe_lo = 0.f, vir = 0.f, vir_lo = 0.f;
    SG_DEV void add(float p, float v) {
        float s = pe + p, bb = s - pe;
        pe_lo += (pe - (s - bb)) + (p - bb);
        pe = s;
        s = vir + v;
        bb = s - vir;
        vir_lo += (vir - (s - bb)) + (v - bb);
        vir = s;
    }
};

// One pair per lane, evaluated and scattered (all 32 lanes call it).
// i, j: the pair's particles (loaded by the caller; ignored when !valid).
// COUNT: 0 nothing, 1 listed and in-range pairs, 2 in-range pairs only.
// HAS_R: r_ij comes from the in-range queue (QueueR potentials).
// PRECISE: the near-contact class of a kTwoClass potential.
template <class Pot, int COUNT, bool HAS_R = false, bool PRECISE = false>
SG_DEV void pair_process(const PairLaunch& L, const Pot& pot, int t, int i, int j, bool valid, EnergySums& es,
                         unsigned long long* sh_stats, float3 rq = make_float3(0.f, 0.f, 0.f)) {
    const int lane = threadIdx.x & 31;
    PairOut o;
    o.f = make_float3(0.f, 0.f, 0.f);
    o.ti = o.f;
    o.tj = o.f;
    o.pe = 0.f;
    o.vir = 0.f;
    o.act = 0;
    if (!valid) {
        i = -1;
        j = 0;
    }
    // called by every lane (warp-cooperative potentials need all 32)
    if constexpr (HAS_R && TwoClass<Pot>::value)
        pot.template eval_r<PRECISE>(valid, valid ? i : 0, j, rq, o);
    else if constexpr (HAS_R)
        pot.eval_r(valid, valid ? i : 0, j, rq, o);
    else
        pot.eval(valid, valid ? i : 0, j, t, o, sh_stats);
    if (COUNT) {
        // stats[0] listed pairs, stats[1] pairs inside the range
        const unsigned va = __ballot_sync(0xffffffffu, valid), ac = __ballot_sync(0xffffffffu, o.act != 0);
        if (lane == 0) {
            if (COUNT == 1) atomicAdd(&sh_stats[0], (unsigned long long)__popc(va));
            if (ac) atomicAdd(&sh_stats[1], (unsigned long long)__popc(ac));
        }
    }
    if (valid && (!Pot::kCountActive || o.act)) {   // out-of-range pairs add nothing
        atomic_add_f3(&L.force[j], make_float3(-o.f.x, -o.f.y, -o.f.z));
        if (Pot::kTorque) atomic_add_f3(&L.torque[j], o.tj);
    }
    es.add(o.pe, o.vir);
    segmented_scatter_i<Pot::kTorque>(L, i, o.f, o.ti);
}

// Per-warp queues of in-range pairs for the filtered kernels: a cheap range
// test runs on every listed pair first; the pairs in range queue up (in list
// order, so rows stay contiguous) and are evaluated 32 at a time, so no lane
// idles on an out-of-range pair. kTwoClass potentials keep a second queue for
// their near-contact class. Slots: storage index, i, j [, r_ij]; 64 per queue.
template <class Pot>
struct PairQueues {
    static constexpr bool kQR = QueueR<Pot>::value;
    static constexpr bool kExact = ExactFilter<Pot>::value;
    static constexpr bool k2 = TwoClass<Pot>::value;
    static constexpr int kQW = kQR ? 6 : 3;   // words per slot
    static constexpr int kNQ = k2 ? 2 : 1;    // queues per warp
    static constexpr int kWords = 64 * kQW * kNQ;   // shared words per warp
    static constexpr int kCnt = (Pot::kCountActive && !kExact) ? 2 : 0;
    int* qbase;   // this warp's queues: t at +0, i at +64, j at +128, r_ij x, y, z at +192, +256, +320
    int qn[2];
    int lane;

    SG_DEV void init(int* warp_words) {
        qbase = warp_words;
        qn[0] = qn[1] = 0;
        lane = threadIdx.x & 31;
    }
    // queue k: append this lane's pair when keep (list order kept)
    SG_DEV void push(int k, bool keep, int t, int i, int j, float3 rr) {
        int* q = qbase + k * 64 * kQW;
        const unsigned km = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const int slot = qn[k] + __popc(km & ((1u << lane) - 1u));
            q[slot] = t;
            q[64 + slot] = i;
            q[128 + slot] = j;
            if constexpr (kQR) {
                float* qr = reinterpret_cast<float*>(q + 192);
                qr[slot] = rr.x;
                qr[64 + slot] = rr.y;
                qr[128 + slot] = rr.z;
            }
        }
        qn[k] += __popc(km);
        __syncwarp();
    }
    // queue K: evaluate its first 32 pairs (or the last n < 32) and shift the rest down
    template <int K>
    SG_DEV void drain(int n, const PairLaunch& L, const Pot& pot, EnergySums& es, unsigned long long* sh_stats) {
        int* q = qbase + K * 64 * kQW;
        [[maybe_unused]] float* qr = reinterpret_cast<float*>(q + 192);
        const bool ok = lane < n;
        const int tq = ok ? q[lane] : 0, iq = ok ? q[64 + lane] : 0, jq = ok ? q[128 + lane] : 0;
        float3 rq = make_float3(0.f, 0.f, 0.f);
        if constexpr (kQR)
            if (ok) rq = make_float3(qr[lane], qr[64 + lane], qr[128 + lane]);
        __syncwarp();
        if (n == 32 && lane < qn[K] - 32) {
            q[lane] = q[32 + lane];
            q[64 + lane] = q[96 + lane];
            q[128 + lane] = q[160 + lane];
            if constexpr (kQR) {
                qr[lane] = qr[32 + lane];
                qr[64 + lane] = qr[96 + lane];
                qr[128 + lane] = qr[160 + lane];
            }
        }
        __syncwarp();
        qn[K] -= n;
        pair_process<Pot, kCnt, kQR, K == 1>(L, pot, tq, iq, jq, ok, es, sh_stats, rq);
    }
    // one listed pair per lane: range test, counters, queue, evaluate full batches
    SG_DEV void feed(const PairLaunch& L, const Pot& pot, int t, int i, int j, bool valid, EnergySums& es,
                     unsigned long long* sh_stats) {
        float3 rr = make_float3(0.f, 0.f, 0.f);
        int cls;
        if constexpr (k2)
            cls = valid ? pot.in_range_r(i, j, rr) : 0;
        else if constexpr (kQR)
            cls = (valid && pot.in_range_r(i, j, rr)) ? 1 : 0;
        else
            cls = (valid && pot.in_range(i, j)) ? 1 : 0;
        const unsigned vm = __ballot_sync(0xffffffffu, valid), km = __ballot_sync(0xffffffffu, cls != 0);
        if (Pot::kCountActive && lane == 0) {
            atomicAdd(&sh_stats[0], (unsigned long long)__popc(vm));
            if (kExact && km) atomicAdd(&sh_stats[1], (unsigned long long)__popc(km));
        }
        if constexpr (k2) {   // stats[3]: pairs of the near-contact class
            const unsigned k2m = __ballot_sync(0xffffffffu, cls == 2);
            if (lane == 0 && k2m) atomicAdd(&sh_stats[3], (unsigned long long)__popc(k2m));
        }
        if constexpr (Pot::kStats) {
            // solver statistics (ECP): a pair turned away counts as listed with
            // no solve (iteration bin 0), and the potential is told of it
            const unsigned rm = vm & ~km;
            if (lane == 0 && rm) {
                atomicAdd(&sh_stats[0], (unsigned long long)__popc(rm));
                atomicAdd(&sh_stats[4], (unsigned long long)__popc(rm));
            }
            if (valid && cls == 0) pot.filtered_out(t);
        }
        push(0, cls == 1, t, i, j, rr);
        if constexpr (k2) push(1, cls == 2, t, i, j, rr);
        if (qn[0] >= 32) drain<0>(32, L, pot, es, sh_stats);
        if constexpr (k2)
            if (qn[1] >= 32) drain<1>(32, L, pot, es, sh_stats);
    }
    // the queues' last pairs (qn is warp-uniform)
    SG_DEV void flush(const PairLaunch& L, const Pot& pot, EnergySums& es, unsigned long long* sh_stats) {
        if (qn[0] > 0) drain<0>(qn[0], L, pot, es, sh_stats);
        if constexpr (k2)
            if (qn[1] > 0) drain<1>(qn[1], L, pot, es, sh_stats);
    }
};

// FILTER: the range test and per-warp queues of PairQueues.
template <class Pot, bool FILTER>
__global__ void __launch_bounds__(SG_PAIR_MAX_BLOCK, FILTER ? Pot::kMinBlocksFiltered : Pot::kMinBlocks)
    k_pair(PairLaunch L, Pot pot) {
    using Q = PairQueues<Pot>;
    __shared__ unsigned long long sh_stats[SG_NSTATS];
    __shared__ int sh_queue[FILTER ? (SG_PAIR_MAX_BLOCK / 32) * Q::kWords : 1];
    constexpr bool kSh = Pot::kStats || Pot::kCountActive;
    if (kSh) {
        for (int k = threadIdx.x; k < SG_NSTATS; k += blockDim.x) sh_stats[k] = 0ull;
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int np = *L.npairs;
    const int b0 = L.begin ? *L.begin : 0;
    EnergySums es;
    Q q;
    q.init(sh_queue + (FILTER ? (threadIdx.x >> 5) * Q::kWords : 0));
    // replica sections: warps walk whole 32-pair chunks, whose first replica is tabulated
    const int bstart = L.sec ? (b0 & ~31) : b0;
    const int stride = nwarps * 32;
    int tn, in_, jn;
    bool vn;
    pair_fetch(L, bstart + gwarp * 32, lane, np, b0, tn, in_, jn, vn);
    for (int base = bstart + gwarp * 32; base < np; base += stride) {
        const int t = tn, i = in_, j = jn;
        const bool valid = vn;
        if (base + stride < np) pair_fetch(L, base + stride, lane, np, b0, tn, in_, jn, vn);   // next indices in flight
        if constexpr (!FILTER)
            pair_process<Pot, Pot::kCountActive ? 1 : 0>(L, pot, t, i, j, valid, es, sh_stats);
        else
            q.feed(L, pot, t, i, j, valid, es, sh_stats);
    }
    if constexpr (FILTER) q.flush(L, pot, es, sh_stats);
    // the pairs are done: a kernel launched after this one with programmatic
    // serialisation (the final half step) may start loading what this one
    // does not write
    pdl_trigger();
    if (kSh) {
        __syncthreads();
        for (int k = threadIdx.x; k < SG_NSTATS; k += blockDim.x)
            if (sh_stats[k]) atomicAdd(&L.stats[k], sh_stats[k]);
    }
    const float e[2] = {es.pe, es.vir}, elo[2] = {es.pe_lo, es.vir_lo};
    if (block_reduce_finish_f<2>(e, L.partials, L.done, L.acc, L.acc_total, elo) && L.count_reset &&
        threadIdx.x == 0)
        *L.count_reset = 0;   // every block has read the compacted count
}

// First pass of the two-pass filtered launch: the range test of every listed
// pair, and the pairs that pass written in list order to (tmap, ci, cj) from
// *count on, one atomic per block and round (a round: blockDim.x * P
// consecutive pairs, P per thread, whose index loads and gathers are in
// flight together). A round's pairs stay together and in row order, so the
// second pass, k_pair over the compacted pairs, keeps the segmented scatter's
// locality and every lane of its warps busy. Pairs turned away are counted as
// listed with no solve (stats[0], stats[4]) and handed to the potential's
// filtered_out. 256 threads: the round's 8 x P warp counts fit one warp scan.
#ifndef SG_COMPACT_P
#define SG_COMPACT_P 4
#endif
template <class Pot>
__global__ void __launch_bounds__(256) k_pair_compact(PairLaunch L, Pot pot, int* __restrict__ count,
                                                     int* __restrict__ tmap, int* __restrict__ ci,
                                                     int* __restrict__ cj) {
    constexpr int P = SG_COMPACT_P;
    static_assert(8 * P <= 32, "one warp scans the round's counts");
    __shared__ int sh_n[8 * P];
    __shared__ unsigned long long sh_away;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) sh_away = 0ull;
    const int np = *L.npairs;
    unsigned away = 0;
    const int per_round = 256 * P;
    for (int base0 = blockIdx.x * per_round; base0 < np; base0 += gridDim.x * per_round) {   // block-uniform
        int t[P], i[P], j[P];
        bool valid[P];
#pragma unroll
        for (int k = 0; k < P; ++k) pair_fetch(L, base0 + (warp * P + k) * 32, lane, np, 0, t[k], i[k], j[k], valid[k]);
        // the P range tests first, with no vote or store between them
        bool keep[P];
#pragma unroll
        for (int k = 0; k < P; ++k) keep[k] = valid[k] && pot.in_range(i[k], j[k]);
        unsigned km[P];
#pragma unroll
        for (int k = 0; k < P; ++k) {
            km[k] = __ballot_sync(full, keep[k]);
            const unsigned vm = __ballot_sync(full, valid[k]);
            if (valid[k] && !keep[k]) pot.filtered_out(t[k]);
            away += __popc(vm & ~km[k]);
            if (lane == 0) sh_n[warp * P + k] = __popc(km[k]);
        }
        __syncthreads();
        if (warp == 0) {   // exclusive scan of the 8 P counts, one atomic for the round
            const int c = lane < 8 * P ? sh_n[lane] : 0;
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(full, incl, o);
                if (lane >= o) incl += y;
            }
            const int total = __shfl_sync(full, incl, 31);
            int base = 0;
            if (lane == 0 && total) base = atomicAdd(count, total);
            base = __shfl_sync(full, base, 0);
            if (lane < 8 * P) sh_n[lane] = base + incl - c;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < P; ++k) {
            if (km[k] & (1u << lane)) {
                const int slot = sh_n[warp * P + k] + __popc(km[k] & ((1u << lane) - 1u));
                tmap[slot] = t[k];
                ci[slot] = i[k];
                cj[slot] = j[k];
            }
        }
        __syncthreads();   // sh_n is rewritten by the next round
    }
    if (lane == 0 && away) atomicAdd(&sh_away, (unsigned long long)away);
    __syncthreads();
    if (threadIdx.x == 0 && sh_away) {
        atomicAdd(&L.stats[0], sh_away);
        atomicAdd(&L.stats[4], sh_away);
    }
}

// Launch shape of the pair kernels: block size and the range filter. The
// autotuner (sg_pair_autotune) times the variants on the live list and
// stores the fastest per (kind, size bucket); untuned kinds use defaults.
PairTune sg_pair_tune_for(sg_ctx* ctx, int kind, bool filterable);

template <class Pot, bool FILTER>
int launch_pair_v(sg_ctx* ctx, PairLaunch L, Pot pot, int block) {
    pot.prefiltered = (FILTER && ExactFilter<Pot>::value) ? 1 : 0;
    const void* fn = (const void*)k_pair<Pot, FILTER>;
    int grid = sg_grid_for(ctx, fn, block, 0);
    int64_t max_useful = (ctx->nl.pair_capacity + block - 1) / block;
    if (grid > max_useful) grid = (int)std::max<int64_t>(1, max_useful);
    if (int rc = sg_ensure_partials(ctx, grid * 2)) return rc;
    L.partials = ctx->partials;
    k_pair<Pot, FILTER><<<grid, block, 0, ctx->stream>>>(L, pot);
    SG_LAUNCH_CHECK(ctx, "k_pair");
    return SG_OK;
}

// The list walk of this context's pair kernels: the whole list, or in a
// replica context the rows of the launch family's replicas.
inline PairLaunch make_pair_launch(sg_ctx* ctx) {
    PairLaunch L;
    L.pair_i = ctx->nl.pair_i;
    L.pair_j = ctx->nl.pair_j;
    L.npairs = ctx->nl.dev_flags + 2;
    L.begin = nullptr;
    L.row_off = ctx->nl.row_off;
    L.rep_off = ctx->rep.off;
    L.sec = nullptr;
    L.chunk_rep = nullptr;
    L.nrep = ctx->nrep;
    if (ctx->nrep) {
        // pairs of one potential family: rows of the family's replicas
        const int f = ctx->launch_family;
        L.begin = ctx->nl.row_off + ctx->fam_pstart[f];
        L.npairs = ctx->nl.row_off + ctx->fam_pstart[f + 1];
        L.sec = ctx->nl.rep_pad_off;
        L.chunk_rep = ctx->nl.chunk_rep;
    }
    L.force = ctx->force;
    L.torque = ctx->torque;
    L.done = ctx->done_counter;
    L.acc = ctx->acc + 4;
    L.acc_total = ctx->acc;
    L.stats = ctx->stats;
    L.partials = nullptr;
    L.tmap = nullptr;
    L.count_reset = nullptr;
    return L;
}

// The two-pass filtered launch of a potential with a superset range test
// (single systems): k_pair_compact, then k_pair over the compacted pairs. The
// compacted arrays hold up to the list's pair capacity.
template <class Pot>
int launch_pair_two_pass(sg_ctx* ctx, Pot pot, int block) {
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "pair forces need sg_nlist_init first");
    PairLaunch L = make_pair_launch(ctx);
    const int64_t cap = ctx->nl.pair_capacity;
    if (ctx->pair_surv_cap < cap) {
        ctx->graph_epoch++;
        if (ctx->pair_surv) cudaFree(ctx->pair_surv);
        ctx->pair_surv = nullptr;
        ctx->pair_surv_cap = 0;
        SG_CUDA(ctx, cudaMalloc(&ctx->pair_surv, sizeof(int) * (size_t)(32 + 3 * cap)));
        SG_CUDA(ctx, cudaMemsetAsync(ctx->pair_surv, 0, sizeof(int) * 32, ctx->stream));
        ctx->pair_surv_cap = cap;
    }
    int* count = ctx->pair_surv;
    int* tmap = count + 32;
    int* ci = tmap + cap;
    int* cj = ci + cap;
    pot.prefiltered = 0;
    int grid = sg_grid_for(ctx, (const void*)k_pair_compact<Pot>, 256, 0);
    const int64_t rounds = (cap + 256 * SG_COMPACT_P - 1) / (256 * SG_COMPACT_P);
    if (grid > rounds) grid = (int)std::max<int64_t>(1, rounds);
    k_pair_compact<Pot><<<grid, 256, 0, ctx->stream>>>(L, pot, count, tmap, ci, cj);
    SG_LAUNCH_CHECK(ctx, "k_pair_compact");
    L.pair_i = ci;
    L.pair_j = cj;
    L.npairs = count;
    L.tmap = tmap;
    L.count_reset = count;
    return launch_pair_v<Pot, false>(ctx, L, pot, block);
}

// Launch helper: persistent grid sized from occupancy.
template <class Pot>
int launch_pair(sg_ctx* ctx, Pot pot, int kind) {
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "pair forces need sg_nlist_init first");
    PairLaunch L = make_pair_launch(ctx);
    const PairTune tune = sg_pair_tune_for(ctx, kind, Pot::kFilterable);
    if (Pot::kFilterable && tune.filter) return launch_pair_v<Pot, Pot::kFilterable>(ctx, L, pot, tune.block);
    return launch_pair_v<Pot, false>(ctx, L, pot, tune.block);
}

struct BoxF {
    float3 box, inv_box;
    float3 box_lo;              // box - (float)box: with box, the FP64 box to ~1e-15
    int periodic;
    const int* rep_of;          // batched replicas: per-particle replica, else nullptr
    const float4* rbox;
    const float4* rinv;
    const float4* rbox_lo;
};

inline BoxF make_boxf(const sg_ctx* ctx) {
    BoxF b;
    b.rep_of = ctx->rep.rep_of;
    b.rbox = ctx->rep.box;
    b.rinv = ctx->rep.inv_box;
    b.rbox_lo = ctx->rep.box_lo;
    b.box_lo = make_float3((float)(ctx->box[0] - (double)(float)ctx->box[0]),
                           (float)(ctx->box[1] - (double)(float)ctx->box[1]),
                           (float)(ctx->box[2] - (double)(float)ctx->box[2]));
    b.box = make_float3((float)ctx->box[0], (float)ctx->box[1], (float)ctx->box[2]);
    b.inv_box = make_float3((float)(1.0 / ctx->box[0]), (float)(1.0 / ctx->box[1]), (float)(1.0 / ctx->box[2]));
    b.periodic = ctx->periodic;
    return b;
}

// r_ij = a - c by the minimum image of the box of i (BoxF).
SG_DEV float3 pair_rij_of(float3 a, float3 c, int i, const BoxF& b) {
    if (b.rep_of) {
        const int r = b.rep_of[i];
        const float4 bx = b.rbox[r], ib = b.rinv[r];
        return min_image(make_float3(a.x - c.x, a.y - c.y, a.z - c.z), make_float3(bx.x, bx.y, bx.z),
                         make_float3(ib.x, ib.y, ib.z), 1);
    }
    return min_image(make_float3(a.x - c.x, a.y - c.y, a.z - c.z), b.box, b.inv_box, b.periodic);
}

// Two float4 from one 32-byte aligned address in a single 256-bit load
// (read-only path): a gather of 32 bytes per lane in one request.
SG_DEV void ld_f4x2(const float4* __restrict__ p, float4& a, float4& c) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(c.x), "=f"(c.y), "=f"(c.z), "=f"(c.w)
        : "l"(p));
}

SG_DEV float3 pair_rij(const float4* __restrict__ pos, int i, int j, const BoxF& b) {
    float4 a = pos[i], c = pos[j];
    if (b.rep_of) {
        // pairs never cross replicas: the replica of i gives the box
        const int r = b.rep_of[i];
        const float4 bx = b.rbox[r], ib = b.rinv[r];
        return min_image(make_float3(a.x - c.x, a.y - c.y, a.z - c.z), make_float3(bx.x, bx.y, bx.z),
                         make_float3(ib.x, ib.y, ib.z), 1);
    }
    return min_image(make_float3(a.x - c.x, a.y - c.y, a.z - c.z), b.box, b.inv_box, b.periodic);
}

// pair_rij that also returns the product of the two charges (pos.w).
SG_DEV float3 pair_rij_q(const float4* __restrict__ pos, int i, int j, const BoxF& b, float& qq) {
    const float4 a = pos[i], c = pos[j];
    qq = a.w * c.w;
    const float3 d = make_float3(a.x - c.x, a.y - c.y, a.z - c.z);
    if (b.rep_of) {
        const int r = b.rep_of[i];
        const float4 bx = b.rbox[r], ib = b.rinv[r];
        return min_image(d, make_float3(bx.x, bx.y, bx.z), make_float3(ib.x, ib.y, ib.z), 1);
    }
    return min_image(d, b.box, b.inv_box, b.periodic);
}

// One component of the minimum image, to about 1e-12 absolute: the FP32
// difference a - c with its exact rounding error (two-sum), the image shift
// n * (box_hi + box_lo) applied to each part (for n = +-1 the difference is
// within a factor two of box_hi, so d - n box_hi is exact). Without it, pairs
// across the boundary carry the rounding of a - c (~ulp(box)/2) and of the
// FP32 box.
SG_DEV float min_image_precise(float a, float c, float L, float iL, float Llo, int periodic) {
    const float d = a - c;
    const float bb = d - a;
    const float e = (a - (d - bb)) + (-c - bb);
    if (!periodic) return d + e;
    const float n = roundf(d * iL);
    return __fsub_rn(d, n * L) + (e - n * Llo);
}

// r_ij = a - c by the minimum image of the box of i, to ~1e-12 absolute
// (min_image_precise), from positions already loaded.
SG_DEV float3 pair_rij_of_precise(float3 a, float3 c, int i, const BoxF& b) {
    float3 L = b.box, iL = b.inv_box, lo = b.box_lo;
    int per = b.periodic;
    if (b.rep_of) {
        const int r = b.rep_of[i];
        const float4 bx = b.rbox[r], ib = b.rinv[r], bl = b.rbox_lo[r];
        L = make_float3(bx.x, bx.y, bx.z);
        iL = make_float3(ib.x, ib.y, ib.z);
        lo = make_float3(bl.x, bl.y, bl.z);
        per = 1;
    }
    return make_float3(min_image_precise(a.x, c.x, L.x, iL.x, lo.x, per),
                       min_image_precise(a.y, c.y, L.y, iL.y, lo.y, per),
                       min_image_precise(a.z, c.z, L.z, iL.z, lo.z, per));
}

// pair_rij for the contact-distance potentials (ECP): see min_image_precise.
SG_DEV float3 pair_rij_precise(const float4* __restrict__ pos, int i, int j, const BoxF& b) {
    const float4 a = pos[i], c = pos[j];
    float3 L = b.box, iL = b.inv_box, lo = b.box_lo;
    int per = b.periodic;
    if (b.rep_of) {
        const int r = b.rep_of[i];
        const float4 bx = b.rbox[r], ib = b.rinv[r], bl = b.rbox_lo[r];
        L = make_float3(bx.x, bx.y, bx.z);
        iL = make_float3(ib.x, ib.y, ib.z);
        lo = make_float3(bl.x, bl.y, bl.z);
        per = 1;
    }
    return make_float3(min_image_precise(a.x, c.x, L.x, iL.x, lo.x, per),
                       min_image_precise(a.y, c.y, L.y, iL.y, lo.y, per),
                       min_image_precise(a.z, c.z, L.z, iL.z, lo.z, per));
}

// Reciprocal by the approximate instruction (at most 1 ulp from 1/x for
// normal x, PTX rcp.approx.ftz.f32): a division costs a dozen instructions,
// this one. Used where a 1-ulp quotient is far inside the force tolerance.
SG_DEV float fast_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// x^n by repeated multiplication, left to right (the rounding of a loop of
// products); n is uniform across the warp. Up to n = 4 the products are
// selected instead of looped.
SG_DEV float ipowf(float x, int n) {
    const float x2 = x * x, x3 = x2 * x, x4 = x3 * x;
    if (n <= 4) return n <= 0 ? 1.f : n == 1 ? x : n == 2 ? x2 : n == 3 ? x3 : x4;
    float r = x4;
    for (int k = 4; k < n; ++k) r *= x;
    return r;
}

// 1/sqrt(x) by the approximate instruction (PTX rsqrt.approx.ftz.f32): for
// superset range tests that carry a slack far above its error.
SG_DEV float fast_rsqrt(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
