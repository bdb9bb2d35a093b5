// The whole timestep as one CUDA graph (sg_step). Every kernel of the step is
// gated on device-side state (list rebuild request, pair count, step counter),
// so a captured step replays without any host decision or synchronisation.
#include <cmath>
#include <vector>

#include "sg_internal.cuh"
#include "step_epi.cuh"

namespace {

__global__ void k_step_incr(int* step) { *step += 1; }

__global__ void k_set_rebuild_condition(cudaGraphConditionalHandle h, const int* flags) {
    cudaGraphSetConditional(h, flags[0] ? 1u : 0u);
}

// List maintenance inside a captured step: the displacement test runs every
// step; a single system with cells then runs the cooperative build kernel,
// which returns at once without a request; a replica context's build kernels
// sit in the body of a conditional graph node that executes only when a
// rebuild was requested. Outside capture the flag-gated kernels are enqueued.
// checked: the displacement test already ran (in the fused initial half step).
int enqueue_list_update(sg_ctx* ctx, bool flat, bool checked) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t nd = 0;
    SG_CUDA(ctx, cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, &edges, &nd));
    // a single system with cells rebuilds in one cooperative kernel that exits
    // at once without a request: no conditional node
    const bool coop = ctx->nl.use_cells && !ctx->nrep;
    if (flat || coop || st != cudaStreamCaptureStatusActive)
        return checked ? sg_nlist_enqueue_build(ctx) : sg_nlist_update(ctx);
    if (!checked)
        if (int rc = sg_nlist_enqueue_check(ctx)) return rc;
    cudaGraphConditionalHandle h;
    SG_CUDA(ctx, cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, &edges, &nd));
    SG_CUDA(ctx, cudaGraphConditionalHandleCreate(&h, cg, 0, cudaGraphCondAssignDefault));
    k_set_rebuild_condition<<<1, 1, 0, ctx->stream>>>(h, ctx->nl.dev_flags);
    SG_LAUNCH_CHECK(ctx, "k_set_rebuild_condition");
    SG_CUDA(ctx, cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, &edges, &nd));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    SG_CUDA(ctx, cudaGraphAddNode(&node, cg, deps, edges, nd, &cp));
    SG_CUDA(ctx, cudaStreamUpdateCaptureDependencies(ctx->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if (!ctx->aux_stream) SG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
    SG_CUDA(ctx, cudaStreamBeginCaptureToGraph(ctx->aux_stream, body, nullptr, nullptr, 0,
                                               cudaStreamCaptureModeThreadLocal));
    cudaStream_t main = ctx->stream;
    ctx->stream = ctx->aux_stream;
    int rc = sg_nlist_enqueue_build(ctx);
    ctx->stream = main;
    cudaGraph_t out = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->aux_stream, &out);
    if (rc) return rc;
    if (e != cudaSuccess) return sg_cuda_check(ctx, e, "capture of the rebuild body");
    return SG_OK;
}

// Whether the step can run in its fused form (four kernels and the rebuild
// node), and which per-particle prep its initial half step writes: the
// Langevin and standard Nose-Hoover integrators without constraints; the
// prep when the pair sets are all ECP kinds with a Newton solver, or all
// Gay-Berne kinds, with one exponent mu.
void plan_fusion(sg_ctx* ctx, const sg_step_config& c) {
    ctx->step_fused = 0;
    ctx->step_prep_kind = SG_PREP_NONE;
    if ((c.flags & SG_STEP_CONSTRAINTS) || !(c.integrator == SG_INT_LANGEVIN || c.integrator == SG_INT_NH)) return;
    ctx->step_fused = 1;
    bool ecp = false, gb = false, other_ecp = false, same_mu = true;
    int mu = -1;
    for (int k = 0; k < ctx->step_npairs; ++k) {
        const sg_pair_params& p = ctx->step_pairs[k];
        int m;
        if (p.kind >= SG_ECP) {
            ecp = true;
            if (p.solver == SG_SOLVER_BRENT_COMPAT) other_ecp = true;
            m = (p.mu == 0 && p.nu == 0) ? 2 : p.mu;
        } else if (p.kind >= SG_GB) {
            gb = true;
            m = (p.mu == 0 && p.nu == 0) ? 1 : p.mu;
        } else {
            continue;
        }
        if (mu >= 0 && m != mu) same_mu = false;
        mu = m;
    }
    if (!same_mu || mu < 1 || (ecp && gb) || other_ecp) return;
    if (ecp) ctx->step_prep_kind = SG_PREP_ECP;
    if (gb) ctx->step_prep_kind = SG_PREP_GB;
    ctx->step_prep_muinv = 1.f / (float)mu;
}

// An event-record node when the stream is being captured (a plain record
// there would only mark a capture dependency), an ordinary record otherwise.
void record_event(cudaEvent_t e, cudaStream_t s) { cudaEventRecordWithFlags(e, s, cudaEventRecordExternal); }

// ev (optional): 6 events recorded before the initial half step, the list
// update, the force zeroing, the pair stage, the final half step and the
// step counter (eager steps only; sg_step_stage_times).
// cont: a step that follows another step of the same sg_step call (its
// Nose-Hoover initial chain reads the sums that step stored; cont_eligible).
int enqueue_step(sg_ctx* ctx, const sg_step_config& c, cudaEvent_t* ev = nullptr, bool cont = false) {
    const double dt = c.dt;
    ctx->lgv_step_dev = ctx->step_dev;
    ctx->lgv_rotations = c.rotations;
    plan_fusion(ctx, c);
    ctx->step_sums_from_acc = cont ? 1 : 0;
    ctx->step_events = ev != nullptr;
    const bool fused = ctx->step_fused != 0;
    int rc = SG_OK;
    if (ev) record_event(ev[0], ctx->stream);
    const bool con = (c.flags & SG_STEP_CONSTRAINTS) != 0;
    if (con) rc = sg_constraints_save(ctx);
    if (!rc) switch (c.integrator) {
        case SG_INT_NVE: rc = sg_vv_initial(ctx, dt); if (!rc && c.rotations) rc = sg_qq_initial(ctx, dt); break;
        case SG_INT_LANGEVIN:
            rc = sg_lgv_initial(ctx, dt, 0, c.damping, c.target_temp, c.has_key ? c.key : nullptr);
            break;
        case SG_INT_NH:   // standard chain: fused kernels, same arithmetic as nht + qq
            rc = sg_nhc_step_initial(ctx, dt, c.target_temp, c.coupling, c.rot_chain, c.rotations);
            break;
        case SG_INT_NH_REF:
            rc = sg_nht_initial(ctx, dt, c.target_temp, c.coupling, 0, 0);
            if (!rc && c.rotations) rc = sg_qq_initial(ctx, dt);
            break;
        default: rc = sg_fail(ctx, SG_EINVAL, "unknown integrator %d", c.integrator);
    }
    if (ev) record_event(ev[1], ctx->stream);
    if (!rc && con) rc = sg_constraints_a(ctx, dt);
    if (ev) record_event(ev[2], ctx->stream);
    if (!rc) rc = enqueue_list_update(ctx, (c.flags & SG_STEP_FLAT) != 0, fused);
    if (ev) record_event(ev[3], ctx->stream);
    if (!rc && !fused) rc = sg_zero_forces(ctx);
    if (ev) record_event(ev[4], ctx->stream);
    for (int k = 0; !rc && k < ctx->step_npairs; ++k) rc = sg_pair_forces_async(ctx, &ctx->step_pairs[k]);
    if (!rc && (c.flags & SG_STEP_REACTION_FIELD)) rc = sg_reaction_field_eval_async(ctx);
    for (int k = 0; !rc && (c.flags & SG_STEP_BONDED) && k < 6; ++k)
        if (ctx->bonded_n[k]) rc = sg_bonded_forces_async(ctx, k);
    if (ev) record_event(ev[5], ctx->stream);
    if (!rc) {
        switch (c.integrator) {
            case SG_INT_NVE: rc = sg_vv_final(ctx, dt, nullptr); if (!rc && c.rotations) rc = sg_qq_final(ctx, dt, nullptr); break;
            case SG_INT_LANGEVIN: rc = sg_lgv_final(ctx, dt, c.damping, nullptr, nullptr); break;
            case SG_INT_NH: rc = sg_nhc_step_final(ctx, dt, c.target_temp, c.coupling, c.rot_chain, c.rotations); break;
            default:
                rc = sg_nht_final(ctx, dt, c.target_temp, c.coupling, 0, 0, nullptr);
                if (!rc && c.rotations) rc = sg_qq_final(ctx, dt, nullptr);
        }
    }
    if (ev) record_event(ev[6], ctx->stream);
    if (!rc && con) rc = sg_constraints_b(ctx, dt);
    if (ev) record_event(ev[7], ctx->stream);
    if (!rc && !fused) {   // the fused final half step advances the counter itself
        k_step_incr<<<1, 1, 0, ctx->stream>>>(ctx->step_dev);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = sg_cuda_check(ctx, e, "k_step_incr");
    }
    ctx->lgv_step_dev = nullptr;
    ctx->lgv_rotations = 1;
    ctx->step_fused = 0;
    ctx->step_events = 0;
    ctx->step_sums_from_acc = 0;
    ctx->step_prep_kind = SG_PREP_NONE;
    return rc;
}

// Whether the step's launches after the first of a call can take the stored
// sums: the fused standard Nose-Hoover step, whose final half stores KE and,
// when the rotational chain is on, KE_rot of the state the next step starts
// from (it sums KE_rot only when rotations are integrated).
bool cont_eligible(sg_ctx* ctx, const sg_step_config& c) {
    if (c.integrator != SG_INT_NH || (c.flags & SG_STEP_CONSTRAINTS)) return false;
    return !c.rot_chain || c.rotations;
}

// Capture one step into an executable graph; kernels: its kernel nodes.
int capture_step(sg_ctx* ctx, const sg_step_config& c, bool cont, cudaGraphExec_t* out, int* kernels) {
    const unsigned epoch = ctx->graph_epoch;
    cudaGraph_t graph = nullptr;
    SG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_step(ctx, c, nullptr, cont);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return sg_cuda_check(ctx, e, "cudaStreamEndCapture");
    if (epoch != ctx->graph_epoch) {
        cudaGraphDestroy(graph);
        return sg_fail(ctx, SG_ECUDA, "a buffer was reallocated while capturing the step");
    }
    if (kernels) {
        size_t nn = 0;
        cudaGraphGetNodes(graph, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        if (nn) cudaGraphGetNodes(graph, nodes.data(), &nn);
        int k = 0;   // kernels launched by a step without a rebuild
        for (size_t m = 0; m < nn; ++m) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[m], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
        }
        *kernels = k;
    }
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return sg_cuda_check(ctx, e, "cudaGraphInstantiate");
    return SG_OK;
}

void drop_graphs(sg_ctx* ctx) {
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph_exec_cont) cudaGraphExecDestroy(ctx->graph_exec_cont);
    ctx->graph_exec = nullptr;
    ctx->graph_exec_cont = nullptr;
}

}  // namespace

extern "C" {

int sg_step_configure(sg_ctx* ctx, const sg_step_config* cfg) {
    if (!ctx || !cfg) return SG_EINVAL;
    static_assert(sizeof(sg_step_config) <= sizeof(ctx->step_cfg), "config size");
    if (!ctx->nl.initialized) return sg_fail(ctx, SG_ENOTREADY, "sg_nlist_init must precede sg_step_configure");
    memcpy(ctx->step_cfg, cfg, sizeof(sg_step_config));
    ctx->step_pairs[0] = cfg->pair;
    ctx->step_npairs = 1;
    if (!ctx->step_dev) SG_CUDA(ctx, cudaMalloc(&ctx->step_dev, sizeof(int)));
    SG_CUDA(ctx, cudaMemcpyAsync(ctx->step_dev, &cfg->first_step, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    drop_graphs(ctx);
    ctx->step_ready = 1;
    return SG_OK;
}

int sg_step_configure_pairs(sg_ctx* ctx, const sg_step_config* cfg, const sg_pair_params* pairs, int32_t npairs) {
    if (!ctx || !cfg || !pairs || npairs < 1 || npairs > 3) return SG_EINVAL;
    if (int rc = sg_step_configure(ctx, cfg)) return rc;
    for (int k = 0; k < npairs; ++k) ctx->step_pairs[k] = pairs[k];
    ctx->step_npairs = npairs;
    return SG_OK;
}

int sg_step(sg_ctx* ctx, int32_t nsteps) {
    if (!ctx || nsteps < 0) return SG_EINVAL;
    if (!ctx->step_ready) return sg_fail(ctx, SG_ENOTREADY, "sg_step_configure must precede sg_step");
    const sg_step_config& c = *reinterpret_cast<const sg_step_config*>(ctx->step_cfg);
    int done = 0;
    if (ctx->graph_exec && ctx->graph_epoch_captured != ctx->graph_epoch) drop_graphs(ctx);
    // no host call wrote the state since the last step: every launch can take
    // the sums that step stored
    const bool clean = ctx->step_clean_version == ctx->state_version;
    if (!ctx->graph_exec && nsteps > 0) {
        // one eager step allocates every buffer the step touches
        if (int rc = enqueue_step(ctx, c)) return rc;
        done = 1;
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const unsigned epoch = ctx->graph_epoch;
        int kernels = 0;
        if (int rc = capture_step(ctx, c, false, &ctx->graph_exec, &kernels)) return rc;
        if (cont_eligible(ctx, c))
            if (int rc = capture_step(ctx, c, true, &ctx->graph_exec_cont, nullptr)) {
                drop_graphs(ctx);
                return rc;
            }
        ctx->graph_kernels = kernels;
        ctx->graph_epoch_captured = epoch;
    }
    // a launch after a step of this call, or after one of an earlier call
    // with no state written since, takes the stored sums; otherwise the step
    // recomputes them
    for (int s = done; s < nsteps; ++s) {
        cudaGraphExec_t ge = ((s > 0 || clean) && ctx->graph_exec_cont) ? ctx->graph_exec_cont : ctx->graph_exec;
        SG_CUDA(ctx, cudaGraphLaunch(ge, ctx->stream));
    }
    if (nsteps > 0) ctx->step_clean_version = ctx->state_version;
    return SG_OK;
}

int sg_step_stage_times(sg_ctx* ctx, int32_t nsteps, double out_ms[7]) {
    if (!ctx || !out_ms || nsteps < 1) return SG_EINVAL;
    if (!ctx->step_ready) return sg_fail(ctx, SG_ENOTREADY, "sg_step_configure must precede sg_step_stage_times");
    sg_state_touched(ctx);
    const sg_step_config& c = *reinterpret_cast<const sg_step_config*>(ctx->step_cfg);
    // one step captured with an event-record node between the stages, so the
    // stages are timed as the captured step runs them (no host launch gaps)
    cudaEvent_t ev[8];
    for (auto& e : ev) SG_CUDA(ctx, cudaEventCreate(&e));
    int rc = enqueue_step(ctx, c);   // eager step: every buffer allocated before the capture
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaSuccess;
    if (!rc) e = cudaStreamSynchronize(ctx->stream);
    if (!rc && e == cudaSuccess) {
        const unsigned epoch = ctx->graph_epoch;
        e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            rc = enqueue_step(ctx, c, ev);
            e = cudaStreamEndCapture(ctx->stream, &graph);
        }
        if (!rc && e == cudaSuccess && epoch != ctx->graph_epoch)
            rc = sg_fail(ctx, SG_ECUDA, "a buffer was reallocated while capturing the step");
        if (!rc && e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    }
    for (int k = 0; k < 7; ++k) out_ms[k] = 0.0;
    for (int s = 0; s < nsteps && !rc && e == cudaSuccess; ++s) {
        e = cudaGraphLaunch(exec, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        for (int k = 0; k < 7 && e == cudaSuccess; ++k) {
            float ms = 0.f;
            e = cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
            out_ms[k] += ms / nsteps;
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (auto& x : ev) cudaEventDestroy(x);
    if (rc) return rc;
    if (e != cudaSuccess) return sg_cuda_check(ctx, e, "sg_step_stage_times");
    return SG_OK;
}

int sg_step_kernel_count(sg_ctx* ctx, int64_t* count) {
    if (!ctx || !count) return SG_EINVAL;
    if (!ctx->graph_exec) return sg_fail(ctx, SG_ENOTREADY, "no captured step yet");
    *count = ctx->graph_kernels;
    return SG_OK;
}

int sg_step_check(sg_ctx* ctx) {
    if (!ctx) return SG_EINVAL;
    int64_t k = 0;
    if (int rc = sg_nlist_count(ctx, &k)) return rc;
    double e[4];
    if (int rc = sg_read_energies(ctx, e)) return rc;
    for (int i = 0; i < 4; ++i)
        if (!std::isfinite(e[i])) return sg_fail(ctx, SG_ENAN, "non-finite energy accumulator %d", i);
    if (ctx->con_n) return sg_constraints_check(ctx);
    return SG_OK;
}

}  // extern "C"
