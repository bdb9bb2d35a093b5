// The whole timestep as one CUDA graph (sg_step). Every kernel of the step is
// gated on device-side state (list rebuild request, pair count, step counter),
// so a captured step replays without any host decision or synchronisation.
#include <cmath>
#include <vector>

#include "sg_internal.cuh"

namespace {

__global__ void k_step_incr(int* step) { *step += 1; }

__global__ void k_set_rebuild_condition(cudaGraphConditionalHandle h, const int* flags) {
    cudaGraphSetConditional(h, flags[0] ? 1u : 0u);
}

// List maintenance inside a captured step: the displacement test runs every
// step; the build kernels sit in the body of a conditional graph node that
// executes only when a rebuild was requested, so a step without a rebuild
// launches none of them. Outside capture the flag-gated kernels are enqueued.
int enqueue_list_update(sg_ctx* ctx, bool flat) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaGraph_t cg = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t nd = 0;
    SG_CUDA(ctx, cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, &edges, &nd));
    if (flat || st != cudaStreamCaptureStatusActive) return sg_nlist_update(ctx);
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

// ev (optional): 6 events recorded before the initial half step, the list
// update, the force zeroing, the pair stage, the final half step and the
// step counter (eager steps only; sg_step_stage_times).
int enqueue_step(sg_ctx* ctx, const sg_step_config& c, cudaEvent_t* ev = nullptr) {
    const double dt = c.dt;
    ctx->lgv_step_dev = ctx->step_dev;
    ctx->lgv_rotations = c.rotations;
    int rc = SG_OK;
    if (ev) cudaEventRecord(ev[0], ctx->stream);
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
    if (ev) cudaEventRecord(ev[1], ctx->stream);
    if (!rc && con) rc = sg_constraints_a(ctx, dt);
    if (ev) cudaEventRecord(ev[2], ctx->stream);
    if (!rc) rc = enqueue_list_update(ctx, (c.flags & SG_STEP_FLAT) != 0);
    if (ev) cudaEventRecord(ev[3], ctx->stream);
    if (!rc) rc = sg_zero_forces(ctx);
    if (ev) cudaEventRecord(ev[4], ctx->stream);
    for (int k = 0; !rc && k < ctx->step_npairs; ++k) rc = sg_pair_forces_async(ctx, &ctx->step_pairs[k]);
    if (!rc && (c.flags & SG_STEP_REACTION_FIELD)) rc = sg_reaction_field_eval_async(ctx);
    for (int k = 0; !rc && (c.flags & SG_STEP_BONDED) && k < 6; ++k)
        if (ctx->bonded_n[k]) rc = sg_bonded_forces_async(ctx, k);
    if (ev) cudaEventRecord(ev[5], ctx->stream);
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
    if (ev) cudaEventRecord(ev[6], ctx->stream);
    if (!rc && con) rc = sg_constraints_b(ctx, dt);
    if (ev) cudaEventRecord(ev[7], ctx->stream);
    if (!rc) {
        k_step_incr<<<1, 1, 0, ctx->stream>>>(ctx->step_dev);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = sg_cuda_check(ctx, e, "k_step_incr");
    }
    ctx->lgv_step_dev = nullptr;
    ctx->lgv_rotations = 1;
    return rc;
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
    if (ctx->graph_exec) {
        cudaGraphExecDestroy(ctx->graph_exec);
        ctx->graph_exec = nullptr;
    }
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
    if (ctx->graph_exec && ctx->graph_epoch_captured != ctx->graph_epoch) {
        cudaGraphExecDestroy(ctx->graph_exec);
        ctx->graph_exec = nullptr;
    }
    if (!ctx->graph_exec && nsteps > 0) {
        // one eager step allocates every buffer the step touches
        if (int rc = enqueue_step(ctx, c)) return rc;
        done = 1;
        SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const unsigned epoch = ctx->graph_epoch;
        cudaGraph_t graph = nullptr;
        SG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_step(ctx, c);
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
        size_t nn = 0;
        cudaGraphGetNodes(graph, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        if (nn) cudaGraphGetNodes(graph, nodes.data(), &nn);
        int kernels = 0;   // kernels launched by a step without a rebuild
        for (size_t k = 0; k < nn; ++k) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
        }
        ctx->graph_kernels = kernels;
        e = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return sg_cuda_check(ctx, e, "cudaGraphInstantiate");
        ctx->graph_epoch_captured = epoch;
    }
    for (int s = done; s < nsteps; ++s) SG_CUDA(ctx, cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    return SG_OK;
}

int sg_step_stage_times(sg_ctx* ctx, int32_t nsteps, double out_ms[7]) {
    if (!ctx || !out_ms || nsteps < 1) return SG_EINVAL;
    if (!ctx->step_ready) return sg_fail(ctx, SG_ENOTREADY, "sg_step_configure must precede sg_step_stage_times");
    const sg_step_config& c = *reinterpret_cast<const sg_step_config*>(ctx->step_cfg);
    std::vector<cudaEvent_t> ev(8 * (size_t)nsteps);
    for (auto& e : ev) SG_CUDA(ctx, cudaEventCreate(&e));
    int rc = SG_OK;
    for (int s = 0; s < nsteps && !rc; ++s) rc = enqueue_step(ctx, c, ev.data() + 8 * s);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    for (int k = 0; k < 7; ++k) out_ms[k] = 0.0;
    if (!rc && e == cudaSuccess) {
        for (int s = 0; s < nsteps; ++s)
            for (int k = 0; k < 7; ++k) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev[8 * s + k], ev[8 * s + k + 1]);
                out_ms[k] += ms / nsteps;
            }
    }
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
