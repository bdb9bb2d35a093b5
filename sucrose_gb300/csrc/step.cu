// The whole timestep as one CUDA graph (sg_step). Every kernel of the step is
// gated on device-side state (list rebuild request, pair count, step counter),
// so a captured step replays without any host decision or synchronisation.
#include <cmath>
#include <vector>

#include "sg_internal.cuh"

namespace {

__global__ void k_step_incr(int* step) { *step += 1; }

int enqueue_step(sg_ctx* ctx, const sg_step_config& c) {
    const double dt = c.dt;
    ctx->lgv_step_dev = ctx->step_dev;
    ctx->lgv_rotations = c.rotations;
    int rc = SG_OK;
    switch (c.integrator) {
        case SG_INT_NVE: rc = sg_vv_initial(ctx, dt); if (!rc && c.rotations) rc = sg_qq_initial(ctx, dt); break;
        case SG_INT_LANGEVIN:
            rc = sg_lgv_initial(ctx, dt, 0, c.damping, c.target_temp, c.has_key ? c.key : nullptr);
            break;
        case SG_INT_NH:
        case SG_INT_NH_REF:
            rc = sg_nht_initial(ctx, dt, c.target_temp, c.coupling, c.integrator == SG_INT_NH ? 1 : 0,
                                c.integrator == SG_INT_NH ? c.rot_chain : 0);
            if (!rc && c.rotations) rc = sg_qq_initial(ctx, dt);
            break;
        default: rc = sg_fail(ctx, SG_EINVAL, "unknown integrator %d", c.integrator);
    }
    if (!rc) rc = sg_nlist_update(ctx);
    if (!rc) rc = sg_zero_forces(ctx);
    if (!rc) rc = sg_pair_forces_async(ctx, &c.pair);
    if (!rc) {
        switch (c.integrator) {
            case SG_INT_NVE: rc = sg_vv_final(ctx, dt, nullptr); if (!rc && c.rotations) rc = sg_qq_final(ctx, dt, nullptr); break;
            case SG_INT_LANGEVIN: rc = sg_lgv_final(ctx, dt, c.damping, nullptr, nullptr); break;
            default:
                rc = sg_nht_final(ctx, dt, c.target_temp, c.coupling, c.integrator == SG_INT_NH ? 1 : 0,
                                  c.integrator == SG_INT_NH ? c.rot_chain : 0, nullptr);
                if (!rc && c.rotations) rc = sg_qq_final(ctx, dt, nullptr);
        }
    }
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
        int kernels = 0;
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
    return SG_OK;
}

}  // extern "C"
