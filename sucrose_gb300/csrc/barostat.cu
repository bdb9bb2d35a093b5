// Monte Carlo barostat (module monte_carlo_barostat, fortran/integrators.f90:
// 858-945). One trial volume move: U_old from the pair sets, a uniform volume
// change of at most max_dV * V, positions and box scaled by (V_new/V_old)^(1/3),
// U_new, and the Metropolis test on
//   -beta dU - beta P (V_new - V_old) + N log(V_new / V_old),
// restoring positions and box on rejection. The reference's
// compute_potential callback becomes the context's own pair kernels (and the
// registered bonded lists, when asked); random_number becomes two Philox
// words from a caller-given counter and key. Forces and torques are restored
// after the energy evaluations, so the integrator state is untouched.
#include <cmath>
#include <vector>

#include "sg_internal.cuh"

namespace {

__global__ void k_scale_pos(int n, float4* pos, float s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    p.x *= s;
    p.y *= s;
    p.z *= s;
    pos[i] = p;
}

struct McScratch {   // one allocation: saved positions, forces, torques
    float4* pos = nullptr;
    float4* force = nullptr;
    float4* torque = nullptr;
};

// sum of the energies of the pair sets (and bonded lists) at the current state
int potential(sg_ctx* ctx, const sg_pair_params* pairs, int npairs, int bonded, double* u) {
    double total = 0.0;
    for (int k = 0; k < npairs; ++k) {
        double pe = 0.0;
        if (int rc = sg_pair_forces(ctx, &pairs[k], &pe, nullptr, nullptr)) return rc;
        total += pe;
    }
    for (int k = 0; bonded && k < 6; ++k) {
        if (!ctx->bonded_n[k]) continue;
        double pe = 0.0;
        if (int rc = sg_bonded_forces(ctx, k, &pe)) return rc;
        total += pe;
    }
    *u = total;
    return SG_OK;
}

}  // namespace

extern "C" {

int sg_mc_barostat(sg_ctx* ctx, const sg_pair_params* pairs, int32_t npairs, int32_t include_bonded,
                   double target_pressure, double temperature, double max_dv, const uint32_t key[2],
                   uint64_t counter, int32_t* accept, double* volume_out) {
    if (!ctx || (npairs > 0 && !pairs) || npairs < 0 || !accept) return SG_EINVAL;
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "the barostat is per system: no replica contexts");
    sg_state_touched(ctx);
    if (!ctx->periodic) return sg_fail(ctx, SG_EINVAL, "the barostat needs a periodic box");
    // the reference stops here (integrators.f90:879-882)
    if (target_pressure <= 1e-3) return sg_fail(ctx, SG_EINVAL, "Target pressure too small.");
    if (!(temperature > 0.0)) return sg_fail(ctx, SG_EINVAL, "temperature must be positive");
    if (!(max_dv > 0.0)) max_dv = 0.01;   // volume_change absent (:884-888)
    *accept = -1;
    const int n = ctx->n;
    const size_t bytes = sizeof(float4) * (size_t)n;
    McScratch s;
    if (!ctx->mc_scratch) SG_CUDA(ctx, cudaMalloc(&ctx->mc_scratch, 3 * bytes));   // kept for later calls
    s.pos = ctx->mc_scratch;
    s.force = s.pos + n;
    s.torque = s.pos + 2 * (size_t)n;
    double acc_save[8];
    auto copy = [&](float4* dst, const float4* src) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
    };
    // restore forces, torques and the energy accumulators, then wait
    auto finish = [&](int rc) {
        cudaError_t e = copy(ctx->force, s.force);
        if (e == cudaSuccess) e = copy(ctx->torque, s.torque);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ctx->acc, acc_save, sizeof(acc_save), cudaMemcpyHostToDevice, ctx->stream);
        const cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
        if (e == cudaSuccess) e = e2;
        if (rc == SG_OK && e != cudaSuccess) rc = sg_cuda_check(ctx, e, "sg_mc_barostat restore");
        return rc;
    };
    cudaError_t e = copy(s.pos, ctx->pos);
    if (e == cudaSuccess) e = copy(s.force, ctx->force);
    if (e == cudaSuccess) e = copy(s.torque, ctx->torque);
    if (e == cudaSuccess) e = cudaMemcpyAsync(acc_save, ctx->acc, sizeof(acc_save), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return sg_cuda_check(ctx, e, "sg_mc_barostat save");

    const double beta = 1.0 / temperature;
    const double box_old[3] = {ctx->box[0], ctx->box[1], ctx->box[2]};
    const double V_old = box_old[0] * box_old[1] * box_old[2];
    double U_old = 0.0, U_new = 0.0;
    if (int rc = potential(ctx, pairs, npairs, include_bonded, &U_old)) return finish(rc);

    // two uniforms u = word * 2^-32 (philox_real, xmath.f90:66-76): the move and the test
    const uint32_t ctr[4] = {(uint32_t)counter, (uint32_t)(counter >> 32), 0x4D43u, 0u};
    uint32_t w[4];
    sg_philox4x32(ctr, key, w);
    const double u1 = w[0] * (1.0 / 4294967296.0), u2 = w[1] * (1.0 / 4294967296.0);
    const double V_new = V_old + max_dv * (2.0 * u1 - 1.0) * V_old;
    if (V_new <= 0.0) {   // unphysical: no move; the reference leaves accept unset (:894-896)
        if (volume_out) *volume_out = V_old;
        return finish(SG_OK);
    }
    const double scale = std::pow(V_new / V_old, 1.0 / 3.0);
    k_scale_pos<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, ctx->pos, (float)scale);
    e = cudaGetLastError();
    if (e != cudaSuccess) return finish(sg_cuda_check(ctx, e, "k_scale_pos"));
    for (int d = 0; d < 3; ++d) ctx->box[d] = box_old[d] * scale;
    sg_nlist_box_changed(ctx);
    int rc = potential(ctx, pairs, npairs, include_bonded, &U_new);
    const double dU = U_new - U_old;
    const double exponent = -beta * dU - beta * target_pressure * (V_new - V_old) + (double)n * std::log(V_new / V_old);
    const bool ok = rc == SG_OK && std::log(u2) < exponent;
    if (!ok) {   // restore the box and the positions (:926-935)
        for (int d = 0; d < 3; ++d) ctx->box[d] = box_old[d];
        sg_nlist_box_changed(ctx);
        e = copy(ctx->pos, s.pos);
        if (e != cudaSuccess && rc == SG_OK) rc = sg_cuda_check(ctx, e, "barostat restore");
    }
    rc = finish(rc);
    if (rc) return rc;
    *accept = ok ? 1 : 0;
    if (volume_out) *volume_out = ctx->box[0] * ctx->box[1] * ctx->box[2];
    return SG_OK;
}

}  // extern "C"
