// Context lifetime, state transfer, accumulators and thermo (C ABI glue).
#include <cstdarg>
#include <cmath>
#include <vector>

#include "sg_internal.cuh"

int sg_fail(sg_ctx* ctx, int code, const char* fmt, ...) {
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

int sg_cuda_check(sg_ctx* ctx, cudaError_t e, const char* what) {
    return sg_fail(ctx, SG_ECUDA, "CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
}

int sg_ensure_partials(sg_ctx* ctx, int slots) {
    if (slots <= ctx->partial_slots) return SG_OK;
    if (ctx->partials) cudaFree(ctx->partials);
    ctx->partials = nullptr;
    ctx->graph_epoch++;
    SG_CUDA(ctx, cudaMalloc(&ctx->partials, sizeof(double) * (size_t)slots));
    ctx->partial_slots = slots;
    return SG_OK;
}

int sg_ensure_stage(sg_ctx* ctx, size_t bytes) {
    if (bytes <= ctx->h_stage_bytes) return SG_OK;
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    SG_CUDA(ctx, cudaMallocHost(&ctx->h_stage, bytes));
    ctx->h_stage_bytes = bytes;
    return SG_OK;
}

int sg_grid_for(sg_ctx* ctx, const void* kernel, int block, size_t smem) {
    int per_sm = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * ctx->num_sms;
}

__global__ void k_set_defaults(int n, float4* vel, float4* angm, float4* quat, float4* shape, float4* eshape,
                               float4* inert, float4* inert_inv, float4* force, float4* torque, float4* pos) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    vel[i] = make_float4(0.f, 0.f, 0.f, 1.f);
    angm[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    quat[i] = make_float4(1.f, 0.f, 0.f, 0.f);
    shape[i] = make_float4(1.f, 1.f, 1.f, 1.f);
    eshape[i] = make_float4(1.f, 1.f, 1.f, 0.f);
    inert[i] = make_float4(0.1f, 0.1f, 0.1f, 0.f);
    inert_inv[i] = make_float4(10.f, 10.f, 10.f, 0.f);
    force[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    torque[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

extern "C" {

int sg_create(sg_ctx** out, int32_t n, int32_t device) {
    if (!out) return SG_EINVAL;
    *out = nullptr;
    if (n < 1) return SG_EINVAL;
    sg_ctx* ctx = new sg_ctx();
    ctx->n = n;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        *out = ctx;
        return sg_cuda_check(ctx, e, "cudaSetDevice");
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    *out = ctx;
    SG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    float4** bufs[] = {&ctx->pos, &ctx->quat, &ctx->vel, &ctx->angm, &ctx->force, &ctx->torque,
                       &ctx->shape, &ctx->eshape, &ctx->inert, &ctx->inert_inv};
    for (float4** b : bufs) SG_CUDA(ctx, cudaMalloc(b, sizeof(float4) * (size_t)n));
    SG_CUDA(ctx, cudaMalloc(&ctx->acc, sizeof(double) * 8));
    SG_CUDA(ctx, cudaMalloc(&ctx->done_counter, sizeof(unsigned int) * 4));
    SG_CUDA(ctx, cudaMalloc(&ctx->stats, sizeof(unsigned long long) * 32));
    SG_CUDA(ctx, cudaMalloc(&ctx->nh, sizeof(double) * 32));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->acc, 0, sizeof(double) * 8, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->done_counter, 0, sizeof(unsigned int) * 4, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->stats, 0, sizeof(unsigned long long) * 32, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->nh, 0, sizeof(double) * 32, ctx->stream));
    if (int rc = sg_ensure_partials(ctx, 8 * 4096)) return rc;
    k_set_defaults<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, ctx->vel, ctx->angm, ctx->quat, ctx->shape,
                                                             ctx->eshape, ctx->inert, ctx->inert_inv, ctx->force,
                                                             ctx->torque, ctx->pos);
    SG_LAUNCH_CHECK(ctx, "k_set_defaults");
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_destroy(sg_ctx* ctx) {
    if (!ctx) return SG_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    sg_nlist_free(ctx);
    sg_mlp_free(ctx);
    sg_constraints_free(ctx);
    sg_bonded_free(ctx);
    void* bufs[] = {ctx->pos, ctx->quat, ctx->vel, ctx->angm, ctx->force, ctx->torque, ctx->shape, ctx->eshape,
                    ctx->inert, ctx->inert_inv, ctx->acc, ctx->partials, ctx->done_counter, ctx->stats, ctx->nh,
                    ctx->ecp_prep, ctx->ecp_prep64, ctx->ecp_lambda, ctx->mlp_w, ctx->mlp_wbf16, ctx->mlp_tc_err,
                    ctx->rf_dip, ctx->rf_mark, ctx->rf_cnt, ctx->rf_field, ctx->mc_scratch, ctx->gb_tile_order,
                    ctx->pair_surv};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    if (ctx->d_stage) cudaFree(ctx->d_stage);
    if (ctx->rep_alloc) cudaFree(ctx->rep_alloc);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph_exec_cont) cudaGraphExecDestroy(ctx->graph_exec_cont);
    if (ctx->step_dev) cudaFree(ctx->step_dev);
    if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SG_OK;
}

const char* sg_last_error(const sg_ctx* ctx) { return ctx ? ctx->err : "null context"; }

void* sg_stream(sg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int sg_synchronize(sg_ctx* ctx) {
    if (!ctx) return SG_EINVAL;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_set_box(sg_ctx* ctx, const double box[3], int32_t periodic) {
    if (!ctx || !box) return SG_EINVAL;
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "replica boxes are fixed by sg_create_replicas");
    for (int d = 0; d < 3; ++d)
        if (!(box[d] > 0.0)) return sg_fail(ctx, SG_EINVAL, "box dimensions must be positive");
    for (int d = 0; d < 3; ++d) ctx->box[d] = box[d];
    ctx->periodic = periodic ? 1 : 0;
    ctx->graph_epoch++;   // captured steps hold the box in their launch arguments
    return sg_nlist_box_changed(ctx);
}

// FP64 SoA <-> float4 packing on the device. Host arrays are copied raw
// into a device FP64 staging area (one cudaMemcpyAsync each), then one kernel
// packs them; a lane whose source is absent keeps its device value, except w
// when wfill applies. Downloads run the other way.
__global__ void k_pack4(int n, float4* __restrict__ dst, const double* __restrict__ src, int mask, const float* wfill) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = dst[i];
    if (mask & 1) v.x = (float)src[i];
    if (mask & 2) v.y = (float)src[(size_t)n + i];
    if (mask & 4) v.z = (float)src[2 * (size_t)n + i];
    if (mask & 8) v.w = (float)src[3 * (size_t)n + i];
    else if (wfill) v.w = wfill[i];
    dst[i] = v;
}

__global__ void k_unpack4(int n, const float4* __restrict__ src, double* __restrict__ dst) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = src[i];
    dst[i] = v.x;
    dst[(size_t)n + i] = v.y;
    dst[2 * (size_t)n + i] = v.z;
    dst[3 * (size_t)n + i] = v.w;
}

// The same conversions reading / writing the caller's host arrays in place.
struct HostCols {
    const double* in[4];
    double* out[4];
};

__global__ void k_pack4_host(int n, float4* __restrict__ dst, HostCols c, int mask, const float* wfill) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = dst[i];
    if (mask & 1) v.x = (float)c.in[0][i];
    if (mask & 2) v.y = (float)c.in[1][i];
    if (mask & 4) v.z = (float)c.in[2][i];
    if (mask & 8) v.w = (float)c.in[3][i];
    else if (wfill) v.w = wfill[i];
    dst[i] = v;
}

__global__ void k_unpack4_host(int n, const float4* __restrict__ src, HostCols c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = src[i];
    if (c.out[0]) c.out[0][i] = v.x;
    if (c.out[1]) c.out[1][i] = v.y;
    if (c.out[2]) c.out[2][i] = v.z;
    if (c.out[3]) c.out[3][i] = v.w;
}

// Device address of a host array that kernels can read and write in place:
// page-locked memory mapped into the device's address space (under unified
// addressing every cudaHostAlloc allocation is), as the CUDA runtime reports it for
// this very pointer; nullptr otherwise (pageable memory: staged by copies).
// Queried on every call: a cached answer could outlive the allocation.
static void* host_view(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return a.devicePointer;
}

// The whole state (pos, quat, vel, angm: 13 columns, absent ones skipped) in
// one pass over mapped host arrays, either way.
struct StateCols {
    double* c[13];
};

__global__ void k_state_from_host(int n, float4* __restrict__ pos, float4* __restrict__ quat,
                                  float4* __restrict__ vel, float4* __restrict__ angm, StateCols s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4* dst[4] = {pos, quat, vel, angm};
    const int first[4] = {0, 3, 7, 10}, width[4] = {3, 4, 3, 3};
#pragma unroll
    for (int gq = 0; gq < 4; ++gq) {
        const int f = first[gq];
        if (!s.c[f] && !s.c[f + 1] && !s.c[f + 2] && (width[gq] < 4 || !s.c[f + 3])) continue;
        float4 v = dst[gq][i];
        if (s.c[f]) v.x = (float)s.c[f][i];
        if (s.c[f + 1]) v.y = (float)s.c[f + 1][i];
        if (s.c[f + 2]) v.z = (float)s.c[f + 2][i];
        if (width[gq] == 4 && s.c[f + 3]) v.w = (float)s.c[f + 3][i];
        dst[gq][i] = v;
    }
}

__global__ void k_state_to_host(int n, const float4* __restrict__ pos, const float4* __restrict__ quat,
                                const float4* __restrict__ vel, const float4* __restrict__ angm, StateCols s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v[4] = {pos[i], quat[i], vel[i], angm[i]};
    const int first[4] = {0, 3, 7, 10}, width[4] = {3, 4, 3, 3};
#pragma unroll
    for (int gq = 0; gq < 4; ++gq) {
        const int f = first[gq];
        if (s.c[f]) s.c[f][i] = v[gq].x;
        if (s.c[f + 1]) s.c[f + 1][i] = v[gq].y;
        if (s.c[f + 2]) s.c[f + 2][i] = v[gq].z;
        if (width[gq] == 4 && s.c[f + 3]) s.c[f + 3][i] = v[gq].w;
    }
}

int sg_ensure_dstage(sg_ctx* ctx) {
    if (ctx->d_stage) return SG_OK;
    SG_CUDA(ctx, cudaMalloc(&ctx->d_stage, sizeof(double) * 16 * (size_t)ctx->n));
    return SG_OK;
}

static int upload4(sg_ctx* ctx, float4* dst, const double* a, const double* b, const double* c, const double* d,
                   const float* wfill_dev, int slot = 0) {
    const int n = ctx->n;
    if (!a && !b && !c && !d) return SG_OK;
    {
        // mapped page-locked arrays: one kernel reads them in place over the link
        HostCols hc{};
        const double* in[4] = {a, b, c, d};
        int mask = 0;
        bool mapped = true;
        for (int k = 0; k < 4 && mapped; ++k)
            if (in[k]) {
                hc.in[k] = (const double*)host_view(in[k]);
                mapped = hc.in[k] != nullptr;
                mask |= 1 << k;
            }
        if (mapped) {
            k_pack4_host<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, dst, hc, mask, wfill_dev);
            SG_LAUNCH_CHECK(ctx, "k_pack4_host");
            return SG_OK;
        }
    }
    if (int rc = sg_ensure_dstage(ctx)) return rc;
    double* st = ctx->d_stage + (size_t)slot * 4 * n;
    const double* src[4] = {a, b, c, d};
    int mask = 0;
    for (int k = 0; k < 4; ++k)
        if (src[k]) {
            mask |= 1 << k;
            SG_CUDA(ctx, cudaMemcpyAsync(st + (size_t)k * n, src[k], sizeof(double) * n, cudaMemcpyHostToDevice,
                                         ctx->stream));
        }
    k_pack4<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, dst, st, mask, wfill_dev);
    SG_LAUNCH_CHECK(ctx, "k_pack4");
    return SG_OK;
}

static int download4(sg_ctx* ctx, const float4* src, double* a, double* b, double* c, double* d, int slot = 0) {
    const int n = ctx->n;
    if (!a && !b && !c && !d) return SG_OK;
    {
        HostCols hc{};
        double* out[4] = {a, b, c, d};
        bool mapped = true;
        for (int k = 0; k < 4 && mapped; ++k)
            if (out[k]) {
                hc.out[k] = (double*)host_view(out[k]);
                mapped = hc.out[k] != nullptr;
            }
        if (mapped) {   // written in place; the caller's synchronisation makes them visible
            k_unpack4_host<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, src, hc);
            SG_LAUNCH_CHECK(ctx, "k_unpack4_host");
            return SG_OK;
        }
    }
    if (int rc = sg_ensure_dstage(ctx)) return rc;
    double* st = ctx->d_stage + (size_t)slot * 4 * n;
    k_unpack4<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, src, st);
    SG_LAUNCH_CHECK(ctx, "k_unpack4");
    double* dst[4] = {a, b, c, d};
    for (int k = 0; k < 4; ++k)
        if (dst[k])
            SG_CUDA(ctx, cudaMemcpyAsync(dst[k], st + (size_t)k * n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                         ctx->stream));
    return SG_OK;
}

int sg_set_particles(sg_ctx* ctx, const double* mass, const double* sig_x, const double* sig_y, const double* sig_z,
                     const double* eps_x, const double* eps_y, const double* eps_z, const double* ixx,
                     const double* iyy, const double* izz) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    const int n = ctx->n;
    std::vector<double> m(n, 1.0), sx(n, 1.0), sy(n, 1.0), sz(n, 1.0), ex(n, 1.0), ey(n, 1.0), ez(n, 1.0);
    std::vector<double> Ix(n), Iy(n), Iz(n), Ixi(n), Iyi(n), Izi(n), im(n);
    for (int i = 0; i < n; ++i) {
        if (mass) m[i] = mass[i];
        if (sig_x && sig_y && sig_z) { sx[i] = sig_x[i]; sy[i] = sig_y[i]; sz[i] = sig_z[i]; }
        if (eps_x && eps_y && eps_z) { ex[i] = eps_x[i]; ey[i] = eps_y[i]; ez[i] = eps_z[i]; }
        if (m[i] < 0.0) return sg_fail(ctx, SG_EINVAL, "negative mass at particle %d", i);
        // initialize_system (fortran/system.f90:614-680)
        if (m[i] == 0.0) {
            im[i] = 0.0;
            Ix[i] = Iy[i] = Iz[i] = 0.0;
            Ixi[i] = Iyi[i] = Izi[i] = 0.0;
            continue;
        }
        im[i] = 1.0 / m[i];
        bool given = ixx && iyy && izz;
        if (!given || ixx[i] < 0 || iyy[i] < 0 || izz[i] < 0) {
            Ix[i] = (sy[i] * sy[i] + sz[i] * sz[i]) / 20.0;
            Iy[i] = (sx[i] * sx[i] + sz[i] * sz[i]) / 20.0;
            Iz[i] = (sx[i] * sx[i] + sy[i] * sy[i]) / 20.0;
        } else {
            Ix[i] = ixx[i]; Iy[i] = iyy[i]; Iz[i] = izz[i];
        }
        if (Ix[i] > 0 && Iy[i] > 0 && Iz[i] > 0) {
            Ixi[i] = 1.0 / Ix[i]; Iyi[i] = 1.0 / Iy[i]; Izi[i] = 1.0 / Iz[i];
        } else {
            Ixi[i] = Iyi[i] = Izi[i] = 0.0;
        }
    }
    std::vector<double> zero(n, 0.0);
    if (int rc = upload4(ctx, ctx->shape, sx.data(), sy.data(), sz.data(), m.data(), nullptr, 0)) return rc;
    if (int rc = upload4(ctx, ctx->eshape, ex.data(), ey.data(), ez.data(), zero.data(), nullptr, 1)) return rc;
    if (int rc = upload4(ctx, ctx->inert, Ix.data(), Iy.data(), Iz.data(), zero.data(), nullptr, 2)) return rc;
    if (int rc = upload4(ctx, ctx->inert_inv, Ixi.data(), Iyi.data(), Izi.data(), zero.data(), nullptr, 3)) return rc;
    // inverse mass lives in vel.w
    if (int rc = upload4(ctx, ctx->vel, nullptr, nullptr, nullptr, im.data(), nullptr, 0)) return rc;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // the host vectors above go out of scope
    return SG_OK;
}

int sg_set_charges(sg_ctx* ctx, const double* charge, int32_t reference_defaults) {
    if (!ctx) return SG_EINVAL;
    std::vector<double> q(ctx->n, 0.0);
    for (int i = 0; i < ctx->n && charge; ++i) {
        q[i] = charge[i];
        // initialize_system (fortran/system.f90:595-598): negative charges become 0
        if (reference_defaults && q[i] < 0.0) q[i] = 0.0;
        if (!std::isfinite(q[i])) return sg_fail(ctx, SG_EINVAL, "non-finite charge at particle %d", i);
    }
    // the charge rides in the position's w lane
    if (int rc = upload4(ctx, ctx->pos, nullptr, nullptr, nullptr, q.data(), nullptr, 0)) return rc;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // q goes out of scope
    return SG_OK;
}

int sg_upload_state(sg_ctx* ctx, const double* rx, const double* ry, const double* rz, const double* qw,
                    const double* qx, const double* qy, const double* qz, const double* vx, const double* vy,
                    const double* vz, const double* lx, const double* ly, const double* lz) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    {
        // every given column mapped page-locked memory: one kernel for the state
        const double* in[13] = {rx, ry, rz, qw, qx, qy, qz, vx, vy, vz, lx, ly, lz};
        StateCols sc{};
        bool mapped = true;
        for (int k = 0; k < 13 && mapped; ++k)
            if (in[k]) mapped = (sc.c[k] = (double*)host_view(in[k])) != nullptr;
        if (mapped) {
            k_state_from_host<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->quat, ctx->vel,
                                                                             ctx->angm, sc);
            SG_LAUNCH_CHECK(ctx, "k_state_from_host");
            if (ctx->sync_transfers) SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            return SG_OK;
        }
    }
    // separate staging slots so that the four copies can be in flight together;
    // quaternion (w x y z) occupies the four lanes in that order
    if (int rc = upload4(ctx, ctx->pos, rx, ry, rz, nullptr, nullptr, 0)) return rc;
    if (int rc = upload4(ctx, ctx->quat, qw, qx, qy, qz, nullptr, 1)) return rc;
    if (int rc = upload4(ctx, ctx->vel, vx, vy, vz, nullptr, nullptr, 2)) return rc;
    if (int rc = upload4(ctx, ctx->angm, lx, ly, lz, nullptr, nullptr, 3)) return rc;
    if (ctx->sync_transfers) SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_download_state(sg_ctx* ctx, double* rx, double* ry, double* rz, double* qw, double* qx, double* qy,
                      double* qz, double* vx, double* vy, double* vz, double* lx, double* ly, double* lz) {
    if (!ctx) return SG_EINVAL;
    {
        double* out[13] = {rx, ry, rz, qw, qx, qy, qz, vx, vy, vz, lx, ly, lz};
        StateCols sc{};
        bool mapped = true;
        for (int k = 0; k < 13 && mapped; ++k)
            if (out[k]) mapped = (sc.c[k] = (double*)host_view(out[k])) != nullptr;
        if (mapped) {
            k_state_to_host<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->quat, ctx->vel,
                                                                           ctx->angm, sc);
            SG_LAUNCH_CHECK(ctx, "k_state_to_host");
            SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            return SG_OK;
        }
    }
    if (int rc = download4(ctx, ctx->pos, rx, ry, rz, nullptr, 0)) return rc;
    if (int rc = download4(ctx, ctx->quat, qw, qx, qy, qz, 1)) return rc;
    if (int rc = download4(ctx, ctx->vel, vx, vy, vz, nullptr, 2)) return rc;
    if (int rc = download4(ctx, ctx->angm, lx, ly, lz, nullptr, 3)) return rc;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_download_forces(sg_ctx* ctx, double* fx, double* fy, double* fz, double* tx, double* ty, double* tz) {
    if (!ctx) return SG_EINVAL;
    if (int rc = download4(ctx, ctx->force, fx, fy, fz, nullptr, 0)) return rc;
    if (int rc = download4(ctx, ctx->torque, tx, ty, tz, nullptr, 1)) return rc;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_upload_forces(sg_ctx* ctx, const double* fx, const double* fy, const double* fz, const double* tx,
                     const double* ty, const double* tz) {
    if (!ctx) return SG_EINVAL;
    if (int rc = upload4(ctx, ctx->force, fx, fy, fz, nullptr, nullptr, 0)) return rc;
    if (int rc = upload4(ctx, ctx->torque, tx, ty, tz, nullptr, nullptr, 1)) return rc;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_zero_forces(sg_ctx* ctx) {
    if (!ctx) return SG_EINVAL;
    SG_CUDA(ctx, cudaMemsetAsync(ctx->force, 0, sizeof(float4) * (size_t)ctx->n, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->torque, 0, sizeof(float4) * (size_t)ctx->n, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->acc, 0, sizeof(double) * 4, ctx->stream));
    SG_CUDA(ctx, cudaMemsetAsync(ctx->acc + 6, 0, sizeof(double), ctx->stream));   // virial_bonded
    return SG_OK;
}

int sg_read_energies(sg_ctx* ctx, double out[4]) {
    if (!ctx || !out) return SG_EINVAL;
    SG_CUDA(ctx, cudaMemcpyAsync(out, ctx->acc, sizeof(double) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- thermo ----
// virial = SUM(RX*FX + RY*FY + RZ*FZ) with absolute positions (fortran/system.f90:733-735).
__global__ void k_virial(int n, const float4* __restrict__ pos, const float4* __restrict__ force, double* partials,
                         unsigned int* done, double* out) {
    double v[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float4 r = pos[i], f = force[i];
        v[0] += (double)r.x * f.x + (double)r.y * f.y + (double)r.z * f.z;
    }
    block_reduce_finish<1>(v, partials, done, out);
}

extern "C" int sg_thermo(sg_ctx* ctx, int32_t dof, double density, int32_t nrigid, double* out3) {
    if (!ctx || !out3 || dof <= 0) return SG_EINVAL;
    SG_CUDA(ctx, cudaMemsetAsync(ctx->acc + 4, 0, sizeof(double), ctx->stream));
    int grid = std::min(1024, (ctx->n + 255) / 256);
    k_virial<<<grid, 256, 0, ctx->stream>>>(ctx->n, ctx->pos, ctx->force, ctx->partials, ctx->done_counter,
                                            ctx->acc + 4);
    SG_LAUNCH_CHECK(ctx, "k_virial");
    double a[7];
    SG_CUDA(ctx, cudaMemcpyAsync(a, ctx->acc, sizeof(double) * 7, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    double kin_tot = a[2] + a[3];
    double temp = 2.0 * kin_tot / (double)dof;
    double volume = ctx->box[0] * ctx->box[1] * ctx->box[2];
    // the bonded virial joins when NC > 0 and it is not negative (system.f90:732-736)
    const double virial = (ctx->con_n > 0 && a[6] >= 0.0) ? a[4] + a[6] : a[4];
    out3[0] = temp;
    out3[1] = virial;
    out3[2] = (density * nrigid * temp) + (virial / (3.0 * volume));
    return SG_OK;
}
