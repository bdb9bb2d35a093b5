// sg_lj_forces_noalloc: the point-particle pair-force kernel in a form that
// allocates no memory at all, for callers that already hold their particle
// data in device memory and cannot call cudaMalloc at this point (code that
// runs while another library captures the stream into a CUDA graph, hosts
// whose device memory comes from their own pool, OpenACC/CUDA Fortran
// programs that keep the reference's module arrays resident on the device).
//
// It evaluates the same lj_ / lj12_ / ljw_ / wca_ formulas as k_pair<PotLJ>
// over a caller-supplied half list, reading FP64 structure-of-arrays
// positions and adding into FP64 structure-of-arrays forces, exactly like the
// reference's pair loop (README.md:86-103) adds into FX, FY, FZ.
//
// Its scratch is one file-scope __device__ array (the struct below), sized
// for at most SG_NOALLOC_MAX_N particles and SG_NOALLOC_MAX_BLOCKS blocks:
// about 2.1 MiB that every GPU which loads the library keeps until the
// process exits. All calls share it, so calls whose work overlaps on the GPU
// (different streams, or different host threads) race and must be serialised
// by the caller. Each call clears the parts that must start at zero.
#include <mutex>

#include "sg_internal.cuh"

#define SG_NOALLOC_MAX_N 131072
#define SG_NOALLOC_MAX_BLOCKS 1024
#define SG_NOALLOC_MAX_DEVICES 64

namespace {

struct NoallocScratch {
    float4 acc[SG_NOALLOC_MAX_N];                 // per-particle force sums (FP32)
    double partials[SG_NOALLOC_MAX_BLOCKS * 2];   // per-block PE and virial
    unsigned int done;                            // blocks finished (last block reduces)
    unsigned int bad;                             // pairs skipped for a bad index
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch, looked up once per device with that
// device current (the host-side name is only a stand-in for the symbol).
NoallocScratch* g_scratch_addr[SG_NOALLOC_MAX_DEVICES] = {nullptr};
std::mutex g_scratch_mutex;

struct LJ64 {
    int kind;
    float sigma, eps, rc, rc2, wf, sig2, pot_cut;
};

__device__ __forceinline__ void lj_pair(const LJ64& p, float3 r, float3& f, float& pe, float& vir) {
    const float rsq = r.x * r.x + r.y * r.y + r.z * r.z;
    f = make_float3(0.f, 0.f, 0.f);
    pe = 0.f;
    vir = 0.f;
    float coeff = 0.f;
    if (p.kind == SG_LJ) {                       // force.f90:26-47
        if (!(rsq < p.rc2)) return;
        const float inv = 1.f / rsq, sr2 = p.sig2 * inv, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        pe = 4.f * p.eps * (sr12 - sr6) - p.pot_cut;
        coeff = 24.f * p.eps * (2.f * sr12 - sr6) * inv;
    } else if (p.kind == SG_LJ12) {              // force.f90:72-91
        if (!(rsq < p.rc2)) return;
        const float inv = 1.f / rsq, sr2 = p.sig2 * inv, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        pe = p.eps * (sr12 - 2.f * sr6) - p.pot_cut;
        coeff = 12.f * p.eps * (sr12 - sr6) * inv;
    } else if (p.kind == SG_LJW) {               // force.f90:116-144
        const float rmag = sqrtf(rsq);
        if (!(rmag < p.rc + p.wf)) return;
        float sr;
        if (rmag < p.sigma) sr = p.sigma / rmag;
        else if (rmag < p.sigma + p.wf) sr = 1.f;
        else sr = p.sigma / (rmag - p.wf);
        const float sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        pe = p.eps * (sr12 - 2.f * sr6) - p.pot_cut;
        coeff = 12.f * p.eps * (sr12 - sr6) * (sr / p.sigma) / rmag;
    } else {                                      // SG_WCA, force.f90:175-188
        if (!(rsq <= p.sig2)) return;
        const float inv = 1.f / rsq, sr2 = p.sig2 * inv, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        pe = p.eps * (sr12 - 2.f * sr6) + p.eps;
        coeff = 12.f * p.eps * (sr12 - sr6) * inv;
    }
    f = coeff * r;
    vir = coeff * rsq;
}

// One lane per pair, 32 consecutive pairs per warp; I-side sums by a
// segmented shuffle scan over runs of equal i, J-side by float4 atomics into
// the scratch accumulator; PE and virial per block in FP64, finished by the
// last block, which adds them to out2[0..1].
//
// The caller's list may hold the pairs of one i in any order, so a run is a
// maximal stretch of adjacent lanes with the same i, and the scan carries a
// head flag: a lane stops adding from below once its partial sum has reached
// the first lane of its run. The last lane of each run flushes its run's sum,
// so an i that appears in two separate runs of a warp is flushed twice, each
// time with only that run's pairs.
//
// A pair whose index (after the one_based shift) lies outside [0, n), or
// whose two indices are equal, is skipped and counted in sc->bad.
__global__ void __launch_bounds__(256) k_pair_noalloc(const double* __restrict__ rx, const double* __restrict__ ry,
                                                      const double* __restrict__ rz, const int* __restrict__ pi_,
                                                      const int* __restrict__ pj_, long long np, int n, int base_index,
                                                      LJ64 p, float3 box, float3 inv_box, int periodic,
                                                      NoallocScratch* sc, double* out2) {
    const int lane = threadIdx.x & 31;
    const long long gwarp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    float pe_t = 0.f, vir_t = 0.f;
    for (long long base = gwarp * 32; base < np; base += nwarps * 32) {
        const long long t = base + lane;
        int i = -1;
        float3 f = make_float3(0.f, 0.f, 0.f);
        if (t < np) {
            // unsigned: a negative or huge index wraps above n and is refused
            const unsigned ii = (unsigned)pi_[t] - (unsigned)base_index;
            const unsigned jj = (unsigned)pj_[t] - (unsigned)base_index;
            if (ii < (unsigned)n && jj < (unsigned)n && ii != jj) {
                i = (int)ii;
                float3 r = make_float3((float)(rx[ii] - rx[jj]), (float)(ry[ii] - ry[jj]), (float)(rz[ii] - rz[jj]));
                r = min_image(r, box, inv_box, periodic);
                float pe, vir;
                lj_pair(p, r, f, pe, vir);
                pe_t += pe;
                vir_t += vir;
                atomicAdd(&sc->acc[jj], make_float4(-f.x, -f.y, -f.z, 0.f));
            } else {
                atomicAdd(&sc->bad, 1u);
            }
        }
        // head flag: lane 0, or a lane whose i differs from the lane below
        const int iprev = __shfl_up_sync(0xffffffffu, i, 1);
        bool head = (lane == 0) || (iprev != i);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float fx = __shfl_up_sync(0xffffffffu, f.x, o);
            const float fy = __shfl_up_sync(0xffffffffu, f.y, o);
            const float fz = __shfl_up_sync(0xffffffffu, f.z, o);
            const bool hup = __shfl_up_sync(0xffffffffu, head, o);
            if (lane >= o && !head) {
                f.x += fx;
                f.y += fy;
                f.z += fz;
                head = hup;
            }
        }
        const int inext = __shfl_down_sync(0xffffffffu, i, 1);
        if ((lane == 31 || inext != i) && i >= 0) atomicAdd(&sc->acc[i], make_float4(f.x, f.y, f.z, 0.f));
    }
    double e[2] = {(double)pe_t, (double)vir_t};
    block_reduce_finish<2>(e, sc->partials, &sc->done, out2);
}

__global__ void k_noalloc_add(int n, const NoallocScratch* __restrict__ sc, double* fx, double* fy, double* fz,
                              int* bad_pairs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && bad_pairs) *bad_pairs = (int)sc->bad;
    if (i >= n) return;
    const float4 a = sc->acc[i];
    fx[i] += a.x;
    fy[i] += a.y;
    fz[i] += a.z;
}

int fail(char* err, int len, int code, const char* msg) {
    if (err && len > 0) {
        strncpy(err, msg, (size_t)len - 1);
        err[len - 1] = 0;
    }
    return code;
}

}  // namespace

extern "C" int sg_lj_forces_noalloc(int32_t n, const double* rx, const double* ry, const double* rz,
                                    const int32_t* pair_i, const int32_t* pair_j, int64_t npairs, int32_t one_based,
                                    const double box[3], int32_t periodic, const sg_pair_params* params, double* fx,
                                    double* fy, double* fz, double* pot_virial, int32_t* bad_pairs, void* stream,
                                    char* err, int32_t err_len) {
    if (!params || !box) return fail(err, err_len, SG_EINVAL, "params and box are required");
    if (params->kind != SG_LJ && params->kind != SG_LJ12 && params->kind != SG_LJW && params->kind != SG_WCA)
        return fail(err, err_len, SG_EINVAL, "sg_lj_forces_noalloc supports SG_LJ, SG_LJ12, SG_LJW and SG_WCA only");
    if (n < 1 || n > SG_NOALLOC_MAX_N)
        return fail(err, err_len, SG_EINVAL,
                    "sg_lj_forces_noalloc: n must be in 1..131072 (the size of its fixed device scratch)");
    if (npairs < 0) return fail(err, err_len, SG_EINVAL, "npairs must be >= 0");
    if (!rx || !ry || !rz || !fx || !fy || !fz || !pot_virial || (npairs > 0 && (!pair_i || !pair_j)))
        return fail(err, err_len, SG_EINVAL, "device arrays must not be NULL");
    if (periodic && !(box[0] > 0.0 && box[1] > 0.0 && box[2] > 0.0))
        return fail(err, err_len, SG_EINVAL, "box dimensions must be positive");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= SG_NOALLOC_MAX_DEVICES)
        return fail(err, err_len, SG_ECUDA, "cudaGetDevice failed");
    NoallocScratch* sc = nullptr;
    {
        // first call on this device: look the scratch up with the device current
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return fail(err, err_len, SG_ECUDA, "cudaGetSymbolAddress failed");
            g_scratch_addr[dev] = static_cast<NoallocScratch*>(p);
        }
        sc = g_scratch_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    LJ64 p;
    p.kind = params->kind;
    p.sigma = (float)params->sigma;
    p.eps = (float)params->epsilon;
    p.rc = (float)params->cutoff;
    p.rc2 = (float)(params->cutoff * params->cutoff);
    p.wf = (float)params->wf;
    p.sig2 = (float)(params->sigma * params->sigma);
    const double sg = params->sigma, ep = params->epsilon, rc = params->cutoff;
    double cut = 0.0;
    if (p.kind == SG_LJ) {
        const double c2 = (sg * sg) / (rc * rc), c6 = c2 * c2 * c2;
        cut = 4.0 * ep * (c6 * c6 - c6);
    } else if (p.kind == SG_LJ12) {
        const double c2 = (sg * sg) / (rc * rc), c6 = c2 * c2 * c2;
        cut = ep * (c6 * c6 - 2.0 * c6);
    } else if (p.kind == SG_LJW) {
        const double c = sg / rc, c2 = c * c, c6 = c2 * c2 * c2;
        cut = ep * (c6 * c6 - 2.0 * c6);
    }
    p.pot_cut = (float)cut;
    const float3 bf = make_float3((float)box[0], (float)box[1], (float)box[2]);
    const float3 ib = periodic ? make_float3((float)(1.0 / box[0]), (float)(1.0 / box[1]), (float)(1.0 / box[2]))
                               : make_float3(0.f, 0.f, 0.f);
    // the scratch keeps the previous call's contents: clear what must start at zero
    if (cudaMemsetAsync(sc->acc, 0, sizeof(float4) * (size_t)n, s) != cudaSuccess ||
        cudaMemsetAsync(&sc->done, 0, 2 * sizeof(unsigned int), s) != cudaSuccess)
        return fail(err, err_len, SG_ECUDA, "cudaMemsetAsync on the scratch failed");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (npairs + 255) / 256;
    if (grid > 4LL * sms) grid = 4LL * sms;
    if (grid > SG_NOALLOC_MAX_BLOCKS) grid = SG_NOALLOC_MAX_BLOCKS;
    if (grid < 1) grid = 1;
    k_pair_noalloc<<<(int)grid, 256, 0, s>>>(rx, ry, rz, pair_i, pair_j, (long long)npairs, n, one_based ? 1 : 0, p,
                                             bf, ib, periodic ? 1 : 0, sc, pot_virial);
    k_noalloc_add<<<(n + 255) / 256, 256, 0, s>>>(n, sc, fx, fy, fz, bad_pairs);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(err, err_len, SG_ECUDA, cudaGetErrorString(e));
    return SG_OK;
}
