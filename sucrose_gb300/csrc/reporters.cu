// Reporters (fortran/reporters.f90): state data, LAMMPS-style trajectory,
// configuration and checkpoint text files, written asynchronously, plus the
// checkpoint loader and an exact binary state file.
//
// A write records an event on the context stream; a reporter-owned copy
// stream waits on it and copies the device state into a pinned slot, and a
// host thread formats and writes the text once that copy is done. The step
// stream never waits for the file system. Two slots per reporter: a third
// write before the first has been formatted waits for it.
//
// Text follows the reference's edit descriptors: F0.d is the shortest fixed
// form with d decimals (leading zero kept), I0 the shortest integer,
// list-directed integers are right-justified in 12 columns, and nX spacing
// after the last item of a record writes nothing.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "sg_internal.cuh"

namespace {

void put_f(std::string& s, double x, int d) {
    char b[64];
    std::snprintf(b, sizeof(b), "%.*f", d, x);
    s += b;
}

// F0.d of a value that came from FP32 (d <= 10): v * 10^d is exact in FP64
// (24-bit mantissa times 5^d, at most 48 bits), so rounding it to the
// nearest integer (ties to even, as printf does) gives printf's digits
// without printf's cost. Anything outside the exact range goes to printf.
void put_f32(std::string& s, float v, int d) {
    static const double p10[11] = {1, 1e1, 1e2, 1e3, 1e4, 1e5, 1e6, 1e7, 1e8, 1e9, 1e10};
    static const long long i10[11] = {1, 10, 100, 1000, 10000, 100000, 1000000, 10000000, 100000000,
                                      1000000000, 10000000000LL};
    const double q = (double)v * p10[d];
    if (!(std::fabs(q) < 4.0e15)) {
        put_f(s, v, d);
        return;
    }
    const long long u = std::llabs((long long)std::nearbyint(q));
    char b[48];
    int k = 0;
    long long ip = u / i10[d], fp = u % i10[d];
    for (int j = 0; j < d; ++j) {   // fraction digits, low to high
        b[k++] = (char)('0' + fp % 10);
        fp /= 10;
    }
    if (d > 0) b[k++] = '.';
    do {
        b[k++] = (char)('0' + ip % 10);
        ip /= 10;
    } while (ip);
    if (std::signbit(v)) b[k++] = '-';
    while (k) s += b[--k];
}
void put_i(std::string& s, long long v) { s += std::to_string(v); }
void put_list_int(std::string& s, long long v) {   // list-directed integer output
    char b[32];
    std::snprintf(b, sizeof(b), "%12lld", v);
    s += b;
}
// the reference's "(1x, k(I0, 2x), m(F0.d, 2x))" records
struct Rec {
    std::string& s;
    bool first = true;
    explicit Rec(std::string& out, bool lead_blank) : s(out) {
        if (lead_blank) s += ' ';
    }
    void sep() {
        if (!first) s += "  ";
        first = false;
    }
    Rec& i(long long v) { sep(); put_i(s, v); return *this; }
    Rec& f(double x, int d) { sep(); put_f(s, x, d); return *this; }
    Rec& g(float x, int d) { sep(); put_f32(s, x, d); return *this; }
    void end() { s += '\n'; }
};

// Per-particle records formatted by up to 8 threads on contiguous ranges,
// joined in order.
template <class LineFn>
void parallel_lines(int n, std::string& out, LineFn&& line) {
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int T = std::min(std::min(8, hw), std::max(1, n / 8192));
    if (T <= 1) {
        for (int i = 0; i < n; ++i) line(i, out);
        return;
    }
    std::vector<std::string> parts(T);
    std::vector<std::thread> th;
    for (int t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            const int a = (int)((long long)n * t / T), b = (int)((long long)n * (t + 1) / T);
            for (int i = a; i < b; ++i) line(i, parts[t]);
        });
    for (auto& x : th) x.join();
    for (auto& p : parts) out += p;
}

// one snapshot of the device state, in pinned host memory
enum { A_POS, A_VEL, A_QUAT, A_ANGM, A_FORCE, A_SHAPE, A_ESHAPE, A_INERT, A_N };

struct Slot {
    float4* host = nullptr;      // A_N arrays of n float4
    double acc[8];
    double box[3];
    cudaEvent_t done = nullptr;
    bool busy = false;
};

struct Job {
    int slot;
    long long step;
};

}  // namespace

struct sg_reporter {
    sg_ctx* ctx = nullptr;
    int kind = 0;
    FILE* f = nullptr;
    int n = 0;
    int dof = 0, nrigid = 1;
    double density = 0.0;
    long long config_index = 0;
    cudaStream_t copy = nullptr;
    cudaEvent_t ready[2] = {nullptr, nullptr};
    Slot slot[2];
    std::deque<Job> queue;
    std::mutex mu;
    std::condition_variable cv;
    bool stop = false, working = false;
    int io_error = 0;
    std::thread worker;
    std::vector<int> types;
    std::vector<int> bbi, bbj;
    std::vector<double> blen;

    const float4* arr(const Slot& s, int a) const { return s.host + (size_t)a * n; }

    void format(const Slot& s, long long step, std::string& out) {
        const float4 *P = arr(s, A_POS), *V = arr(s, A_VEL), *Q = arr(s, A_QUAT), *L = arr(s, A_ANGM);
        const float4 *F = arr(s, A_FORCE), *S = arr(s, A_SHAPE), *E = arr(s, A_ESHAPE), *I = arr(s, A_INERT);
        if (kind == SG_REPORT_STATE) {   // report_state_data (reporters.f90:21-37)
            const double pot_av = s.acc[0] / n, kin_av = s.acc[2] / n, rot_av = s.acc[3] / n;
            const double kin_tot = kin_av + rot_av, tot = pot_av + kin_tot;
            // calculate_thermo (system.f90:725-741) from the same snapshot
            const double temp = dof > 0 ? 2.0 * (s.acc[2] + s.acc[3]) / dof : 0.0;
            double vir = 0.0;
            for (int i = 0; i < n; ++i)
                vir += (double)P[i].x * F[i].x + (double)P[i].y * F[i].y + (double)P[i].z * F[i].z;
            if (!bbi.empty() && s.acc[6] >= 0.0) vir += s.acc[6];
            const double vol = s.box[0] * s.box[1] * s.box[2];
            const double pres = density * nrigid * temp + vir / (3.0 * vol);
            Rec r(out, false);
            r.i(step).f(pot_av, 10).f(kin_tot, 10).f(tot, 10).f(temp, 10).f(pres, 10).f(density, 10).end();
        } else if (kind == SG_REPORT_TRAJECTORY) {   // report_trajectory (reporters.f90:66-92)
            out += "ITEM: TIMESTEP\n";
            put_list_int(out, step);
            out += "\nITEM: NUMBER OF ATOMS\n";
            put_list_int(out, n);
            out += "\nITEM: BOX BOUNDS pp pp pp\n";
            for (int d = 0; d < 3; ++d) Rec(out, true).f(-s.box[d] / 2.0, 3).f(s.box[d] / 2.0, 3).end();
            out += "ITEM: ATOMS id type shapex shapey shapez x y z vx vy vz fx fy fz quatw quati quatj quatk\n";
            parallel_lines(n, out, [&](int i, std::string& o) {
                const double w = Q[i].x, x = Q[i].y, y = Q[i].z, z = Q[i].w;
                // the columns headed vx vy vz hold the body z axis (:82-84)
                const double ux = 2.0 * (x * z + w * y), uy = 2.0 * (y * z - w * x), uz = w * w - x * x - y * y + z * z;
                Rec r(o, true);
                r.i(i + 1).i(types[i]).g(S[i].x, 3).g(S[i].y, 3).g(S[i].z, 3).g(P[i].x, 3).g(P[i].y, 3).g(P[i].z, 3);
                r.f(ux, 3).f(uy, 3).f(uz, 3).g(F[i].x, 3).g(F[i].y, 3).g(F[i].z, 3);
                r.g(Q[i].x, 3).g(Q[i].y, 3).g(Q[i].z, 3).g(Q[i].w, 3).end();
            });
        } else if (kind == SG_REPORT_CONFIG) {   // report_confwriter (reporters.f90:120-129)
            parallel_lines(n, out, [&](int i, std::string& o) {
                Rec r(o, false);
                r.g(P[i].x, 3).g(P[i].y, 3).g(P[i].z, 3).g(V[i].x, 3).g(V[i].y, 3).g(V[i].z, 3);
                r.g(L[i].x, 3).g(L[i].y, 3).g(L[i].z, 3).g(Q[i].x, 3).g(Q[i].y, 3).g(Q[i].z, 3).g(Q[i].w, 3).end();
            });
        } else {   // report_checkpoint (reporters.f90:158-184)
            out += "ATOMS ";
            put_i(out, n);
            out += "\n\nBONDS ";
            put_i(out, (long long)bbi.size());
            out += "\n\nBOX ";
            Rec(out, false).f(s.box[0], 10).f(s.box[1], 10).f(s.box[2], 10).end();
            out += "\nATOM: ID TYPE MASS CHARGE SHAPEX SHAPEY SHAPEZ ESHAPEX ESHAPEY ESHAPEZ IXX IYY IZZ RX RY RZ VX VY "
                   "VZ LX LY LZ QW QX QY QZ\n\n";
            parallel_lines(n, out, [&](int i, std::string& o) {
                Rec r(o, true);
                r.i(i + 1).i(types[i]).g(S[i].w, 10).g(P[i].w, 10).g(S[i].x, 10).g(S[i].y, 10).g(S[i].z, 10);
                r.g(E[i].x, 10).g(E[i].y, 10).g(E[i].z, 10).g(I[i].x, 10).g(I[i].y, 10).g(I[i].z, 10);
                r.g(P[i].x, 10).g(P[i].y, 10).g(P[i].z, 10).g(V[i].x, 10).g(V[i].y, 10).g(V[i].z, 10);
                r.g(L[i].x, 10).g(L[i].y, 10).g(L[i].z, 10).g(Q[i].x, 10).g(Q[i].y, 10).g(Q[i].z, 10);
                r.g(Q[i].w, 10).end();
            });
            out += "\nBOND: ID I J LEN\n\n";
            for (size_t k = 0; k < bbi.size(); ++k)
                Rec(out, true).i((long long)k + 1).i(bbi[k] + 1).i(bbj[k] + 1).f(blen[k], 10).end();
            out += "\n";
            put_list_int(out, config_index);   // never advanced by the reference (:156, :184)
            out += "\n";
        }
    }

    void run() {
        cudaSetDevice(ctx->device);
        std::string text;
        for (;;) {
            Job j;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || !queue.empty(); });
                if (queue.empty()) return;
                j = queue.front();
                queue.pop_front();
                working = true;
            }
            Slot& s = slot[j.slot];
            int err = cudaEventSynchronize(s.done) == cudaSuccess ? 0 : SG_ECUDA;
            if (!err) {
                text.clear();
                format(s, j.step, text);
                if (std::fwrite(text.data(), 1, text.size(), f) != text.size() || std::fflush(f) != 0) err = SG_EINVAL;
            }
            {
                std::lock_guard<std::mutex> lk(mu);
                s.busy = false;
                working = false;
                if (err && !io_error) io_error = err;
            }
            cv.notify_all();
        }
    }
};

extern "C" {

int sg_set_types(sg_ctx* ctx, const int32_t* type) {
    if (!ctx) return SG_EINVAL;
    sg_state_touched(ctx);
    ctx->h_types.assign(ctx->n, 0);
    // initialize_system (fortran/system.f90:590-593): a negative type becomes 0
    for (int i = 0; type && i < ctx->n; ++i) ctx->h_types[i] = type[i] < 0 ? 0 : type[i];
    return SG_OK;
}

int sg_reporter_open(sg_ctx* ctx, int32_t kind, const char* path, sg_reporter** out) {
    if (!ctx || !path || !out || kind < 0 || kind > 3) return SG_EINVAL;
    *out = nullptr;
    if (ctx->nrep) return sg_fail(ctx, SG_EINVAL, "reporters write one system: no replica contexts");
    FILE* f = std::fopen(path, "w");
    if (!f) return sg_fail(ctx, SG_EINVAL, "cannot open %s for writing (errno %d)", path, errno);
    auto* r = new sg_reporter();
    r->ctx = ctx;
    r->kind = kind;
    r->f = f;
    r->n = ctx->n;
    r->types = ctx->h_types;
    r->types.resize(ctx->n, 0);
    r->bbi = ctx->h_bbi;
    r->bbj = ctx->h_bbj;
    r->blen = ctx->h_blen;
    auto fail = [&](cudaError_t e) {
        sg_reporter_close(r);
        return sg_cuda_check(ctx, e, "sg_reporter_open");
    };
    cudaError_t e = cudaStreamCreateWithFlags(&r->copy, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        e = cudaEventCreateWithFlags(&r->ready[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&r->slot[k].done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaMallocHost(&r->slot[k].host, sizeof(float4) * A_N * (size_t)r->n);
    }
    if (e != cudaSuccess) return fail(e);
    if (kind == SG_REPORT_STATE)   // open_state_data_file (reporters.f90:7-19)
        std::fputs("Step  Potential_Energy  Kinetic_Energy  Total_Energy  Temperature  Pressure  Density\n", f);
    r->worker = std::thread([r] { r->run(); });
    *out = r;
    return SG_OK;
}

int sg_reporter_set_thermo(sg_reporter* r, int32_t dof, double density, int32_t nrigid) {
    if (!r) return SG_EINVAL;
    r->dof = dof;
    r->density = density;
    r->nrigid = nrigid;
    return SG_OK;
}

int sg_reporter_write(sg_reporter* r, int64_t step) {
    if (!r) return SG_EINVAL;
    sg_ctx* ctx = r->ctx;
    int k;
    {
        std::unique_lock<std::mutex> lk(r->mu);
        r->cv.wait(lk, [&] { return !r->slot[0].busy || !r->slot[1].busy || r->io_error; });
        if (r->io_error) return sg_fail(ctx, r->io_error, "reporter: an earlier write failed");
        k = r->slot[0].busy ? 1 : 0;
        r->slot[k].busy = true;
    }
    Slot& s = r->slot[k];
    for (int d = 0; d < 3; ++d) s.box[d] = ctx->box[d];
    const float4* src[A_N] = {ctx->pos, ctx->vel, ctx->quat, ctx->angm, ctx->force, ctx->shape, ctx->eshape,
                              ctx->inert};
    const size_t bytes = sizeof(float4) * (size_t)r->n;
    cudaError_t e = cudaEventRecord(r->ready[k], ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(r->copy, r->ready[k], 0);
    for (int a = 0; a < A_N && e == cudaSuccess; ++a)
        e = cudaMemcpyAsync(s.host + (size_t)a * r->n, src[a], bytes, cudaMemcpyDeviceToHost, r->copy);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.acc, ctx->acc, sizeof(s.acc), cudaMemcpyDeviceToHost, r->copy);
    if (e == cudaSuccess) e = cudaEventRecord(s.done, r->copy);
    if (e != cudaSuccess) {
        std::lock_guard<std::mutex> lk(r->mu);
        s.busy = false;
        return sg_cuda_check(ctx, e, "sg_reporter_write");
    }
    {
        std::lock_guard<std::mutex> lk(r->mu);
        r->queue.push_back({k, (long long)step});
    }
    r->cv.notify_all();
    return SG_OK;
}

int sg_reporter_flush(sg_reporter* r) {
    if (!r) return SG_EINVAL;
    std::unique_lock<std::mutex> lk(r->mu);
    r->cv.wait(lk, [&] { return r->queue.empty() && !r->working; });
    if (r->io_error) return sg_fail(r->ctx, r->io_error, "reporter: a write failed");
    return SG_OK;
}

int sg_reporter_close(sg_reporter* r) {
    if (!r) return SG_OK;
    int rc = SG_OK;
    if (r->worker.joinable()) {
        rc = sg_reporter_flush(r);
        {
            std::lock_guard<std::mutex> lk(r->mu);
            r->stop = true;
        }
        r->cv.notify_all();
        r->worker.join();
    }
    if (r->f) std::fclose(r->f);
    for (int k = 0; k < 2; ++k) {
        if (r->slot[k].host) cudaFreeHost(r->slot[k].host);
        if (r->slot[k].done) cudaEventDestroy(r->slot[k].done);
        if (r->ready[k]) cudaEventDestroy(r->ready[k]);
    }
    if (r->copy) cudaStreamDestroy(r->copy);
    delete r;
    return rc;
}

// ---- checkpoint text loader (load_checkpoint, reporters.f90:186-223) ----------
int sg_load_checkpoint(const char* path, int32_t device, sg_ctx** out, int64_t* config_index) {
    if (!path || !out) return SG_EINVAL;
    *out = nullptr;
    FILE* f = std::fopen(path, "r");
    if (!f) return SG_EINVAL;
    int na = 0, nb = 0;
    double box[3];
    char label[64];
    auto line = [&](char* buf, int cap) { return std::fgets(buf, cap, f) != nullptr; };
    std::vector<char> buf(1 << 16);
    bool ok = line(buf.data(), (int)buf.size()) && std::sscanf(buf.data(), "%63s %d", label, &na) == 2;
    ok = ok && line(buf.data(), (int)buf.size());
    ok = ok && line(buf.data(), (int)buf.size()) && std::sscanf(buf.data(), "%63s %d", label, &nb) == 2;
    ok = ok && line(buf.data(), (int)buf.size());
    ok = ok && line(buf.data(), (int)buf.size()) &&
         std::sscanf(buf.data(), "%63s %lf %lf %lf", label, &box[0], &box[1], &box[2]) == 4;
    ok = ok && line(buf.data(), (int)buf.size()) && line(buf.data(), (int)buf.size()) &&
         line(buf.data(), (int)buf.size());
    if (!ok || na < 1 || nb < 0) {
        std::fclose(f);
        return SG_EINVAL;
    }
    std::vector<std::vector<double>> col(26, std::vector<double>(na));
    std::vector<int> type(na);
    for (int i = 0; i < na && ok; ++i) {
        ok = line(buf.data(), (int)buf.size());
        double v[26];
        int id = 0, t = 0;
        ok = ok && std::sscanf(buf.data(),
                               " %d %d %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf "
                               "%lf %lf %lf %lf",
                               &id, &t, &v[2], &v[3], &v[4], &v[5], &v[6], &v[7], &v[8], &v[9], &v[10], &v[11],
                               &v[12], &v[13], &v[14], &v[15], &v[16], &v[17], &v[18], &v[19], &v[20], &v[21],
                               &v[22], &v[23], &v[24], &v[25]) == 26;
        ok = ok && id >= 1 && id <= na;
        if (ok) {
            type[id - 1] = t;
            for (int c = 2; c < 26; ++c) col[c][id - 1] = v[c];
        }
    }
    ok = ok && line(buf.data(), (int)buf.size()) && line(buf.data(), (int)buf.size()) &&
         line(buf.data(), (int)buf.size());
    std::vector<int32_t> bi(nb), bj(nb);
    std::vector<double> bl(nb);
    for (int k = 0; k < nb && ok; ++k) {
        int id = 0;
        ok = line(buf.data(), (int)buf.size()) &&
             std::sscanf(buf.data(), " %d %d %d %lf", &id, &bi[k], &bj[k], &bl[k]) == 4;
    }
    long long cfg = 0;
    if (ok && line(buf.data(), (int)buf.size()) && line(buf.data(), (int)buf.size()))
        std::sscanf(buf.data(), " %lld", &cfg);
    std::fclose(f);
    if (!ok) return SG_EINVAL;
    sg_ctx* ctx = nullptr;
    int rc = sg_create(&ctx, na, device);
    *out = ctx;
    if (rc) return rc;
    if ((rc = sg_set_box(ctx, box, 1))) return rc;
    // columns: 2 mass 3 charge 4-6 shape 7-9 eshape 10-12 inertia 13-15 r 16-18 v 19-21 L 22-25 q
    if ((rc = sg_set_particles(ctx, col[2].data(), col[4].data(), col[5].data(), col[6].data(), col[7].data(),
                               col[8].data(), col[9].data(), col[10].data(), col[11].data(), col[12].data())))
        return rc;
    if ((rc = sg_set_charges(ctx, col[3].data(), 0))) return rc;
    if ((rc = sg_set_types(ctx, type.data()))) return rc;
    if ((rc = sg_upload_state(ctx, col[13].data(), col[14].data(), col[15].data(), col[22].data(), col[23].data(),
                              col[24].data(), col[25].data(), col[16].data(), col[17].data(), col[18].data(),
                              col[19].data(), col[20].data(), col[21].data())))
        return rc;
    if (nb > 0 && (rc = sg_set_constraints(ctx, nb, bi.data(), bj.data(), bl.data(), 1))) return rc;
    if (config_index) *config_index = cfg;
    return SG_OK;
}

// ---- exact binary state ------------------------------------------------------
// Layout: "SGST", version 1, n, periodic, box[3] (FP64), the ten float4
// particle arrays in the context's order, the thermostat chain (32 FP64), the
// captured step's counter and the energy accumulators (8 FP64).
int sg_save_state(sg_ctx* ctx, const char* path) {
    if (!ctx || !path) return SG_EINVAL;
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // the copies below use the default stream
    FILE* f = std::fopen(path, "wb");
    if (!f) return sg_fail(ctx, SG_EINVAL, "cannot open %s", path);
    const size_t n = (size_t)ctx->n;
    std::vector<float4> h(n);
    const float4* arrs[10] = {ctx->pos, ctx->quat, ctx->vel, ctx->angm, ctx->force, ctx->torque, ctx->shape,
                              ctx->eshape, ctx->inert, ctx->inert_inv};
    const int32_t head[4] = {0x54534753, 1, ctx->n, ctx->periodic};
    bool ok = std::fwrite(head, sizeof(head), 1, f) == 1 && std::fwrite(ctx->box, sizeof(double), 3, f) == 3;
    for (int a = 0; a < 10 && ok; ++a) {
        if (cudaMemcpy(h.data(), arrs[a], sizeof(float4) * n, cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
        ok = ok && std::fwrite(h.data(), sizeof(float4), n, f) == n;
    }
    double nh[32], acc[8];
    int step = 0;
    ok = ok && cudaMemcpy(nh, ctx->nh, sizeof(nh), cudaMemcpyDeviceToHost) == cudaSuccess;
    ok = ok && cudaMemcpy(acc, ctx->acc, sizeof(acc), cudaMemcpyDeviceToHost) == cudaSuccess;
    if (ok && ctx->step_dev) ok = cudaMemcpy(&step, ctx->step_dev, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
    ok = ok && std::fwrite(nh, sizeof(nh), 1, f) == 1 && std::fwrite(&step, sizeof(int), 1, f) == 1 &&
         std::fwrite(acc, sizeof(acc), 1, f) == 1;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? SG_OK : sg_fail(ctx, SG_EINVAL, "writing %s failed", path);
}

int sg_load_state(sg_ctx* ctx, const char* path) {
    if (!ctx || !path) return SG_EINVAL;
    sg_state_touched(ctx);
    SG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    FILE* f = std::fopen(path, "rb");
    if (!f) return sg_fail(ctx, SG_EINVAL, "cannot open %s", path);
    int32_t head[4];
    double box[3];
    bool ok = std::fread(head, sizeof(head), 1, f) == 1 && head[0] == 0x54534753 && head[1] == 1 &&
              head[2] == ctx->n && std::fread(box, sizeof(double), 3, f) == 3;
    if (!ok) {
        std::fclose(f);
        return sg_fail(ctx, SG_EINVAL, "%s is not a state file of %d particles", path, ctx->n);
    }
    const size_t n = (size_t)ctx->n;
    std::vector<float4> h(n);
    float4* arrs[10] = {ctx->pos, ctx->quat, ctx->vel, ctx->angm, ctx->force, ctx->torque, ctx->shape,
                        ctx->eshape, ctx->inert, ctx->inert_inv};
    for (int a = 0; a < 10 && ok; ++a) {
        ok = std::fread(h.data(), sizeof(float4), n, f) == n;
        ok = ok && cudaMemcpy(arrs[a], h.data(), sizeof(float4) * n, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    double nh[32], acc[8];
    int step = 0;
    ok = ok && std::fread(nh, sizeof(nh), 1, f) == 1 && std::fread(&step, sizeof(int), 1, f) == 1 &&
         std::fread(acc, sizeof(acc), 1, f) == 1;
    std::fclose(f);
    ok = ok && cudaMemcpy(ctx->nh, nh, sizeof(nh), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMemcpy(ctx->acc, acc, sizeof(acc), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok && ctx->step_dev) ok = cudaMemcpy(ctx->step_dev, &step, sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) return sg_fail(ctx, SG_EINVAL, "reading %s failed", path);
    for (int d = 0; d < 3; ++d) ctx->box[d] = box[d];
    ctx->periodic = head[3];
    ctx->graph_epoch++;
    return sg_nlist_box_changed(ctx);
}

}  // extern "C"
