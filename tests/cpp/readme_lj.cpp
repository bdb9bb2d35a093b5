// The README's Lennard-Jones time loop (README.md:57-119) written against the
// C++ adapters of sucrose_gpu.hpp, with a System shaped like the reference's
// (include/system.h:10-28). Reads the initial state from a binary file
// (n, box[3], then rx ry rz vx vy vz as n doubles each), runs `steps` steps of
// velocity Verlet with the Verlet list and LJ (rc 2.5, skin 0.3), and prints
// "step pot_eng kin_eng" every `every` steps.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sucrose_gpu.hpp"

struct Atom {
    std::vector<double> rx, ry, rz, vx, vy, vz, fx, fy, fz;
    std::vector<double> qw, qx, qy, qz, lx, ly, lz, tx, ty, tz;
};
struct System {
    int N = 0;
    double box[3] = {0, 0, 0};
    Atom atom;
};

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s state.bin steps every\n", argv[0]);
        return 2;
    }
    System s;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    double hdr[4];
    if (std::fread(hdr, sizeof(double), 4, f) != 4) return 2;
    s.N = (int)hdr[0];
    for (int d = 0; d < 3; ++d) s.box[d] = hdr[1 + d];
    std::vector<double>* cols[6] = {&s.atom.rx, &s.atom.ry, &s.atom.rz, &s.atom.vx, &s.atom.vy, &s.atom.vz};
    for (auto* c : cols) {
        c->resize(s.N);
        if (std::fread(c->data(), sizeof(double), s.N, f) != (size_t)s.N) return 2;
    }
    std::fclose(f);
    const int steps = std::atoi(argv[2]), every = std::atoi(argv[3]);
    try {
        sucrose_gpu::Context ctx(s.N, s.box, true, 0);
        ctx.upload(s);
        ctx.init_nlist(0.3, 2.5);
        sucrose_gpu::LennardJones lj(ctx, 1.0, 1.0, 2.5);
        sucrose_gpu::VerletIntegrator vv(ctx, 0.0005);
        ctx.zero_forces();
        lj.compute();
        for (int step = 1; step <= steps; ++step) {
            vv.initial_step();
            if (ctx.needs_rebuild()) ctx.build_nlist();
            ctx.zero_forces();
            const double pot_eng = lj.compute();
            vv.final_step();
            if (step % every == 0) std::printf("%d %.12e %.12e\n", step, pot_eng, vv.kinetic_energy);
        }
        ctx.download(s);
        ctx.download_forces(s);
        std::printf("final %.12e %.12e %.12e\n", s.atom.rx[0], s.atom.vx[0], s.atom.fx[0]);
    } catch (const sucrose_gpu::Error& e) {
        std::fprintf(stderr, "%s (status %d)\n", e.what(), e.code());
        return 1;
    }
    return 0;
}
