// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A thin extern "C" shim over the reference's own C++ port (include/force.h,
// include/integrators.h, src/force.cpp, src/integrators.cpp, src/xmath.cpp),
// compiled from the reference sources in place by build_oracle.py into
// oracle/_ref/. It lets the tests pin the FP64 restatement in
// sucrose_oracle.cpp against code the reference itself ships:
//   LennardJones::calculate_forces   src/force.cpp:6-37 (untruncated 12-6, rint image)
//   MorsePotential::calculate_forces src/force.cpp:113-140 (no cutoff, no shift)
//   VerletIntegrator                  src/integrators.cpp:7-38 (unit mass)
//   Matrix3::determinant              src/xmath.cpp:55
#include <vector>
#include "xmath.h"
#include "system.h"
#include "force.h"
#include "integrators.h"

static void load(System& s, int n, double box_len, int periodic, const double* rx, const double* ry, const double* rz) {
    s.set_num_atoms(n);
    s.box.box_length = box_len;
    s.box.box_xlen = s.box.box_ylen = s.box.box_zlen = box_len;
    s.box.is_periodic = periodic != 0;
    for (int i = 0; i < n; ++i) {
        s.atom.rx[i] = rx[i]; s.atom.ry[i] = ry[i]; s.atom.rz[i] = rz[i];
        s.atom.fx[i] = s.atom.fy[i] = s.atom.fz[i] = 0.0;
        s.atom.vx[i] = s.atom.vy[i] = s.atom.vz[i] = 0.0;
    }
    s.potential_energy = 0.0;
    s.virial = 0.0;
}

extern "C" {

// Calls LennardJones::calculate_forces(i, j) for each listed pair (0-based).
void ref_lj_forces(int n, double box_len, int periodic, const double* rx, const double* ry, const double* rz,
                   double sigma, double epsilon, int npairs, const int* pi, const int* pj, double* fx, double* fy,
                   double* fz, double* pot) {
    System s;
    load(s, n, box_len, periodic, rx, ry, rz);
    LennardJones lj(s, epsilon, sigma);
    for (int k = 0; k < npairs; ++k) lj.calculate_forces(pi[k], pj[k]);
    for (int i = 0; i < n; ++i) { fx[i] = s.atom.fx[i]; fy[i] = s.atom.fy[i]; fz[i] = s.atom.fz[i]; }
    *pot = s.potential_energy;
}

// Calls MorsePotential::calculate_forces(i, j) (src/force.cpp:113-140: no
// cutoff, no shift) for each listed pair (0-based).
void ref_morse_forces(int n, double box_len, int periodic, const double* rx, const double* ry, const double* rz,
                      double dissoc, double rmin, double width, int npairs, const int* pi, const int* pj, double* fx,
                      double* fy, double* fz, double* pot) {
    System s;
    load(s, n, box_len, periodic, rx, ry, rz);
    MorsePotential m(s, dissoc, rmin, width);
    for (int k = 0; k < npairs; ++k) m.calculate_forces(pi[k], pj[k]);
    for (int i = 0; i < n; ++i) { fx[i] = s.atom.fx[i]; fy[i] = s.atom.fy[i]; fz[i] = s.atom.fz[i]; }
    *pot = s.potential_energy;
}

// One VerletIntegrator initial_step + final_step with the given forces.
void ref_vv_step(int n, double box_len, int periodic, double dt, double* rx, double* ry, double* rz, double* vx,
                 double* vy, double* vz, const double* fx, const double* fy, const double* fz, int which) {
    System s;
    load(s, n, box_len, periodic, rx, ry, rz);
    for (int i = 0; i < n; ++i) {
        s.atom.vx[i] = vx[i]; s.atom.vy[i] = vy[i]; s.atom.vz[i] = vz[i];
        s.atom.fx[i] = fx[i]; s.atom.fy[i] = fy[i]; s.atom.fz[i] = fz[i];
    }
    VerletIntegrator vv(s, dt);
    if (which == 0) vv.initial_step(); else vv.final_step();
    for (int i = 0; i < n; ++i) {
        rx[i] = s.atom.rx[i]; ry[i] = s.atom.ry[i]; rz[i] = s.atom.rz[i];
        vx[i] = s.atom.vx[i]; vy[i] = s.atom.vy[i]; vz[i] = s.atom.vz[i];
    }
}

double ref_det3(const double* m9) {
    Matrix3 m;
    for (int k = 0; k < 9; ++k) m(k) = m9[k];
    return m.determinant();
}

}
