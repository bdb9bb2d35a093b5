// ORACLE — TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement, in FP64 (templated so it can also run in FP32 to predict
// single-precision error), of the SUCROSE Fortran hot path:
//   Philox4x32-10 and Box-Muller normals   fortran/xmath.f90:1-113
//   3x3 algebra and Cholesky solve         fortran/xmath.f90:117-318
//   Verlet list and rebuild trigger        fortran/system.f90:885-1053
//   LJ / LJ12 / LJW / WCA                  fortran/force.f90:6-190
//   Gay-Berne family                       fortran/force.f90:237-1030
//   ECP family and its Brent solve         fortran/force.f90:1034-2236
//   VV / quaternion / Nose-Hoover / Langevin  fortran/integrators.f90:1-392,494-676
//   velocity init, defaults, thermo        fortran/system.f90:362-741
//
// Only tests, the smoke check and the CPU-baseline leg of the benchmark load
// this library, and only as the checker or as the timed CPU reference. The GPU
// product never links it.
//
// Numerical contract: compiled without FMA contraction and without fast-math
// (see build_oracle.py) so that every FP64 operation is one IEEE-754 rounding
// in the reference's own evaluation order. Indices are 0-based here; the
// exported Verlet list uses the reference's 1-based CSR when asked.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>
#include <algorithm>
#include <vector>

namespace {

// ---------------------------------------------------------------- Philox ---
// fortran/xmath.f90:5-11 constants; :14-26 mulhilo32; :42-76 the 10 rounds.
const uint32_t PHILOX_M0 = 0xD2511F53u;
const uint32_t PHILOX_M1 = 0xCD9E8D57u;
const uint32_t PHILOX_W0 = 0x9E3779B9u;
const uint32_t PHILOX_W1 = 0xBB67AE85u;
const uint32_t PHILOX_KEY0 = 0x6D2B79F5u;
const uint32_t PHILOX_KEY1 = 0x1B873593u;

inline void mulhilo32(uint32_t a, uint32_t b, uint32_t& hi, uint32_t& lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    lo = (uint32_t)(p & 0xFFFFFFFFull);
    hi = (uint32_t)(p >> 32);
}

void philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 1; round <= 10; ++round) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(PHILOX_M0, c0, hi0, lo0);
        mulhilo32(PHILOX_M1, c2, hi1, lo1);
        uint32_t n0 = hi1 ^ (c1 ^ k0);
        uint32_t n2 = hi0 ^ (c3 ^ k1);
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        if (round < 10) { k0 += PHILOX_W0; k1 += PHILOX_W1; }
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

inline double philox_real(uint32_t w) { return (double)w * (1.0 / 4294967296.0); }

// fortran/xmath.f90:78-113 (u1, u3 clamped to 1e-35; the fourth normal dropped)
void normal_3seq(const uint32_t ctr[4], const uint32_t key[2], double& n1, double& n2, double& n3) {
    const double TWOPI = 6.283185307179586;
    const double TINY = 1.0e-35;
    uint32_t w[4];
    philox(ctr, key, w);
    double u1 = philox_real(w[0]), u2 = philox_real(w[1]);
    double u3 = philox_real(w[2]), u4 = philox_real(w[3]);
    u1 = std::max(u1, TINY);
    u3 = std::max(u3, TINY);
    double r1 = std::sqrt(-2.0 * std::log(u1));
    double th1 = TWOPI * u2;
    double r2 = std::sqrt(-2.0 * std::log(u3));
    double th2 = TWOPI * u4;
    n1 = r1 * std::cos(th1);
    n2 = r1 * std::sin(th1);
    n3 = r2 * std::cos(th2);
}

// ---------------------------------------------------------------- xmath ---
// Matrices are M[row][col] = Fortran M(row+1, col+1).
template <class T> struct M3 { T m[3][3]; };

template <class T> inline T rnd(T x) { return std::round(x); }  // ANINT: half away from zero

template <class T> inline void cross(const T a[3], const T b[3], T o[3]) {   // xmath.f90:130
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

template <class T> inline T determinant(const M3<T>& M) {                    // xmath.f90:141
    const T (*m)[3] = M.m;
    return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2])
         - m[0][1] * (m[1][0] * m[2][2] - m[2][0] * m[1][2])
         + m[0][2] * (m[1][0] * m[2][1] - m[2][0] * m[1][1]);
}

template <class T> inline M3<T> inverse(const M3<T>& M) {                     // xmath.f90:152
    const T (*m)[3] = M.m;
    M3<T> o;
    o.m[0][0] = m[1][1] * m[2][2] - m[2][1] * m[1][2];
    o.m[0][1] = m[0][2] * m[2][1] - m[0][1] * m[2][2];
    o.m[0][2] = m[0][1] * m[1][2] - m[0][2] * m[1][1];
    o.m[1][0] = m[1][2] * m[2][0] - m[1][0] * m[2][2];
    o.m[1][1] = m[0][0] * m[2][2] - m[0][2] * m[2][0];
    o.m[1][2] = m[0][2] * m[1][0] - m[0][0] * m[1][2];
    o.m[2][0] = m[1][0] * m[2][1] - m[1][1] * m[2][0];
    o.m[2][1] = m[0][1] * m[2][0] - m[0][0] * m[2][1];
    o.m[2][2] = m[0][0] * m[1][1] - m[0][1] * m[1][0];
    T det = determinant(M);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) o.m[i][j] = o.m[i][j] / det;
    return o;
}

// rotation_matrix form used by ECP and the integrators (force.f90:1244-1252,
// integrators.f90:144-152): row k is body axis k in the lab frame.
template <class T> inline M3<T> rotmat(T w, T x, T y, T z) {
    M3<T> r;
    r.m[0][0] = w * w + x * x - y * y - z * z;
    r.m[0][1] = T(2.0) * (x * y + w * z);
    r.m[0][2] = T(2.0) * (x * z - w * y);
    r.m[1][0] = T(2.0) * (x * y - w * z);
    r.m[1][1] = w * w - x * x + y * y - z * z;
    r.m[1][2] = T(2.0) * (y * z + w * x);
    r.m[2][0] = T(2.0) * (x * z + w * y);
    r.m[2][1] = T(2.0) * (y * z - w * x);
    r.m[2][2] = w * w - x * x - y * y + z * z;
    return r;
}

template <class T> inline void mvdot(const M3<T>& a, const T b[3], T o[3]) { // xmath.f90:231
    for (int i = 0; i < 3; ++i) o[i] = a.m[i][0] * b[0] + a.m[i][1] * b[1] + a.m[i][2] * b[2];
}
template <class T> inline void vmdot(const T a[3], const M3<T>& b, T o[3]) { // xmath.f90:219
    for (int j = 0; j < 3; ++j) o[j] = a[0] * b.m[0][j] + a[1] * b.m[1][j] + a[2] * b.m[2][j];
}
template <class T> inline M3<T> mmdot(const M3<T>& a, const M3<T>& b) {      // xmath.f90:243
    M3<T> o;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            o.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return o;
}
// A^T B A for diagonal B (xmath.f90:262-279)
template <class T> inline M3<T> matmul_atba(const M3<T>& A, const M3<T>& B) {
    const T (*a)[3] = A.m;
    T b0 = B.m[0][0], b1 = B.m[1][1], b2 = B.m[2][2];
    M3<T> o;
    o.m[0][0] = a[0][0] * b0 * a[0][0] + a[1][0] * b1 * a[1][0] + a[2][0] * b2 * a[2][0];
    o.m[0][1] = a[0][0] * b0 * a[0][1] + a[1][0] * b1 * a[1][1] + a[2][0] * b2 * a[2][1];
    o.m[0][2] = a[0][0] * b0 * a[0][2] + a[1][0] * b1 * a[1][2] + a[2][0] * b2 * a[2][2];
    o.m[1][0] = o.m[0][1];
    o.m[1][1] = a[0][1] * b0 * a[0][1] + a[1][1] * b1 * a[1][1] + a[2][1] * b2 * a[2][1];
    o.m[1][2] = a[0][1] * b0 * a[0][2] + a[1][1] * b1 * a[1][2] + a[2][1] * b2 * a[2][2];
    o.m[2][0] = o.m[0][2];
    o.m[2][1] = o.m[1][2];
    o.m[2][2] = a[0][2] * b0 * a[0][2] + a[1][2] * b1 * a[1][2] + a[2][2] * b2 * a[2][2];
    return o;
}
// 3x3 SPD solve, lower triangle read (xmath.f90:281-304)
template <class T> inline void cholesky_solve(const M3<T>& A, const T b[3], T o[3]) {
    const T (*a)[3] = A.m;
    T inv_l11 = T(1.0) / std::sqrt(a[0][0]);
    T l21 = a[1][0] * inv_l11;
    T l31 = a[2][0] * inv_l11;
    T inv_l22 = T(1.0) / std::sqrt(a[1][1] - l21 * l21);
    T l32 = (a[2][1] - l31 * l21) * inv_l22;
    T inv_l33 = T(1.0) / std::sqrt(a[2][2] - l31 * l31 - l32 * l32);
    T y1 = b[0] * inv_l11;
    T y2 = (b[1] - l21 * y1) * inv_l22;
    T y3 = (b[2] - l31 * y1 - l32 * y2) * inv_l33;
    o[2] = y3 * inv_l33;
    o[1] = (y2 - l32 * o[2]) * inv_l22;
    o[0] = (y1 - l21 * o[1] - l31 * o[2]) * inv_l11;
}

template <class T> inline T ipow(T x, int n) {
    T r = T(1.0);
    for (int k = 0; k < n; ++k) r = r * x;
    return r;
}

} // namespace

// ================================================================ C ABI ====
extern "C" {

// State of one system, SoA FP64, borrowed from the caller (numpy arrays).
typedef struct OrSys {
    int n, periodic, nc, nrigid, dof;
    int target_temp_set;
    double box[3];
    double *rx, *ry, *rz, *vx, *vy, *vz, *fx, *fy, *fz;
    double *qw, *qx, *qy, *qz, *lx, *ly, *lz, *tx, *ty, *tz;
    double *mass, *inv_mass;
    double *sig_x, *sig_y, *sig_z, *eps_x, *eps_y, *eps_z;
    double *ixx, *iyy, *izz, *ixx_inv, *iyy_inv, *izz_inv;
    double pot_eng, kin_eng, kin_rot, temp, pressure, density, virial, target_temp;
    double eta[3], p_eta[3];       // Nose-Hoover chain (integrators.f90:230)
    double eta_r[3], p_eta_r[3];   // rotational chain of the standard NHC mode
    double* charge;                // system.f90:7 (NULL: all zero)
    double *dipx, *dipy, *dipz;    // module dipole DIP arrays (force.f90:2671)
    double rfl[3];                 // RFL: every element of the reference's RFL arrays holds this vector
    double *rx_old, *ry_old, *rz_old;   // system.f90:22
    int *bbi, *bbj;                // constraint atoms, 0-based, nc of them (system.f90:32-33)
    double* bb_len;
    double virial_bonded;          // system.f90:29
    int rattle_sweeps;             // sweeps of the last apply_constraints_a / _b call
} OrSys;

// Pair-potential parameters shared by every family.
typedef struct OrPairParams {
    int kind;        // see OR_* below
    int mu, nu;      // GB / ECP exponents
    int solver;      // ECP: 0 = reference Brent, 1 = tightly converged FP64, 2 = use lam_in
    double sigma, epsilon, cutoff, wf, chirality;
    double lam_in;   // ECP with solver 2
    double dissoc, width, rmin;   // morse
    double db_len, dielectric;    // dh, coulombic, dipole
} OrPairParams;

enum {
    OR_LJ = 0, OR_LJ12 = 1, OR_LJW = 2, OR_WCA = 3, OR_MORSE = 4, OR_DH = 5, OR_COULOMB = 6, OR_DIPOLE = 7,
    OR_GB = 10, OR_GBR = 11, OR_GBW = 12, OR_GBC = 13, OR_GBWC = 14,
    OR_ECP = 20, OR_ECPR = 21, OR_ECPW = 22, OR_ECPC = 23, OR_ECPWC = 24,
};

void or_philox4x32(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { philox(ctr, key, out); }

void or_philox4x32_batch(int n, const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    for (int i = 0; i < n; ++i) philox(ctr + 4 * i, key, out + 4 * i);
}

// philox_normal_3seq with the reference key (xmath.f90:78)
void or_philox_normal_3seq(int32_t c1, int32_t c2, int32_t c3, int32_t c4, double* n) {
    uint32_t ctr[4] = {(uint32_t)c1, (uint32_t)c2, (uint32_t)c3, (uint32_t)c4};
    uint32_t key[2] = {PHILOX_KEY0, PHILOX_KEY1};
    normal_3seq(ctr, key, n[0], n[1], n[2]);
}

} // extern "C"

namespace {

// ------------------------------------------------------- pair inputs -------
template <class T> struct PairIn {
    T rij[3];                 // minimum image r_i - r_j
    T qi[4], qj[4];           // (w,x,y,z)
    T si[3], sj[3], ei[3], ej[3];
    T ci, cj;                 // charges
};

template <class T> inline void min_image(T r[3], const double box[3], int periodic) {
    if (!periodic) return;
    for (int d = 0; d < 3; ++d) {
        T b = T(box[d]);
        r[d] = r[d] - rnd(r[d] / b) * b;
    }
}

template <class T> PairIn<T> load_pair(const OrSys* s, int i, int j) {
    PairIn<T> p;
    p.rij[0] = T(s->rx[i]) - T(s->rx[j]);
    p.rij[1] = T(s->ry[i]) - T(s->ry[j]);
    p.rij[2] = T(s->rz[i]) - T(s->rz[j]);
    min_image(p.rij, s->box, s->periodic);
    if (s->qw) {
        p.qi[0] = T(s->qw[i]); p.qi[1] = T(s->qx[i]); p.qi[2] = T(s->qy[i]); p.qi[3] = T(s->qz[i]);
        p.qj[0] = T(s->qw[j]); p.qj[1] = T(s->qx[j]); p.qj[2] = T(s->qy[j]); p.qj[3] = T(s->qz[j]);
    }
    if (s->sig_x) {
        p.si[0] = T(s->sig_x[i]); p.si[1] = T(s->sig_y[i]); p.si[2] = T(s->sig_z[i]);
        p.sj[0] = T(s->sig_x[j]); p.sj[1] = T(s->sig_y[j]); p.sj[2] = T(s->sig_z[j]);
    }
    p.ci = s->charge ? T(s->charge[i]) : T(0.0);
    p.cj = s->charge ? T(s->charge[j]) : T(0.0);
    if (s->eps_x) {
        p.ei[0] = T(s->eps_x[i]); p.ei[1] = T(s->eps_y[i]); p.ei[2] = T(s->eps_z[i]);
        p.ej[0] = T(s->eps_x[j]); p.ej[1] = T(s->eps_y[j]); p.ej[2] = T(s->eps_z[j]);
    }
    return p;
}

struct PairOut {
    double pe, f[3], ti[3], tj[3], lam;
    int nevals;
    int rf;                  // dipole pair in range: DIP(I) = u1, RFL += u2 dip_coeff
    double u1[3], u2[3];
};

// ----------------------------------------------------------- LJ family -----
template <class T> void lj_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) { // force.f90:6-49
    const T* r = in.rij;
    T sigma = T(pp.sigma), eps = T(pp.epsilon), rc = T(pp.cutoff);
    T rsq = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    T rcsq = rc * rc;
    bool cmask = rsq < rcsq;
    T sr2 = (sigma * sigma) / rsq, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
    T sc2 = (sigma * sigma) / rcsq, sc6 = sc2 * sc2 * sc2, sc12 = sc6 * sc6;
    T pot = T(4.0) * eps * (sr12 - sr6);
    T potc = T(4.0) * eps * (sc12 - sc6);
    T coeff = T(24.0) * eps * (T(2.0) * sr12 - sr6);
    o.pe = cmask ? double(pot - potc) : 0.0;
    for (int d = 0; d < 3; ++d) o.f[d] = cmask ? double(coeff * r[d] / rsq) : 0.0;
}

template <class T> void lj12_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) { // force.f90:51-93
    const T* r = in.rij;
    T sigma = T(pp.sigma), eps = T(pp.epsilon), rc = T(pp.cutoff);
    T rsq = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    T rcsq = rc * rc;
    if (rsq < rcsq) {
        T sr2 = (sigma * sigma) / rsq, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        T sc2 = (sigma * sigma) / rcsq, sc6 = sc2 * sc2 * sc2, sc12 = sc6 * sc6;
        T pot = eps * (sr12 - T(2.0) * sr6);
        T potc = eps * (sc12 - T(2.0) * sc6);
        T coeff = T(12.0) * eps * (sr12 - sr6);
        o.pe = double(pot - potc);
        for (int d = 0; d < 3; ++d) o.f[d] = double(coeff * r[d] / rsq);
    }
}

template <class T> void ljw_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) { // force.f90:95-146
    const T* r = in.rij;
    T sigma = T(pp.sigma), eps = T(pp.epsilon), rc = T(pp.cutoff), wf = T(pp.wf);
    T rsq = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    T rmag = std::sqrt(rsq);
    if (rmag < rc + wf) {
        T sr;
        if (rmag < sigma) sr = sigma / rmag;
        else if (rmag >= sigma && rmag < sigma + wf) sr = T(1.0);
        else sr = sigma / (rmag - wf);
        T sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        T sc = sigma / rc, sc2 = sc * sc, sc6 = sc2 * sc2 * sc2, sc12 = sc6 * sc6;
        T pot = eps * (sr12 - T(2.0) * sr6);
        T potc = eps * (sc12 - T(2.0) * sc6);
        T coeff = T(12.0) * eps * (sr12 - sr6) * (sr / sigma);
        o.pe = double(pot - potc);
        for (int d = 0; d < 3; ++d) o.f[d] = double(coeff * r[d] / rmag);
    }
}

template <class T> void wca_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) { // force.f90:155-190
    const T* r = in.rij;
    T sigma = T(pp.sigma), eps = T(pp.epsilon);
    T rsq = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    T ssq = sigma * sigma;
    if (rsq <= ssq) {
        T sr2 = ssq / rsq, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        o.pe = double(eps * (sr12 - T(2.0) * sr6) + eps);
        T coeff = T(12.0) * eps * (sr12 - sr6);
        for (int d = 0; d < 3; ++d) o.f[d] = double(coeff * r[d] / rsq);
    }
}

// ------------------------------------------------ Morse and charges -----
template <class T> void morse_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) { // force.f90:199-233
    const T* r = in.rij;
    T D = T(pp.dissoc), w = T(pp.width), r0 = T(pp.rmin), rc = T(pp.cutoff);
    T rmag = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (rmag < rc) {
        T e = std::exp(-w * (rmag - r0));
        T ec = std::exp(-w * (rc - r0));
        T pot = D * ((T(1.0) - e) * (T(1.0) - e) - T(1.0));
        T potc = D * ((T(1.0) - ec) * (T(1.0) - ec) - T(1.0));
        o.pe = double(pot - potc);
        for (int d = 0; d < 3; ++d) o.f[d] = double(T(-2.0) * w * D * (T(1.0) - e) * e * r[d] / rmag);
    }
}

template <class T> void dh_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) { // force.f90:2589-2617
    const T* r = in.rij;
    T rc = T(pp.cutoff), db = T(pp.db_len), diel = T(pp.dielectric);
    T rsq = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    T rmag = std::sqrt(rsq);
    if (rmag < rc) {
        T pe = (in.ci * in.cj * std::exp(-rmag / db)) / (T(4.0) * T(M_PI) * diel * rmag);
        o.pe = double(pe);
        for (int d = 0; d < 3; ++d) o.f[d] = double(pe * (T(1.0) + rmag / db) * r[d] / rsq);
    }
}

template <class T> void coulomb_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) { // force.f90:2627-2665
    const T* r = in.rij;
    T rc = T(pp.cutoff), diel = T(pp.dielectric);
    T rsq = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    T rmag = std::sqrt(rsq);
    T sw = rc - T(2.0);
    T factor = T(1.0) / (rc - sw);
    T x = (rmag - sw) * factor;
    T sx = T(1.0) - T(6.0) * x * x * x * x * x + T(15.0) * x * x * x * x - T(10.0) * x * x * x;
    T sdx = T(-30.0) * x * x * x * x + T(60.0) * x * x * x - T(30.0) * x * x;
    if (rmag < rc) {
        T pe = in.ci * in.cj / (T(4.0) * T(M_PI) * diel * rmag);
        T f[3];
        for (int d = 0; d < 3; ++d) f[d] = pe * r[d] / rsq;
        if (rmag >= sw) {
            pe = sx * pe;
            // the scaled PE, subtracted from every component (:2660-2661)
            for (int d = 0; d < 3; ++d) f[d] = sx * f[d] - sdx * pe * factor;
        }
        o.pe = double(pe);
        for (int d = 0; d < 3; ++d) o.f[d] = double(f[d]);
    }
}

template <class T> void dipole_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) { // force.f90:2687-2751
    const T* r = in.rij;
    T rc = T(pp.cutoff);
    T rsq = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    T rmag = std::sqrt(rsq);
    const T* a = in.qi;
    const T* b = in.qj;   // (w, x, y, z)
    T U1[3] = {T(2.0) * (a[1] * a[3] + a[0] * a[2]), T(2.0) * (a[2] * a[3] - a[0] * a[1]),
               a[0] * a[0] - a[1] * a[1] - a[2] * a[2] + a[3] * a[3]};
    T U2[3] = {T(2.0) * (b[1] * b[3] + b[0] * b[2]), T(2.0) * (b[2] * b[3] - b[0] * b[1]),
               b[0] * b[0] - b[1] * b[1] - b[2] * b[2] + b[3] * b[3]};
    for (int d = 0; d < 3; ++d) { U1[d] = U1[d] * in.ci; U2[d] = U2[d] * in.cj; }
    if (rmag < rc) {
        T ci = U1[0] * r[0] + U1[1] * r[1] + U1[2] * r[2];
        T cj = U2[0] * r[0] + U2[1] * r[1] + U2[2] * r[2];
        T cij = U1[0] * U2[0] + U1[1] * U2[1] + U1[2] * U2[2];
        T t1[3], t2[3], t3[3], c1[3], c2[3];
        for (int d = 0; d < 3; ++d) {
            t1[d] = (cij - (T(5.0) * ci * cj / rsq)) * r[d] + cj * U1[d] + ci * U2[d];
            t2[d] = T(3.0) * cj * (r[d] / rsq) - U2[d];
            t3[d] = T(3.0) * ci * (r[d] / rsq) - U1[d];
        }
        T r3 = rsq * rmag, r5 = r3 * rsq;
        cross(U1, t2, c1);
        cross(U2, t3, c2);
        o.pe = double((cij / r3) - ((T(3.0) * ci * cj) / r5));
        for (int d = 0; d < 3; ++d) {
            o.f[d] = double((T(3.0) / r5) * t1[d]);
            o.ti[d] = double((T(1.0) / r3) * c1[d]);
            o.tj[d] = double((T(1.0) / r3) * c2[d]);
            o.u1[d] = double(U1[d]);
            o.u2[d] = double(U2[d]);
        }
        o.rf = 1;
    }
}

// ----------------------------------------------------------- Gay-Berne -----
// force.f90:252-306 helpers, :308-1030 the five flavours. The reference fixes
// (mu, nu) = (1, 2) at :240; here they are parameters.
template <class T> struct GBP { T ru1, ru2, uu; T U1[3], U2[3], rij[3], rsq; };

template <class T> inline T g_func(T chie, const GBP<T>& p) {
    T t1 = (p.ru1 + p.ru2) * (p.ru1 + p.ru2) / (T(1) + chie * p.uu);
    T t2 = (p.ru1 - p.ru2) * (p.ru1 - p.ru2) / (T(1) - chie * p.uu);
    return T(1) - (chie / T(2.0) / p.rsq) * (t1 + t2);
}
template <class T> inline void dG_dr(T chie, const GBP<T>& p, T o[3]) {
    T a = (p.ru1 + p.ru2) / (T(1) + chie * p.uu);
    T b = (p.ru1 - p.ru2) / (T(1) - chie * p.uu);
    T g = g_func(chie, p);
    for (int d = 0; d < 3; ++d) {
        T t1 = a * (p.U1[d] + p.U2[d]);
        T t2 = b * (p.U1[d] - p.U2[d]);
        o[d] = (-chie / p.rsq) * (t1 + t2) + (T(2) * p.rij[d] / p.rsq) * (T(1) - g);
    }
}
template <class T> inline void dG_du(T chie, const GBP<T>& p, int which, T o[3]) {
    T t1 = (p.ru1 + p.ru2) / (T(1) + chie * p.uu);
    T t2 = (p.ru1 - p.ru2) / (T(1) - chie * p.uu);
    const T* Uo = which == 1 ? p.U2 : p.U1;
    T s = which == 1 ? (t1 + t2) : (t1 - t2);
    for (int d = 0; d < 3; ++d)
        o[d] = (-chie * p.rij[d] / p.rsq) * s + ((chie * chie * Uo[d]) / (T(2) * p.rsq)) * (t1 * t1 - t2 * t2);
}

template <class T> void gb_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) {
    const int kind = pp.kind;
    const int meu = pp.mu, neu = pp.nu;
    const bool weld = (kind == OR_GBW || kind == OR_GBWC);
    const bool taper = (kind != OR_GBR);
    const bool chiral = (kind == OR_GBC || kind == OR_GBWC);
    const T cutoff = T(pp.cutoff), wf = T(pp.wf), chirality = T(pp.chirality);
    T pot = 0, FIJ[3] = {0, 0, 0}, TQ1[3] = {0, 0, 0}, TQ2[3] = {0, 0, 0};
    const T sigma_0 = T(1.0);
    GBP<T> p;
    for (int d = 0; d < 3; ++d) p.rij[d] = in.rij[d];
    p.rsq = p.rij[0] * p.rij[0] + p.rij[1] * p.rij[1] + p.rij[2] * p.rij[2];
    T rmag = std::sqrt(p.rsq);
    T rhat[3];
    for (int d = 0; d < 3; ++d) rhat[d] = p.rij[d] / rmag;
    const T *qi = in.qi, *qj = in.qj;  // w x y z
    p.U1[0] = T(2.0) * (qi[1] * qi[3] + qi[0] * qi[2]);
    p.U1[1] = T(2.0) * (qi[2] * qi[3] - qi[0] * qi[1]);
    p.U1[2] = qi[0] * qi[0] - qi[1] * qi[1] - qi[2] * qi[2] + qi[3] * qi[3];
    p.U2[0] = T(2.0) * (qj[1] * qj[3] + qj[0] * qj[2]);
    p.U2[1] = T(2.0) * (qj[2] * qj[3] - qj[0] * qj[1]);
    p.U2[2] = qj[0] * qj[0] - qj[1] * qj[1] - qj[2] * qj[2] + qj[3] * qj[3];
    T lpar = in.si[2], lprp = in.si[0], epar = in.ei[2], eprp = in.ei[0];
    T muinv = T(1.0) / T(meu);
    p.ru1 = p.rij[0] * p.U1[0] + p.rij[1] * p.U1[1] + p.rij[2] * p.U1[2];
    p.ru2 = p.rij[0] * p.U2[0] + p.rij[1] * p.U2[1] + p.rij[2] * p.U2[2];
    p.uu = p.U1[0] * p.U2[0] + p.U1[1] * p.U2[1] + p.U1[2] * p.U2[2];
    T chi = (lpar * lpar - lprp * lprp) / (lpar * lpar + lprp * lprp);
    T xhi = (std::pow(eprp, muinv) - std::pow(epar, muinv)) / (std::pow(eprp, muinv) + std::pow(epar, muinv));
    T gchi = g_func(chi, p), gxhi = g_func(xhi, p);
    T eps1 = T(1.0) / std::sqrt(T(1) - (chi * p.uu) * (chi * p.uu));
    T eps2 = gxhi / in.ei[2];
    T sigma = lprp / std::sqrt(gchi);
    T s0inv = T(1.0) / sigma_0;
    T ginv = sigma / gchi;
    T reach = weld ? (sigma + cutoff + wf - sigma_0) : (sigma + cutoff - sigma_0);
    T sw = T(0.9) * reach;
    T factor = T(1.0) / (reach - sw);
    T xx = (rmag - sw) * factor;
    T sx = T(1.0) - T(6.0) * xx * xx * xx * xx * xx + T(15.0) * xx * xx * xx * xx - T(10.0) * xx * xx * xx;
    T sdx = T(-30.0) * xx * xx * xx * xx + T(60.0) * xx * xx * xx - T(30.0) * xx * xx;
    bool active = (kind == OR_GBR) ? (rmag <= sigma) : (rmag < reach);
    if (active) {
        T sr;
        if (weld) {
            if (rmag < sigma) sr = sigma_0 / (rmag - sigma + sigma_0);
            else if (rmag >= sigma && rmag <= sigma + wf) sr = T(1.0);
            else sr = sigma_0 / (rmag - sigma + sigma_0 - wf);
        } else {
            sr = sigma_0 / (rmag - sigma + sigma_0);
        }
        T sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        T srx = (sr12 - T(2.0) * sr6);
        if (kind == OR_GBR) srx = srx + T(1.0);
        T srd = T(12.0) * (sr6 - sr12) * sr;
        T e1n = ipow(eps1, neu), e2m = ipow(eps2, meu);
        T dGr_chi[3], dGr_xhi[3], dGu1_chi[3], dGu1_xhi[3], dGu2_chi[3], dGu2_xhi[3];
        dG_dr(chi, p, dGr_chi); dG_dr(xhi, p, dGr_xhi);
        dG_du(chi, p, 1, dGu1_chi); dG_du(xhi, p, 1, dGu1_xhi);
        dG_du(chi, p, 2, dGu2_chi); dG_du(xhi, p, 2, dGu2_xhi);
        T dR_dr[3], de2_dr[3], de1_du1[3], de2_du1[3], dR_du1[3], de1_du2[3], de2_du2[3], dR_du2[3];
        T TI[3], TJ[3];
        T pe_fac = e1n * (T(meu) * ipow(eps2, meu - 1));
        T e1_fac = e2m * (T(neu) * ipow(eps1, neu + 2));
        if (!chiral) {
            // gb_/gbr_/gbw_ ordering (force.f90:392-412)
            for (int d = 0; d < 3; ++d) {
                dR_dr[d] = s0inv * (rhat[d] + T(0.5) * dGr_chi[d] * ginv);
                de2_dr[d] = pe_fac * dGr_xhi[d];
                de1_du1[d] = e1_fac * (chi * chi * p.uu * p.U2[d]);
                de2_du1[d] = pe_fac * dGu1_xhi[d];
                dR_du1[d] = srd * T(0.5) * s0inv * dGu1_chi[d] * ginv;
                de1_du2[d] = e1_fac * (chi * chi * p.uu * p.U1[d]);
                de2_du2[d] = pe_fac * dGu2_xhi[d];
                dR_du2[d] = srd * T(0.5) * s0inv * dGu2_chi[d] * ginv;
            }
            pot = e1n * e2m * srx;
            for (int d = 0; d < 3; ++d) {
                FIJ[d] = T(-1.0) * (e1n * e2m * srd * dR_dr[d] + de2_dr[d] * srx);
                TI[d] = T(-1.0) * (srx * (de1_du1[d] + de2_du1[d]) + (e1n * e2m * dR_du1[d]));
                TJ[d] = T(-1.0) * (srx * (de1_du2[d] + de2_du2[d]) + (e1n * e2m * dR_du2[d]));
            }
            cross(p.U1, TI, TQ1);
            cross(p.U2, TJ, TQ2);
        } else {
            // gbc_/gbwc_ ordering (force.f90:755-827, :942-1014)
            for (int d = 0; d < 3; ++d) {
                dR_dr[d] = e1n * e2m * s0inv * (rhat[d] + T(0.5) * dGr_chi[d] * ginv);
                de2_dr[d] = pe_fac * dGr_xhi[d];
                de1_du1[d] = e1_fac * (chi * chi * p.uu * p.U2[d]);
                de2_du1[d] = pe_fac * dGu1_xhi[d];
                dR_du1[d] = e1n * e2m * T(0.5) * s0inv * dGu1_chi[d] * ginv;
                de1_du2[d] = e1_fac * (chi * chi * p.uu * p.U1[d]);
                de2_du2[d] = pe_fac * dGu2_xhi[d];
                dR_du2[d] = e1n * e2m * T(0.5) * s0inv * dGu2_chi[d] * ginv;
            }
            pot = e1n * e2m * srx;
            for (int d = 0; d < 3; ++d) {
                FIJ[d] = T(-1.0) * (srx * de2_dr[d] + srd * dR_dr[d]);
                TI[d] = T(-1.0) * (srx * (de1_du1[d] + de2_du1[d]) + srd * dR_du1[d]);
                TJ[d] = T(-1.0) * (srx * (de1_du2[d] + de2_du2[d]) + srd * dR_du2[d]);
            }
            cross(p.U1, TI, TQ1);
            cross(p.U2, TJ, TQ2);
            // chiral terms
            if (kind == OR_GBC) {
                srx = sr6 * sr;
                srd = T(-7.0) * sr6 * sr2;
            } else {
                srx = (sr12 - (T(12.0) / T(7.0)) * sr6 * sr);
                srd = T(12.0) * (sr6 * sr2 - sr12 * sr);
            }
            T u1xu2[3], u2xr[3], rxu1[3];
            cross(p.U1, p.U2, u1xu2);
            cross(p.U2, rhat, u2xr);
            cross(rhat, p.U1, rxu1);
            T uur = u1xu2[0] * rhat[0] + u1xu2[1] * rhat[1] + u1xu2[2] * rhat[2];
            T uu = p.uu;
            T duur_dr[3], duur_du1[3], duu_du1[3], duur_du2[3], duu_du2[3];
            for (int d = 0; d < 3; ++d) {
                dR_dr[d] = dR_dr[d] * srd * uur * uu;
                de2_dr[d] = de2_dr[d] * srx * uur * uu;
                duur_dr[d] = e1n * e2m * srx * uu * (u1xu2[d] - uur * rhat[d]) / rmag;
                de1_du1[d] = de1_du1[d] * srx * uur * uu;
                de2_du1[d] = de2_du1[d] * srx * uur * uu;
                dR_du1[d] = dR_du1[d] * srd * uur * uu;
                duur_du1[d] = e1n * e2m * srx * uu * u2xr[d];
                duu_du1[d] = e1n * e2m * srx * uur * p.U2[d];
                de1_du2[d] = de1_du2[d] * srx * uur * uu;
                de2_du2[d] = de2_du2[d] * srx * uur * uu;
                dR_du2[d] = dR_du2[d] * srd * uur * uu;
                duur_du2[d] = e1n * e2m * srx * uu * rxu1[d];
                duu_du2[d] = e1n * e2m * srx * uur * p.U1[d];
            }
            T pot_c = e1n * e2m * srx * uur * uu;
            T Fc[3], TIc[3], TJc[3], TQ1c[3], TQ2c[3];
            for (int d = 0; d < 3; ++d) {
                Fc[d] = T(-1.0) * (de2_dr[d] + dR_dr[d] + duur_dr[d]);
                TIc[d] = T(-1.0) * (de1_du1[d] + de2_du1[d] + dR_du1[d] + duur_du1[d] + duu_du1[d]);
                TJc[d] = T(-1.0) * (de1_du2[d] + de2_du2[d] + dR_du2[d] + duur_du2[d] + duu_du2[d]);
            }
            cross(p.U1, TIc, TQ1c);
            cross(p.U2, TJc, TQ2c);
            pot = pot + chirality * pot_c;
            for (int d = 0; d < 3; ++d) {
                FIJ[d] = FIJ[d] + chirality * Fc[d];
                TQ1[d] = TQ1[d] + chirality * TQ1c[d];
                TQ2[d] = TQ2[d] + chirality * TQ2c[d];
            }
        }
        if (taper && rmag >= sw && rmag <= reach) {
            for (int d = 0; d < 3; ++d) {           // Q7: scalar subtracted from each component
                FIJ[d] = sx * FIJ[d] - sdx * pot * factor;
                TQ1[d] = sx * TQ1[d] - sdx * pot * factor;
                TQ2[d] = sx * TQ2[d] - sdx * pot * factor;
            }
            pot = sx * pot;
        }
    }
    o.pe = double(pot);
    for (int d = 0; d < 3; ++d) { o.f[d] = double(FIJ[d]); o.ti[d] = double(TQ1[d]); o.tj[d] = double(TQ2[d]); }
}

// ----------------------------------------------------------------- ECP -----
template <class T> struct EcpPair { M3<T> AE, BE, AR, BR; T rij[3]; };

// optim_dist (force.f90:1188-1200)
template <class T> inline T optim_dist(T L, const EcpPair<T>& p) {
    M3<T> G;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) G.m[i][j] = (T(1) - L) * p.AR.m[i][j] + L * p.BR.m[i][j];
    T K[3];
    cholesky_solve(G, p.rij, K);
    return -(L * (T(1) - L) * (p.rij[0] * K[0] + p.rij[1] * K[1] + p.rij[2] * K[2]));
}

// brent (force.f90:1046-1172), including the two evaluations at a and b that
// are never used.
template <class T> T brent(const EcpPair<T>& pair, int& nevals) {
    const int max_iter = 10000;
    const T psi = T(0.5) * (T(3.0) - std::sqrt(T(5.0)));
    T a, b, c, x, w, v, u, fa, fb, fc, ft, fw, fv, fu;
    T deltax = 0, atol = T(1e-3), rtol = T(1e-2);
    T tol1, tol2, xmid, tmp1, tmp2, rat = 0, pp, dx_temp;
    int iter = 0;
    a = 0; b = 1;
    c = (T(1) - psi) * a + psi * b;
    fa = optim_dist(a, pair); fb = optim_dist(b, pair); fc = optim_dist(c, pair);
    (void)fa; (void)fb;
    nevals = 3;
    v = c; w = v; x = w;
    fv = fc; fw = fv; ft = fw;
    while (iter < max_iter) {
        tol1 = rtol * std::fabs(x) + atol;
        tol2 = T(2.0) * tol1;
        xmid = T(0.5) * (a + b);
        if (std::fabs(x - xmid) < (tol2 - T(0.5) * (b - a))) break;
        if (std::fabs(deltax) <= tol1) {
            deltax = (x >= xmid) ? (a - x) : (b - x);
            rat = psi * deltax;
        } else {
            tmp1 = (x - w) * (ft - fv);
            tmp2 = (x - v) * (ft - fw);
            pp = (x - v) * tmp2 - (x - w) * tmp1;
            tmp2 = T(2.0) * (tmp2 - tmp1);
            if (tmp2 > T(0.0)) pp = -pp;
            tmp2 = std::fabs(tmp2);
            dx_temp = deltax;
            deltax = rat;
            if ((pp > tmp2 * (a - x)) && (pp < tmp2 * (b - x)) && (std::fabs(pp) < std::fabs(T(0.5) * tmp2 * dx_temp))) {
                rat = pp * T(1.0) / tmp2;
                u = x + rat;
                if ((u - a) < tol2 || (b - u) < tol2) rat = (xmid - x >= 0) ? tol1 : -tol1;
            } else {
                deltax = (x >= xmid) ? (a - x) : (b - x);
                rat = psi * deltax;
            }
        }
        if (std::fabs(rat) < tol1) u = (rat >= 0) ? (x + tol1) : (x - tol1);
        else u = x + rat;
        fu = optim_dist(u, pair);
        ++nevals;
        if (fu > ft) {
            if (u < x) a = u; else b = u;
            if ((fu <= fw) || (w == x)) { v = w; w = u; fv = fw; fw = fu; }
            else if ((fu <= fv) || (v == x) || (v == w)) { v = u; fv = fu; }
        } else {
            if (u >= x) a = x; else b = x;
            v = w; w = x; x = u;
            fv = fw; fw = ft; ft = fu;
        }
        ++iter;
    }
    return x;
}

// Tightly converged maximiser of S(l) = l(1-l) r^T G(l)^-1 r on [0,1]:
// bracketed Newton on S'(l) in the working precision, to |dl| < 1e-15.
// Not in the reference; it is the FP64 check of the Newton and MLP paths.
template <class T> T tight_lambda(const EcpPair<T>& p, int& nevals) {
    T lo = 0, hi = 1, L = T(0.5);
    nevals = 0;
    M3<T> D;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D.m[i][j] = p.BR.m[i][j] - p.AR.m[i][j];
    for (int it = 0; it < 200; ++it) {
        M3<T> G;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) G.m[i][j] = (T(1) - L) * p.AR.m[i][j] + L * p.BR.m[i][j];
        T K[3], DK[3], Z[3];
        cholesky_solve(G, p.rij, K);
        mvdot(D, K, DK);
        cholesky_solve(G, DK, Z);
        T rK = p.rij[0] * K[0] + p.rij[1] * K[1] + p.rij[2] * K[2];
        T KDK = K[0] * DK[0] + K[1] * DK[1] + K[2] * DK[2];
        T DKZ = DK[0] * Z[0] + DK[1] * Z[1] + DK[2] * Z[2];
        T s1 = (T(1) - T(2) * L) * rK - L * (T(1) - L) * KDK;
        T s2 = T(-2) * rK - T(2) * (T(1) - T(2) * L) * KDK + T(2) * L * (T(1) - L) * DKZ;
        ++nevals;
        if (s1 == T(0)) break;
        if (s1 > 0) lo = L; else hi = L;
        T Ln = (s2 < 0) ? L - s1 / s2 : T(0.5) * (lo + hi);
        if (!(Ln > lo && Ln < hi)) Ln = T(0.5) * (lo + hi);
        T dl = std::fabs(Ln - L);
        L = Ln;
        if (dl < T(1e-13) || hi - lo < T(1e-15)) break;
    }
    return L;
}

template <class T> void ecp_pair(const PairIn<T>& in, const OrPairParams& pp, PairOut& o) {
    const int kind = pp.kind;
    const int meu = pp.mu, neu = pp.nu;
    const bool weld = (kind == OR_ECPW || kind == OR_ECPWC);
    const bool chiral = (kind == OR_ECPC || kind == OR_ECPWC);
    const bool rep = (kind == OR_ECPR);
    const T cutoff = T(pp.cutoff), wf = T(pp.wf), chirality = T(pp.chirality);
    const T sigma_0 = T(1.0);
    T pot = 0, FIJ[3] = {0, 0, 0}, TQ1[3] = {0, 0, 0}, TQ2[3] = {0, 0, 0};
    EcpPair<T> pr;
    for (int d = 0; d < 3; ++d) pr.rij[d] = in.rij[d];
    T rsq = pr.rij[0] * pr.rij[0] + pr.rij[1] * pr.rij[1] + pr.rij[2] * pr.rij[2];
    T rmag = std::sqrt(rsq);
    T rhat[3];
    for (int d = 0; d < 3; ++d) rhat[d] = pr.rij[d] / rmag;
    M3<T> U1 = rotmat(in.qi[0], in.qi[1], in.qi[2], in.qi[3]);
    M3<T> U2 = rotmat(in.qj[0], in.qj[1], in.qj[2], in.qj[3]);
    T e10 = std::max(std::max(in.ei[0], in.ei[1]), in.ei[2]);
    T e20 = std::max(std::max(in.ej[0], in.ej[1]), in.ej[2]);
    T muinv = T(1.0) / T(meu);
    M3<T> E1{}, E2{}, S1{}, S2{}, S1sq{}, S2sq{};
    for (int d = 0; d < 3; ++d) {
        E1.m[d][d] = std::pow(e10 / in.ei[d], muinv) / T(4.0);
        E2.m[d][d] = std::pow(e20 / in.ej[d], muinv) / T(4.0);
        S1.m[d][d] = in.si[d] / T(2.0);
        S2.m[d][d] = in.sj[d] / T(2.0);
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { S1sq.m[i][j] = S1.m[i][j] * S1.m[i][j]; S2sq.m[i][j] = S2.m[i][j] * S2.m[i][j]; }
    M3<T> U1t, U2t;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) { U1t.m[i][j] = U1.m[j][i]; U2t.m[i][j] = U2.m[j][i]; }
    M3<T> MM1 = mmdot(U1t, S1), MM2 = mmdot(U2t, S2);
    pr.AR = matmul_atba(U1, S1sq);
    pr.BR = matmul_atba(U2, S2sq);
    pr.AE = matmul_atba(U1, E1);
    pr.BE = matmul_atba(U2, E2);
    T st1 = (in.si[0] * in.si[1] + in.si[2] * in.si[2]) * std::sqrt(T(2.0) * in.si[0] * in.si[1]) / T(8.0);
    T st2 = (in.sj[0] * in.sj[1] + in.sj[2] * in.sj[2]) * std::sqrt(T(2.0) * in.sj[0] * in.sj[1]) / T(8.0);
    T sigma_t = std::sqrt(st1 * st2);
    M3<T> EAB;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) EAB.m[i][j] = pr.AR.m[i][j] + pr.BR.m[i][j];
    M3<T> EM = inverse(EAB);
    T eps1 = sigma_t * std::sqrt(determinant(EM));
    int nev = 0;
    T lam;
    if (pp.solver == 0) lam = brent(pr, nev);
    else if (pp.solver == 1) lam = tight_lambda(pr, nev);
    else lam = T(pp.lam_in);
    o.lam = double(lam);
    o.nevals = nev;
    T lamE = lam, lamR = lam;
    M3<T> GE, GR;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            GE.m[i][j] = (T(1) - lamE) * pr.AE.m[i][j] + lamE * pr.BE.m[i][j];
            GR.m[i][j] = (T(1) - lamR) * pr.AR.m[i][j] + lamR * pr.BR.m[i][j];
        }
    T KE[3], KR[3];
    cholesky_solve(GE, pr.rij, KE);
    T eps2 = lamE * (T(1.0) - lamE) * (rhat[0] * KE[0] + rhat[1] * KE[1] + rhat[2] * KE[2]) / rmag;
    cholesky_solve(GR, pr.rij, KR);
    T phi = lamR * (T(1.0) - lamR) * (rhat[0] * KR[0] + rhat[1] * KR[1] + rhat[2] * KR[2]) / rmag;
    T sigma = T(1.0) / std::sqrt(phi);
    T efac = T(2.0) * lamE * (T(1.0) - lamE) / rsq;
    T rfac = T(2.0) * lamR * (T(1.0) - lamR) / rsq;
    T s0inv = T(1.0) / sigma_0;
    T pi32 = sigma * sigma * sigma;
    T reach = weld ? (sigma + cutoff + wf - sigma_0) : (sigma + cutoff - sigma_0);
    T sw = T(0.9) * reach;
    T factor = T(1.0) / (reach - sw);
    T xx = (rmag - sw) * factor;
    T sx = T(1.0) - T(6.0) * xx * xx * xx * xx * xx + T(15.0) * xx * xx * xx * xx - T(10.0) * xx * xx * xx;
    T sdx = T(-30.0) * xx * xx * xx * xx + T(60.0) * xx * xx * xx - T(30.0) * xx * xx;
    bool active = rep ? (rmag <= sigma) : (rmag < reach);
    if (active) {
        T sr;
        if (weld) {
            if (rmag < sigma) sr = sigma_0 / (rmag - sigma + sigma_0);
            else if (rmag >= sigma && rmag <= sigma + wf) sr = T(1.0);
            else sr = sigma_0 / (rmag - sigma + sigma_0 - wf);
        } else {
            sr = sigma_0 / (rmag - sigma + sigma_0);
        }
        T sr2 = sr * sr, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        T srx = (sr12 - T(2.0) * sr6);
        if (rep) srx = srx + T(1.0);
        T srd = T(12.0) * (sr6 - sr12) * sr;
        T e1n = ipow(eps1, neu), e2m = ipow(eps2, meu);
        T e2fac = e1n * (T(meu) * ipow(eps2, meu - 1));
        T e1fac = e2m * (T(neu) * ipow(eps1, neu));
        T rKR = rhat[0] * KR[0] + rhat[1] * KR[1] + rhat[2] * KR[2];
        T rKE = rhat[0] * KE[0] + rhat[1] * KE[1] + rhat[2] * KE[2];
        T dR_dr[3], de2_dr[3];
        for (int d = 0; d < 3; ++d) {
            if (chiral) dR_dr[d] = e1n * e2m * s0inv * (rhat[d] + T(0.5) * rfac * (KR[d] - rKR * rhat[d]) * pi32);
            else dR_dr[d] = s0inv * (rhat[d] + T(0.5) * rfac * (KR[d] - rKR * rhat[d]) * pi32);
            de2_dr[d] = e2fac * efac * (KE[d] - rKE * rhat[d]);
        }
        // d eps1 / d u : sum over the three body axes (force.f90:1346-1352)
        T de1_du1[3] = {0, 0, 0}, de1_du2[3] = {0, 0, 0};
        T d1x[3], d1y[3], d1z[3], d2x[3], d2y[3], d2z[3];
        for (int ax = 0; ax < 3; ++ax) {
            T c1[3] = {MM1.m[0][ax], MM1.m[1][ax], MM1.m[2][ax]};
            T c2[3] = {MM2.m[0][ax], MM2.m[1][ax], MM2.m[2][ax]};
            T e1c[3], e2c[3], x1[3], x2[3];
            mvdot(EM, c1, e1c);
            mvdot(EM, c2, e2c);
            cross(c1, e1c, x1);
            cross(c2, e2c, x2);
            T* o1 = ax == 0 ? d1x : (ax == 1 ? d1y : d1z);
            T* o2 = ax == 0 ? d2x : (ax == 1 ? d2y : d2z);
            for (int d = 0; d < 3; ++d) {
                o1[d] = chiral ? e1fac * x1[d] : e1fac * srx * x1[d];
                o2[d] = chiral ? e1fac * x2[d] : e1fac * srx * x2[d];
            }
        }
        for (int d = 0; d < 3; ++d) { de1_du1[d] = (d1x[d] + d1y[d]) + d1z[d]; de1_du2[d] = (d2x[d] + d2y[d]) + d2z[d]; }
        T KEAE[3], KRAR[3], KEBE[3], KRBR[3], xa[3], xb[3], xc[3], xd[3];
        vmdot(KE, pr.AE, KEAE); vmdot(KR, pr.AR, KRAR);
        vmdot(KE, pr.BE, KEBE); vmdot(KR, pr.BR, KRBR);
        cross(KEAE, KE, xa); cross(KRAR, KR, xb);
        cross(KEBE, KE, xc); cross(KRBR, KR, xd);
        T de2_du1[3], dR_du1[3], de2_du2[3], dR_du2[3];
        for (int d = 0; d < 3; ++d) {
            if (!chiral) {
                de2_du1[d] = e2fac * srx * (T(1) - lamE) * efac * xa[d];
                dR_du1[d] = e1n * e2m * srd * (T(0.5) * s0inv) * (T(1) - lamR) * rfac * xb[d] * pi32;
                de2_du2[d] = e2fac * srx * lamE * efac * xc[d];
                dR_du2[d] = e1n * e2m * srd * (T(0.5) * s0inv) * lamR * rfac * xd[d] * pi32;
            } else {
                de2_du1[d] = e2fac * (T(1) - lamE) * efac * xa[d];
                dR_du1[d] = e1n * e2m * (T(0.5) * s0inv) * (T(1) - lamR) * rfac * xb[d] * pi32;
                de2_du2[d] = e2fac * lamE * efac * xc[d];
                dR_du2[d] = e1n * e2m * (T(0.5) * s0inv) * lamR * rfac * xd[d] * pi32;
            }
        }
        pot = e1n * e2m * srx;
        if (!chiral) {
            for (int d = 0; d < 3; ++d) {
                FIJ[d] = T(-1.0) * (e1n * e2m * srd * dR_dr[d] + srx * de2_dr[d]);
                TQ1[d] = (de1_du1[d] + de2_du1[d] + dR_du1[d]);
                TQ2[d] = (de1_du2[d] + de2_du2[d] + dR_du2[d]);
            }
        } else {
            for (int d = 0; d < 3; ++d) {
                FIJ[d] = T(-1.0) * (srx * de2_dr[d] + srd * dR_dr[d]);
                TQ1[d] = (srx * (de1_du1[d] + de2_du1[d]) + srd * dR_du1[d]);
                TQ2[d] = (srx * (de1_du2[d] + de2_du2[d]) + srd * dR_du2[d]);
            }
            // chiral terms (force.f90:1774-1826 for ecpc_, :2021-2073 for ecpwc_)
            if (kind == OR_ECPC) { srx = sr6 * sr; srd = T(-7.0) * sr6 * sr2; }
            else { srx = (sr12 - (T(12.0) / T(7.0)) * sr6 * sr); srd = T(12.0) * (sr6 * sr2 - sr12 * sr); }
            T u1z[3] = {U1.m[2][0], U1.m[2][1], U1.m[2][2]};
            T u2z[3] = {U2.m[2][0], U2.m[2][1], U2.m[2][2]};
            T u1xu2[3], u2xr[3], rxu1[3];
            cross(u1z, u2z, u1xu2);
            cross(u2z, rhat, u2xr);
            cross(rhat, u1z, rxu1);
            T uur = u1xu2[0] * rhat[0] + u1xu2[1] * rhat[1] + u1xu2[2] * rhat[2];
            T uu = u1z[0] * u2z[0] + u1z[1] * u2z[1] + u1z[2] * u2z[2];
            T duur_dr[3], t1[3], t2[3];
            for (int d = 0; d < 3; ++d) {
                dR_dr[d] = dR_dr[d] * srd * uur * uu;
                de2_dr[d] = de2_dr[d] * srx * uur * uu;
                duur_dr[d] = e1n * e2m * srx * uu * (u1xu2[d] - uur * rhat[d]) / rmag;
                de1_du1[d] = de1_du1[d] * srx * uur * uu;
                de2_du1[d] = de2_du1[d] * srx * uur * uu;
                dR_du1[d] = dR_du1[d] * srd * uur * uu;
                de1_du2[d] = de1_du2[d] * srx * uur * uu;
                de2_du2[d] = de2_du2[d] * srx * uur * uu;
                dR_du2[d] = dR_du2[d] * srd * uur * uu;
                T duur_du1z = e1n * e2m * srx * uu * u2xr[d];
                T duu_du1z = e1n * e2m * srx * uur * u2z[d];
                T duur_du2z = e1n * e2m * srx * uu * rxu1[d];
                T duu_du2z = e1n * e2m * srx * uur * u1z[d];
                t1[d] = (duur_du1z + duu_du1z);
                t2[d] = (duur_du2z + duu_du2z);
            }
            T tu1[3], tu2[3];
            cross(u1z, t1, tu1);
            cross(u2z, t2, tu2);
            T pot_c = e1n * e2m * srx * uur * uu;
            pot = pot + chirality * pot_c;
            for (int d = 0; d < 3; ++d) {
                T Fc = T(-1.0) * (de2_dr[d] + dR_dr[d] + duur_dr[d]);
                T T1c = (de1_du1[d] + de2_du1[d] + dR_du1[d] - tu1[d]);
                T T2c = (de1_du2[d] + de2_du2[d] + dR_du2[d] - tu2[d]);
                FIJ[d] = FIJ[d] + chirality * Fc;
                TQ1[d] = TQ1[d] + chirality * T1c;
                TQ2[d] = TQ2[d] + chirality * T2c;
            }
        }
        if (!rep && rmag >= sw && rmag <= reach) {
            for (int d = 0; d < 3; ++d) {
                FIJ[d] = sx * FIJ[d] - sdx * pot * factor;
                TQ1[d] = sx * TQ1[d] - sdx * pot * factor;
                TQ2[d] = sx * TQ2[d] - sdx * pot * factor;
            }
            pot = sx * pot;
        }
    }
    o.pe = double(pot);
    for (int d = 0; d < 3; ++d) { o.f[d] = double(FIJ[d]); o.ti[d] = double(TQ1[d]); o.tj[d] = double(TQ2[d]); }
}

template <class T> void eval_pair(const OrSys* s, int i, int j, const OrPairParams& pp, PairOut& o) {
    std::memset(&o, 0, sizeof(o));
    PairIn<T> in = load_pair<T>(s, i, j);
    switch (pp.kind) {
        case OR_LJ: lj_pair(in, pp, o); break;
        case OR_LJ12: lj12_pair(in, pp, o); break;
        case OR_LJW: ljw_pair(in, pp, o); break;
        case OR_WCA: wca_pair(in, pp, o); break;
        case OR_MORSE: morse_pair(in, pp, o); break;
        case OR_DH: dh_pair(in, pp, o); break;
        case OR_COULOMB: coulomb_pair(in, pp, o); break;
        case OR_DIPOLE: dipole_pair(in, pp, o); break;
        case OR_GB: case OR_GBR: case OR_GBW: case OR_GBC: case OR_GBWC: gb_pair(in, pp, o); break;
        default: ecp_pair(in, pp, o); break;
    }
}

} // namespace

extern "C" {

// One pair, reference argument meaning (I, J) 0-based: PE, FXIJ (force on I),
// TXI, TXJ. prec = 64 or 32 (the FP32 prediction of the same formulas).
void or_pair(const OrSys* s, int i, int j, const OrPairParams* pp, int prec, double* out /*11: pe f3 ti3 tj3 lam*/,
             int* nevals) {
    PairOut o;
    if (prec == 32) eval_pair<float>(s, i, j, *pp, o);
    else eval_pair<double>(s, i, j, *pp, o);
    out[0] = o.pe;
    for (int d = 0; d < 3; ++d) { out[1 + d] = o.f[d]; out[4 + d] = o.ti[d]; out[7 + d] = o.tj[d]; }
    out[10] = o.lam;
    if (nevals) *nevals = o.nevals;
}

// Per-pair outputs for a list of pairs, evaluated by nthreads threads when the
// library is built with OpenMP (the fast CPU-baseline build); no accumulation,
// so the threads never share an output. out holds 11 doubles per pair.
void or_pair_batch(const OrSys* s, const OrPairParams* pp, long long npairs, const int* pi, const int* pj,
                   double* out, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
#endif
    for (long long k = 0; k < npairs; ++k) {
        PairOut o;
        eval_pair<double>(s, pi[k], pj[k], *pp, o);
        double* w = out + 11 * k;
        w[0] = o.pe;
        for (int d = 0; d < 3; ++d) { w[1 + d] = o.f[d]; w[4 + d] = o.ti[d]; w[7 + d] = o.tj[d]; }
        w[10] = o.lam;
    }
    (void)nthreads;
}

// The README pair loop (README.md:86-103) over an explicit pair list: adds
// F(I) += f, F(J) -= f, T(I) += TXI, T(J) += TXJ and pot_eng += PE. Per-pair
// lambda and evaluation counts are returned when the arrays are given.
void or_forces(OrSys* s, const OrPairParams* pp, int npairs, const int* pi, const int* pj, int prec,
               double* lam_out, int* nevals_out, double* lam_in) {
    for (int k = 0; k < npairs; ++k) {
        int i = pi[k], j = pj[k];
        PairOut o;
        OrPairParams q = *pp;
        if (lam_in) { q.solver = 2; q.lam_in = lam_in[k]; }
        if (prec == 32) eval_pair<float>(s, i, j, q, o);
        else eval_pair<double>(s, i, j, q, o);
        s->pot_eng += o.pe;
        s->fx[i] += o.f[0]; s->fy[i] += o.f[1]; s->fz[i] += o.f[2];
        s->fx[j] -= o.f[0]; s->fy[j] -= o.f[1]; s->fz[j] -= o.f[2];
        if (s->tx) {
            s->tx[i] += o.ti[0]; s->ty[i] += o.ti[1]; s->tz[i] += o.ti[2];
            s->tx[j] += o.tj[0]; s->ty[j] += o.tj[1]; s->tz[j] += o.tj[2];
        }
        if (lam_out) lam_out[k] = o.lam;
        if (nevals_out) nevals_out[k] = o.nevals;
        if (o.rf && s->dipx) {   // force.f90:2739-2745
            const double rc = pp->cutoff, eps = pp->dielectric;
            const double dip_coeff = ((2.0 * (eps - 1.0)) / (2.0 * eps + 1.0)) / (rc * rc * rc);
            s->dipx[i] = o.u1[0]; s->dipy[i] = o.u1[1]; s->dipz[i] = o.u1[2];
            for (int d = 0; d < 3; ++d) s->rfl[d] = s->rfl[d] + o.u2[d] * dip_coeff;
        }
    }
}

// mc_barostat (integrators.f90:858-945) with compute_potential = the summed
// energy of nsets pair parameter sets over the given pair list, and the two
// random_number draws replaced by Philox words of counter (lo, hi, 0x4D43, 0)
// under key. Forces and pot_eng are left as they were. Returns accept: 1, 0,
// or -1 for no move (V_new <= 0).
int or_mc_barostat(OrSys* s, const OrPairParams* sets, int nsets, int npairs, const int* pi, const int* pj,
                   double target_pres, double temp, double max_dv, const uint32_t* key, unsigned long long counter,
                   double* u_out) {
    const int n = s->n;
    std::vector<double> f(6 * (size_t)n), r(3 * (size_t)n);
    double* F[6] = {s->fx, s->fy, s->fz, s->tx, s->ty, s->tz};
    for (int k = 0; k < 6; ++k)
        if (F[k]) std::memcpy(&f[(size_t)k * n], F[k], sizeof(double) * n);
    const double pe_save = s->pot_eng;
    auto potential = [&]() {
        s->pot_eng = 0.0;
        for (int k = 0; k < nsets; ++k) or_forces(s, &sets[k], npairs, pi, pj, 64, nullptr, nullptr, nullptr);
        return s->pot_eng;
    };
    auto restore = [&]() {
        for (int k = 0; k < 6; ++k)
            if (F[k]) std::memcpy(F[k], &f[(size_t)k * n], sizeof(double) * n);
        s->pot_eng = pe_save;
    };
    if (!(max_dv > 0.0)) max_dv = 0.01;
    const double beta = 1.0 / temp;
    const double L[3] = {s->box[0], s->box[1], s->box[2]};
    const double V_old = L[0] * L[1] * L[2];
    std::memcpy(&r[0], s->rx, sizeof(double) * n);
    std::memcpy(&r[n], s->ry, sizeof(double) * n);
    std::memcpy(&r[2 * (size_t)n], s->rz, sizeof(double) * n);
    const double U_old = potential();
    const uint32_t ctr[4] = {(uint32_t)counter, (uint32_t)(counter >> 32), 0x4D43u, 0u};
    const uint32_t k0[2] = {PHILOX_KEY0, PHILOX_KEY1};
    uint32_t w[4];
    philox(ctr, key ? key : k0, w);
    const double u1 = w[0] * (1.0 / 4294967296.0), u2 = w[1] * (1.0 / 4294967296.0);
    const double V_new = V_old + max_dv * (2.0 * u1 - 1.0) * V_old;
    if (u_out) { u_out[0] = U_old; u_out[1] = 0.0; u_out[2] = V_new; }
    if (V_new <= 0.0) {
        restore();
        return -1;
    }
    const double scale = std::pow(V_new / V_old, 1.0 / 3.0);
    for (int d = 0; d < 3; ++d) s->box[d] = L[d] * scale;
    for (int i = 0; i < n; ++i) {
        s->rx[i] = r[i] * scale;
        s->ry[i] = r[n + i] * scale;
        s->rz[i] = r[2 * (size_t)n + i] * scale;
    }
    const double U_new = potential();
    if (u_out) u_out[1] = U_new;
    const double dU = U_new - U_old;
    const double exponent = -beta * dU - beta * target_pres * (V_new - V_old) + double(n) * std::log(V_new / V_old);
    int accept;
    if (std::log(u2) < exponent) {
        accept = 1;
        s->density = double(n) / (s->box[0] * s->box[1] * s->box[2]);
    } else {
        for (int d = 0; d < 3; ++d) s->box[d] = L[d];
        std::memcpy(s->rx, &r[0], sizeof(double) * n);
        std::memcpy(s->ry, &r[n], sizeof(double) * n);
        std::memcpy(s->rz, &r[2 * (size_t)n], sizeof(double) * n);
        accept = 0;
    }
    restore();
    return accept;
}

// init_reaction_field (force.f90:2677-2685): DIP and RFL to zero.
void or_reaction_field_init(OrSys* s) {
    for (int i = 0; i < s->n; ++i) s->dipx[i] = s->dipy[i] = s->dipz[i] = 0.0;
    s->rfl[0] = s->rfl[1] = s->rfl[2] = 0.0;
}

// ---------------------------------------------------------------- bonded -----
// module bonded (force.f90:2238-2581). kind: 0 bend, 1 dih, 2 cosine_bend,
// 3 cosine_dih, 4 angle_bend, 5 angle_dih. atoms: I J K [L] 0-based. out:
// PE, FXI, FXJ, FXK, FXL (13 doubles; FXL zero for three-body kinds).
void or_bonded(const OrSys* s, int kind, const int* at, double coeff, double angle, double* out) {
    const double PI_ = 3.1415926535897932384626433832795;
    auto vec = [&](int a, int b, double v[3]) {   // r_b - r_a, minimum image
        v[0] = s->rx[b] - s->rx[a];
        v[1] = s->ry[b] - s->ry[a];
        v[2] = s->rz[b] - s->rz[a];
        min_image(v, s->box, s->periodic);
    };
    auto dot = [](const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    for (int k = 0; k < 13; ++k) out[k] = 0.0;
    double* FI = out + 1;
    double* FJ = out + 4;
    double* FK = out + 7;
    double* FL = out + 10;
    double VI[3], VJ[3], VK[3];
    vec(at[0], at[1], VI);
    vec(at[1], at[2], VJ);
    if (kind == 0 || kind == 2 || kind == 4) {   // bend family (:2244-2284, :2345-2390, :2464-2506)
        const double C11 = dot(VI, VI), C12 = dot(VI, VJ), C22 = dot(VJ, VJ);
        const double prefac = 1.0 / std::sqrt(C11 * C22);
        const double fac = C12, fac1 = fac / C22, fac2 = fac / C11;
        double strength = coeff;
        if (kind == 0) {
            out[0] = coeff * (1.0 - prefac * fac);
        } else if (kind == 2) {
            const double th0 = PI_ - (PI_ / 180.0) * angle;
            const double c0 = std::cos(th0), c = prefac * fac;
            strength = coeff * (c - c0);
            out[0] = (coeff / 2.0) * (c - c0) * (c - c0);
        } else {
            const double th0 = PI_ - (PI_ / 180.0) * angle;
            const double th = std::acos(prefac * fac);
            strength = coeff * (th - th0) / std::sin(th);
            out[0] = (coeff / 2.0) * (th - th0) * (th - th0);
        }
        for (int d = 0; d < 3; ++d) {
            FK[d] = -strength * prefac * (fac1 * VJ[d] - VI[d]);
            FJ[d] = strength * prefac * (fac1 * VJ[d] - fac2 * VI[d] + VJ[d] - VI[d]);
            FI[d] = strength * prefac * (fac2 * VI[d] - VJ[d]);
        }
        return;
    }
    // dihedral family (:2286-2343, :2392-2462, :2508-2579)
    vec(at[2], at[3], VK);
    const double C11 = dot(VI, VI), C12 = dot(VI, VJ), C13 = dot(VI, VK);
    const double C22 = dot(VJ, VJ), C23 = dot(VJ, VK), C33 = dot(VK, VK);
    const double D12 = C11 * C22 - C12 * C12, D23 = C22 * C33 - C23 * C23;
    const double prefac = 1.0 / std::sqrt(D23 * D12);
    const double fac = C23 * C12 - C13 * C22, fac1 = fac / D23, fac2 = fac / D12;
    double strength = coeff;
    if (kind == 1) {
        out[0] = coeff * (1.0 + prefac * fac);
    } else {
        const double x[3] = {VI[1] * VJ[2] - VI[2] * VJ[1], VI[2] * VJ[0] - VI[0] * VJ[2],
                             VI[0] * VJ[1] - VI[1] * VJ[0]};
        const double fac_sin = dot(x, VK);
        const double ph0 = PI_ - (PI_ / 180.0) * angle;
        const double cph = -prefac * fac;
        const double sph = prefac * fac_sin * std::sqrt(dot(VJ, VJ));
        if (kind == 3) {
            const double c0 = std::cos(ph0), cs = std::cos(std::atan2(sph, cph));
            strength = coeff * (cs - c0);
            out[0] = (coeff / 2.0) * (cs - c0) * (cs - c0);
        } else {
            const double c0 = std::cos(ph0), s0 = std::sin(ph0);
            strength = coeff * (c0 - s0 * (cph / sph));
            out[0] = coeff * (1.0 - cph * c0 - sph * s0);
        }
    }
    const double a = -strength * prefac;
    for (int d = 0; d < 3; ++d) {
        FL[d] = a * (C12 * VJ[d] - C22 * VI[d] - fac1 * (C22 * VK[d] - C23 * VJ[d]));
        FK[d] = a * (C12 * VK[d] - C12 * VJ[d] + C23 * VI[d] + C22 * VI[d] - 2.0 * C13 * VJ[d] -
                     fac2 * (C11 * VJ[d] - C12 * VI[d]) - fac1 * (C33 * VJ[d] - C22 * VK[d] - C23 * VK[d] + C23 * VJ[d]));
        FJ[d] = a * (-C12 * VK[d] + C23 * VJ[d] - C23 * VI[d] - C22 * VK[d] + 2.0 * C13 * VJ[d] -
                     fac2 * (C22 * VI[d] - C11 * VJ[d] - C12 * VJ[d] + C12 * VI[d]) - fac1 * (-C33 * VJ[d] + C23 * VK[d]));
        FI[d] = a * (-C23 * VJ[d] + C22 * VK[d] - fac2 * (-C22 * VI[d] + C12 * VJ[d]));
    }
}

// The user's loop over a bonded term list: F(I) += FXI, F(J) += FXJ,
// F(K) += FXK [, F(L) += FXL], pot_eng += PE. nat = 3 or 4 atoms per term.
void or_bonded_forces(OrSys* s, int kind, int nterms, const int* atoms, const double* coeff, const double* angle) {
    const int nat = (kind == 1 || kind == 3 || kind == 5) ? 4 : 3;
    double out[13];
    for (int t = 0; t < nterms; ++t) {
        const int* at = atoms + (size_t)nat * t;
        or_bonded(s, kind, at, coeff[t], angle ? angle[t] : 0.0, out);
        s->pot_eng += out[0];
        for (int a = 0; a < nat; ++a) {
            s->fx[at[a]] += out[1 + 3 * a];
            s->fy[at[a]] += out[2 + 3 * a];
            s->fz[at[a]] += out[3 + 3 * a];
        }
    }
}

// eval_reaction_field (force.f90:2753-2766)
void or_reaction_field_eval(OrSys* s) {
    const double* R = s->rfl;
    for (int i = 0; i < s->n; ++i) {
        if (s->charge[i] != 0.0) {
            s->pot_eng = s->pot_eng + 0.5 * (s->dipx[i] * R[0] + s->dipy[i] * R[1] + s->dipz[i] * R[2]);
            s->tx[i] = s->tx[i] - (s->dipy[i] * R[2] - s->dipz[i] * R[1]);
            s->ty[i] = s->ty[i] - (s->dipz[i] * R[0] - s->dipx[i] * R[2]);
            s->tz[i] = s->tz[i] - (s->dipx[i] * R[1] - s->dipy[i] * R[0]);
        }
    }
}

// ---------------------------------------------------------- Verlet list ----
// build_nlist (system.f90:966-1003): O(N^2), J > I ascending, strict
// r^2 < (rc+skin)^2 with SUM(RIJ*RIJ). Returns the pair count K, or -1 if the
// cutoff exceeds half the box (system.f90:902-906), or -(K+2) when K exceeds cap.
// With one_based != 0 the output is the reference CSR: offset[I] is the
// 1-based start of row I, offset[N-1] = K+1, nlist holds 1-based J.
// With one_based == 0 offset has N+1 entries and values are 0-based.
long long or_nlist_build(const OrSys* s, double cutoff, double skin, int* nlist, long long cap, int* offset,
                         int one_based) {
    for (int d = 0; d < 3; ++d)
        if (cutoff > s->box[d] / 2.0) return -1;
    double rskin = cutoff + skin;
    double rsq_skin = rskin * rskin;
    long long K = 0;
    int n = s->n;
    for (int i = 0; i < n - 1; ++i) {
        offset[i] = (int)(one_based ? K + 1 : K);
        for (int j = i + 1; j < n; ++j) {
            double r[3] = {s->rx[i] - s->rx[j], s->ry[i] - s->ry[j], s->rz[i] - s->rz[j]};
            min_image(r, s->box, s->periodic);
            double rsq = (r[0] * r[0] + r[1] * r[1]) + r[2] * r[2];
            if (rsq < rsq_skin) {
                if (K < cap) nlist[K] = one_based ? j + 1 : j;
                ++K;
            }
        }
    }
    if (n >= 1) offset[n - 1] = (int)(one_based ? K + 1 : K);
    if (!one_based) offset[n] = (int)K;
    if (K > cap) return -(K + 2);
    return K;
}

// needs_rebuild (system.f90:1005-1039). r_skin_sq is (rc+skin)^2 after a
// build in the reference (trigger_mode 0) or skin^2 (trigger_mode 1).
int or_needs_rebuild(const OrSys* s, const double* xl, const double* yl, const double* zl, double cutoff,
                     double skin, int trigger_mode) {
    double max_disp = 0.0;
    for (int i = 0; i < s->n; ++i) {
        double d[3] = {s->rx[i] - xl[i], s->ry[i] - yl[i], s->rz[i] - zl[i]};
        min_image(d, s->box, s->periodic);
        double r = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        max_disp = std::max(max_disp, r);
    }
    double rs = trigger_mode == 0 ? (cutoff + skin) * (cutoff + skin) : skin * skin;
    return (4.0 * max_disp > rs) ? 1 : 0;
}

// ---------------------------------------------------------- integrators ----
static inline void wrap(OrSys* s, int i) {
    if (!s->periodic) return;
    s->rx[i] = s->rx[i] - std::round(s->rx[i] / s->box[0]) * s->box[0];
    s->ry[i] = s->ry[i] - std::round(s->ry[i] / s->box[1]) * s->box[1];
    s->rz[i] = s->rz[i] - std::round(s->rz[i] / s->box[2]) * s->box[2];
}

void or_vv_initial(OrSys* s, double dt) {                        // integrators.f90:7-34
    for (int i = 0; i < s->n; ++i) {
        s->vx[i] = s->vx[i] + 0.5 * dt * (s->fx[i] * s->inv_mass[i]);
        s->vy[i] = s->vy[i] + 0.5 * dt * (s->fy[i] * s->inv_mass[i]);
        s->vz[i] = s->vz[i] + 0.5 * dt * (s->fz[i] * s->inv_mass[i]);
        s->rx[i] = s->rx[i] + dt * s->vx[i];
        s->ry[i] = s->ry[i] + dt * s->vy[i];
        s->rz[i] = s->rz[i] + dt * s->vz[i];
        wrap(s, i);
    }
}

void or_vv_final(OrSys* s, double dt) {                          // integrators.f90:36-53
    s->kin_eng = 0.0;
    for (int i = 0; i < s->n; ++i) {
        s->vx[i] = s->vx[i] + 0.5 * dt * (s->fx[i] * s->inv_mass[i]);
        s->vy[i] = s->vy[i] + 0.5 * dt * (s->fy[i] * s->inv_mass[i]);
        s->vz[i] = s->vz[i] + 0.5 * dt * (s->fz[i] * s->inv_mass[i]);
        s->kin_eng = s->kin_eng + 0.5 * s->mass[i] * (s->vx[i] * s->vx[i] + s->vy[i] * s->vy[i] + s->vz[i] * s->vz[i]);
    }
}

// Mid-point quaternion derivative with two fixed-point passes
// (integrators.f90:140-168 and :572-604). body_frame_L selects the Langevin
// form, which returns L_body and leaves RM of the last pass in rm.
static void q_midpoint(const OrSys* s, int i, double dt, double qd[4], double rm[3][3], double Lb[3]) {
    double qn[4] = {s->qw[i], s->qx[i], s->qy[i], s->qz[i]};
    for (int it = 0; it < 2; ++it) {
        double qo[4] = {qn[0], qn[1], qn[2], qn[3]};
        M3<double> R = rotmat(qo[0], qo[1], qo[2], qo[3]);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) rm[a][b] = R.m[a][b];
        Lb[0] = (R.m[0][0] * s->lx[i] + R.m[0][1] * s->ly[i] + R.m[0][2] * s->lz[i]);
        Lb[1] = (R.m[1][0] * s->lx[i] + R.m[1][1] * s->ly[i] + R.m[1][2] * s->lz[i]);
        Lb[2] = (R.m[2][0] * s->lx[i] + R.m[2][1] * s->ly[i] + R.m[2][2] * s->lz[i]);
        double wx = Lb[0] * s->ixx_inv[i], wy = Lb[1] * s->iyy_inv[i], wz = Lb[2] * s->izz_inv[i];
        qd[0] = 0.5 * (-qo[1] * wx - qo[2] * wy - qo[3] * wz);
        qd[1] = 0.5 * (qo[0] * wx + qo[2] * wz - qo[3] * wy);
        qd[2] = 0.5 * (qo[0] * wy - qo[1] * wz + qo[3] * wx);
        qd[3] = 0.5 * (qo[0] * wz + qo[1] * wy - qo[2] * wx);
        qn[0] = s->qw[i] + 0.5 * dt * qd[0];
        qn[1] = s->qx[i] + 0.5 * dt * qd[1];
        qn[2] = s->qy[i] + 0.5 * dt * qd[2];
        qn[3] = s->qz[i] + 0.5 * dt * qd[3];
    }
}

static void q_advance(OrSys* s, int i, double dt, const double qd[4]) {
    s->qw[i] = s->qw[i] + dt * qd[0];
    s->qx[i] = s->qx[i] + dt * qd[1];
    s->qy[i] = s->qy[i] + dt * qd[2];
    s->qz[i] = s->qz[i] + dt * qd[3];
    double qm = std::sqrt(s->qw[i] * s->qw[i] + s->qx[i] * s->qx[i] + s->qy[i] * s->qy[i] + s->qz[i] * s->qz[i]);
    s->qw[i] = s->qw[i] / qm; s->qx[i] = s->qx[i] / qm; s->qy[i] = s->qy[i] / qm; s->qz[i] = s->qz[i] / qm;
}

void or_qq_initial(OrSys* s, double dt) {                        // integrators.f90:123-183
    for (int i = 0; i < s->n; ++i) {
        s->lx[i] = s->lx[i] + 0.5 * dt * s->tx[i];
        s->ly[i] = s->ly[i] + 0.5 * dt * s->ty[i];
        s->lz[i] = s->lz[i] + 0.5 * dt * s->tz[i];
        double qd[4], rm[3][3], Lb[3];
        q_midpoint(s, i, dt, qd, rm, Lb);
        q_advance(s, i, dt, qd);
    }
}

static double kin_rot_one(const OrSys* s, int i) {
    M3<double> R = rotmat(s->qw[i], s->qx[i], s->qy[i], s->qz[i]);
    double Lb0 = (R.m[0][0] * s->lx[i] + R.m[0][1] * s->ly[i] + R.m[0][2] * s->lz[i]);
    double Lb1 = (R.m[1][0] * s->lx[i] + R.m[1][1] * s->ly[i] + R.m[1][2] * s->lz[i]);
    double Lb2 = (R.m[2][0] * s->lx[i] + R.m[2][1] * s->ly[i] + R.m[2][2] * s->lz[i]);
    return 0.5 * ((Lb0 * Lb0) * s->ixx_inv[i] + (Lb1 * Lb1) * s->iyy_inv[i] + (Lb2 * Lb2) * s->izz_inv[i]);
}

void or_qq_final(OrSys* s, double dt) {                          // integrators.f90:185-218
    s->kin_rot = 0.0;
    for (int i = 0; i < s->n; ++i) {
        s->lx[i] = s->lx[i] + 0.5 * dt * s->tx[i];
        s->ly[i] = s->ly[i] + 0.5 * dt * s->ty[i];
        s->lz[i] = s->lz[i] + 0.5 * dt * s->tz[i];
        s->kin_rot = s->kin_rot + kin_rot_one(s, i);
    }
}

// Langevin (integrators.f90:507-627); philox key as given (reference key by
// default), counter (I 1-based, step, int(T*1000), stream).
void or_lgv_initial(OrSys* s, double dt, int step, double damp, const uint32_t* key) {
    double kk1 = 1.0 - (damp * dt) / 2.0;
    double kk2 = 1.0 / (1.0 + (damp * dt) / 2.0);
    int32_t temp_int = (int32_t)(s->target_temp * 1000.0);
    uint32_t kref[2] = {PHILOX_KEY0, PHILOX_KEY1};
    const uint32_t* k = key ? key : kref;
    for (int i = 0; i < s->n; ++i) {
        s->vx[i] = s->vx[i] + 0.5 * dt * (s->fx[i] * s->inv_mass[i]);
        s->vy[i] = s->vy[i] + 0.5 * dt * (s->fy[i] * s->inv_mass[i]);
        s->vz[i] = s->vz[i] + 0.5 * dt * (s->fz[i] * s->inv_mass[i]);
        s->rx[i] = s->rx[i] + 0.5 * dt * s->vx[i];
        s->ry[i] = s->ry[i] + 0.5 * dt * s->vy[i];
        s->rz[i] = s->rz[i] + 0.5 * dt * s->vz[i];
        uint32_t c0[4] = {(uint32_t)(i + 1), (uint32_t)step, (uint32_t)temp_int, 0u};
        uint32_t c1[4] = {(uint32_t)(i + 1), (uint32_t)step, (uint32_t)temp_int, 1u};
        double n1[3], n2[3];
        normal_3seq(c0, k, n1[0], n1[1], n1[2]);
        normal_3seq(c1, k, n2[0], n2[1], n2[2]);
        double ed = std::exp(-damp * dt);
        double amp = std::sqrt(s->target_temp * s->inv_mass[i] * (1 - std::exp(-2.0 * damp * dt)));
        s->vx[i] = ed * s->vx[i] + amp * n1[0];
        s->vy[i] = ed * s->vy[i] + amp * n1[1];
        s->vz[i] = ed * s->vz[i] + amp * n1[2];
        s->rx[i] = s->rx[i] + 0.5 * dt * s->vx[i];
        s->ry[i] = s->ry[i] + 0.5 * dt * s->vy[i];
        s->rz[i] = s->rz[i] + 0.5 * dt * s->vz[i];
        wrap(s, i);
        s->lx[i] = s->lx[i] + 0.5 * dt * s->tx[i];
        s->ly[i] = s->ly[i] + 0.5 * dt * s->ty[i];
        s->lz[i] = s->lz[i] + 0.5 * dt * s->tz[i];
        double qd[4], rm[3][3], Lb[3];
        q_midpoint(s, i, dt, qd, rm, Lb);
        double Ii[3] = {s->ixx[i], s->iyy[i], s->izz[i]};
        for (int d = 0; d < 3; ++d)
            Lb[d] = kk2 * kk1 * Lb[d] + kk2 * std::sqrt(2.0 * damp * s->target_temp * dt * Ii[d]) * n2[d];
        s->lx[i] = (rm[0][0] * Lb[0] + rm[1][0] * Lb[1] + rm[2][0] * Lb[2]);
        s->ly[i] = (rm[0][1] * Lb[0] + rm[1][1] * Lb[1] + rm[2][1] * Lb[2]);
        s->lz[i] = (rm[0][2] * Lb[0] + rm[1][2] * Lb[1] + rm[2][2] * Lb[2]);
        q_advance(s, i, dt, qd);
    }
}

void or_lgv_final(OrSys* s, double dt) {                         // integrators.f90:629-676
    s->kin_eng = 0.0;
    s->kin_rot = 0.0;
    for (int i = 0; i < s->n; ++i) {
        s->vx[i] = s->vx[i] + 0.5 * dt * (s->fx[i] * s->inv_mass[i]);
        s->vy[i] = s->vy[i] + 0.5 * dt * (s->fy[i] * s->inv_mass[i]);
        s->vz[i] = s->vz[i] + 0.5 * dt * (s->fz[i] * s->inv_mass[i]);
        s->lx[i] = s->lx[i] + 0.5 * dt * s->tx[i];
        s->ly[i] = s->ly[i] + 0.5 * dt * s->ty[i];
        s->lz[i] = s->lz[i] + 0.5 * dt * s->tz[i];
        double kr = kin_rot_one(s, i);
        s->kin_eng = s->kin_eng + 0.5 * s->mass[i] * (s->vx[i] * s->vx[i] + s->vy[i] * s->vy[i] + s->vz[i] * s->vz[i]);
        s->kin_rot = s->kin_rot + kr;
    }
}

// ---------------------------------------------------------- Nose-Hoover ----
// integrators.f90:233-301
static double polyval(double x, const double* c, int upper) {
    double f = c[upper];
    for (int i = upper - 1; i >= 0; --i) f = f * x + c[i];
    return f;
}
static double exprel(double x) {
    const double g[5] = {1.0 / 1, 1.0 / 6, 1.0 / 120, 1.0 / 5040, 1.0 / 362880};
    if (std::fabs(x) > 0.01) return (std::exp(x) - 1.0) / x;
    return std::exp(x / 2) * polyval((x / 2) * (x / 2), g, 4);
}
static void u4(double t, int j_start, int j_stop, int stride, double* p_eta, const double* HB, double sum_mv2,
               double ndof, double T) {
    const int N_th = 3;
    for (int j = j_start; stride > 0 ? j <= j_stop : j >= j_stop; j += stride) {
        double gj = (j == 1) ? (sum_mv2 - ndof * T) : ((p_eta[j - 2] * p_eta[j - 2] / HB[j - 2]) - T);
        if (j == N_th) {
            p_eta[j - 1] = p_eta[j - 1] + t * gj;
        } else {
            double x = t * p_eta[j] / HB[j];
            double c = exprel(-x);
            p_eta[j - 1] = p_eta[j - 1] * std::exp(-x) + t * gj * c;
        }
    }
}
static double sum_mv2(const OrSys* s) {
    double acc = 0.0;
    for (int i = 0; i < s->n; ++i) acc += s->mass[i] * (s->vx[i] * s->vx[i] + s->vy[i] * s->vy[i] + s->vz[i] * s->vz[i]);
    return acc;
}
static void nh_masses(const OrSys* s, double coupling, int has_coupling, double HB[3], double& ndof) {
    const double tau = 2.0;
    ndof = 3 * (s->n / s->nrigid) - 3;
    if (has_coupling) { HB[0] = HB[1] = HB[2] = coupling; }
    else {
        HB[0] = HB[1] = HB[2] = s->target_temp * std::pow(tau, 2.0);
        HB[0] = ndof * s->target_temp * std::pow(tau, 2.0);
    }
}

// mode 0: the reference's per-particle chain (integrators.f90:303-354), with
// the O(N) SUM re-evaluated at every particle exactly as written.
// mode 1: standard NHC, one chain update per half step (not in the reference).
void or_nht_initial(OrSys* s, double dt, double coupling, int has_coupling, int mode) {
    double HB[3], ndof;
    nh_masses(s, coupling, has_coupling, HB, ndof);
    double T = s->target_temp;
    if (mode == 0) {
        for (int i = 0; i < s->n; ++i) {
            u4(dt / 4.0, 3, 1, -1, s->p_eta, HB, sum_mv2(s), ndof, T);
            double sc = std::exp(-0.5 * dt * s->p_eta[0] / HB[0]);
            s->vx[i] = s->vx[i] * sc; s->vy[i] = s->vy[i] * sc; s->vz[i] = s->vz[i] * sc;
            for (int k = 0; k < 3; ++k) s->eta[k] = s->eta[k] + 0.5 * dt * s->p_eta[k] / HB[k];
            u4(dt / 4.0, 1, 3, 1, s->p_eta, HB, sum_mv2(s), ndof, T);
            s->vx[i] = s->vx[i] + 0.5 * dt * (s->fx[i] * s->inv_mass[i]);
            s->vy[i] = s->vy[i] + 0.5 * dt * (s->fy[i] * s->inv_mass[i]);
            s->vz[i] = s->vz[i] + 0.5 * dt * (s->fz[i] * s->inv_mass[i]);
            s->rx[i] = s->rx[i] + dt * s->vx[i];
            s->ry[i] = s->ry[i] + dt * s->vy[i];
            s->rz[i] = s->rz[i] + dt * s->vz[i];
            wrap(s, i);
        }
    } else {
        u4(dt / 4.0, 3, 1, -1, s->p_eta, HB, sum_mv2(s), ndof, T);
        double sc = std::exp(-0.5 * dt * s->p_eta[0] / HB[0]);
        for (int i = 0; i < s->n; ++i) { s->vx[i] *= sc; s->vy[i] *= sc; s->vz[i] *= sc; }
        for (int k = 0; k < 3; ++k) s->eta[k] = s->eta[k] + 0.5 * dt * s->p_eta[k] / HB[k];
        u4(dt / 4.0, 1, 3, 1, s->p_eta, HB, sum_mv2(s), ndof, T);
        or_vv_initial(s, dt);
    }
}

void or_nht_final(OrSys* s, double dt, double coupling, int has_coupling, int mode) {
    double HB[3], ndof;
    nh_masses(s, coupling, has_coupling, HB, ndof);
    double T = s->target_temp;
    s->kin_eng = 0.0;
    if (mode == 0) {
        for (int i = 0; i < s->n; ++i) {
            s->vx[i] = s->vx[i] + 0.5 * dt * (s->fx[i] * s->inv_mass[i]);
            s->vy[i] = s->vy[i] + 0.5 * dt * (s->fy[i] * s->inv_mass[i]);
            s->vz[i] = s->vz[i] + 0.5 * dt * (s->fz[i] * s->inv_mass[i]);
            u4(dt / 4.0, 3, 1, -1, s->p_eta, HB, sum_mv2(s), ndof, T);
            double sc = std::exp(-0.5 * dt * s->p_eta[0] / HB[0]);
            s->vx[i] = s->vx[i] * sc; s->vy[i] = s->vy[i] * sc; s->vz[i] = s->vz[i] * sc;
            for (int k = 0; k < 3; ++k) s->eta[k] = s->eta[k] + 0.5 * dt * s->p_eta[k] / HB[k];
            u4(dt / 4.0, 1, 3, 1, s->p_eta, HB, sum_mv2(s), ndof, T);
            s->kin_eng = s->kin_eng + 0.5 * s->mass[i] * (s->vx[i] * s->vx[i] + s->vy[i] * s->vy[i] + s->vz[i] * s->vz[i]);
        }
    } else {
        for (int i = 0; i < s->n; ++i) {
            s->vx[i] = s->vx[i] + 0.5 * dt * (s->fx[i] * s->inv_mass[i]);
            s->vy[i] = s->vy[i] + 0.5 * dt * (s->fy[i] * s->inv_mass[i]);
            s->vz[i] = s->vz[i] + 0.5 * dt * (s->fz[i] * s->inv_mass[i]);
        }
        u4(dt / 4.0, 3, 1, -1, s->p_eta, HB, sum_mv2(s), ndof, T);
        double sc = std::exp(-0.5 * dt * s->p_eta[0] / HB[0]);
        for (int i = 0; i < s->n; ++i) { s->vx[i] *= sc; s->vy[i] *= sc; s->vz[i] *= sc; }
        for (int k = 0; k < 3; ++k) s->eta[k] = s->eta[k] + 0.5 * dt * s->p_eta[k] / HB[k];
        u4(dt / 4.0, 1, 3, 1, s->p_eta, HB, sum_mv2(s), ndof, T);
        s->kin_eng = 0.5 * sum_mv2(s);
    }
}

// Rotational chain of the standard mode (not in the reference): the same
// propagator on G1 = sum L_body^2 / I - 3N T, scaling every angular momentum.
void or_nhr_half(OrSys* s, double dt, double coupling, int has_coupling) {
    const double tau = 2.0;
    double T = s->target_temp;
    double nrot = 3.0 * s->n;
    double HB[3];
    if (has_coupling) { HB[0] = HB[1] = HB[2] = coupling; }
    else { HB[0] = HB[1] = HB[2] = T * tau * tau; HB[0] = nrot * T * tau * tau; }
    double k2 = 0.0;
    for (int i = 0; i < s->n; ++i) k2 += 2.0 * kin_rot_one(s, i);
    u4(dt / 4.0, 3, 1, -1, s->p_eta_r, HB, k2, nrot, T);
    double sc = std::exp(-0.5 * dt * s->p_eta_r[0] / HB[0]);
    for (int i = 0; i < s->n; ++i) { s->lx[i] *= sc; s->ly[i] *= sc; s->lz[i] *= sc; }
    for (int k = 0; k < 3; ++k) s->eta_r[k] = s->eta_r[k] + 0.5 * dt * s->p_eta_r[k] / HB[k];
    k2 = 0.0;
    for (int i = 0; i < s->n; ++i) k2 += 2.0 * kin_rot_one(s, i);
    u4(dt / 4.0, 1, 3, 1, s->p_eta_r, HB, k2, nrot, T);
}

// ------------------------------------------------------ setup and thermo ----
void or_calculate_thermo(OrSys* s) {                             // system.f90:725-741
    double kin_tot = s->kin_eng + s->kin_rot;
    s->temp = 2.0 * kin_tot / (double)s->dof;
    double vir = 0.0;
    for (int i = 0; i < s->n; ++i) vir += s->rx[i] * s->fx[i] + s->ry[i] * s->fy[i] + s->rz[i] * s->fz[i];
    s->virial = vir;
    if (s->nc > 0 && s->virial_bonded >= 0.0) s->virial = vir + s->virial_bonded;   // :732-736
    double volume = s->box[0] * s->box[1] * s->box[2];
    s->pressure = (s->density * s->nrigid * s->temp) + (s->virial / (3.0 * volume));
}

// ------------------------------------------------------------- RATTLE -----
// apply_constraints_a (system.f90:1060-1142): one global Gauss-Seidel loop over
// the constraint list in order, moved flags per atom, at most 100 sweeps.
// Returns 0, or 1 + the index of the constraint whose vdot test failed (the
// reference prints and stops there).
int or_constraints_a(OrSys* s, double dt) {
    const double r_tol = 1.0e-5;
    const int max_rattle = 100;
    std::vector<char> moved(s->n, 1);
    int rattle = 0;
    auto any = [&]() {
        for (char m : moved)
            if (m) return true;
        return false;
    };
    while (any() && rattle < max_rattle) {
        for (int ix = 0; ix < s->nc; ++ix) {
            const int i = s->bbi[ix], j = s->bbj[ix];
            const double len = s->bb_len[ix];
            if (moved[i] || moved[j]) {
                double r[3] = {s->rx[i] - s->rx[j], s->ry[i] - s->ry[j], s->rz[i] - s->rz[j]};
                min_image(r, s->box, s->periodic);
                const double chi = len * len - (r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
                if (std::fabs(chi) > 2 * r_tol * len * len) {
                    double ro[3] = {s->rx_old[i] - s->rx_old[j], s->ry_old[i] - s->ry_old[j],
                                    s->rz_old[i] - s->rz_old[j]};
                    min_image(ro, s->box, s->periodic);
                    const double vdot = r[0] * ro[0] + r[1] * ro[1] + r[2] * ro[2];
                    if (vdot < r_tol * len * len) {
                        s->rattle_sweeps = rattle;
                        return ix + 1;
                    }
                    const double L = chi / (2.0 * vdot * (s->inv_mass[i] + s->inv_mass[j]));
                    s->virial_bonded = s->virial_bonded + (L * len * len) / (dt * dt);
                    const double ai = L * s->inv_mass[i], aj = L * s->inv_mass[j];
                    s->rx[i] += ai * ro[0]; s->ry[i] += ai * ro[1]; s->rz[i] += ai * ro[2];
                    s->rx[j] -= aj * ro[0]; s->ry[j] -= aj * ro[1]; s->rz[j] -= aj * ro[2];
                    s->vx[i] += ai * ro[0] / dt; s->vy[i] += ai * ro[1] / dt; s->vz[i] += ai * ro[2] / dt;
                    s->vx[j] -= aj * ro[0] / dt; s->vy[j] -= aj * ro[1] / dt; s->vz[j] -= aj * ro[2] / dt;
                    moved[i] = 1;
                    moved[j] = 1;
                } else {
                    moved[i] = 0;
                    moved[j] = 0;
                }
            }
        }
        rattle = rattle + 1;
    }
    s->rattle_sweeps = rattle;
    return 0;
}

// apply_constraints_b (system.f90:1144-1208)
void or_constraints_b(OrSys* s, double dt) {
    const double r_tol = 1.0e-5;
    const int max_rattle = 100;
    std::vector<char> moved(s->n, 1);
    int rattle = 0;
    auto any = [&]() {
        for (char m : moved)
            if (m) return true;
        return false;
    };
    while (any() && rattle < max_rattle) {
        for (int ix = 0; ix < s->nc; ++ix) {
            const int i = s->bbi[ix], j = s->bbj[ix];
            const double len = s->bb_len[ix];
            if (moved[i] || moved[j]) {
                double r[3] = {s->rx[i] - s->rx[j], s->ry[i] - s->ry[j], s->rz[i] - s->rz[j]};
                min_image(r, s->box, s->periodic);
                const double v[3] = {s->vx[i] - s->vx[j], s->vy[i] - s->vy[j], s->vz[i] - s->vz[j]};
                const double vdot = r[0] * v[0] + r[1] * v[1] + r[2] * v[2];
                const double L = -vdot / ((s->inv_mass[i] + s->inv_mass[j]) * len * len);
                if (std::fabs(L) > r_tol) {
                    s->virial_bonded = s->virial_bonded + (L * len * len) / dt;
                    const double ai = L * s->inv_mass[i], aj = L * s->inv_mass[j];
                    s->vx[i] += ai * r[0]; s->vy[i] += ai * r[1]; s->vz[i] += ai * r[2];
                    s->vx[j] -= aj * r[0]; s->vy[j] -= aj * r[1]; s->vz[j] -= aj * r[2];
                    moved[i] = 1;
                    moved[j] = 1;
                } else {
                    moved[i] = 0;
                    moved[j] = 0;
                }
            }
        }
        rattle = rattle + 1;
    }
    s->rattle_sweeps = rattle;
}

// RX_old(I) = RX(I), taken by vvc_ / nhtc_ / lgvc_ before the drift
// (integrators.f90:67-69, 432-434, 714-716).
void or_constraints_save(OrSys* s) {
    for (int i = 0; i < s->n; ++i) {
        s->rx_old[i] = s->rx[i];
        s->ry_old[i] = s->ry[i];
        s->rz_old[i] = s->rz[i];
    }
}

// set_velocity_to_temperature (system.f90:362-421), quirk: scales sum v^2 to
// (6N - NC - 3) * T * Nrigid regardless of mass.
void or_set_velocity_to_temperature(OrSys* s, double rtemp, int seed, int remove_com) {
    int32_t temp_int = (int32_t)(rtemp * 1000);
    for (int i = 0; i < s->n; ++i) {
        double n[3];
        or_philox_normal_3seq(i + 1, temp_int, seed, 42, n);
        s->vx[i] = n[0]; s->vy[i] = n[1]; s->vz[i] = n[2];
    }
    int n_dof = 6 * s->n - s->nc;
    if (remove_com) {
        double cx = 0, cy = 0, cz = 0;
        for (int i = 0; i < s->n; ++i) { cx += s->vx[i]; cy += s->vy[i]; cz += s->vz[i]; }
        cx /= (double)s->n; cy /= (double)s->n; cz /= (double)s->n;
        for (int i = 0; i < s->n; ++i) { s->vx[i] -= cx; s->vy[i] -= cy; s->vz[i] -= cz; }
        n_dof -= 3;
    }
    double v2 = 0.0;
    for (int i = 0; i < s->n; ++i) v2 += (s->vx[i] * s->vx[i] + s->vy[i] * s->vy[i] + s->vz[i] * s->vz[i]);
    double factor = std::sqrt((double)n_dof * rtemp * s->nrigid / v2);
    for (int i = 0; i < s->n; ++i) { s->vx[i] *= factor; s->vy[i] *= factor; s->vz[i] *= factor; }
}

// generate_fcc_lattice positions and orientations (system.f90:438-523)
void or_generate_fcc(int cells, double box_len, double* rx, double* ry, double* rz, double* qw, double* qx, double* qy,
                     double* qz) {
    double cell = box_len / (double)cells;
    double half = cell / 2.0;
    double rr3 = 1.0 / std::sqrt(3.0);
    double a = std::sqrt((1.0 + rr3) / 2.0), b = std::sqrt((1.0 - rr3) / 2.0);
    double c = rr3 / std::sqrt(1.0 - std::pow(rr3, 2.0));
    double bx[4] = {0.0, half, 0.0, half}, by[4] = {0.0, half, half, 0.0}, bz[4] = {0.0, 0.0, half, half};
    double bw[4] = {a, b, b, a}, bqx[4] = {b * c, a * -c, a * c, b * -c}, bqy[4] = {b * -c, a * -c, a * c, b * c};
    int m = 0;
    for (int I = 1; I <= cells; ++I)
        for (int J = 1; J <= cells; ++J)
            for (int K = 1; K <= cells; ++K) {
                for (int r = 0; r < 4; ++r) {
                    rx[m + r] = bx[r] + cell * (I - 1);
                    ry[m + r] = by[r] + cell * (J - 1);
                    rz[m + r] = bz[r] + cell * (K - 1);
                    qw[m + r] = bw[r]; qx[m + r] = bqx[r]; qy[m + r] = bqy[r]; qz[m + r] = 0.0;
                }
                m += 4;
            }
    for (int i = 0; i < m; ++i) { rx[i] -= box_len / 2.0; ry[i] -= box_len / 2.0; rz[i] -= box_len / 2.0; }
}

} // extern "C"
