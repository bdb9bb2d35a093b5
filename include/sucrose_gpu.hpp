// C++ adapters over the C ABI of sucrose_gpu.h, shaped like the reference's
// C++ classes: Force with calculate_forces (include/force.h:8-17),
// Integrator with initial_step / final_step and get/set_timestep
// (include/integrators.h:8-27), and a System whose Atom arrays are SoA
// std::vector<double> (include/system.h:10-28).
//
// The reference calls Force::calculate_forces(i, j) once per listed pair from
// the user's loop; here compute() evaluates the whole list on the GPU in one
// call and leaves the forces on the device, where the integrators use them.
// upload / download move the System's arrays across explicitly. Errors throw
// sucrose_gpu::Error carrying the C status and sg_last_error's message (the
// reference prints to std::cerr and exits, src/system.cpp:162-165).
//
// Header-only; link with -lsucrose_gb300.
#pragma once

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "sucrose_gpu.h"

namespace sucrose_gpu {

class Error : public std::runtime_error {
  public:
    Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

  private:
    int code_;
};

inline void check(sg_ctx* ctx, int rc) {
    if (rc != SG_OK) throw Error(rc, std::string("sucrose_gpu: ") + (ctx ? sg_last_error(ctx) : "no context"));
}

// Owns one device context (one system, its list and its stream).
class Context {
  public:
    Context(int n, const double box[3], bool periodic = true, int device = 0) : n_(n) {
        check(ctx_, sg_create(&ctx_, n, device));
        check(ctx_, sg_set_box(ctx_, box, periodic ? 1 : 0));
    }
    ~Context() {
        if (ctx_) sg_destroy(ctx_);
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;

    sg_ctx* get() const { return ctx_; }
    int size() const { return n_; }

    // per-particle constants; NULL (nullptr) keeps the defaults
    void set_particles(const double* mass, const double* sig_x, const double* sig_y, const double* sig_z,
                       const double* eps_x, const double* eps_y, const double* eps_z, const double* ixx,
                       const double* iyy, const double* izz) {
        check(ctx_, sg_set_particles(ctx_, mass, sig_x, sig_y, sig_z, eps_x, eps_y, eps_z, ixx, iyy, izz));
    }

    // set_atom_charge for every particle (fortran/system.f90:148); reference_defaults
    // applies initialize_system's negative-to-zero rule (:595-598)
    void set_charges(const double* charge, bool reference_defaults = false) {
        check(ctx_, sg_set_charges(ctx_, charge, reference_defaults ? 1 : 0));
    }

    // init_nlist (fortran/system.f90:895); trigger 0 = the reference's (rc+skin)^2 bound
    void init_nlist(double skin, double cutoff, int trigger_mode = 0) {
        check(ctx_, sg_nlist_init(ctx_, skin, cutoff, trigger_mode));
    }
    bool needs_rebuild() {
        int32_t f = 0;
        check(ctx_, sg_nlist_needs_rebuild(ctx_, &f));
        return f != 0;
    }
    void build_nlist() { check(ctx_, sg_nlist_build(ctx_)); }
    void update_nlist() { check(ctx_, sg_nlist_update(ctx_)); }

    // initialize_forces (fortran/system.f90:423)
    void zero_forces() { check(ctx_, sg_zero_forces(ctx_)); }
    void synchronize() { check(ctx_, sg_synchronize(ctx_)); }
    // set_velocity_to_temperature (fortran/system.f90:361-421), on the device
    void set_velocity_to_temperature(double rtemp, int seed, bool remove_com_velocity = true, int nrigid = 1) {
        check(ctx_, sg_set_velocity_to_temperature(ctx_, rtemp, seed, remove_com_velocity ? 1 : 0, nrigid));
    }

    // State of a reference-shaped System (atom.rx ... atom.lz, 0-based).
    template <class SystemT>
    void upload(const SystemT& s) {
        const auto& a = s.atom;
        check(ctx_, sg_upload_state(ctx_, a.rx.data(), a.ry.data(), a.rz.data(), opt(a.qw), opt(a.qx), opt(a.qy),
                                    opt(a.qz), a.vx.data(), a.vy.data(), a.vz.data(), opt(a.lx), opt(a.ly),
                                    opt(a.lz)));
    }
    template <class SystemT>
    void download(SystemT& s) {
        auto& a = s.atom;
        fit(a.rx); fit(a.ry); fit(a.rz); fit(a.vx); fit(a.vy); fit(a.vz);
        fit(a.qw); fit(a.qx); fit(a.qy); fit(a.qz); fit(a.lx); fit(a.ly); fit(a.lz);
        check(ctx_, sg_download_state(ctx_, a.rx.data(), a.ry.data(), a.rz.data(), a.qw.data(), a.qx.data(),
                                      a.qy.data(), a.qz.data(), a.vx.data(), a.vy.data(), a.vz.data(), a.lx.data(),
                                      a.ly.data(), a.lz.data()));
    }
    template <class SystemT>
    void download_forces(SystemT& s) {
        auto& a = s.atom;
        fit(a.fx); fit(a.fy); fit(a.fz); fit(a.tx); fit(a.ty); fit(a.tz);
        check(ctx_, sg_download_forces(ctx_, a.fx.data(), a.fy.data(), a.fz.data(), a.tx.data(), a.ty.data(),
                                       a.tz.data()));
    }

    // Device accumulators since the last zero_forces: pot_eng, pair virial, KE, KE_rot.
    void energies(double out[4]) { check(ctx_, sg_read_energies(ctx_, out)); }

  private:
    static const double* opt(const std::vector<double>& v) { return v.empty() ? nullptr : v.data(); }
    void fit(std::vector<double>& v) const {
        if ((int)v.size() != n_) v.assign(n_, 0.0);
    }
    sg_ctx* ctx_ = nullptr;
    int n_;
};

// ---- forces (include/force.h) ------------------------------------------------
class Force {
  protected:
    Context& ctx_;
    sg_pair_params p_{};
    explicit Force(Context& c) : ctx_(c) {}

  public:
    virtual ~Force() = default;
    // The batched calculate_forces: every listed pair, accumulated into the
    // device forces and torques; adds PE to *pot_eng and r.F to *virial.
    double compute(double* virial = nullptr, sg_ecp_stats* stats = nullptr) {
        double pe = 0.0, vir = 0.0;
        check(ctx_.get(), sg_pair_forces(ctx_.get(), &p_, &pe, &vir, stats));
        if (virial) *virial += vir;
        return pe;
    }
    // The same without waiting (results stay in the device accumulators).
    void compute_async() { check(ctx_.get(), sg_pair_forces_async(ctx_.get(), &p_)); }
    const sg_pair_params& params() const { return p_; }
};

class LennardJones : public Force {       // LennardJones (src/force.cpp:6); lj_ (fortran/force.f90:6)
  public:
    LennardJones(Context& c, double epsilon, double sigma, double cutoff) : Force(c) {
        p_.kind = SG_LJ; p_.epsilon = epsilon; p_.sigma = sigma; p_.cutoff = cutoff;
    }
};
class LennardJones12 : public Force {     // LennardJones12 (src/force.cpp:39); lj12_ (force.f90:51)
  public:
    LennardJones12(Context& c, double epsilon, double sigma, double cutoff) : Force(c) {
        p_.kind = SG_LJ12; p_.epsilon = epsilon; p_.sigma = sigma; p_.cutoff = cutoff;
    }
};
class LennardJones_WCA : public Force {   // LennardJones_WCA (src/force.cpp:71); wca_ (force.f90:155)
  public:
    LennardJones_WCA(Context& c, double epsilon, double sigma) : Force(c) {
        p_.kind = SG_WCA; p_.epsilon = epsilon; p_.sigma = sigma; p_.cutoff = sigma;
    }
};
class MorsePotential : public Force {     // MorsePotential (src/force.cpp:113): no cutoff, no shift
  public:
    MorsePotential(Context& c, double dissociation_energy, double equilibrium_distance, double width,
                   double cutoff = HUGE_VAL)   // a finite cutoff gives morse_ (force.f90:199-233)
        : Force(c) {
        p_.kind = SG_MORSE; p_.dissoc = dissociation_energy; p_.rmin = equilibrium_distance; p_.width = width;
        p_.cutoff = cutoff;
    }
};
class DebyeHuckel : public Force {        // dh_calculate_forces (force.f90:2589-2617)
  public:
    DebyeHuckel(Context& c, double cutoff, double db_len, double dielectric) : Force(c) {
        p_.kind = SG_DH; p_.cutoff = cutoff; p_.db_len = db_len; p_.dielectric = dielectric;
    }
};
class Coulombic : public Force {          // coulombic_calculate_forces (force.f90:2627-2665)
  public:
    Coulombic(Context& c, double cutoff, double dielectric) : Force(c) {
        p_.kind = SG_COULOMB; p_.cutoff = cutoff; p_.dielectric = dielectric;
    }
};
class Dipole : public Force {             // module dipole (force.f90:2669-2767)
  public:
    Dipole(Context& c, double cutoff, double dielectric) : Force(c) {
        p_.kind = SG_DIPOLE; p_.cutoff = cutoff; p_.dielectric = dielectric;
    }
    void init_reaction_field() { check(ctx_.get(), sg_reaction_field_init(ctx_.get())); }
    // adds 0.5 DIP.RFL over charged particles to the returned energy and DIP x RFL to the torques
    double eval_reaction_field() {
        double e = 0.0;
        check(ctx_.get(), sg_reaction_field_eval(ctx_.get(), &e));
        return e;
    }
};
class GayBerne : public Force {           // gb_ family (force.f90:308-1030); kind SG_GB .. SG_GBWC
  public:
    GayBerne(Context& c, double cutoff, int mu = 1, int nu = 2, int kind = SG_GB, double wf = 0.0,
             double chirality = 0.0)
        : Force(c) {
        p_.kind = kind; p_.cutoff = cutoff; p_.mu = mu; p_.nu = nu; p_.wf = wf; p_.chirality = chirality;
    }
};
class EllipsoidContact : public Force {   // ecp_ family (force.f90:1202-2234); kind SG_ECP .. SG_ECPWC
  public:
    EllipsoidContact(Context& c, double cutoff, int kind = SG_ECP, int solver = SG_SOLVER_NEWTON, double wf = 0.0,
                     double chirality = 0.0)
        : Force(c) {
        p_.kind = kind; p_.cutoff = cutoff; p_.solver = solver; p_.wf = wf; p_.chirality = chirality;
        p_.newton_tol = 1e-6; p_.newton_max_iter = 20; p_.fp64_check = 1;
    }
};

// ---- integrators (include/integrators.h) ------------------------------------
class Integrator {
  protected:
    Context& ctx_;
    double dt;

  public:
    Integrator(Context& c, double dt) : ctx_(c), dt(dt) {}
    virtual ~Integrator() = default;
    double get_timestep() { return dt; }
    void set_timestep(double dt) { this->dt = dt; }
    virtual void initial_step() = 0;
    virtual void final_step() = 0;
    double kinetic_energy = 0.0;
    double rotational_energy = 0.0;
};

class VerletIntegrator : public Integrator {   // vv_* (fortran/integrators.f90:7-53)
  public:
    using Integrator::Integrator;
    void initial_step() override { check(ctx_.get(), sg_vv_initial(ctx_.get(), dt)); }
    void final_step() override { check(ctx_.get(), sg_vv_final(ctx_.get(), dt, &kinetic_energy)); }
};

class RigidVerletIntegrator : public Integrator {   // vv_* + qq_* (integrators.f90:123-218)
  public:
    using Integrator::Integrator;
    void initial_step() override {
        check(ctx_.get(), sg_vv_initial(ctx_.get(), dt));
        check(ctx_.get(), sg_qq_initial(ctx_.get(), dt));
    }
    void final_step() override {
        check(ctx_.get(), sg_vv_final(ctx_.get(), dt, &kinetic_energy));
        check(ctx_.get(), sg_qq_final(ctx_.get(), dt, &rotational_energy));
    }
};

class LangevinIntegrator : public Integrator {   // lgv_* (integrators.f90:507-676)
  public:
    LangevinIntegrator(Context& c, double dt, double target_temp, double damping = 1.0, int first_step = 1)
        : Integrator(c, dt), T_(target_temp), gamma_(damping), step_(first_step) {}
    void initial_step() override {
        check(ctx_.get(), sg_lgv_initial(ctx_.get(), dt, step_, gamma_, T_, nullptr));
        ++step_;
    }
    void final_step() override {
        check(ctx_.get(), sg_lgv_final(ctx_.get(), dt, gamma_, &kinetic_energy, &rotational_energy));
    }

  private:
    double T_, gamma_;
    int step_;
};

class NoseHooverIntegrator : public Integrator {   // nht_* (integrators.f90:233-392), + qq_* with rotations
  public:
    // mode 1: standard chain (rot_chain adds one on rotation); mode 0: the reference's per-particle chain
    NoseHooverIntegrator(Context& c, double dt, double target_temp, bool rotations = false, int mode = 1,
                         bool rot_chain = false, double coupling = 0.0)
        : Integrator(c, dt), T_(target_temp), Q_(coupling), mode_(mode), rot_(rotations), chain_(rot_chain) {}
    void initial_step() override {
        check(ctx_.get(), sg_nht_initial(ctx_.get(), dt, T_, Q_, mode_, chain_ ? 1 : 0));
        if (rot_) check(ctx_.get(), sg_qq_initial(ctx_.get(), dt));
    }
    void final_step() override {
        check(ctx_.get(), sg_nht_final(ctx_.get(), dt, T_, Q_, mode_, chain_ ? 1 : 0, &kinetic_energy));
        if (rot_) check(ctx_.get(), sg_qq_final(ctx_.get(), dt, &rotational_energy));
    }

  private:
    double T_, Q_;
    int mode_;
    bool rot_, chain_;
};

}  // namespace sucrose_gpu
