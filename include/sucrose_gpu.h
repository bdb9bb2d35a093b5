/*
 * sucrose_gpu.h — C ABI of the GB300 (sm_103a) SUCROSE molecular-dynamics hot path.
 *
 * One context (sg_ctx) owns one system's device state on one GPU and one CUDA
 * stream. State is FP32 structure-of-arrays in HBM (float4 position,
 * quaternion, velocity, angular momentum, force, torque, shape, energy scales,
 * inertia); energy, virial and kinetic-energy totals are FP64 (kinetic terms
 * and their partial sums in double-float, ~48 bits).
 *
 * Host arrays crossing this boundary are FP64 structure-of-arrays of length N
 * in the reference's own layout (module globals RX..RZ, QW..QZ, VX..VZ, LX..LZ,
 * FX..FZ, TX..TY, fortran/system.f90:7-30), 0-based. The caller keeps
 * ownership of every host array; the context copies in and out explicitly.
 *
 * Every entry point returns an sg_status; on error sg_last_error() holds a
 * one-line message. Nothing here exits the process, and no kernel traps:
 * per-pair non-convergence and list overflow are counted in device status
 * words, then reported by the call that reads them.
 *
 * Threading: one context per host thread; calls on one context are serialised
 * by the caller; contexts are independent.
 */
#ifndef SUCROSE_GPU_H
#define SUCROSE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sg_ctx sg_ctx;

typedef enum {
    SG_OK = 0,
    SG_EINVAL = 1,               /* bad argument                                   */
    SG_ECUTOFF_GT_HALFBOX = 2,   /* init_nlist guard, fortran/system.f90:902-906   */
    SG_ENOCONV = 3,              /* contact solve did not converge for some pairs */
    SG_ENAN = 4,                 /* non-finite energy or force                      */
    SG_ECAPACITY = 5,            /* neighbour list overflowed its capacity          */
    SG_ECUDA = 6,                /* CUDA runtime error                              */
    SG_ENOTREADY = 7             /* call order (e.g. forces before a list build)    */
} sg_status;

/* Pair-potential kinds; one entry point per family. */
typedef enum {
    SG_LJ = 0,     /* lj_calculate_forces     fortran/force.f90:6-49     */
    SG_LJ12 = 1,   /* lj12_calculate_forces   fortran/force.f90:51-93    */
    SG_LJW = 2,    /* ljw_calculate_forces    fortran/force.f90:95-146   */
    SG_WCA = 3,    /* wca_calculate_forces    fortran/force.f90:155-190  */
    SG_MORSE = 4,  /* morse_calculate_forces  fortran/force.f90:199-233  */
    SG_DH = 5,     /* dh_calculate_forces     fortran/force.f90:2589-2617 (charges) */
    SG_COULOMB = 6,/* coulombic_calculate_forces fortran/force.f90:2627-2665 (charges) */
    SG_DIPOLE = 7, /* dipole_calculate_forces fortran/force.f90:2687-2751 (charge x body z axis) */
    SG_GB = 10,    /* gb_calculate_forces     fortran/force.f90:308-428  */
    SG_GBR = 11,   /* gbr_calculate_forces    fortran/force.f90:430-533  */
    SG_GBW = 12,   /* gbw_calculate_forces    fortran/force.f90:535-663  */
    SG_GBC = 13,   /* gbc_calculate_forces    fortran/force.f90:665-843  */
    SG_GBWC = 14,  /* gbwc_calculate_forces   fortran/force.f90:845-1030 */
    SG_ECP = 20,   /* ecp_calculate_forces    fortran/force.f90:1202-1385 */
    SG_ECPR = 21,  /* ecpr_calculate_forces   fortran/force.f90:1387-1551 */
    SG_ECPW = 22,  /* ecpw_calculate_forces   fortran/force.f90:1553-1742 */
    SG_ECPC = 23,  /* ecpc_calculate_forces   fortran/force.f90:1744-1984 */
    SG_ECPWC = 24  /* ecpwc_calculate_forces  fortran/force.f90:1986-2234 */
} sg_pair_kind;

/* ECP contact-parameter solvers. */
typedef enum {
    SG_SOLVER_BRENT_COMPAT = 0,  /* the reference's Brent (fortran/force.f90:1046-1172), FP64, same lambda bits */
    SG_SOLVER_NEWTON = 1,        /* Newton on dS/dlambda from lambda = 1/2, FP32, FP64 residual check */
    SG_SOLVER_MLP_NEWTON = 2,    /* MLP initial guess, <= 3 Newton steps, else the plain Newton */
    SG_SOLVER_NEWTON_SUPPORT = 3 /* the same Newton from lambda = h_A / (h_A + h_B), h the support
                                    functions sqrt(r.A r), sqrt(r.B r) of the two ellipsoids along r
                                    (the maximiser for spheres); same tolerance and check */
} sg_ecp_solver;

/* Parameters of one pair-force call (the arguments of *_calculate_forces). */
typedef struct {
    int32_t kind;       /* sg_pair_kind                                            */
    int32_t mu, nu;     /* GB / ECP exponents; 0,0 selects the reference's (1,2) for GB, (2,1) for ECP */
    int32_t solver;     /* sg_ecp_solver (ECP only)                                 */
    double sigma;       /* LJ/WCA sigma                                             */
    double epsilon;     /* LJ/WCA epsilon                                           */
    double cutoff;      /* rc (LJ), GB/ECP cutoff argument                          */
    double wf;          /* weld width (ljw, gbw, gbwc, ecpw, ecpwc)                 */
    double chirality;   /* gbc, gbwc, ecpc, ecpwc                                   */
    double newton_tol;  /* bound on |S'(lambda)| / (r.K) checked in FP64; 0 selects 1e-6 */
    int32_t newton_max_iter;  /* 0 selects 20                                       */
    int32_t fp64_check; /* Newton residual check: 1 = FP64 (default), 2 = double-float on the FP32 pipe,
                           0 = none (FP32 step-size test only) */
    double dissoc;      /* Morse well depth D (dissoc)                              */
    double width;       /* Morse width alpha (width)                                */
    double rmin;        /* Morse equilibrium distance r0 (rmin)                     */
    double db_len;      /* Debye length (dh)                                        */
    double dielectric;  /* relative permittivity (dh, coulombic, dipole)            */
} sg_pair_params;

/* Per-call statistics of a pair-force evaluation. ECP kinds fill every field;
 * LJ and GB kinds fill pairs and, in solver_evals, the pairs that were inside
 * the potential's range (the rest were listed but out of range). */
typedef struct {
    int64_t pairs;          /* pairs evaluated                                      */
    int64_t solver_evals;   /* ECP: total objective / Newton evaluations; LJ, GB: pairs in range */
    int64_t nonconverged;   /* pairs whose solve hit its iteration cap              */
    int64_t fallbacks;      /* MLP path: pairs that fell back to the plain Newton;
                               GB kinds: pairs evaluated in the near-contact class
                               (contact distance in double-float)                */
    int64_t iter_hist[24];  /* Newton iterations per pair (last bin: >= 23); bin 0:
                               pairs the support-filtered launch turned away
                               unsolved (beyond any contact)                       */
    int64_t fp64_refined;   /* Newton: pairs that needed the FP64-residual correction */
} sg_ecp_stats;

/* ---- context -------------------------------------------------------------- */
int sg_create(sg_ctx** out, int32_t n, int32_t device);
int sg_destroy(sg_ctx* ctx);
const char* sg_last_error(const sg_ctx* ctx);
/* Opaque: the context's CUDA stream (cudaStream_t), for callers that overlap work. */
void* sg_stream(sg_ctx* ctx);
int sg_synchronize(sg_ctx* ctx);

/* set_box / set_periodic_boundary (fortran/system.f90:185-213). On a context
 * with a list, the cell grid follows the new box (the pair list itself waits
 * for the next rebuild, as the reference's does); captured steps re-capture. */
int sg_set_box(sg_ctx* ctx, const double box[3], int32_t periodic);

/* Per-particle constants: mass, shape (sig_*), energy scales (eps_*) and
 * principal moments (I*). NULL arrays take initialize_system's defaults
 * (fortran/system.f90:586-682): mass 1, shape and energy (1,1,1), inertia
 * ((sy^2+sz^2)/20, ...). A zero mass freezes the particle. */
int sg_set_particles(sg_ctx* ctx, const double* mass, const double* sig_x, const double* sig_y,
                     const double* sig_z, const double* eps_x, const double* eps_y, const double* eps_z,
                     const double* ixx, const double* iyy, const double* izz);

/* set_atom_charge (fortran/system.f90:148-165) for every particle; NULL sets
 * all charges to 0. reference_defaults = 1 also applies initialize_system's
 * rule (fortran/system.f90:595-598): a negative charge becomes 0. The charges
 * feed SG_DH, SG_COULOMB and SG_DIPOLE. */
int sg_set_charges(sg_ctx* ctx, const double* charge, int32_t reference_defaults);

/* Reaction field of the dipole potential (module dipole, fortran/force.f90:2669-2767).
 * init_reaction_field (:2677-2685): zero DIP (per particle) and RFL. Every
 * SG_DIPOLE call then sets DIP(I) for the I side of each pair in range and adds
 * U2 * dip_coeff to RFL, which the reference adds to every element of its RFL
 * arrays (:2743-2745), so RFL is one vector shared by all particles; it keeps
 * growing across calls until the next init, as in the reference.
 * eval_reaction_field (:2753-2766): for every particle with charge != 0 adds
 * 0.5 DIP.RFL to the potential energy and subtracts DIP x RFL from its torque;
 * *pot_eng (may be NULL) gets the energy added. Single-system contexts only. */
int sg_reaction_field_init(sg_ctx* ctx);
int sg_reaction_field_eval(sg_ctx* ctx, double* pot_eng);
/* RFL (3 doubles) and DIP (NULL arrays skip). */
int sg_reaction_field_read(sg_ctx* ctx, double rfl[3], double* dipx, double* dipy, double* dipz);

/* Copy state in / out. Any array may be NULL to skip it. Quaternions are (w,x,y,z). */
int sg_upload_state(sg_ctx* ctx, const double* rx, const double* ry, const double* rz, const double* qw,
                    const double* qx, const double* qy, const double* qz, const double* vx, const double* vy,
                    const double* vz, const double* lx, const double* ly, const double* lz);
int sg_download_state(sg_ctx* ctx, double* rx, double* ry, double* rz, double* qw, double* qx, double* qy,
                      double* qz, double* vx, double* vy, double* vz, double* lx, double* ly, double* lz);
int sg_download_forces(sg_ctx* ctx, double* fx, double* fy, double* fz, double* tx, double* ty, double* tz);
int sg_upload_forces(sg_ctx* ctx, const double* fx, const double* fy, const double* fz, const double* tx,
                     const double* ty, const double* tz);

/* initialize_forces (fortran/system.f90:423-436): zero F, T and the accumulators. */
int sg_zero_forces(sg_ctx* ctx);

/* ---- neighbour list (fortran/system.f90:885-1053) ---------------------------- */
/* init_nlist(skin, cutoff) :895 + build_init_nlist :927. trigger_mode 0 reproduces
 * the reference trigger (displacement^2 * 4 > (rc+skin)^2, quirk at :933,:1033);
 * trigger_mode 1 uses skin^2. Returns SG_ECUTOFF_GT_HALFBOX like the reference stop. */
int sg_nlist_init(sg_ctx* ctx, double skin, double cutoff, int32_t trigger_mode);
/* needs_rebuild() :1005 — reads the device flag (synchronises). */
int sg_nlist_needs_rebuild(sg_ctx* ctx, int32_t* flag);
/* build_nlist() :966 — unconditional rebuild. */
int sg_nlist_build(sg_ctx* ctx);
/* needs_rebuild + conditional build on the device, no host synchronisation
 * (safe inside a captured CUDA graph). */
int sg_nlist_update(sg_ctx* ctx);
/* Number of listed (half) pairs; synchronises. */
int sg_nlist_count(sg_ctx* ctx, int64_t* npairs);
/* The list in the reference's CSR (rows J>I ascending): with one_based = 1,
 * offset[I] is the 1-based start of row I and offset[N-1] = K+1, nlist holds
 * 1-based J, exactly as nlist/offset after build_nlist (:977-1000). With
 * one_based = 0, offset has N+1 entries and values are 0-based. */
int sg_nlist_export(sg_ctx* ctx, int32_t* nlist, int64_t capacity, int32_t* offset, int64_t* npairs,
                    int32_t one_based);
/* The listed pairs (I < J, 0-based) in the device's internal order, which is
 * the order of per-pair outputs such as sg_ecp_lambda. */
int sg_nlist_pairs(sg_ctx* ctx, int32_t* pi, int32_t* pj, int64_t capacity, int64_t* npairs);
/* Number of list rebuilds performed since sg_nlist_init. */
int sg_nlist_builds(sg_ctx* ctx, int64_t* builds);

/* ---- pair forces (fortran/force.f90, README.md:86-103 accumulation) ----------- */
/* Batched drop-in for the user's pair loop over the Verlet list calling
 * X_calculate_forces(I, J, ...): adds F(I) += FXIJ, F(J) -= FXIJ,
 * T(I) += TXI, T(J) += TXJ on the device and adds the summed PE to *pot_eng
 * and the pair virial sum r_ij . F_ij to *virial (either may be NULL).
 * stats may be NULL. */
int sg_pair_forces(sg_ctx* ctx, const sg_pair_params* params, double* pot_eng, double* virial,
                   sg_ecp_stats* stats);
/* Same, without reading results back (no host synchronisation): the sums stay
 * in the device accumulators, read by sg_read_energies. */
int sg_pair_forces_async(sg_ctx* ctx, const sg_pair_params* params);
/* Device accumulators: pot_eng, pair virial, kin_eng, kin_rot (FP64). */
int sg_read_energies(sg_ctx* ctx, double out[4]);
/* Per-pair contact parameter of the last ECP call, in the device list order
 * that sg_nlist_pairs returns (debug / parity). After a call with the
 * support-filtered launch (sg_pair_set_launch filter 2), pairs that it did not
 * solve read NaN. */
int sg_ecp_lambda(sg_ctx* ctx, float* lam, int64_t capacity);

/* ---- integrators (fortran/integrators.f90) ----------------------------------- */
int sg_vv_initial(sg_ctx* ctx, double dt);                       /* :7-34    */
int sg_vv_final(sg_ctx* ctx, double dt, double* kin_eng);          /* :36-53   */
int sg_qq_initial(sg_ctx* ctx, double dt);                       /* :123-183 */
int sg_qq_final(sg_ctx* ctx, double dt, double* kin_rot);          /* :185-218 */
/* Langevin :507-627 / :629-676. Noise counter (I 1-based, step, int(T*1000), stream 0|1);
 * key NULL selects the reference's fixed key (fortran/xmath.f90:10-11). */
int sg_lgv_initial(sg_ctx* ctx, double dt, int32_t step, double damping, double target_temp,
                   const uint32_t* key);
int sg_lgv_final(sg_ctx* ctx, double dt, double damping, double* kin_eng, double* kin_rot);
/* Nose-Hoover chain (length 3, tau 2) :303-354 / :356-392. coupling <= 0 selects
 * the reference masses. mode 0 = the reference's per-particle chain recurrence,
 * mode 1 = standard NHC (one chain update per half step). rot_chain = 1 adds a
 * second chain on the rotational kinetic energy (mode 1 only). */
int sg_nht_initial(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t mode,
                   int32_t rot_chain);
int sg_nht_final(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t mode, int32_t rot_chain,
                 double* kin_eng);
/* Chain state (eta[3], p_eta[3], eta_rot[3], p_eta_rot[3]) in / out. */
int sg_nht_state(sg_ctx* ctx, double* get12, const double* set12);
/* calculate_thermo (fortran/system.f90:725-741): out = {temp, virial, pressure};
 * dof and density as in initialize_system; kin_eng/kin_rot from the last integrator call.
 * With constraints set, virial_bonded (reset by sg_zero_forces, like initialize_forces)
 * joins the virial when it is not negative (:732-736). */
int sg_thermo(sg_ctx* ctx, int32_t dof, double density, int32_t nrigid, double* out3);

/* ---- reporters (fortran/reporters.f90) ------------------------------------------ */
/* set_atom_type (fortran/system.f90:110-127) for every particle (NULL: all 0;
 * negative types become 0 as initialize_system does). Used by the reporters. */
int sg_set_types(sg_ctx* ctx, const int32_t* type);

typedef struct sg_reporter sg_reporter;
typedef enum {
    SG_REPORT_STATE = 0,       /* state_data_reporter   reporters.f90:1-48    */
    SG_REPORT_TRAJECTORY = 1,  /* trajectory_reporter   reporters.f90:50-101  */
    SG_REPORT_CONFIG = 2,      /* config_reporter       reporters.f90:103-138 */
    SG_REPORT_CHECKPOINT = 3   /* checkpoint_reporter   reporters.f90:140-231 */
} sg_report_kind;
/* open_*_file(unit, filename): the state-data kind writes its header line. */
int sg_reporter_open(sg_ctx* ctx, int32_t kind, const char* path, sg_reporter** out);
/* dof, density, Nrigid of calculate_thermo for the state-data kind. */
int sg_reporter_set_thermo(sg_reporter* r, int32_t dof, double density, int32_t nrigid);
/* report_*(unit, step): snapshots the device state at this point of the
 * context stream and returns; a host thread formats and writes the record. */
int sg_reporter_write(sg_reporter* r, int64_t step);
/* Wait until every snapshot so far is written. */
int sg_reporter_flush(sg_reporter* r);
/* close_*_file: flush and close. */
int sg_reporter_close(sg_reporter* r);
/* load_checkpoint (reporters.f90:186-223): a new context from a checkpoint
 * text file (atoms, masses, charges, shapes, energies, inertia, state, box,
 * bonds as constraints); *out is set (and must be destroyed) whenever a
 * context was created, also on a later error. */
int sg_load_checkpoint(const char* path, int32_t device, sg_ctx** out, int64_t* config_index);
/* Exact binary state (no counterpart in the reference): every particle array
 * as stored on the device, box, thermostat chain, step counter, accumulators.
 * Loading needs a context of the same particle count. */
int sg_save_state(sg_ctx* ctx, const char* path);
int sg_load_state(sg_ctx* ctx, const char* path);

/* ---- Monte Carlo barostat (fortran/integrators.f90:858-945) --------------------- */
/* mc_barostat(compute_potential, accept, volume_change): one trial volume move.
 * compute_potential is the sum of the npairs pair sets (plus every registered
 * bonded list when include_bonded = 1) evaluated by this context's kernels;
 * beta = 1 / temperature (the reference uses the last calculate_thermo's
 * temperature); max_dv <= 0 selects 0.01. random_number is replaced by two
 * Philox words of counter (counter lo, counter hi, 0x4D43, 0) under key (NULL:
 * the reference key). Positions (atoms, not molecules) and the box are scaled
 * by (V_new / V_old)^(1/3) and restored on rejection; forces, torques and the
 * energy accumulators are left as they were. *accept = 1 accepted, 0 rejected,
 * -1 no move (V_new <= 0, where the reference leaves accept unset). Waits. */
int sg_mc_barostat(sg_ctx* ctx, const sg_pair_params* pairs, int32_t npairs, int32_t include_bonded,
                   double target_pressure, double temperature, double max_dv, const uint32_t key[2],
                   uint64_t counter, int32_t* accept, double* volume_out);

/* ---- bonded terms (module bonded, fortran/force.f90:2238-2581) ---------------- */
typedef enum {
    SG_BEND = 0,          /* bend_calculate_forces         fortran/force.f90:2244-2284 */
    SG_DIH = 1,           /* dih_calculate_forces          fortran/force.f90:2286-2343 */
    SG_COSINE_BEND = 2,   /* cosine_bend_calculate_forces  fortran/force.f90:2345-2390 */
    SG_COSINE_DIH = 3,    /* cosine_dih_calculate_forces   fortran/force.f90:2392-2462 */
    SG_ANGLE_BEND = 4,    /* angle_bend_calculate_forces   fortran/force.f90:2464-2506 */
    SG_ANGLE_DIH = 5      /* angle_dih_calculate_forces    fortran/force.f90:2508-2579 */
} sg_bonded_kind;
/* Register the term list of one kind (replacing any earlier list of that kind):
 * nterms terms of 3 (bends) or 4 (dihedrals) atoms, I J K [L] in the routine's
 * argument order (one_based selects 1-based indices), coeff per term and, for
 * the cosine_ and angle_ kinds, angle per term in degrees (NULL otherwise). */
int sg_bonded_set(sg_ctx* ctx, int32_t kind, int32_t nterms, const int32_t* atoms, const double* coeff,
                  const double* angle, int32_t one_based);
/* The user's loop over that list: F(I) += FXI, F(J) += FXJ, F(K) += FXK
 * [, F(L) += FXL], pot_eng += PE; *pot_eng (may be NULL) gets the energy. */
int sg_bonded_forces(sg_ctx* ctx, int32_t kind, double* pot_eng);
int sg_bonded_forces_async(sg_ctx* ctx, int32_t kind);

/* ---- bond constraints (module constraints, fortran/system.f90:1055-1210) ------ */
/* set_num_constraints + add_constraint for every bond (fortran/system.f90:97-108,
 * 345-360): atoms I, J (one_based selects 1-based indices) at fixed distance
 * length. The list is split into molecules (connected components); each is
 * solved by one device thread in the list's order. Single-system contexts only. */
int sg_set_constraints(sg_ctx* ctx, int32_t nc, const int32_t* bbi, const int32_t* bbj, const double* length,
                       int32_t one_based);
/* RX_old = RX: the start-of-step positions apply_constraints_a measures against. */
int sg_constraints_save(sg_ctx* ctx);
/* apply_constraints_a(DT) :1060-1142 and apply_constraints_b(DT) :1144-1208, enqueued
 * without waiting; both add to virial_bonded. Where the reference stops on a
 * constraint failure (:1102-1106) the kernel records it and leaves that molecule;
 * sg_constraints_check (and sg_step_check) then returns SG_ENOCONV. */
int sg_constraints_a(sg_ctx* ctx, double dt);
int sg_constraints_b(sg_ctx* ctx, double dt);
int sg_constraints_check(sg_ctx* ctx);
int sg_constraints_clear_error(sg_ctx* ctx);
/* Counters since the last reset: {max sweeps a, molecules still moving after 100
 * sweeps a, corrections a, the same three for b}. */
int sg_constraint_stats(sg_ctx* ctx, int64_t out[6], int32_t reset);
/* Constrained integrators (fortran/integrators.f90): vvc_ :55-106, nhtc_ :394-490,
 * lgvc_ :678-855. Each is the plain half step of this header with RX_old saved
 * before it and apply_constraints_a / _b after it; the initial steps wait and
 * report a constraint failure. */
int sg_vvc_initial(sg_ctx* ctx, double dt);
int sg_vvc_final(sg_ctx* ctx, double dt, double* kin_eng);
int sg_nhtc_initial(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t mode, int32_t rot_chain);
int sg_nhtc_final(sg_ctx* ctx, double dt, double target_temp, double coupling, int32_t mode, int32_t rot_chain,
                  double* kin_eng);
int sg_lgvc_initial(sg_ctx* ctx, double dt, int32_t step, double damping, double target_temp,
                    const uint32_t* key);
int sg_lgvc_final(sg_ctx* ctx, double dt, double damping, double* kin_eng, double* kin_rot);

/* ---- batched replicas (no counterpart in the reference: its state is one
 * global system, fortran/system.f90:7-39) ------------------------------------ */
/* nrep independent periodic systems of uneven size in one context: replica r
 * holds n_per_rep[r] particles, box boxes[3r..3r+2], potential family
 * family[r] (0 = LJ kinds, 1 = GB kinds, 2 = ECP kinds; replicas grouped by
 * family in increasing order), Langevin temperature temps[r] and Philox key
 * keys[2r..2r+1] (NULL: the reference key). State arrays are the replicas'
 * arrays concatenated, each in its own box centred on the origin. Every other
 * entry point then acts on all replicas at once: pair calls evaluate the
 * replicas of the params' family, Langevin uses each replica's T and key with
 * the particle's index within its replica in the counter, so a replica draws
 * the numbers of its own single-system run. Nose-Hoover is per system and not
 * available here. */
int sg_create_replicas(sg_ctx** out, int32_t nrep, const int32_t* n_per_rep, const double* boxes,
                       const int32_t* family, const double* temps, const uint32_t* keys, int32_t device);
/* Verlet lists of every replica; skin[f], cutoff[f] per family f (3 each). */
int sg_rep_nlist_init(sg_ctx* ctx, const double* skin, const double* cutoff, int32_t trigger_mode);
/* Rebuilds of each replica's rows since sg_rep_nlist_init (counts[nrep]; the
 * initial build counts one). */
int sg_nlist_replica_builds(sg_ctx* ctx, int64_t* counts);
/* Per-replica kinetic energies: ke2[2r] translational, ke2[2r+1] rotational (FP64). */
int sg_rep_kinetic(sg_ctx* ctx, double* ke2);

/* ---- whole timestep, captured in a CUDA graph ------------------------------- */
/* One timestep in the reference's README order (README.md:83-115, with the
 * Verlet list of fortran/system.f90:1005 and :966): integrator initial half
 * step, list check with device-side conditional rebuild, initialize_forces,
 * the pair loop, integrator final half step. */
typedef enum {
    SG_INT_NVE = 0,        /* vv_* (+ qq_* with rotations)                          */
    SG_INT_LANGEVIN = 1,   /* lgv_* (rotation included when rotations = 1)          */
    SG_INT_NH = 2,         /* nht_* standard chain (+ qq_*), optional rotational chain */
    SG_INT_NH_REF = 3      /* nht_* with the reference's per-particle chain (+ qq_*) */
} sg_integrator;

typedef struct {
    int32_t integrator;    /* sg_integrator                                       */
    int32_t rotations;     /* 1: quaternion dynamics                               */
    int32_t rot_chain;     /* SG_INT_NH: second chain on rotation                  */
    int32_t first_step;    /* Langevin step counter of the next step               */
    double dt, target_temp, damping, coupling;
    uint32_t key[2];       /* Langevin Philox key (has_key = 1), else the reference key */
    int32_t has_key;
    int32_t flags;         /* SG_STEP_FLAT: list build as flag-gated kernels in the
                              graph instead of a conditional node (same results; for
                              profilers that do not follow conditional nodes)      */
    sg_pair_params pair;   /* the pair potential evaluated every step              */
} sg_step_config;
#define SG_STEP_FLAT 1
#define SG_STEP_REACTION_FIELD 2   /* eval_reaction_field after the pair stage (SG_DIPOLE) */
#define SG_STEP_BONDED 8           /* every registered bonded list after the pair stage */
#define SG_STEP_CONSTRAINTS 4      /* RATTLE around the integrator: RX_old saved before the initial half
                                      step, apply_constraints_a after it, apply_constraints_b after the
                                      final half step (vvc_, nhtc_, lgvc_ with the chosen integrator) */

/* Set the step program. The first sg_step call runs one step eagerly (which
 * allocates every buffer), then captures one step as a CUDA graph; later
 * steps launch the graph. Reallocation (list regrowth) forces a re-capture. */
int sg_step_configure(sg_ctx* ctx, const sg_step_config* cfg);
/* Same, with the step's pair stage given as npairs (1..3) parameter sets run in
 * order, their forces and energies summed as the reference's user loop sums
 * several calculate_forces calls (e.g. WCA plus Coulomb). In a replica context
 * each set acts on the replicas of its potential family (LJ-like kinds < 10,
 * GB, ECP): one replica context holding LJ and GB replicas passes one LJ and
 * one GB set. cfg->pair is ignored. */
int sg_step_configure_pairs(sg_ctx* ctx, const sg_step_config* cfg, const sg_pair_params* pairs, int32_t npairs);
/* Enqueue nsteps timesteps on the context stream; returns without waiting. */
int sg_step(sg_ctx* ctx, int32_t nsteps);
/* Wait, then report list overflow (SG_ECAPACITY) or a non-finite energy (SG_ENAN). */
int sg_step_check(sg_ctx* ctx);
/* Run nsteps steps (one eager step, then a captured step with an event-record
 * node between its stages, launched nsteps times) and return the mean
 * milliseconds of: initial half step, constraints a, list check and rebuild,
 * force zeroing, pair forces, final half step, constraints b (the constraint
 * stages are 0 without SG_STEP_CONSTRAINTS). */
int sg_step_stage_times(sg_ctx* ctx, int32_t nsteps, double out_ms[7]);
/* Kernel launches in one captured step (after the first sg_step call). */
int sg_step_kernel_count(sg_ctx* ctx, int64_t* count);

/* The learned guess for every listed pair on the tensor cores (tcgen05.mma,
 * accumulators in tensor memory), into out_dev (device, >= pair count): the
 * pass that SG_SOLVER_MLP_NEWTON runs before the Newton kernel. */
int sg_mlp_guess_tc(sg_ctx* ctx, float* out_dev, int64_t capacity);
/* Failure-path test hook: the next tensor-core guess pass issues no MMA, so
 * its completion waits run out after a short bound; the pass stops, releases
 * its tensor memory and the call reports SG_ECUDA. No fault, no hang. */
int sg_mlp_test_wait_timeout(sg_ctx* ctx);
/* Clear the tensor-core pass's error flag (after a reported timeout). */
int sg_mlp_clear_error(sg_ctx* ctx);
/* inline_guess = 1: the ECP kernel evaluates the guess itself with warp-level
 * mma.sync instead (one kernel, more registers); 0 (default): separate pass. */
int sg_mlp_set_inline(sg_ctx* ctx, int32_t inline_guess);

/* ---- autotuner of the pair kernels (no counterpart in the reference) ------- */
typedef struct {
    int32_t block;       /* chosen threads per block (64, 128 or 256)           */
    int32_t filter;      /* chosen: 1 = range filter + per-warp in-range queue;
                            2 = Gay-Berne replicas: one replica per block, its
                            records staged in shared memory (replaces (256, 0));
                            ECP kinds: 0 = one kernel per pair, 1 = split Newton
                            path (solve kernel, then force kernel), 2 = one
                            kernel behind the support-function range test (pairs
                            beyond h_A + h_B + reach - sigma are not solved)   */
    int32_t candidates;  /* variants timed (ms[0..candidates-1])                 */
    int32_t reserved;
    float ms[8];         /* mean launch time of the variants (block, filter), in
                            order (256,0) (128,0) (256,1) (128,1) (64,0) (64,1);
                            GB replicas: (256,2) in place of (256,0); ECP with a
                            Newton solver: (256,2) (128,2) (256,0) (128,0)
                            (256,1) (128,1) (64,2) (64,0); kinds without the
                            second axis: (256,0) (128,0) (64,0)              */
} sg_tune_result;
/* Time each launch variant of the params' pair kernel on the current list
 * (reps launches each), keep the fastest for this context's (kind, size,
 * density) bucket; a variant with the same second axis and a smaller block
 * within 1 % of the fastest is kept instead (a tie goes to the smaller
 * block). Forces, torques and energy accumulators are restored.
 * Captured steps are re-captured at their next sg_step. */
int sg_pair_autotune(sg_ctx* ctx, const sg_pair_params* params, int32_t reps, sg_tune_result* out);
/* Set a launch variant by hand (block 64, 128 or 256; filter 0, 1, or 2 for
 * the Gay-Berne replica tiles; for ECP kinds, filter 1 selects the split
 * Newton path and 2 the support-filtered one kernel, both of which the Brent
 * solver ignores). */
int sg_pair_set_launch(sg_ctx* ctx, int32_t kind, int32_t block, int32_t filter);

/* Measured FP32 (fp64 = 0) or FP64 (fp64 = 1) FMA throughput of this GPU in
 * TFLOP/s: the roofline denominator of the FP32-pipe pair kernels. */
int sg_peak_fma(sg_ctx* ctx, int32_t fp64, double* tflops);

/* ---- pair forces without any allocation -------------------------------------- */
/* No counterpart in the reference. For callers that keep their particle data
 * in device memory and cannot call cudaMalloc where they call this: code that
 * runs while another library captures the stream into a CUDA graph, hosts
 * whose device memory comes from their own pool, OpenACC / CUDA Fortran
 * programs that keep RX, RY, RZ and FX, FY, FZ resident on the device.
 *
 * Evaluates lj_ / lj12_ / ljw_ / wca_ (params->kind) over a half list that
 * names each unordered pair once, in any order and either way round, and
 * ADDS the forces into fx, fy, fz and {pot_eng, pair virial} into
 * pot_virial[0..1], like the reference's pair loop (README.md:86-103): the
 * force of pair k acts on pair_i[k] with r = r_i - r_j, and its negative on
 * pair_j[k]. Indices are 0-based, or 1-based (Fortran's RX(1..N)) when
 * one_based is nonzero. A pair whose index lies outside the n particles, or
 * whose two indices are equal, is skipped; when bad_pairs is not NULL the call
 * sets *bad_pairs (a DEVICE int32) to the number of pairs it skipped.
 * rx..rz, pair_i, pair_j, fx..fz, pot_virial and bad_pairs are DEVICE
 * pointers owned by the caller; box and params are host memory; the work is
 * enqueued on `stream` (a cudaStream_t, NULL for the default stream) and the
 * call returns without waiting.
 *
 * It allocates nothing: its scratch is a fixed device array inside the
 * library (about 2.1 MiB, held by every GPU that loads the library until the
 * process exits), which limits n to 131072 particles; larger n returns
 * SG_EINVAL with a message in err. The first call on a device looks the
 * scratch up for that device, so make that first call before any stream
 * capture. All calls share the scratch: calls whose work overlaps on the GPU
 * (other streams, other host threads) race and must be serialised by the
 * caller. err (may be NULL) receives a message on failure. */
int sg_lj_forces_noalloc(int32_t n, const double* rx, const double* ry, const double* rz, const int32_t* pair_i,
                         const int32_t* pair_j, int64_t npairs, int32_t one_based, const double box[3],
                         int32_t periodic, const sg_pair_params* params, double* fx, double* fy, double* fz,
                         double* pot_virial, int32_t* bad_pairs, void* stream, char* err, int32_t err_len);

/* ---- seeded isotropic ellipsoid placement ---------------------------------- */
/* No counterpart in the reference, whose only generator is the FCC lattice
 * (fortran/system.f90:438-523). n hard ellipsoids of the given semi-axes in a
 * periodic box centred on 0, built on the current device: positions start
 * uniform in the box and orientations uniform on the unit 3-sphere (Philox
 * words of the seed); the ellipsoids grow from a fifth of their size to full
 * size while Jacobi sweeps move and turn every overlapping pair apart
 * (Perram-Wertheim test and its gradient) until no pair is closer than gap
 * times contact. The same seed gives the same bits on every run (per-particle
 * sums in fixed point). r_out: n x 3, q_out: n x 4 (w, x, y, z), HOST arrays.
 * Returns SG_ENOCONV if the sweeps could not relax the packing (too dense),
 * SG_ECUTOFF_GT_HALFBOX if the box is narrower than about four semi-axes. */
typedef struct {
    int32_t stages;              /* growth steps taken                         */
    int32_t sweeps;              /* Jacobi sweeps in all                       */
    int64_t overlaps;            /* pairs closer than gap x contact at the end */
    double min_contact_ratio;    /* min |r| / contact distance over close pairs */
    double final_scale;          /* size reached, 1 on success                 */
} sg_place_report;
int sg_place_isotropic(int64_t n, const double semi_axes[3], const double box[3], uint64_t seed, double gap,
                       double* r_out, double* q_out, sg_place_report* rep);

/* ---- Philox4x32-10 (fortran/xmath.f90:42-113) -------------------------------- */
/* Host-side single block, for callers that mirror philox_uniform. */
void sg_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* n counters (4 words each) from a HOST array through a device kernel. */
int sg_philox4x32_device(sg_ctx* ctx, int64_t n, const uint32_t* ctr, const uint32_t key[2], uint32_t* out);
/* philox_normal_3seq on the device for n counters; out holds 3 doubles per counter. */
int sg_philox_normal_3seq_device(sg_ctx* ctx, int64_t n, const int32_t* ctr, double* out);
/* set_velocity_to_temperature (fortran/system.f90:361-421) on the device:
 * particle I (1-based) takes the normals of counter (I, int(rtemp*1000), seed,
 * 42) under the default key; with remove_com the mean velocity is subtracted
 * and n_dof = 6N - NC - 3, else n_dof = 6N - NC (NC: the constraints given to
 * sg_set_constraints, as the reference's module count); the velocities are
 * then scaled so that sum |v|^2 = n_dof * rtemp * nrigid (mass ignored, as in
 * the reference). Sums in FP64, the result rounded once to the FP32 state.
 * Enqueued on the context's stream (no synchronisation). Single systems only;
 * SG_EINVAL for a replica context, no particles, remove_com with one particle,
 * rtemp outside (0, 2147483.647), nrigid < 1 or no degrees of freedom. */
int sg_set_velocity_to_temperature(sg_ctx* ctx, double rtemp, int32_t seed, int32_t remove_com, int32_t nrigid);

/* ---- learned contact-parameter guess (no counterpart in the reference) -------- */
/* Weights of the 14(16)->64->64->64->1 MLP, FP32 master copy, packed
 * W1[64x16] b1[64] W2[64x64] b2[64] W3[64x64] b3[64] W4[64] b4[1]. */
int sg_mlp_set_weights(sg_ctx* ctx, const float* w, int64_t count);
int sg_mlp_get_weights(sg_ctx* ctx, float* w, int64_t count);
int64_t sg_mlp_weight_count(void);
/* Seeded Kaiming-uniform initialisation; resets the Adam state. */
int sg_mlp_init(sg_ctx* ctx, uint64_t seed);
/* Features (BF16, 16 per pair, x_bf16 is a DEVICE buffer) and labels (the
 * lambda of the last ECP call, FP32, DEVICE) for the current list. */
int sg_mlp_features(sg_ctx* ctx, void* x_bf16, float* y, int64_t capacity, int64_t* count);
/* Tensor-core training: one Adam step on a minibatch (DEVICE x_bf16 rows x 16,
 * y rows), MSE on the sigmoid output; loss_host may be NULL. */
int sg_mlp_train_step(sg_ctx* ctx, const void* x_bf16, const float* y, int64_t rows, float lr, float* loss_host);
/* Gradients of the MSE loss (packed like the weights) without an update. */
int sg_mlp_grad(sg_ctx* ctx, const void* x_bf16, const float* y, int64_t rows, float* grad_host, float* loss_host);
/* The in-kernel guess (warp-level MMA inference, clamped to [0.02, 0.98]) for
 * every listed pair, in sg_nlist_pairs order, into a DEVICE buffer. */
int sg_mlp_guess(sg_ctx* ctx, float* out_dev, int64_t capacity);
/* Forward pass of the training path: yhat (DEVICE, rows). */
int sg_mlp_predict(sg_ctx* ctx, const void* x_bf16, int64_t rows, float* yhat_dev);

#ifdef __cplusplus
}
#endif
#endif
