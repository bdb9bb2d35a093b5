! ISO_C_BINDING interface to libsucrose_gb300.so (include/sucrose_gpu.h).
!
! The reference's users drive the time loop from a Fortran program that
! calls `X_calculate_forces(I, J, ...)` inside their own pair loop
! (README.md:57-119) and the integrator routines of fortran/integrators.f90.
! This module lets such a program call the GB300 path instead: one batched
! call per pair potential fills FX..TZ and pot_eng, and the integrator,
! thermostat and neighbour-list routines keep their names with an `sg_`
! prefix. Every interface below names the C entry point it binds; the C
! header states what each does and which reference routine it replaces.
!
! Conventions of the binding:
!   * the context is an opaque type(c_ptr) made by sg_create;
!   * host state arrays are real(c_double) columns, RX(1:N) etc. (assumed
!     size; the C side reads them as 0-based views of the same memory);
!   * optional outputs and the Philox key are type(c_ptr), value: pass
!     c_null_ptr to skip them, or c_loc(x) of a TARGET variable;
!   * unsigned C integers (the Philox key, the placement seed) are carried
!     in the signed Fortran kind of the same width, bit for bit;
!   * every function returns the sg_status code (0 = SG_OK); sg_error_message
!     returns the context's last message as a Fortran string.
!
! No Fortran compiler exists in the image this library is built in, so this
! file is checked by a test against the C header and the library's exported
! symbols (names, argument counts, structure sizes), not by compiling it.
module sucrose_gpu
    use iso_c_binding
    implicit none
    private :: c_strlen

    ! sg_status
    integer(c_int), parameter :: SG_OK = 0, SG_EINVAL = 1, SG_ECUTOFF_GT_HALFBOX = 2, SG_ENOCONV = 3, &
        SG_ENAN = 4, SG_ECAPACITY = 5, SG_ECUDA = 6, SG_ENOTREADY = 7
    ! sg_pair_kind
    integer(c_int32_t), parameter :: SG_LJ = 0, SG_LJ12 = 1, SG_LJW = 2, SG_WCA = 3, SG_MORSE = 4, &
        SG_DH = 5, SG_COULOMB = 6, SG_DIPOLE = 7, SG_GB = 10, SG_GBR = 11, SG_GBW = 12, SG_GBC = 13, &
        SG_GBWC = 14, SG_ECP = 20, SG_ECPR = 21, SG_ECPW = 22, SG_ECPC = 23, SG_ECPWC = 24
    ! sg_ecp_solver
    integer(c_int32_t), parameter :: SG_SOLVER_BRENT_COMPAT = 0, SG_SOLVER_NEWTON = 1, SG_SOLVER_MLP_NEWTON = 2, &
        SG_SOLVER_NEWTON_SUPPORT = 3
    ! sg_integrator and step flags
    integer(c_int32_t), parameter :: SG_INT_NVE = 0, SG_INT_LANGEVIN = 1, SG_INT_NH = 2, SG_INT_NH_REF = 3
    integer(c_int32_t), parameter :: SG_STEP_FLAT = 1, SG_STEP_REACTION_FIELD = 2, SG_STEP_CONSTRAINTS = 4, &
        SG_STEP_BONDED = 8

    ! sg_pair_params: the arguments of one *_calculate_forces family
    type, bind(c) :: sg_pair_params
        integer(c_int32_t) :: kind = 0, mu = 0, nu = 0, solver = SG_SOLVER_NEWTON
        real(c_double)     :: sigma = 1.0d0, epsilon = 1.0d0, cutoff = 0.0d0, wf = 0.0d0
        real(c_double)     :: chirality = 0.0d0, newton_tol = 0.0d0
        integer(c_int32_t) :: newton_max_iter = 0, fp64_check = 1
        real(c_double)     :: dissoc = 0.0d0, width = 0.0d0, rmin = 0.0d0, db_len = 0.0d0, dielectric = 1.0d0
    end type sg_pair_params

    ! sg_ecp_stats
    type, bind(c) :: sg_ecp_stats
        integer(c_int64_t) :: pairs, solver_evals, nonconverged, fallbacks
        integer(c_int64_t) :: iter_hist(24)
        integer(c_int64_t) :: fp64_refined
    end type sg_ecp_stats

    ! sg_step_config: one timestep in the README's order
    type, bind(c) :: sg_step_config
        integer(c_int32_t)   :: integrator = SG_INT_NVE, rotations = 0, rot_chain = 0, first_step = 1
        real(c_double)       :: dt = 0.0d0, target_temp = 0.0d0, damping = 0.0d0, coupling = 0.0d0
        integer(c_int32_t)   :: key(2) = 0
        integer(c_int32_t)   :: has_key = 0, flags = 0
        type(sg_pair_params) :: pair
    end type sg_step_config

    interface
        ! ---- context --------------------------------------------------------
        integer(c_int) function sg_create(ctx, n, device) bind(c, name="sg_create")
            import :: c_ptr, c_int, c_int32_t
            type(c_ptr), intent(out)      :: ctx
            integer(c_int32_t), value     :: n, device
        end function
        integer(c_int) function sg_destroy(ctx) bind(c, name="sg_destroy")
            import :: c_ptr, c_int
            type(c_ptr), value            :: ctx
        end function
        type(c_ptr) function sg_last_error(ctx) bind(c, name="sg_last_error")
            import :: c_ptr
            type(c_ptr), value            :: ctx
        end function
        integer(c_int) function sg_synchronize(ctx) bind(c, name="sg_synchronize")
            import :: c_ptr, c_int
            type(c_ptr), value            :: ctx
        end function
        ! set_box / set_periodic_boundary (fortran/system.f90:185-213)
        integer(c_int) function sg_set_box(ctx, box, periodic) bind(c, name="sg_set_box")
            import :: c_ptr, c_int, c_double, c_int32_t
            type(c_ptr), value            :: ctx
            real(c_double), intent(in)    :: box(3)
            integer(c_int32_t), value     :: periodic
        end function
        ! per-particle constants (initialize_system, fortran/system.f90:586-682); c_null_ptr = default
        integer(c_int) function sg_set_particles(ctx, mass, sig_x, sig_y, sig_z, eps_x, eps_y, eps_z, &
                ixx, iyy, izz) bind(c, name="sg_set_particles")
            import :: c_ptr, c_int
            type(c_ptr), value            :: ctx, mass, sig_x, sig_y, sig_z, eps_x, eps_y, eps_z, ixx, iyy, izz
        end function
        ! set_atom_charge for every particle (fortran/system.f90:148-165)
        integer(c_int) function sg_set_charges(ctx, charge, reference_defaults) bind(c, name="sg_set_charges")
            import :: c_ptr, c_int, c_int32_t
            type(c_ptr), value            :: ctx, charge
            integer(c_int32_t), value     :: reference_defaults
        end function
        ! ---- state in / out ---------------------------------------------------
        integer(c_int) function sg_upload_state(ctx, rx, ry, rz, qw, qx, qy, qz, vx, vy, vz, lx, ly, lz) &
                bind(c, name="sg_upload_state")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), intent(in)    :: rx(*), ry(*), rz(*), qw(*), qx(*), qy(*), qz(*)
            real(c_double), intent(in)    :: vx(*), vy(*), vz(*), lx(*), ly(*), lz(*)
        end function
        integer(c_int) function sg_download_state(ctx, rx, ry, rz, qw, qx, qy, qz, vx, vy, vz, lx, ly, lz) &
                bind(c, name="sg_download_state")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), intent(out)   :: rx(*), ry(*), rz(*), qw(*), qx(*), qy(*), qz(*)
            real(c_double), intent(out)   :: vx(*), vy(*), vz(*), lx(*), ly(*), lz(*)
        end function
        integer(c_int) function sg_download_forces(ctx, fx, fy, fz, tx, ty, tz) bind(c, name="sg_download_forces")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), intent(out)   :: fx(*), fy(*), fz(*), tx(*), ty(*), tz(*)
        end function
        integer(c_int) function sg_upload_forces(ctx, fx, fy, fz, tx, ty, tz) bind(c, name="sg_upload_forces")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), intent(in)    :: fx(*), fy(*), fz(*), tx(*), ty(*), tz(*)
        end function
        ! initialize_forces (fortran/system.f90:423-436)
        integer(c_int) function sg_zero_forces(ctx) bind(c, name="sg_zero_forces")
            import :: c_ptr, c_int
            type(c_ptr), value            :: ctx
        end function
        ! ---- neighbour list (fortran/system.f90:885-1053) ---------------------
        integer(c_int) function sg_nlist_init(ctx, skin, cutoff, trigger_mode) bind(c, name="sg_nlist_init")
            import :: c_ptr, c_int, c_double, c_int32_t
            type(c_ptr), value            :: ctx
            real(c_double), value         :: skin, cutoff
            integer(c_int32_t), value     :: trigger_mode
        end function
        integer(c_int) function sg_nlist_needs_rebuild(ctx, flag) bind(c, name="sg_nlist_needs_rebuild")
            import :: c_ptr, c_int, c_int32_t
            type(c_ptr), value            :: ctx
            integer(c_int32_t), intent(out) :: flag
        end function
        integer(c_int) function sg_nlist_build(ctx) bind(c, name="sg_nlist_build")
            import :: c_ptr, c_int
            type(c_ptr), value            :: ctx
        end function
        integer(c_int) function sg_nlist_update(ctx) bind(c, name="sg_nlist_update")
            import :: c_ptr, c_int
            type(c_ptr), value            :: ctx
        end function
        integer(c_int) function sg_nlist_count(ctx, npairs) bind(c, name="sg_nlist_count")
            import :: c_ptr, c_int, c_int64_t
            type(c_ptr), value            :: ctx
            integer(c_int64_t), intent(out) :: npairs
        end function
        ! nlist / offset exactly as build_nlist leaves them when one_based = 1
        integer(c_int) function sg_nlist_export(ctx, nlist, capacity, offset, npairs, one_based) &
                bind(c, name="sg_nlist_export")
            import :: c_ptr, c_int, c_int32_t, c_int64_t
            type(c_ptr), value            :: ctx
            integer(c_int32_t), intent(out) :: nlist(*), offset(*)
            integer(c_int64_t), value     :: capacity
            integer(c_int64_t), intent(out) :: npairs
            integer(c_int32_t), value     :: one_based
        end function
        ! ---- pair forces: the user's loop over X_calculate_forces -------------
        integer(c_int) function sg_pair_forces(ctx, params, pot_eng, virial, stats) bind(c, name="sg_pair_forces")
            import :: c_ptr, c_int, c_double, sg_pair_params
            type(c_ptr), value            :: ctx
            type(sg_pair_params), intent(in) :: params
            real(c_double), intent(inout) :: pot_eng, virial
            type(c_ptr), value            :: stats
        end function
        integer(c_int) function sg_pair_forces_async(ctx, params) bind(c, name="sg_pair_forces_async")
            import :: c_ptr, c_int, sg_pair_params
            type(c_ptr), value            :: ctx
            type(sg_pair_params), intent(in) :: params
        end function
        integer(c_int) function sg_read_energies(ctx, out) bind(c, name="sg_read_energies")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), intent(out)   :: out(4)
        end function
        ! ---- integrators (fortran/integrators.f90) ----------------------------
        integer(c_int) function sg_vv_initial(ctx, dt) bind(c, name="sg_vv_initial")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), value         :: dt
        end function
        integer(c_int) function sg_vv_final(ctx, dt, kin_eng) bind(c, name="sg_vv_final")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), value         :: dt
            real(c_double), intent(out)   :: kin_eng
        end function
        integer(c_int) function sg_qq_initial(ctx, dt) bind(c, name="sg_qq_initial")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), value         :: dt
        end function
        integer(c_int) function sg_qq_final(ctx, dt, kin_rot) bind(c, name="sg_qq_final")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), value         :: dt
            real(c_double), intent(out)   :: kin_rot
        end function
        ! lgv_initial_step / lgv_final_step; key = c_null_ptr selects the reference key
        integer(c_int) function sg_lgv_initial(ctx, dt, step, damping, target_temp, key) &
                bind(c, name="sg_lgv_initial")
            import :: c_ptr, c_int, c_double, c_int32_t
            type(c_ptr), value            :: ctx
            real(c_double), value         :: dt
            integer(c_int32_t), value     :: step
            real(c_double), value         :: damping, target_temp
            type(c_ptr), value            :: key
        end function
        integer(c_int) function sg_lgv_final(ctx, dt, damping, kin_eng, kin_rot) bind(c, name="sg_lgv_final")
            import :: c_ptr, c_int, c_double
            type(c_ptr), value            :: ctx
            real(c_double), value         :: dt, damping
            real(c_double), intent(out)   :: kin_eng, kin_rot
        end function
        ! nht_initial_step / nht_final_step; mode 0 = the reference's per-particle chain
        integer(c_int) function sg_nht_initial(ctx, dt, target_temp, coupling, mode, rot_chain) &
                bind(c, name="sg_nht_initial")
            import :: c_ptr, c_int, c_double, c_int32_t
            type(c_ptr), value            :: ctx
            real(c_double), value         :: dt, target_temp, coupling
            integer(c_int32_t), value     :: mode, rot_chain
        end function
        integer(c_int) function sg_nht_final(ctx, dt, target_temp, coupling, mode, rot_chain, kin_eng) &
                bind(c, name="sg_nht_final")
            import :: c_ptr, c_int, c_double, c_int32_t
            type(c_ptr), value            :: ctx
            real(c_double), value         :: dt, target_temp, coupling
            integer(c_int32_t), value     :: mode, rot_chain
            real(c_double), intent(out)   :: kin_eng
        end function
        ! calculate_thermo (fortran/system.f90:725-741): out = temp, virial, pressure
        integer(c_int) function sg_thermo(ctx, dof, density, nrigid, out3) bind(c, name="sg_thermo")
            import :: c_ptr, c_int, c_double, c_int32_t
            type(c_ptr), value            :: ctx
            integer(c_int32_t), value     :: dof
            real(c_double), value         :: density
            integer(c_int32_t), value     :: nrigid
            real(c_double), intent(out)   :: out3(3)
        end function
        ! set_velocity_to_temperature (fortran/system.f90:361-421) on the device
        integer(c_int) function sg_set_velocity_to_temperature(ctx, rtemp, seed, remove_com, nrigid) &
                bind(c, name="sg_set_velocity_to_temperature")
            import :: c_ptr, c_int, c_double, c_int32_t
            type(c_ptr), value            :: ctx
            real(c_double), value         :: rtemp
            integer(c_int32_t), value     :: seed, remove_com, nrigid
        end function
        ! ---- whole timestep as a captured CUDA graph ---------------------------
        integer(c_int) function sg_step_configure(ctx, cfg) bind(c, name="sg_step_configure")
            import :: c_ptr, c_int, sg_step_config
            type(c_ptr), value            :: ctx
            type(sg_step_config), intent(in) :: cfg
        end function
        integer(c_int) function sg_step(ctx, nsteps) bind(c, name="sg_step")
            import :: c_ptr, c_int, c_int32_t
            type(c_ptr), value            :: ctx
            integer(c_int32_t), value     :: nsteps
        end function
        integer(c_int) function sg_step_check(ctx) bind(c, name="sg_step_check")
            import :: c_ptr, c_int
            type(c_ptr), value            :: ctx
        end function
        ! ---- Lennard-Jones forces on device-resident arrays, no allocation -----
        ! For OpenACC / CUDA Fortran programs that keep RX..RZ and FX..FZ on the
        ! device: pass c_loc of the device copies (e.g. inside !$acc host_data
        ! use_device), and one_based = 1 for Fortran's 1-based pair indices.
        integer(c_int) function sg_lj_forces_noalloc(n, rx, ry, rz, pair_i, pair_j, npairs, one_based, box, &
                periodic, params, fx, fy, fz, pot_virial, bad_pairs, stream, err, err_len) &
                bind(c, name="sg_lj_forces_noalloc")
            import :: c_ptr, c_int, c_int32_t, c_int64_t, c_double, c_char, sg_pair_params
            integer(c_int32_t), value     :: n
            type(c_ptr), value            :: rx, ry, rz, pair_i, pair_j
            integer(c_int64_t), value     :: npairs
            integer(c_int32_t), value     :: one_based
            real(c_double), intent(in)    :: box(3)
            integer(c_int32_t), value     :: periodic
            type(sg_pair_params), intent(in) :: params
            type(c_ptr), value            :: fx, fy, fz, pot_virial, bad_pairs, stream
            character(kind=c_char), intent(out) :: err(*)
            integer(c_int32_t), value     :: err_len
        end function
        ! ---- Philox4x32-10 (fortran/xmath.f90:42-76) ------------------------------
        subroutine sg_philox4x32(ctr, key, out) bind(c, name="sg_philox4x32")
            import :: c_int32_t
            integer(c_int32_t), intent(in)  :: ctr(4), key(2)
            integer(c_int32_t), intent(out) :: out(4)
        end subroutine
        ! ---- seeded isotropic ellipsoid placement ----------------------------------
        integer(c_int) function sg_place_isotropic(n, semi_axes, box, seed, gap, r_out, q_out, rep) &
                bind(c, name="sg_place_isotropic")
            import :: c_ptr, c_int, c_int64_t, c_double
            integer(c_int64_t), value     :: n
            real(c_double), intent(in)    :: semi_axes(3), box(3)
            integer(c_int64_t), value     :: seed
            real(c_double), value         :: gap
            real(c_double), intent(out)   :: r_out(*), q_out(*)
            type(c_ptr), value            :: rep
        end function
        ! strlen of the C library, for sg_error_message
        function c_strlen(s) bind(c, name="strlen")
            import :: c_ptr, c_size_t
            type(c_ptr), value            :: s
            integer(c_size_t)             :: c_strlen
        end function
    end interface

contains

    ! The context's last error message (sg_last_error) as a Fortran string.
    function sg_error_message(ctx) result(msg)
        type(c_ptr), intent(in) :: ctx
        character(len=:), allocatable :: msg
        type(c_ptr) :: p
        character(kind=c_char), pointer :: chars(:)
        integer :: k, n
        p = sg_last_error(ctx)
        if (.not. c_associated(p)) then
            msg = ""
            return
        end if
        n = int(c_strlen(p))
        call c_f_pointer(p, chars, [n])
        allocate(character(len=n) :: msg)
        do k = 1, n
            msg(k:k) = chars(k)
        end do
    end function sg_error_message

end module sucrose_gpu
