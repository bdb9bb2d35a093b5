"""ctypes declarations of the C ABI in include/sucrose_gpu.h.

Loads sucrose_gb300/lib/libsucrose_gb300.so (built in-tree by
sucrose_gb300/build.py). There is no fallback: if the library is missing or
fails to load, import raises.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libsucrose_gb300.so")

SG_OK, SG_EINVAL, SG_ECUTOFF_GT_HALFBOX, SG_ENOCONV, SG_ENAN, SG_ECAPACITY, SG_ECUDA, SG_ENOTREADY = range(8)
STATUS_NAMES = {0: "SG_OK", 1: "SG_EINVAL", 2: "SG_ECUTOFF_GT_HALFBOX", 3: "SG_ENOCONV", 4: "SG_ENAN",
                5: "SG_ECAPACITY", 6: "SG_ECUDA", 7: "SG_ENOTREADY"}

LJ, LJ12, LJW, WCA = 0, 1, 2, 3
MORSE, DH, COULOMB, DIPOLE = 4, 5, 6, 7
GB, GBR, GBW, GBC, GBWC = 10, 11, 12, 13, 14
ECP, ECPR, ECPW, ECPC, ECPWC = 20, 21, 22, 23, 24
SOLVER_BRENT_COMPAT, SOLVER_NEWTON, SOLVER_MLP_NEWTON, SOLVER_NEWTON_SUPPORT = 0, 1, 2, 3


class PairParams(C.Structure):
    _fields_ = [("kind", C.c_int32), ("mu", C.c_int32), ("nu", C.c_int32), ("solver", C.c_int32),
                ("sigma", C.c_double), ("epsilon", C.c_double), ("cutoff", C.c_double), ("wf", C.c_double),
                ("chirality", C.c_double), ("newton_tol", C.c_double), ("newton_max_iter", C.c_int32),
                ("fp64_check", C.c_int32), ("dissoc", C.c_double), ("width", C.c_double), ("rmin", C.c_double),
                ("db_len", C.c_double), ("dielectric", C.c_double)]


class StepConfig(C.Structure):
    _fields_ = [("integrator", C.c_int32), ("rotations", C.c_int32), ("rot_chain", C.c_int32),
                ("first_step", C.c_int32), ("dt", C.c_double), ("target_temp", C.c_double),
                ("damping", C.c_double), ("coupling", C.c_double), ("key", C.c_uint32 * 2),
                ("has_key", C.c_int32), ("flags", C.c_int32), ("pair", PairParams)]


INT_NVE, INT_LANGEVIN, INT_NH, INT_NH_REF = 0, 1, 2, 3
STEP_FLAT = 1
STEP_REACTION_FIELD = 2
STEP_CONSTRAINTS = 4
STEP_BONDED = 8
REPORT_STATE, REPORT_TRAJECTORY, REPORT_CONFIG, REPORT_CHECKPOINT = range(4)
BEND, DIH, COSINE_BEND, COSINE_DIH, ANGLE_BEND, ANGLE_DIH = range(6)


class TuneResult(C.Structure):
    _fields_ = [("block", C.c_int32), ("filter", C.c_int32), ("candidates", C.c_int32), ("reserved", C.c_int32),
                ("ms", C.c_float * 8)]


class PlaceReport(C.Structure):
    _fields_ = [("stages", C.c_int32), ("sweeps", C.c_int32), ("overlaps", C.c_int64),
                ("min_contact_ratio", C.c_double), ("final_scale", C.c_double)]


class EcpStats(C.Structure):
    _fields_ = [("pairs", C.c_int64), ("solver_evals", C.c_int64), ("nonconverged", C.c_int64),
                ("fallbacks", C.c_int64), ("iter_hist", C.c_int64 * 24), ("fp64_refined", C.c_int64)]


_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_U32 = C.POINTER(C.c_uint32)
_F = C.POINTER(C.c_float)
_P = C.c_void_p

# (name, restype, argtypes) for every entry point of include/sucrose_gpu.h
SIGNATURES = [
    ("sg_create", C.c_int, [C.POINTER(_P), C.c_int32, C.c_int32]),
    ("sg_destroy", C.c_int, [_P]),
    ("sg_last_error", C.c_char_p, [_P]),
    ("sg_stream", C.c_void_p, [_P]),
    ("sg_synchronize", C.c_int, [_P]),
    ("sg_set_box", C.c_int, [_P, _D, C.c_int32]),
    ("sg_set_particles", C.c_int, [_P] + [_D] * 10),
    ("sg_set_charges", C.c_int, [_P, _D, C.c_int32]),
    ("sg_reaction_field_init", C.c_int, [_P]),
    ("sg_reaction_field_eval", C.c_int, [_P, _D]),
    ("sg_reaction_field_read", C.c_int, [_P, _D, _D, _D, _D]),
    ("sg_upload_state", C.c_int, [_P] + [_D] * 13),
    ("sg_download_state", C.c_int, [_P] + [_D] * 13),
    ("sg_download_forces", C.c_int, [_P] + [_D] * 6),
    ("sg_upload_forces", C.c_int, [_P] + [_D] * 6),
    ("sg_zero_forces", C.c_int, [_P]),
    ("sg_nlist_init", C.c_int, [_P, C.c_double, C.c_double, C.c_int32]),
    ("sg_nlist_needs_rebuild", C.c_int, [_P, _I32]),
    ("sg_nlist_build", C.c_int, [_P]),
    ("sg_nlist_update", C.c_int, [_P]),
    ("sg_nlist_count", C.c_int, [_P, _I64]),
    ("sg_nlist_export", C.c_int, [_P, _I32, C.c_int64, _I32, _I64, C.c_int32]),
    ("sg_nlist_builds", C.c_int, [_P, _I64]),
    ("sg_nlist_replica_builds", C.c_int, [_P, _I64]),
    ("sg_nlist_pairs", C.c_int, [_P, _I32, _I32, C.c_int64, _I64]),
    ("sg_pair_forces", C.c_int, [_P, C.POINTER(PairParams), _D, _D, C.POINTER(EcpStats)]),
    ("sg_pair_forces_async", C.c_int, [_P, C.POINTER(PairParams)]),
    ("sg_read_energies", C.c_int, [_P, _D]),
    ("sg_ecp_lambda", C.c_int, [_P, _F, C.c_int64]),
    ("sg_vv_initial", C.c_int, [_P, C.c_double]),
    ("sg_vv_final", C.c_int, [_P, C.c_double, _D]),
    ("sg_qq_initial", C.c_int, [_P, C.c_double]),
    ("sg_qq_final", C.c_int, [_P, C.c_double, _D]),
    ("sg_lgv_initial", C.c_int, [_P, C.c_double, C.c_int32, C.c_double, C.c_double, _U32]),
    ("sg_lgv_final", C.c_int, [_P, C.c_double, C.c_double, _D, _D]),
    ("sg_nht_initial", C.c_int, [_P, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32]),
    ("sg_nht_final", C.c_int, [_P, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32, _D]),
    ("sg_nht_state", C.c_int, [_P, _D, _D]),
    ("sg_thermo", C.c_int, [_P, C.c_int32, C.c_double, C.c_int32, _D]),
    ("sg_set_types", C.c_int, [_P, _I32]),
    ("sg_reporter_open", C.c_int, [_P, C.c_int32, C.c_char_p, C.POINTER(_P)]),
    ("sg_reporter_set_thermo", C.c_int, [_P, C.c_int32, C.c_double, C.c_int32]),
    ("sg_reporter_write", C.c_int, [_P, C.c_int64]),
    ("sg_reporter_flush", C.c_int, [_P]),
    ("sg_reporter_close", C.c_int, [_P]),
    ("sg_load_checkpoint", C.c_int, [C.c_char_p, C.c_int32, C.POINTER(_P), _I64]),
    ("sg_save_state", C.c_int, [_P, C.c_char_p]),
    ("sg_load_state", C.c_int, [_P, C.c_char_p]),
    ("sg_mc_barostat", C.c_int, [_P, C.POINTER(PairParams), C.c_int32, C.c_int32, C.c_double, C.c_double,
                                 C.c_double, _U32, C.c_uint64, _I32, _D]),
    ("sg_bonded_set", C.c_int, [_P, C.c_int32, C.c_int32, _I32, _D, _D, C.c_int32]),
    ("sg_bonded_forces", C.c_int, [_P, C.c_int32, _D]),
    ("sg_bonded_forces_async", C.c_int, [_P, C.c_int32]),
    ("sg_set_constraints", C.c_int, [_P, C.c_int32, _I32, _I32, _D, C.c_int32]),
    ("sg_constraints_save", C.c_int, [_P]),
    ("sg_constraints_a", C.c_int, [_P, C.c_double]),
    ("sg_constraints_b", C.c_int, [_P, C.c_double]),
    ("sg_constraints_check", C.c_int, [_P]),
    ("sg_constraints_clear_error", C.c_int, [_P]),
    ("sg_constraint_stats", C.c_int, [_P, _I64, C.c_int32]),
    ("sg_vvc_initial", C.c_int, [_P, C.c_double]),
    ("sg_vvc_final", C.c_int, [_P, C.c_double, _D]),
    ("sg_nhtc_initial", C.c_int, [_P, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32]),
    ("sg_nhtc_final", C.c_int, [_P, C.c_double, C.c_double, C.c_double, C.c_int32, C.c_int32, _D]),
    ("sg_lgvc_initial", C.c_int, [_P, C.c_double, C.c_int32, C.c_double, C.c_double, _U32]),
    ("sg_lgvc_final", C.c_int, [_P, C.c_double, C.c_double, _D, _D]),
    ("sg_create_replicas", C.c_int, [C.POINTER(_P), C.c_int32, _I32, _D, _I32, _D, _U32, C.c_int32]),
    ("sg_rep_nlist_init", C.c_int, [_P, _D, _D, C.c_int32]),
    ("sg_rep_kinetic", C.c_int, [_P, _D]),
    ("sg_mlp_guess_tc", C.c_int, [_P, C.c_void_p, C.c_int64]),
    ("sg_mlp_set_inline", C.c_int, [_P, C.c_int32]),
    ("sg_mlp_test_wait_timeout", C.c_int, [_P]),
    ("sg_mlp_clear_error", C.c_int, [_P]),
    ("sg_pair_autotune", C.c_int, [_P, C.POINTER(PairParams), C.c_int32, C.POINTER(TuneResult)]),
    ("sg_pair_set_launch", C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    ("sg_step_configure", C.c_int, [_P, C.POINTER(StepConfig)]),
    ("sg_step_configure_pairs", C.c_int, [_P, C.POINTER(StepConfig), C.POINTER(PairParams), C.c_int32]),
    ("sg_step_stage_times", C.c_int, [_P, C.c_int32, _D]),
    ("sg_step", C.c_int, [_P, C.c_int32]),
    ("sg_step_check", C.c_int, [_P]),
    ("sg_step_kernel_count", C.c_int, [_P, _I64]),
    ("sg_peak_fma", C.c_int, [_P, C.c_int32, _D]),
    ("sg_lj_forces_noalloc", C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_int64, C.c_int32, _D, C.c_int32, C.POINTER(PairParams), C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p,
                                       C.c_int32]),
    ("sg_place_isotropic", C.c_int, [C.c_int64, _D, _D, C.c_uint64, C.c_double, _D, _D, C.POINTER(PlaceReport)]),
    ("sg_philox4x32", None, [_U32, _U32, _U32]),
    ("sg_philox4x32_device", C.c_int, [_P, C.c_int64, _U32, _U32, _U32]),
    ("sg_philox_normal_3seq_device", C.c_int, [_P, C.c_int64, _I32, _D]),
    ("sg_set_velocity_to_temperature", C.c_int, [_P, C.c_double, C.c_int32, C.c_int32, C.c_int32]),
    ("sg_mlp_set_weights", C.c_int, [_P, _F, C.c_int64]),
    ("sg_mlp_get_weights", C.c_int, [_P, _F, C.c_int64]),
    ("sg_mlp_weight_count", C.c_int64, []),
    ("sg_mlp_init", C.c_int, [_P, C.c_uint64]),
    ("sg_mlp_features", C.c_int, [_P, C.c_void_p, C.c_void_p, C.c_int64, _I64]),
    ("sg_mlp_train_step", C.c_int, [_P, C.c_void_p, C.c_void_p, C.c_int64, C.c_float, _F]),
    ("sg_mlp_grad", C.c_int, [_P, C.c_void_p, C.c_void_p, C.c_int64, _F, _F]),
    ("sg_mlp_predict", C.c_int, [_P, C.c_void_p, C.c_int64, C.c_void_p]),
    ("sg_mlp_guess", C.c_int, [_P, C.c_void_p, C.c_int64]),
]

_lib = None


def load():
    """Load the CUDA library; raises if it is absent (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libsucrose_gb300.so is not built: run __graft_entry__.build() "
                               "or python sucrose_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class SgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def check(ctx, code):
    if code != SG_OK:
        msg = load().sg_last_error(ctx).decode() if ctx else ""
        raise SgError(code, msg)
    return code
