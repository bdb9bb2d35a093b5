"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes front end of the CPU restatement in sucrose_oracle.cpp. Only tests,
the smoke check and the benchmark's CPU-baseline leg import this package, and
only as the checker (or as the timed CPU reference). The GPU product never
imports it.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

HERE = os.path.dirname(os.path.abspath(__file__))

# Pair kinds (shared numbering with the product's C-ABI)
LJ, LJ12, LJW, WCA = 0, 1, 2, 3
MORSE, DH, COULOMB, DIPOLE = 4, 5, 6, 7
BEND, DIH, COSINE_BEND, COSINE_DIH, ANGLE_BEND, ANGLE_DIH = range(6)
GB, GBR, GBW, GBC, GBWC = 10, 11, 12, 13, 14
ECP, ECPR, ECPW, ECPC, ECPWC = 20, 21, 22, 23, 24
SOLVER_BRENT, SOLVER_TIGHT, SOLVER_GIVEN = 0, 1, 2

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_U = C.POINTER(C.c_uint32)


class OrSys(C.Structure):
    _fields_ = [("n", C.c_int), ("periodic", C.c_int), ("nc", C.c_int), ("nrigid", C.c_int), ("dof", C.c_int),
                ("target_temp_set", C.c_int), ("box", C.c_double * 3)] + \
               [(k, _D) for k in ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz",
                                  "qw", "qx", "qy", "qz", "lx", "ly", "lz", "tx", "ty", "tz",
                                  "mass", "inv_mass", "sig_x", "sig_y", "sig_z", "eps_x", "eps_y", "eps_z",
                                  "ixx", "iyy", "izz", "ixx_inv", "iyy_inv", "izz_inv")] + \
               [(k, C.c_double) for k in ("pot_eng", "kin_eng", "kin_rot", "temp", "pressure", "density", "virial",
                                          "target_temp")] + \
               [("eta", C.c_double * 3), ("p_eta", C.c_double * 3), ("eta_r", C.c_double * 3),
                ("p_eta_r", C.c_double * 3)] + \
               [(k, _D) for k in ("charge", "dipx", "dipy", "dipz")] + [("rfl", C.c_double * 3)] + \
               [(k, _D) for k in ("rx_old", "ry_old", "rz_old")] + [("bbi", _I), ("bbj", _I), ("bb_len", _D),
                                                                    ("virial_bonded", C.c_double),
                                                                    ("rattle_sweeps", C.c_int)]


class OrPairParams(C.Structure):
    _fields_ = [("kind", C.c_int), ("mu", C.c_int), ("nu", C.c_int), ("solver", C.c_int),
                ("sigma", C.c_double), ("epsilon", C.c_double), ("cutoff", C.c_double), ("wf", C.c_double),
                ("chirality", C.c_double), ("lam_in", C.c_double), ("dissoc", C.c_double), ("width", C.c_double),
                ("rmin", C.c_double), ("db_len", C.c_double), ("dielectric", C.c_double)]


_libs = {}


def lib(fast=False):
    key = "fast" if fast else "strict"
    if key not in _libs:
        build_oracle.build()
        path = os.path.join(HERE, "_build", "liboracle_fast.so" if fast else "liboracle.so")
        L = C.CDLL(path)
        P = C.POINTER(OrSys)
        L.or_philox4x32.argtypes = [_U, _U, _U]
        L.or_philox4x32_batch.argtypes = [C.c_int, _U, _U, _U]
        L.or_philox_normal_3seq.argtypes = [C.c_int32] * 4 + [_D]
        L.or_pair.argtypes = [P, C.c_int, C.c_int, C.POINTER(OrPairParams), C.c_int, _D, _I]
        L.or_forces.argtypes = [P, C.POINTER(OrPairParams), C.c_int, _I, _I, C.c_int, _D, _I, _D]
        L.or_pair_batch.argtypes = [P, C.POINTER(OrPairParams), C.c_longlong, _I, _I, _D, C.c_int]
        L.or_nlist_build.argtypes = [P, C.c_double, C.c_double, _I, C.c_longlong, _I, C.c_int]
        L.or_nlist_build.restype = C.c_longlong
        L.or_needs_rebuild.argtypes = [P, _D, _D, _D, C.c_double, C.c_double, C.c_int]
        for f in ("or_vv_initial", "or_vv_final", "or_qq_initial", "or_qq_final", "or_lgv_final"):
            getattr(L, f).argtypes = [P, C.c_double]
        L.or_lgv_initial.argtypes = [P, C.c_double, C.c_int, C.c_double, _U]
        L.or_nht_initial.argtypes = [P, C.c_double, C.c_double, C.c_int, C.c_int]
        L.or_nht_final.argtypes = [P, C.c_double, C.c_double, C.c_int, C.c_int]
        L.or_nhr_half.argtypes = [P, C.c_double, C.c_double, C.c_int]
        L.or_calculate_thermo.argtypes = [P]
        L.or_reaction_field_init.argtypes = [P]
        L.or_constraints_a.argtypes = [P, C.c_double]
        L.or_constraints_a.restype = C.c_int
        L.or_constraints_b.argtypes = [P, C.c_double]
        L.or_constraints_save.argtypes = [P]
        L.or_bonded.argtypes = [P, C.c_int, _I, C.c_double, C.c_double, _D]
        L.or_mc_barostat.argtypes = [P, C.POINTER(OrPairParams), C.c_int, C.c_int, _I, _I, C.c_double, C.c_double,
                                     C.c_double, _U, C.c_ulonglong, _D]
        L.or_mc_barostat.restype = C.c_int
        L.or_bonded_forces.argtypes = [P, C.c_int, C.c_int, _I, _D, _D]
        L.or_reaction_field_eval.argtypes = [P]
        L.or_set_velocity_to_temperature.argtypes = [P, C.c_double, C.c_int, C.c_int]
        L.or_generate_fcc.argtypes = [C.c_int, C.c_double] + [_D] * 7
        _libs[key] = L
    return _libs[key]


def ref_lib():
    """The reference's own C++ port compiled in place (None when absent)."""
    if "ref" not in _libs:
        build_oracle.build()
        path = os.path.join(HERE, "_ref", "libsucrose_ref.so")
        if not os.path.exists(path):
            _libs["ref"] = None
        else:
            L = C.CDLL(path)
            L.ref_lj_forces.argtypes = [C.c_int, C.c_double, C.c_int, _D, _D, _D, C.c_double, C.c_double, C.c_int,
                                        _I, _I, _D, _D, _D, _D]
            L.ref_morse_forces.argtypes = [C.c_int, C.c_double, C.c_int, _D, _D, _D, C.c_double, C.c_double,
                                           C.c_double, C.c_int, _I, _I, _D, _D, _D, _D]
            L.ref_vv_step.argtypes = [C.c_int, C.c_double, C.c_int, C.c_double] + [_D] * 9 + [C.c_int]
            L.ref_det3.argtypes = [_D]
            L.ref_det3.restype = C.c_double
            _libs["ref"] = L
    return _libs["ref"]


def dptr(a):
    return a.ctypes.data_as(_D)


def iptr(a):
    return a.ctypes.data_as(_I)


def uptr(a):
    return a.ctypes.data_as(_U)


PARTICLE_FIELDS = ("rx", "ry", "rz", "vx", "vy", "vz", "fx", "fy", "fz", "qw", "qx", "qy", "qz",
                   "lx", "ly", "lz", "tx", "ty", "tz", "mass", "inv_mass", "sig_x", "sig_y", "sig_z",
                   "eps_x", "eps_y", "eps_z", "ixx", "iyy", "izz", "ixx_inv", "iyy_inv", "izz_inv",
                   "charge", "dipx", "dipy", "dipz", "rx_old", "ry_old", "rz_old")


class System:
    """FP64 SoA state mirroring the reference's module globals (system.f90:7-30)."""

    def __init__(self, n, box, periodic=True, fast=False):
        self.n = int(n)
        self.L = lib(fast)
        for f in PARTICLE_FIELDS:
            setattr(self, f, np.zeros(self.n, dtype=np.float64))
        self.qw[:] = 1.0
        self.s = OrSys()
        self.s.n = self.n
        self.s.periodic = 1 if periodic else 0
        self.s.nc = 0
        self.s.nrigid = 1
        self.s.dof = 6 * self.n - 3
        b = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
        for d in range(3):
            self.s.box[d] = float(b[d])
        for f in PARTICLE_FIELDS:
            setattr(self.s, f, dptr(getattr(self, f)))
        self.set_defaults()

    @property
    def box(self):
        return np.array([self.s.box[0], self.s.box[1], self.s.box[2]])

    def set_defaults(self, mass=1.0, sig=(1.0, 1.0, 1.0), eps=(1.0, 1.0, 1.0)):
        """initialize_system defaults (system.f90:586-682): unit mass, inertia (s_y^2+s_z^2)/20 ..."""
        self.mass[:] = mass
        self.inv_mass[:] = 1.0 / mass
        self.sig_x[:], self.sig_y[:], self.sig_z[:] = sig
        self.eps_x[:], self.eps_y[:], self.eps_z[:] = eps
        self.ixx[:] = (self.sig_y ** 2.0 + self.sig_z ** 2.0) / 20.0
        self.iyy[:] = (self.sig_x ** 2.0 + self.sig_z ** 2.0) / 20.0
        self.izz[:] = (self.sig_x ** 2.0 + self.sig_y ** 2.0) / 20.0
        self.ixx_inv[:] = 1.0 / self.ixx
        self.iyy_inv[:] = 1.0 / self.iyy
        self.izz_inv[:] = 1.0 / self.izz

    def ptr(self):
        return C.byref(self.s)

    def zero_forces(self):
        """initialize_forces (system.f90:423-436)."""
        for f in ("fx", "fy", "fz", "tx", "ty", "tz"):
            getattr(self, f)[:] = 0.0
        self.s.pot_eng = 0.0
        self.s.virial_bonded = 0.0

    # --- pair potentials -------------------------------------------------
    def pair(self, i, j, params, prec=64):
        out = np.zeros(11)
        nev = C.c_int(0)
        self.L.or_pair(self.ptr(), int(i), int(j), C.byref(params), prec, dptr(out), C.byref(nev))
        return out, nev.value

    def forces(self, params, pi, pj, prec=64, lam_in=None, want_lambda=False):
        pi = np.ascontiguousarray(pi, dtype=np.int32)
        pj = np.ascontiguousarray(pj, dtype=np.int32)
        lam = np.zeros(len(pi)) if want_lambda else None
        nev = np.zeros(len(pi), dtype=np.int32) if want_lambda else None
        lin = np.ascontiguousarray(lam_in, dtype=np.float64) if lam_in is not None else None
        self.L.or_forces(self.ptr(), C.byref(params), len(pi), iptr(pi), iptr(pj), prec,
                         dptr(lam) if lam is not None else None, iptr(nev) if nev is not None else None,
                         dptr(lin) if lin is not None else None)
        return (lam, nev) if want_lambda else None

    def pair_batch(self, params, pi, pj, nthreads=1):
        """Per-pair (pe, f3, ti3, tj3, lambda) for every listed pair, in parallel."""
        pi = np.ascontiguousarray(pi, dtype=np.int32)
        pj = np.ascontiguousarray(pj, dtype=np.int32)
        out = np.zeros((len(pi), 11))
        self.L.or_pair_batch(self.ptr(), C.byref(params), len(pi), iptr(pi), iptr(pj), dptr(out), int(nthreads))
        return out

    # --- neighbour list --------------------------------------------------
    def nlist(self, cutoff, skin, one_based=False, cap=None):
        cap = cap or max(1, 50 * self.n)
        while True:
            nl = np.zeros(cap, dtype=np.int32)
            off = np.zeros(self.n + 1, dtype=np.int32)
            k = self.L.or_nlist_build(self.ptr(), cutoff, skin, iptr(nl), cap, iptr(off), 1 if one_based else 0)
            if k == -1:
                raise ValueError("cutoff larger than half the box")
            if k < -1:
                cap = int(-k - 2)
                continue
            return nl[:k], (off[: self.n] if one_based else off)

    def pairs(self, cutoff, skin):
        """The reference half list as (i, j) arrays, 0-based, i < j, row-major."""
        nl, off = self.nlist(cutoff, skin)
        counts = np.diff(off)
        pi = np.repeat(np.arange(self.n, dtype=np.int32), counts)
        return pi, nl

    def needs_rebuild(self, xl, yl, zl, cutoff, skin, trigger_mode=0):
        return bool(self.L.or_needs_rebuild(self.ptr(), dptr(xl), dptr(yl), dptr(zl), cutoff, skin, trigger_mode))

    # --- integrators -------------------------------------------------------
    def vv_initial(self, dt): self.L.or_vv_initial(self.ptr(), dt)
    def vv_final(self, dt): self.L.or_vv_final(self.ptr(), dt)
    def qq_initial(self, dt): self.L.or_qq_initial(self.ptr(), dt)
    def qq_final(self, dt): self.L.or_qq_final(self.ptr(), dt)

    def lgv_initial(self, dt, step, damping=1.0, key=None):
        k = np.asarray(key, dtype=np.uint32) if key is not None else None
        self.L.or_lgv_initial(self.ptr(), dt, step, damping, uptr(k) if k is not None else None)

    def lgv_final(self, dt): self.L.or_lgv_final(self.ptr(), dt)

    def nht_initial(self, dt, coupling=None, mode=0):
        self.L.or_nht_initial(self.ptr(), dt, 0.0 if coupling is None else coupling, 0 if coupling is None else 1, mode)

    def nht_final(self, dt, coupling=None, mode=0):
        self.L.or_nht_final(self.ptr(), dt, 0.0 if coupling is None else coupling, 0 if coupling is None else 1, mode)

    def nhr_half(self, dt, coupling=None):
        self.L.or_nhr_half(self.ptr(), dt, 0.0 if coupling is None else coupling, 0 if coupling is None else 1)

    # --- bond constraints (module constraints, system.f90:1055-1210) ----------
    def set_constraints(self, bbi, bbj, length):
        """set_num_constraints + add_constraint, 0-based atom indices."""
        self.bbi = np.ascontiguousarray(bbi, dtype=np.int32)
        self.bbj = np.ascontiguousarray(bbj, dtype=np.int32)
        self.bb_len = np.ascontiguousarray(np.broadcast_to(np.asarray(length, dtype=np.float64), self.bbi.shape))
        self.s.nc = len(self.bbi)
        self.s.bbi = iptr(self.bbi)
        self.s.bbj = iptr(self.bbj)
        self.s.bb_len = dptr(self.bb_len)

    def constraints_save(self):
        self.L.or_constraints_save(self.ptr())

    def constraints_a(self, dt):
        """0, or 1 + the index of the failing constraint."""
        return self.L.or_constraints_a(self.ptr(), dt)

    def constraints_b(self, dt):
        self.L.or_constraints_b(self.ptr(), dt)

    # --- Monte Carlo barostat (integrators.f90:858-945) ---------------------
    def mc_barostat(self, sets, pi, pj, target_pressure, temperature, max_dv=0.01, key=None, counter=0):
        """One trial move; returns (accept, U_old, U_new, V_new)."""
        arr = (OrPairParams * len(sets))(*sets)
        pi = np.ascontiguousarray(pi, dtype=np.int32)
        pj = np.ascontiguousarray(pj, dtype=np.int32)
        k = None if key is None else np.ascontiguousarray(key, dtype=np.uint32)
        u = np.zeros(3)
        a = self.L.or_mc_barostat(self.ptr(), arr, len(sets), len(pi), iptr(pi), iptr(pj), float(target_pressure),
                                  float(temperature), float(max_dv), None if k is None else uptr(k), int(counter),
                                  dptr(u))
        return a, u[0], u[1], u[2]

    # --- bonded terms (module bonded, force.f90:2238-2581) -------------------
    def bonded(self, kind, atoms, coeff, angle=0.0):
        """One term: (PE, F on each of its 3 or 4 atoms as an (4, 3) array)."""
        at = np.ascontiguousarray(atoms, dtype=np.int32)
        out = np.zeros(13)
        self.L.or_bonded(self.ptr(), int(kind), iptr(at), float(coeff), float(angle), dptr(out))
        return out[0], out[1:].reshape(4, 3)

    def bonded_forces(self, kind, atoms, coeff, angle=None):
        """The user's loop over a term list, accumulating into F and pot_eng."""
        at = np.ascontiguousarray(atoms, dtype=np.int32)
        nt = len(at)
        c = np.ascontiguousarray(np.broadcast_to(np.asarray(coeff, dtype=np.float64), (nt,)))
        a = None if angle is None else np.ascontiguousarray(np.broadcast_to(np.asarray(angle, dtype=np.float64),
                                                                             (nt,)))
        self.L.or_bonded_forces(self.ptr(), int(kind), nt, iptr(at), dptr(c), None if a is None else dptr(a))

    def reaction_field_init(self):
        self.L.or_reaction_field_init(self.ptr())

    def reaction_field_eval(self):
        self.L.or_reaction_field_eval(self.ptr())

    @property
    def rfl(self):
        return np.array([self.s.rfl[0], self.s.rfl[1], self.s.rfl[2]])

    def thermo(self):
        self.L.or_calculate_thermo(self.ptr())

    def set_velocity_to_temperature(self, T, seed, remove_com=True):
        self.L.or_set_velocity_to_temperature(self.ptr(), T, seed, 1 if remove_com else 0)


def pair_params(kind, sigma=1.0, epsilon=1.0, cutoff=2.5, wf=0.0, chirality=0.0, mu=None, nu=None,
                solver=SOLVER_BRENT, lam_in=0.0, dissoc=1.0, width=1.0, rmin=1.0, db_len=1.0, dielectric=1.0):
    if mu is None:
        mu, nu = (1, 2) if 10 <= kind < 20 else (2, 1)
    return OrPairParams(kind, mu, nu, solver, sigma, epsilon, cutoff, wf, chirality, lam_in, dissoc, width, rmin,
                        db_len, dielectric)


def philox4x32(ctr, key=(0x6D2B79F5, 0x1B873593)):
    c = np.ascontiguousarray(ctr, dtype=np.uint32).reshape(-1, 4)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros_like(c)
    lib().or_philox4x32_batch(len(c), uptr(c), uptr(k), uptr(out))
    return out


def philox_normal_3seq(c1, c2, c3, c4):
    out = np.zeros(3)
    lib().or_philox_normal_3seq(c1, c2, c3, c4, dptr(out))
    return out


def fcc_lattice(cells, density):
    """generate_fcc_lattice(cells, density): positions, quaternions and box (system.f90:438-523)."""
    n = 4 * cells ** 3
    box_len = (float(n) / density) ** (1.0 / 3.0)
    arrs = [np.zeros(n) for _ in range(7)]
    lib().or_generate_fcc(cells, box_len, *[dptr(a) for a in arrs])
    return arrs, box_len
