"""Host-side mirror of the reference's system / neighbour_list / force /
integrator modules (fortran/system.f90, fortran/force.f90,
fortran/integrators.f90), backed by the CUDA library through its C ABI.

A GpuSystem owns one device context. Arrays handed in and out are FP64
structure-of-arrays in the reference's layout (RX..RZ, QW..QZ, VX..VZ,
LX..LZ, FX..FZ, TX..TZ), 0-based; the device state is FP32. Errors come back
as SgError carrying the C status (the reference stops the program instead).
"""
import ctypes as C

import numpy as np

from . import capi
from .capi import PairParams, EcpStats, check

_D = C.POINTER(C.c_double)


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _f64(a, n):
    if a is None:
        return None
    a = np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (n,)))
    return a


class GpuSystem:
    def __init__(self, n, box, periodic=True, device=0):
        self.L = capi.load()
        self.n = int(n)
        ctx = C.c_void_p()
        rc = self.L.sg_create(C.byref(ctx), self.n, int(device))
        self.ctx = ctx
        check(ctx, rc)
        self.set_box(box, periodic)

    @classmethod
    def replicas(cls, n_per_rep, boxes, family, temps=None, keys=None, device=0):
        """A batched context of independent periodic replicas (sg_create_replicas):
        replica r has n_per_rep[r] particles in box boxes[r] (3 lengths) and
        potential family family[r] (0 LJ, 1 GB, 2 ECP; non-decreasing)."""
        self = cls.__new__(cls)
        self.L = capi.load()
        npr = np.ascontiguousarray(n_per_rep, dtype=np.int32)
        bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(-1, 3))
        fam = np.ascontiguousarray(family, dtype=np.int32)
        R = len(npr)
        T = None if temps is None else np.ascontiguousarray(temps, dtype=np.float64)
        K = None if keys is None else np.ascontiguousarray(np.asarray(keys, dtype=np.uint32).reshape(R, 2))
        self.n = int(npr.sum())
        self.nrep = R
        self.rep_off = np.concatenate([[0], np.cumsum(npr)]).astype(np.int64)
        self.rep_box = bx.copy()
        self.box = bx.max(axis=0)
        self.periodic = True
        ctx = C.c_void_p()
        P32 = C.POINTER(C.c_int32)
        rc = self.L.sg_create_replicas(C.byref(ctx), R, npr.ctypes.data_as(P32), _dp(bx), fam.ctypes.data_as(P32),
                                       _dp(T), None if K is None else K.ctypes.data_as(C.POINTER(C.c_uint32)),
                                       int(device))
        self.ctx = ctx
        check(ctx, rc)
        return self

    def init_rep_nlist(self, skin, cutoff, trigger_mode=0):
        """Lists of every replica; skin and cutoff are 3-vectors indexed by family."""
        s = np.ascontiguousarray(np.broadcast_to(np.asarray(skin, dtype=np.float64), (3,)))
        c = np.ascontiguousarray(np.broadcast_to(np.asarray(cutoff, dtype=np.float64), (3,)))
        self._c(self.L.sg_rep_nlist_init(self.ctx, _dp(s), _dp(c), int(trigger_mode)))

    def rep_nlist_builds(self):
        """Rebuilds of each replica's list since init_rep_nlist, shape (nrep,)."""
        out = np.zeros(self.nrep, dtype=np.int64)
        self._c(self.L.sg_nlist_replica_builds(self.ctx, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def rep_kinetic(self):
        """Per-replica (KE, KE_rot), FP64, shape (nrep, 2)."""
        out = np.zeros((self.nrep, 2))
        self._c(self.L.sg_rep_kinetic(self.ctx, _dp(out)))
        return out

    def close(self):
        if getattr(self, "ctx", None):
            self.L.sg_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, rc):
        return check(self.ctx, rc)

    # ---- configuration ----------------------------------------------------
    def set_box(self, box, periodic=True):
        b = np.ascontiguousarray(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
        self.box = b.copy()
        self.periodic = bool(periodic)
        self._c(self.L.sg_set_box(self.ctx, _dp(b), 1 if periodic else 0))

    def set_particles(self, mass=None, sig=None, eps=None, inertia=None):
        """Per-particle constants; each of sig, eps, inertia is None, a 3-tuple
        applied to every particle, or an (n, 3) array."""
        n = self.n

        def cols(a):
            if a is None:
                return [None] * 3
            a = np.asarray(a, dtype=np.float64)
            if a.ndim == 1:
                return [_f64(a[k], n) for k in range(3)]
            return [np.ascontiguousarray(a[:, k]) for k in range(3)]

        m = _f64(mass, n)
        s, e, I = cols(sig), cols(eps), cols(inertia)
        self._keep = (m, s, e, I)
        self._c(self.L.sg_set_particles(self.ctx, _dp(m), *[_dp(a) for a in s], *[_dp(a) for a in e],
                                        *[_dp(a) for a in I]))

    def set_charges(self, charge, reference_defaults=False):
        """Per-particle charges (set_atom_charge); reference_defaults applies
        initialize_system's rule that a negative charge becomes 0."""
        q = _f64(charge, self.n) if charge is not None else None
        self._keep_q = q
        self._c(self.L.sg_set_charges(self.ctx, _dp(q), 1 if reference_defaults else 0))

    def reaction_field_init(self):
        self._c(self.L.sg_reaction_field_init(self.ctx))

    def reaction_field_eval(self):
        """eval_reaction_field: returns the energy it added."""
        e = C.c_double(0.0)
        self._c(self.L.sg_reaction_field_eval(self.ctx, C.byref(e)))
        return e.value

    def reaction_field(self):
        """(RFL (3,), DIP (n, 3))."""
        rfl = np.zeros(3)
        d = [np.zeros(self.n) for _ in range(3)]
        self._c(self.L.sg_reaction_field_read(self.ctx, _dp(rfl), *[_dp(a) for a in d]))
        return rfl, np.stack(d, 1)

    # ---- state transfer -------------------------------------------------------
    def upload(self, r=None, q=None, v=None, l=None):
        """r, v, l: (n,3) FP64; q: (n,4) (w,x,y,z)."""
        cols = []
        for a, k in ((r, 3), (q, 4), (v, 3), (l, 3)):
            if a is None:
                cols += [None] * k
            else:
                a = np.asarray(a, dtype=np.float64)
                cols += [np.ascontiguousarray(a[:, d]) for d in range(k)]
        self._c(self.L.sg_upload_state(self.ctx, *[_dp(c) for c in cols]))

    def download(self):
        n = self.n
        arrs = [np.empty(n) for _ in range(13)]
        self._c(self.L.sg_download_state(self.ctx, *[_dp(a) for a in arrs]))
        r = np.stack(arrs[0:3], 1)
        q = np.stack(arrs[3:7], 1)
        v = np.stack(arrs[7:10], 1)
        l = np.stack(arrs[10:13], 1)
        return r, q, v, l

    def forces(self):
        n = self.n
        arrs = [np.empty(n) for _ in range(6)]
        self._c(self.L.sg_download_forces(self.ctx, *[_dp(a) for a in arrs]))
        return np.stack(arrs[0:3], 1), np.stack(arrs[3:6], 1)

    def set_forces(self, f, t=None):
        f = np.asarray(f, dtype=np.float64)
        cols = [np.ascontiguousarray(f[:, d]) for d in range(3)]
        tc = [None] * 3 if t is None else [np.ascontiguousarray(np.asarray(t, dtype=np.float64)[:, d]) for d in range(3)]
        self._c(self.L.sg_upload_forces(self.ctx, *[_dp(c) for c in cols], *[_dp(c) for c in tc]))

    def zero_forces(self):
        """initialize_forces (system.f90:423)."""
        self._c(self.L.sg_zero_forces(self.ctx))

    # ---- neighbour list -----------------------------------------------------
    def init_nlist(self, skin, cutoff, trigger_mode=0):
        self._c(self.L.sg_nlist_init(self.ctx, float(skin), float(cutoff), int(trigger_mode)))

    def needs_rebuild(self):
        f = C.c_int32(0)
        self._c(self.L.sg_nlist_needs_rebuild(self.ctx, C.byref(f)))
        return bool(f.value)

    def build_nlist(self):
        self._c(self.L.sg_nlist_build(self.ctx))

    def update_nlist(self):
        self._c(self.L.sg_nlist_update(self.ctx))

    def npairs(self):
        k = C.c_int64(0)
        self._c(self.L.sg_nlist_count(self.ctx, C.byref(k)))
        return k.value

    def nlist_builds(self):
        k = C.c_int64(0)
        self._c(self.L.sg_nlist_builds(self.ctx, C.byref(k)))
        return k.value

    def export_nlist(self, one_based=False):
        k = self.npairs()
        nl = np.zeros(max(k, 1), dtype=np.int32)
        off = np.zeros(self.n + 1, dtype=np.int32)
        kk = C.c_int64(0)
        self._c(self.L.sg_nlist_export(self.ctx, nl.ctypes.data_as(C.POINTER(C.c_int32)), len(nl),
                                       off.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(kk), 1 if one_based else 0))
        return nl[:k], (off[: self.n] if one_based else off)

    def raw_pairs(self):
        """Listed pairs in the device's internal order (the order of per-pair outputs)."""
        k = self.npairs()
        pi = np.zeros(max(k, 1), dtype=np.int32)
        pj = np.zeros(max(k, 1), dtype=np.int32)
        kk = C.c_int64(0)
        P = C.POINTER(C.c_int32)
        self._c(self.L.sg_nlist_pairs(self.ctx, pi.ctypes.data_as(P), pj.ctypes.data_as(P), len(pi), C.byref(kk)))
        return pi[:k], pj[:k]

    def pairs(self):
        """Listed pairs as (i, j) arrays, 0-based, i < j, rows ascending."""
        nl, off = self.export_nlist()
        counts = np.diff(off)
        return np.repeat(np.arange(self.n, dtype=np.int32), counts), nl

    # ---- pair forces ------------------------------------------------------------
    @staticmethod
    def params(kind, sigma=1.0, epsilon=1.0, cutoff=2.5, wf=0.0, chirality=0.0, mu=0, nu=0,
               solver=capi.SOLVER_NEWTON, newton_tol=1e-6, newton_max_iter=20, fp64_check=1, dissoc=1.0, width=1.0,
               rmin=1.0, db_len=1.0, dielectric=1.0):
        return PairParams(kind, mu, nu, solver, sigma, epsilon, cutoff, wf, chirality, newton_tol, newton_max_iter,
                          fp64_check, dissoc, width, rmin, db_len, dielectric)

    def pair_forces(self, params, want_stats=False, allow=()):
        pe = C.c_double(0.0)
        vir = C.c_double(0.0)
        st = EcpStats()
        rc = self.L.sg_pair_forces(self.ctx, C.byref(params), C.byref(pe), C.byref(vir), C.byref(st))
        if rc not in allow:
            self._c(rc)
        if want_stats:
            return pe.value, vir.value, st
        return pe.value, vir.value

    def autotune(self, params, reps=5):
        """Time the pair kernel's launch variants on the current list and keep
        the fastest (sg_pair_autotune). Returns the capi.TuneResult."""
        res = capi.TuneResult()
        self._c(self.L.sg_pair_autotune(self.ctx, C.byref(params), int(reps), C.byref(res)))
        return res

    def set_launch(self, kind, block=256, filter=0):
        self._c(self.L.sg_pair_set_launch(self.ctx, int(kind), int(block), int(filter)))

    def pair_forces_async(self, params):
        self._c(self.L.sg_pair_forces_async(self.ctx, C.byref(params)))

    def energies(self):
        out = np.zeros(4)
        self._c(self.L.sg_read_energies(self.ctx, _dp(out)))
        return out

    def ecp_lambda(self):
        k = self.npairs()
        lam = np.zeros(max(k, 1), dtype=np.float32)
        self._c(self.L.sg_ecp_lambda(self.ctx, lam.ctypes.data_as(C.POINTER(C.c_float)), len(lam)))
        return lam[:k]

    # ---- integrators --------------------------------------------------------------
    def vv_initial(self, dt):
        self._c(self.L.sg_vv_initial(self.ctx, dt))

    def vv_final(self, dt):
        ke = C.c_double(0.0)
        self._c(self.L.sg_vv_final(self.ctx, dt, C.byref(ke)))
        return ke.value

    def qq_initial(self, dt):
        self._c(self.L.sg_qq_initial(self.ctx, dt))

    def qq_final(self, dt):
        kr = C.c_double(0.0)
        self._c(self.L.sg_qq_final(self.ctx, dt, C.byref(kr)))
        return kr.value

    def lgv_initial(self, dt, step, damping=1.0, target_temp=1.0, key=None):
        k = None if key is None else np.asarray(key, dtype=np.uint32)
        self._c(self.L.sg_lgv_initial(self.ctx, dt, int(step), damping, target_temp,
                                      None if k is None else k.ctypes.data_as(C.POINTER(C.c_uint32))))

    def lgv_final(self, dt, damping=1.0):
        ke = C.c_double(0.0)
        kr = C.c_double(0.0)
        self._c(self.L.sg_lgv_final(self.ctx, dt, damping, C.byref(ke), C.byref(kr)))
        return ke.value, kr.value

    def nht_initial(self, dt, target_temp, coupling=0.0, mode=1, rot_chain=0):
        self._c(self.L.sg_nht_initial(self.ctx, dt, target_temp, coupling, mode, rot_chain))

    def nht_final(self, dt, target_temp, coupling=0.0, mode=1, rot_chain=0):
        ke = C.c_double(0.0)
        self._c(self.L.sg_nht_final(self.ctx, dt, target_temp, coupling, mode, rot_chain, C.byref(ke)))
        return ke.value

    def nht_state(self, set_values=None):
        out = np.zeros(12)
        s = None if set_values is None else np.ascontiguousarray(set_values, dtype=np.float64)
        self._c(self.L.sg_nht_state(self.ctx, _dp(out), _dp(s)))
        return out

    # ---- reporters ---------------------------------------------------------------------
    def set_types(self, types):
        t = None if types is None else np.ascontiguousarray(np.broadcast_to(np.asarray(types, dtype=np.int32),
                                                                             (self.n,)))
        self._c(self.L.sg_set_types(self.ctx, None if t is None else t.ctypes.data_as(C.POINTER(C.c_int32))))

    def reporter(self, kind, path, dof=None, density=None, nrigid=1):
        """An asynchronous reporter (use as a context manager or close())."""
        return Reporter(self, kind, path, dof, density, nrigid)

    def save_state(self, path):
        self._c(self.L.sg_save_state(self.ctx, str(path).encode()))

    def load_state(self, path):
        self._c(self.L.sg_load_state(self.ctx, str(path).encode()))

    @classmethod
    def load_checkpoint(cls, path, device=0):
        """load_checkpoint: a new system from a checkpoint text file; returns
        (system, config_index)."""
        self = cls.__new__(cls)
        self.L = capi.load()
        ctx = C.c_void_p()
        cfg = C.c_int64(0)
        rc = self.L.sg_load_checkpoint(str(path).encode(), int(device), C.byref(ctx), C.byref(cfg))
        self.ctx = ctx
        if rc != 0 and not ctx.value:
            raise capi.SgError(rc, f"cannot read checkpoint {path}")
        check(ctx, rc)
        with open(path) as f:
            f.readline(); f.readline(); f.readline(); f.readline()
            b = f.readline().split()[1:4]
        self.n = int(open(path).readline().split()[1])
        self.box = np.array([float(x) for x in b])
        self.periodic = True
        return self, cfg.value

    # ---- Monte Carlo barostat -----------------------------------------------------------
    def mc_barostat(self, pairs, target_pressure, temperature, max_dv=0.01, key=None, counter=0,
                    include_bonded=False):
        """One trial volume move; returns (accept: 1 / 0 / -1, volume)."""
        arr = (PairParams * len(pairs))(*pairs)
        k = None if key is None else np.asarray(key, dtype=np.uint32)
        acc = C.c_int32(0)
        vol = C.c_double(0.0)
        self._c(self.L.sg_mc_barostat(self.ctx, arr, len(pairs), 1 if include_bonded else 0, float(target_pressure),
                                      float(temperature), float(max_dv),
                                      None if k is None else k.ctypes.data_as(C.POINTER(C.c_uint32)),
                                      int(counter), C.byref(acc), C.byref(vol)))
        b = self.box
        if acc.value == 1:
            s = (vol.value / float(np.prod(b))) ** (1.0 / 3.0)
            self.box = b * s
        return acc.value, vol.value

    # ---- bonded terms -----------------------------------------------------------------
    def bonded_set(self, kind, atoms, coeff, angle=None, one_based=False):
        """Register the term list of one bonded kind: atoms (nterms, 3|4)."""
        at = np.ascontiguousarray(atoms, dtype=np.int32)
        nt = len(at)
        c = np.ascontiguousarray(np.broadcast_to(np.asarray(coeff, dtype=np.float64), (nt,)))
        a = None if angle is None else np.ascontiguousarray(np.broadcast_to(np.asarray(angle, dtype=np.float64),
                                                                             (nt,)))
        self._c(self.L.sg_bonded_set(self.ctx, int(kind), nt, at.ctypes.data_as(C.POINTER(C.c_int32)), _dp(c),
                                     _dp(a), 1 if one_based else 0))

    def bonded_forces(self, kind):
        e = C.c_double(0.0)
        self._c(self.L.sg_bonded_forces(self.ctx, int(kind), C.byref(e)))
        return e.value

    # ---- bond constraints -------------------------------------------------------------
    def set_constraints(self, bbi, bbj, length, one_based=False):
        """set_num_constraints + add_constraint for every bond."""
        i = np.ascontiguousarray(bbi, dtype=np.int32)
        j = np.ascontiguousarray(bbj, dtype=np.int32)
        ln = np.ascontiguousarray(np.broadcast_to(np.asarray(length, dtype=np.float64), i.shape))
        P = C.POINTER(C.c_int32)
        self._c(self.L.sg_set_constraints(self.ctx, len(i), i.ctypes.data_as(P), j.ctypes.data_as(P), _dp(ln),
                                          1 if one_based else 0))

    def constraints_save(self):
        self._c(self.L.sg_constraints_save(self.ctx))

    def constraints_a(self, dt):
        self._c(self.L.sg_constraints_a(self.ctx, dt))

    def constraints_b(self, dt):
        self._c(self.L.sg_constraints_b(self.ctx, dt))

    def constraints_check(self):
        self._c(self.L.sg_constraints_check(self.ctx))

    def constraints_clear_error(self):
        self._c(self.L.sg_constraints_clear_error(self.ctx))

    def constraint_stats(self, reset=False):
        out = np.zeros(6, dtype=np.int64)
        self._c(self.L.sg_constraint_stats(self.ctx, out.ctypes.data_as(C.POINTER(C.c_int64)), 1 if reset else 0))
        return dict(zip(("sweeps_a", "unconverged_a", "corrections_a", "sweeps_b", "unconverged_b",
                         "corrections_b"), out.tolist()))

    def vvc_initial(self, dt):
        self._c(self.L.sg_vvc_initial(self.ctx, dt))

    def vvc_final(self, dt):
        ke = C.c_double(0.0)
        self._c(self.L.sg_vvc_final(self.ctx, dt, C.byref(ke)))
        return ke.value

    def nhtc_initial(self, dt, target_temp, coupling=0.0, mode=0, rot_chain=0):
        self._c(self.L.sg_nhtc_initial(self.ctx, dt, target_temp, coupling, mode, rot_chain))

    def nhtc_final(self, dt, target_temp, coupling=0.0, mode=0, rot_chain=0):
        ke = C.c_double(0.0)
        self._c(self.L.sg_nhtc_final(self.ctx, dt, target_temp, coupling, mode, rot_chain, C.byref(ke)))
        return ke.value

    def lgvc_initial(self, dt, step, damping=1.0, target_temp=1.0, key=None):
        k = None if key is None else np.asarray(key, dtype=np.uint32)
        self._c(self.L.sg_lgvc_initial(self.ctx, dt, int(step), damping, target_temp,
                                       None if k is None else k.ctypes.data_as(C.POINTER(C.c_uint32))))

    def lgvc_final(self, dt, damping=1.0):
        ke = C.c_double(0.0)
        kr = C.c_double(0.0)
        self._c(self.L.sg_lgvc_final(self.ctx, dt, damping, C.byref(ke), C.byref(kr)))
        return ke.value, kr.value

    def thermo(self, dof, density, nrigid=1):
        out = np.zeros(3)
        self._c(self.L.sg_thermo(self.ctx, int(dof), float(density), int(nrigid), _dp(out)))
        return out

    def set_velocity_to_temperature(self, rtemp, seed, remove_com_velocity=True, nrigid=1):
        """set_velocity_to_temperature (fortran/system.f90:361-421) on the device:
        Philox normals of counter (I, int(rtemp*1000), seed, 42), the mean
        removed (n_dof = 6N - NC - 3) unless remove_com_velocity is False
        (6N - NC), scaled to sum |v|^2 = n_dof * rtemp * nrigid."""
        self._c(self.L.sg_set_velocity_to_temperature(self.ctx, float(rtemp), int(seed),
                                                      1 if remove_com_velocity else 0, int(nrigid)))

    def synchronize(self):
        self._c(self.L.sg_synchronize(self.ctx))

    # ---- captured timestep -------------------------------------------------------------
    def configure_step(self, pair, integrator=capi.INT_NVE, dt=0.001, target_temp=1.0, damping=1.0, coupling=0.0,
                       rotations=0, rot_chain=0, first_step=1, key=None, flags=0):
        cfg = capi.StepConfig()
        cfg.flags = flags
        cfg.integrator, cfg.rotations, cfg.rot_chain, cfg.first_step = integrator, rotations, rot_chain, first_step
        cfg.dt, cfg.target_temp, cfg.damping, cfg.coupling = dt, target_temp, damping, coupling
        if key is not None:
            cfg.key[0], cfg.key[1] = int(key[0]), int(key[1])
            cfg.has_key = 1
        cfg.pair = pair
        self._step_cfg = cfg
        self._c(self.L.sg_step_configure(self.ctx, C.byref(cfg)))

    def configure_step_pairs(self, pairs, integrator=capi.INT_NVE, dt=0.001, target_temp=1.0, damping=1.0,
                             coupling=0.0, rotations=0, rot_chain=0, first_step=1, key=None, flags=0):
        """Step whose pair stage runs several parameter sets in order (summed
        potentials; in replica contexts each set acts on its family's replicas)."""
        cfg = capi.StepConfig()
        cfg.flags = flags
        cfg.integrator, cfg.rotations, cfg.rot_chain, cfg.first_step = integrator, rotations, rot_chain, first_step
        cfg.dt, cfg.target_temp, cfg.damping, cfg.coupling = dt, target_temp, damping, coupling
        if key is not None:
            cfg.key[0], cfg.key[1] = int(key[0]), int(key[1])
            cfg.has_key = 1
        arr = (PairParams * len(pairs))(*pairs)
        self._step_cfg = (cfg, arr)
        self._c(self.L.sg_step_configure_pairs(self.ctx, C.byref(cfg), arr, len(pairs)))

    def step(self, nsteps=1):
        self._c(self.L.sg_step(self.ctx, int(nsteps)))

    def step_stage_times(self, nsteps=10):
        """Mean ms per stage of nsteps eager steps: initial half step,
        constraints a, list, zero forces, pairs, final half step, constraints b."""
        out = np.zeros(7)
        self._c(self.L.sg_step_stage_times(self.ctx, int(nsteps), _dp(out)))
        return dict(zip(("initial", "constraints_a", "list", "zero_forces", "pairs", "final", "constraints_b"),
                        out.tolist()))

    def step_check(self):
        self._c(self.L.sg_step_check(self.ctx))

    def step_kernel_count(self):
        k = C.c_int64(0)
        self._c(self.L.sg_step_kernel_count(self.ctx, C.byref(k)))
        return k.value

    def peak_fma(self, fp64=False):
        t = C.c_double(0.0)
        self._c(self.L.sg_peak_fma(self.ctx, 1 if fp64 else 0, C.byref(t)))
        return t.value

    def stream_ptr(self):
        return self.L.sg_stream(self.ctx)

    # ---- Philox ---------------------------------------------------------------------
    def philox(self, ctr, key=(0x6D2B79F5, 0x1B873593)):
        c = np.ascontiguousarray(ctr, dtype=np.uint32).reshape(-1, 4)
        k = np.asarray(key, dtype=np.uint32)
        out = np.zeros_like(c)
        P = C.POINTER(C.c_uint32)
        self._c(self.L.sg_philox4x32_device(self.ctx, len(c), c.ctypes.data_as(P), k.ctypes.data_as(P),
                                            out.ctypes.data_as(P)))
        return out

    def normal_3seq(self, ctr):
        c = np.ascontiguousarray(ctr, dtype=np.int32).reshape(-1, 4)
        out = np.zeros((len(c), 3))
        self._c(self.L.sg_philox_normal_3seq_device(self.ctx, len(c), c.ctypes.data_as(C.POINTER(C.c_int32)), _dp(out)))
        return out

    # ---- MLP ---------------------------------------------------------------------------
    def set_mlp_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._c(self.L.sg_mlp_set_weights(self.ctx, w.ctypes.data_as(C.POINTER(C.c_float)), len(w)))

    def get_mlp_weights(self):
        n = self.L.sg_mlp_weight_count()
        w = np.zeros(n, dtype=np.float32)
        self._c(self.L.sg_mlp_get_weights(self.ctx, w.ctypes.data_as(C.POINTER(C.c_float)), n))
        return w


class Reporter:
    """sg_reporter: open_*_file / report_* / close_*_file of fortran/reporters.f90."""

    def __init__(self, system, kind, path, dof=None, density=None, nrigid=1):
        self.g = system
        self.L = system.L
        h = C.c_void_p()
        system._c(self.L.sg_reporter_open(system.ctx, int(kind), str(path).encode(), C.byref(h)))
        self.h = h
        if dof is not None:
            system._c(self.L.sg_reporter_set_thermo(h, int(dof), float(density or 0.0), int(nrigid)))

    def write(self, step):
        self.g._c(self.L.sg_reporter_write(self.h, int(step)))

    def flush(self):
        self.g._c(self.L.sg_reporter_flush(self.h))

    def close(self):
        if self.h:
            rc = self.L.sg_reporter_close(self.h)
            self.h = None
            self.g._c(rc)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
