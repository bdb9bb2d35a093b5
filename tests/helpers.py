"""Shared builders for the parity tests: one seeded state, rounded to FP32,
loaded into both the oracle (FP64) and the device (FP32)."""
import numpy as np

import oracle as O
from sucrose_gb300 import configs


def f32(a):
    return np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)


def rel(a, b):
    """Norm-wise relative error ||a - b|| / ||b|| over the whole array."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def per_particle_max(a, b, floor_frac=1e-3):
    """max_i ||a_i - b_i|| / max(||b_i||, floor_frac * rms||b||)."""
    nb = np.linalg.norm(b, axis=1)
    fl = floor_frac * np.sqrt(np.mean(nb ** 2))
    return float(np.max(np.linalg.norm(a - b, axis=1) / np.maximum(nb, fl))) if len(nb) else 0.0


class Pair:
    """Matched oracle / device systems."""

    def __init__(self, r, q, box, sig=(1.0, 1.0, 1.0), eps=(1.0, 1.0, 1.0), v=None, l=None, mass=1.0,
                 periodic=True, device=True):
        from sucrose_gb300 import GpuSystem
        self.r = f32(r)
        self.q = f32(q) if q is not None else np.tile([1.0, 0.0, 0.0, 0.0], (len(r), 1))
        self.n = len(self.r)
        self.box = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)).copy()
        self.sig, self.eps = sig, eps
        self.v = f32(v) if v is not None else np.zeros((self.n, 3))
        self.l = f32(l) if l is not None else np.zeros((self.n, 3))
        s = O.System(self.n, self.box, periodic=periodic)
        s.set_defaults(mass=mass, sig=sig, eps=eps)
        s.rx[:], s.ry[:], s.rz[:] = self.r.T
        s.qw[:], s.qx[:], s.qy[:], s.qz[:] = self.q.T
        s.vx[:], s.vy[:], s.vz[:] = self.v.T
        s.lx[:], s.ly[:], s.lz[:] = self.l.T
        # inertia as the device stores it (FP32)
        for f in ("ixx", "iyy", "izz", "ixx_inv", "iyy_inv", "izz_inv", "inv_mass", "mass"):
            getattr(s, f)[:] = f32(getattr(s, f))
        self.o = s
        if device:
            g = GpuSystem(self.n, self.box, periodic=periodic)
            g.set_particles(mass=mass, sig=sig, eps=eps)
            g.upload(r=self.r, q=self.q, v=self.v, l=self.l)
            self.g = g

    def oracle_forces(self):
        return np.stack([self.o.fx, self.o.fy, self.o.fz], 1), np.stack([self.o.tx, self.o.ty, self.o.tz], 1)

    def set_oracle_forces(self, F, T):
        self.o.fx[:], self.o.fy[:], self.o.fz[:] = F.T
        self.o.tx[:], self.o.ty[:], self.o.tz[:] = T.T


def lj_fcc():
    r, q, box = configs.fcc_lattice(3, 0.8442)
    v = configs.velocities_to_temperature(108, 0.722, 15)
    return r, q, box, v


def jittered_fcc(cells, density, seed, amp=0.08):
    r, q, box = configs.fcc_lattice(cells, density)
    d = configs.normal_3seq(np.arange(1, len(r) + 1), seed, 3, 1)
    return r + amp * np.clip(d, -3, 3), q, box


def ellipsoids(counts, sig, density, seed, tilt, jitter=0.03):
    return configs.aligned_lattice(counts, sig, density, seed=seed, jitter=jitter, tilt=tilt)


def kdtree_reference_pairs(r, box, cutoff, skin):
    """The reference's half list at sizes where its O(N^2) build is too slow:
    candidates from a periodic k-d tree (a superset, radius widened by 1e-6),
    then build_nlist's own acceptance test on each (system.f90:977-1000):
    FP64 difference, ANINT minimum image (ties away from zero), and the strict
    (x^2 + y^2) + z^2 < (rc+skin)^2. Returns (pi, pj) 0-based, i < j, in row
    order. Checked against the oracle's O(N^2) build in tests/test_oracle.py."""
    from scipy.spatial import cKDTree
    r = np.asarray(r, dtype=np.float64)
    box = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)).copy()
    rl = cutoff + skin
    w = np.mod(r + box / 2.0, box)
    w = np.minimum(w, np.nextafter(box, 0.0))
    cand = cKDTree(w, boxsize=box).query_pairs(rl * (1.0 + 1e-6), output_type="ndarray")
    if len(cand) == 0:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    cand.sort(axis=1)
    i, j = cand[:, 0], cand[:, 1]
    d = r[i] - r[j]
    x = d / box
    d = d - np.sign(x) * np.floor(np.abs(x) + 0.5) * box
    rsq = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    keep = rsq < rl * rl
    i, j = i[keep], j[keep]
    o = np.lexsort((j, i))
    return i[o].astype(np.int32), j[o].astype(np.int32)
