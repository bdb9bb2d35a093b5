"""Seeded synthetic initial configurations (host-side set-up, not the hot path).

fcc_lattice and velocities_to_temperature follow the reference's own
generate_fcc_lattice (fortran/system.f90:438-523) and
set_velocity_to_temperature (:362-421, Philox counter (I, int(T*1000), seed, 42)),
so the Lennard-Jones README case starts from the reference's state.

The reference has no placement routine for dense ellipsoid fluids. The
ellipsoid systems here start from an aligned orthorhombic lattice whose cell
is the particle's bounding box scaled to the target number density (no
overlaps by construction), with a seeded jitter of positions and a seeded
small rotation of every particle; the benchmark then equilibrates them with
the repulsive potentials on the device before timing.
"""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
KEY = (0x6D2B79F5, 0x1B873593)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32(ctr, key=KEY):
    """Vectorised Philox4x32-10 (fortran/xmath.f90:42-76); ctr: (n, 4) uint32."""
    c = np.asarray(ctr, dtype=np.uint32).reshape(-1, 4)
    c0, c1, c2, c3 = (c[:, k].astype(np.uint64) for k in range(4))
    k0, k1 = np.uint32(key[0]), np.uint32(key[1])
    with np.errstate(over="ignore"):
        for rnd in range(10):
            p0 = M0 * c0
            p1 = M1 * c2
            hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
            hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
            n0 = hi1 ^ c1 ^ np.uint64(k0)
            n2 = hi0 ^ c3 ^ np.uint64(k1)
            c0, c1, c2, c3 = n0, lo1, n2, lo0
            if rnd < 9:
                k0 = np.uint32(k0 + W0)
                k1 = np.uint32(k1 + W1)
    return np.stack([c0, c1, c2, c3], 1).astype(np.uint32)


def normal_3seq(c1, c2, c3, c4, key=KEY):
    """philox_normal_3seq (fortran/xmath.f90:78-113), vectorised; FP64."""
    n = np.broadcast(c1, c2, c3, c4).shape[0] if np.ndim(c1) else 1
    ctr = np.zeros((n, 4), dtype=np.uint32)
    for k, c in enumerate((c1, c2, c3, c4)):
        ctr[:, k] = np.broadcast_to(np.asarray(c, dtype=np.int64) & 0xFFFFFFFF, (n,)).astype(np.uint32)
    w = philox4x32(ctr, key).astype(np.float64) * (1.0 / 4294967296.0)
    u1 = np.maximum(w[:, 0], 1.0e-35)
    u3 = np.maximum(w[:, 2], 1.0e-35)
    twopi = 6.283185307179586
    r1 = np.sqrt(-2.0 * np.log(u1))
    r2 = np.sqrt(-2.0 * np.log(u3))
    return np.stack([r1 * np.cos(twopi * w[:, 1]), r1 * np.sin(twopi * w[:, 1]), r2 * np.cos(twopi * w[:, 3])], 1)


def fcc_lattice(cells, density):
    """generate_fcc_lattice: 4 cells^3 points in a cubic box centred on 0, with
    the reference's four basis orientations. Returns r (n,3), q (n,4), box."""
    n = 4 * cells ** 3
    box = (float(n) / density) ** (1.0 / 3.0)
    cell = box / cells
    h = cell / 2.0
    rr3 = 1.0 / np.sqrt(3.0)
    a, b = np.sqrt((1.0 + rr3) / 2.0), np.sqrt((1.0 - rr3) / 2.0)
    c = rr3 / np.sqrt(1.0 - rr3 ** 2.0)
    basis = np.array([[0.0, 0.0, 0.0], [h, h, 0.0], [0.0, h, h], [h, 0.0, h]])
    qb = np.array([[a, b * c, -b * c, 0.0], [b, -a * c, -a * c, 0.0], [b, a * c, a * c, 0.0], [a, -b * c, b * c, 0.0]])
    r = np.zeros((n, 3))
    q = np.zeros((n, 4))
    m = 0
    for I in range(cells):
        for J in range(cells):
            for K in range(cells):
                r[m:m + 4] = basis + cell * np.array([I, J, K], dtype=np.float64)
                q[m:m + 4] = qb
                m += 4
    r -= box / 2.0
    return r, q, box


def velocities_to_temperature(n, temp, seed, nc=0, nrigid=1, remove_com=True):
    """set_velocity_to_temperature: Philox normals with counter
    (I, int(T*1000), seed, 42), COM removal, then sum v^2 scaled to
    (6N - NC [-3]) * T * Nrigid (the reference's convention, mass ignored)."""
    idx = np.arange(1, n + 1, dtype=np.int64)
    v = normal_3seq(idx, int(temp * 1000), seed, 42)
    n_dof = 6 * n - nc
    if remove_com:
        v = v - v.sum(0) / float(n)
        n_dof -= 3
    factor = np.sqrt(float(n_dof) * temp * nrigid / np.sum(v ** 2))
    return v * factor


def random_quaternions(n, seed, key=(0x2545F491, 0x4F6CDD1D)):
    """Uniform unit quaternions from four Philox normals, seeded."""
    idx = np.arange(1, n + 1, dtype=np.int64)
    a = normal_3seq(idx, seed, 7, 0, key)
    b = normal_3seq(idx, seed, 7, 1, key)
    q = np.concatenate([a, b[:, :1]], 1)
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    return q


def _small_rotations(n, seed, angle):
    """Rotations by a seeded random angle <= angle about seeded random axes."""
    idx = np.arange(1, n + 1, dtype=np.int64)
    ax = normal_3seq(idx, seed, 11, 0)
    ax /= np.linalg.norm(ax, axis=1, keepdims=True)
    u = philox4x32(np.stack([idx, np.full(n, seed), np.full(n, 13), np.zeros(n)], 1).astype(np.uint32))
    th = angle * (u[:, 0].astype(np.float64) / 4294967296.0)
    return np.concatenate([np.cos(th / 2)[:, None], np.sin(th / 2)[:, None] * ax], 1)


def quat_mul(a, b):
    w1, x1, y1, z1 = a.T
    w2, x2, y2, z2 = b.T
    return np.stack([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2], 1)


def aligned_lattice(counts, sig, density, seed, jitter=0.02, tilt=0.05):
    """Orthorhombic lattice of nx*ny*nz particles of full axes sig = (sx, sy, sz),
    body axes along the lab axes, cell = s * sig with s fixed by the density.
    Returns r (n,3), q (n,4), box (3,)."""
    nx, ny, nz = counts
    n = nx * ny * nz
    sx, sy, sz = sig
    s = (1.0 / (density * sx * sy * sz)) ** (1.0 / 3.0)
    cell = s * np.array([sx, sy, sz])
    box = cell * np.array([nx, ny, nz], dtype=np.float64)
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    r = (g + 0.5) * cell - box / 2.0
    idx = np.arange(1, n + 1, dtype=np.int64)
    d = normal_3seq(idx, seed, 5, 0)
    r = r + jitter * np.clip(d, -2.0, 2.0) * cell.min()
    q = _small_rotations(n, seed, tilt)
    return r, q, box


def isotropic_placement(n, sig, density, seed, gap=1.0, box=None):
    """Seeded isotropic, non-overlapping placement of n ellipsoids of full axes
    sig = (sx, sy, sz) at the given number density in a cubic periodic box
    (sg_place_isotropic, on the current GPU: uniform positions and
    orientations, growth from a fifth of full size with overlap relaxation).
    The same bits on every run. Returns r (n,3), q (n,4), box (3,), report."""
    import ctypes as C
    from sucrose_gb300 import capi
    L = capi.load()
    if box is None:
        box = np.full(3, (float(n) / density) ** (1.0 / 3.0))
    box = np.ascontiguousarray(box, dtype=np.float64)
    semi = np.ascontiguousarray(np.asarray(sig, dtype=np.float64) / 2.0)
    r = np.zeros((n, 3))
    q = np.zeros((n, 4))
    rep = capi.PlaceReport()
    D = C.POINTER(C.c_double)
    rc = L.sg_place_isotropic(n, semi.ctypes.data_as(D), box.ctypes.data_as(D), seed, gap,
                              r.ctypes.data_as(D), q.ctypes.data_as(D), C.byref(rep))
    if rc != capi.SG_OK:
        raise capi.SgError(rc, f"isotropic placement of {n} ellipsoids {tuple(sig)} at density {density}: "
                               f"{rep.overlaps} overlapping pairs left at size {rep.final_scale:.3f} "
                               f"after {rep.sweeps} sweeps")
    return r, q, box, rep


def nematic_order(q, axis=2):
    """Nematic order parameter P2 of body axis `axis` (largest eigenvalue of
    the Q tensor <3/2 u u^T - 1/2 I>): 0 for isotropic orientations (about
    1/sqrt(n) from sampling), 1 for perfect alignment."""
    w, x, y, z = np.asarray(q, dtype=np.float64).T
    rows = [np.stack([w * w + x * x - y * y - z * z, 2 * (x * y + w * z), 2 * (x * z - w * y)], 1),
            np.stack([2 * (x * y - w * z), w * w - x * x + y * y - z * z, 2 * (y * z + w * x)], 1),
            np.stack([2 * (x * z + w * y), 2 * (y * z - w * x), w * w - x * x - y * y + z * z], 1)]
    u = rows[axis]
    u = u / np.linalg.norm(u, axis=1, keepdims=True)
    Q = 1.5 * (u.T @ u) / len(u) - 0.5 * np.eye(3)
    return float(np.linalg.eigvalsh(Q)[-1])


def angular_momenta(q, inertia, temp, seed):
    """Thermal body-frame angular momenta L_b ~ sqrt(T I) N(0,1), returned in the lab frame."""
    n = len(q)
    idx = np.arange(1, n + 1, dtype=np.int64)
    lb = normal_3seq(idx, seed, 17, 3) * np.sqrt(temp * inertia)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0] = np.stack([w * w + x * x - y * y - z * z, 2 * (x * y + w * z), 2 * (x * z - w * y)], 1)
    R[:, 1] = np.stack([2 * (x * y - w * z), w * w - x * x + y * y - z * z, 2 * (y * z + w * x)], 1)
    R[:, 2] = np.stack([2 * (x * z + w * y), 2 * (y * z - w * x), w * w - x * x - y * y + z * z], 1)
    return np.einsum("nji,nj->ni", R, lb)


def default_inertia(sig, mass=1.0):
    """initialize_system default (system.f90:619-621): I_x = (s_y^2 + s_z^2)/20 ..."""
    sx, sy, sz = sig
    return np.array([(sy ** 2 + sz ** 2) / 20.0, (sx ** 2 + sz ** 2) / 20.0, (sx ** 2 + sy ** 2) / 20.0]) * mass


# ---------------------------------------------------------------- replicas ---
LJ_REPLICA = dict(family=0, cutoff=2.5, list_cutoff=2.5, skin=0.3, rho=(0.7, 0.9), T=(0.7, 1.5),
                  sig=(1.0, 1.0, 1.0), eps=(1.0, 1.0, 1.0))
GB_REPLICA = dict(family=1, cutoff=4.0, list_cutoff=6.0, skin=0.4, rho=(0.2, 0.35), T=(0.8, 1.6),
                  sig=(1.0, 1.0, 3.0), eps=(1.0, 1.0, 0.2))


def _replica_lattice(n, sig, density, seed, rng, tilt):
    """n particles on an orthorhombic lattice of cell s*sig with about three
    times as many cells across x and y as along the long axis, seeded
    vacancies removed; box fixed by the density. Returns r, q, box."""
    sx, sy, sz = sig
    aspect = sz / sx
    nz = max(1, int(round((n / aspect ** 2) ** (1.0 / 3.0))))
    nxy = int(np.ceil(np.sqrt(n / nz)))
    m = nxy * nxy * nz
    s = (n / (density * m * sx * sy * sz)) ** (1.0 / 3.0)
    cell = s * np.array([sx, sy, sz])
    box = cell * np.array([nxy, nxy, nz], dtype=np.float64)
    g = np.stack(np.meshgrid(np.arange(nxy), np.arange(nxy), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    keep = np.sort(rng.choice(m, size=n, replace=False))
    r = (g[keep] + 0.5) * cell - box / 2.0
    r = r + 0.02 * np.clip(rng.standard_normal((n, 3)), -2.0, 2.0) * cell.min()
    q = _small_rotations(n, seed, tilt) if tilt > 0 else np.tile([1.0, 0.0, 0.0, 0.0], (n, 1))
    return r, q, box


def replica_ensemble(nrep=4096, seed=1005, nmin=64, nmax=2048, lj=LJ_REPLICA, gb=GB_REPLICA, max_redraw=1000):
    """Seeded ensemble of nrep independent periodic replicas: the first half
    Lennard-Jones point fluids, the second half Gay-Berne (3, 5, 2, 1)
    ellipsoid fluids. Particle counts are log-uniform in [nmin, nmax]; a
    count whose box would be narrower than twice its list cut-off (the
    reference's init_nlist guard, fortran/system.f90:902-906) is redrawn from
    the same stream. Each replica has its own density, temperature and
    Philox key (two words derived from (seed, replica)).

    Returns a dict of per-replica arrays (n, box, family, temp, key, density)
    and the concatenated r, q (each replica centred in its own box)."""
    rng = np.random.default_rng(seed)
    fams = [lj] * (nrep // 2) + [gb] * (nrep - nrep // 2)
    out = dict(n=[], box=[], family=[], temp=[], density=[], redraws=0)
    rs, qs = [], []
    for k, p in enumerate(fams):
        rho = rng.uniform(*p["rho"])
        T = rng.uniform(*p["T"])
        for attempt in range(max_redraw):
            n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
            r, q, box = _replica_lattice(n, p["sig"], rho, seed * 7919 + k, rng, 0.1 if p["family"] == 1 else 0.0)
            if box.min() >= 2.0 * p["list_cutoff"]:
                break
            out["redraws"] += 1
        else:
            raise RuntimeError("replica %d: no count in range fits the cut-off" % k)
        out["n"].append(n)
        out["box"].append(box)
        out["family"].append(p["family"])
        out["temp"].append(T)
        out["density"].append(rho)
        rs.append(r)
        qs.append(q)
    R = np.arange(nrep, dtype=np.int64)
    words = philox4x32(np.stack([R, np.full(nrep, seed), np.full(nrep, 0x5EED), np.zeros(nrep)], 1).astype(np.uint32))
    out["key"] = words[:, :2].copy()
    for k in ("n", "family"):
        out[k] = np.asarray(out[k], dtype=np.int32)
    for k in ("temp", "density"):
        out[k] = np.asarray(out[k], dtype=np.float64)
    out["box"] = np.asarray(out["box"])
    out["r"] = np.concatenate(rs)
    out["q"] = np.concatenate(qs)
    out["off"] = np.concatenate([[0], np.cumsum(out["n"])]).astype(np.int64)
    return out
