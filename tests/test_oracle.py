"""The oracle (CPU restatement) pinned against the reference's own code and
known answers. CPU only."""
import os

import numpy as np
import pytest

import oracle as O
from sucrose_gb300 import configs

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def system_from(r, box, sig=(1.0, 1.0, 1.0), eps=(1.0, 1.0, 1.0), q=None, periodic=True):
    s = O.System(len(r), box, periodic=periodic)
    s.set_defaults(sig=sig, eps=eps)
    s.rx[:], s.ry[:], s.rz[:] = np.asarray(r).T
    if q is not None:
        s.qw[:], s.qx[:], s.qy[:], s.qz[:] = np.asarray(q).T
    return s


# ---------------------------------------------- pins to the reference's code ---
def test_lj_matches_reference_cpp_golden():
    g = np.load(os.path.join(GOLD, "ref_lj_untruncated.npz"))
    r, L = g["r"], float(g["box"])
    s = system_from(r, L)
    pi, pj = np.triu_indices(len(r), 1)
    # untruncated LJ == lj_ with an infinite cutoff (the shift vanishes)
    s.forces(O.pair_params(O.LJ, cutoff=1e150), pi, pj)
    F = np.stack([s.fx, s.fy, s.fz], 1)
    Fr = np.stack([g["fx"], g["fy"], g["fz"]], 1)
    assert np.linalg.norm(F - Fr) <= 1e-12 * np.linalg.norm(Fr)
    assert abs(s.s.pot_eng - float(g["pot"])) <= 1e-12 * abs(float(g["pot"]))


def test_lj_matches_reference_cpp_live():
    R = O.ref_lib()
    if R is None:
        pytest.skip("reference tree absent (GPU host): the committed fixture covers this")
    rng = np.random.default_rng(5)
    (rx, ry, rz, *_), L = O.fcc_lattice(3, 0.8)
    r = np.stack([rx, ry, rz], 1) + rng.uniform(-0.2, 0.2, size=(108, 3))
    s = system_from(r, L)
    pi, pj = [a.astype(np.int32) for a in np.triu_indices(108, 1)]
    s.forces(O.pair_params(O.LJ, cutoff=1e150), pi, pj)
    a = [np.ascontiguousarray(r[:, k]) for k in range(3)]
    fx, fy, fz, pot = np.zeros(108), np.zeros(108), np.zeros(108), np.zeros(1)
    R.ref_lj_forces(108, L, 1, *[O.dptr(x) for x in a], 1.0, 1.0, len(pi), O.iptr(pi), O.iptr(pj), O.dptr(fx),
                    O.dptr(fy), O.dptr(fz), O.dptr(pot))
    assert np.allclose(s.fx, fx, rtol=1e-11, atol=1e-11)
    assert abs(s.s.pot_eng - pot[0]) <= 1e-11 * abs(pot[0])


def test_vv_matches_reference_cpp_golden():
    g = np.load(os.path.join(GOLD, "ref_vv_step.npz"))
    r, v, f, L, dt = g["r"], g["v"], g["f"], float(g["box"]), float(g["dt"])
    s = system_from(r, L)
    s.vx[:], s.vy[:], s.vz[:] = v.T
    s.fx[:], s.fy[:], s.fz[:] = f.T
    s.vv_initial(dt)
    assert np.allclose(np.stack([s.rx, s.ry, s.rz], 1), g["r0"], rtol=0, atol=1e-13)
    assert np.allclose(np.stack([s.vx, s.vy, s.vz], 1), g["v0"], rtol=0, atol=1e-13)
    s2 = system_from(r, L)
    s2.vx[:], s2.vy[:], s2.vz[:] = v.T
    s2.fx[:], s2.fy[:], s2.fz[:] = f.T
    s2.vv_final(dt)
    assert np.allclose(np.stack([s2.vx, s2.vy, s2.vz], 1), g["v1"], rtol=0, atol=1e-13)


def test_philox_golden_and_host_copy():
    g = np.load(os.path.join(GOLD, "philox_words.npz"))
    assert np.array_equal(O.philox4x32(g["ctr"]), g["words"])
    # an independent vectorised restatement (product host code) agrees bit for bit
    assert np.array_equal(configs.philox4x32(g["ctr"]), g["words"])


def test_readme_velocities_golden():
    g = np.load(os.path.join(GOLD, "readme_velocities.npz"))
    v = configs.velocities_to_temperature(108, 0.722, 15)
    assert np.allclose(v, g["v"], rtol=0, atol=1e-13)
    # the reference's dof convention: sum v^2 = (6N - 3) T
    assert abs(np.sum(v ** 2) - (6 * 108 - 3) * 0.722) < 1e-9
    # the fixture is the oracle's own output: a regression anchor
    o = O.System(108, 10.0)
    o.set_velocity_to_temperature(0.722, 15)
    assert np.array_equal(np.stack([o.vx, o.vy, o.vz], 1), g["v"])


@pytest.mark.parametrize("n,temp,seed,nc,nrigid,com", [(500, 1.37, -3, 120, 2, False), (777, 0.8, 2024, 0, 1, True)])
def test_velocity_init_host_matches_oracle(n, temp, seed, nc, nrigid, com):
    # the host routine used for replica set-up against the oracle's
    # set_velocity_to_temperature, with NC, Nrigid, a negative seed and no
    # mean removal
    o = O.System(n, 10.0)
    o.s.nc, o.s.nrigid = nc, nrigid
    o.set_velocity_to_temperature(temp, seed, com)
    v = configs.velocities_to_temperature(n, temp, seed, nc=nc, nrigid=nrigid, remove_com=com)
    np.testing.assert_allclose(v, np.stack([o.vx, o.vy, o.vz], 1), rtol=1e-13, atol=1e-13)
    dof = 6 * n - nc - (3 if com else 0)
    assert abs(np.sum(v ** 2) - dof * temp * nrigid) < 1e-9 * dof * temp * nrigid


# ----------------------------------------------------------- Philox structure ---
def test_philox_structure():
    n = 1 << 16
    ctr = np.zeros((n, 4), dtype=np.uint32)
    ctr[:, 0] = np.arange(n)
    w = O.philox4x32(ctr)
    assert len(np.unique(w[:, 0])) > n - 5            # distinct words for distinct counters
    u = w.astype(np.float64) / 2 ** 32
    assert np.all((u >= 0) & (u < 1))
    hist, _ = np.histogram(u.ravel(), bins=64, range=(0, 1))
    expect = u.size / 64
    chi2 = np.sum((hist - expect) ** 2 / expect)
    assert chi2 < 150                                   # 63 dof
    z = O.philox_normal_3seq(1, 2, 3, 4)
    assert np.all(np.isfinite(z))


# ------------------------------------------------------------ known answers ---
def test_lj_known_answers():
    rmin = 2 ** (1 / 6)
    s = system_from([[0, 0, 0], [rmin, 0, 0]], 50.0)
    out, _ = s.pair(0, 1, O.pair_params(O.LJ, cutoff=1e150))
    assert abs(out[1]) < 1e-12 and abs(out[0] + 1.0) < 1e-12
    s = system_from([[0, 0, 0], [2.5 - 1e-12, 0, 0]], 50.0)
    out, _ = s.pair(0, 1, O.pair_params(O.LJ, cutoff=2.5))
    assert abs(out[0]) < 1e-9                           # shifted energy vanishes at rc
    s = system_from([[0, 0, 0], [1.0, 0, 0]], 50.0)
    out, _ = s.pair(0, 1, O.pair_params(O.WCA, sigma=1.0))
    assert abs(out[0]) < 1e-12 and abs(out[1]) < 1e-12  # WCA: zero at its minimum sigma


def test_ecp_spheres():
    # equal spheres of radius 1.2: lambda = 1/2, contact at 2.4
    for d in (2.0, 2.4, 3.0):
        s = system_from([[0, 0, 0], [d, 0.0, 0.0]], 50.0, sig=(2.4, 2.4, 2.4))
        for solver in (O.SOLVER_BRENT, O.SOLVER_TIGHT):
            out, _ = s.pair(0, 1, O.pair_params(O.ECP, cutoff=3.0, solver=solver))
            assert abs(out[10] - 0.5) < 1e-12
    # unequal spheres a, b: lambda = a / (a + b)
    s = system_from([[0, 0, 0], [3.0, 0.0, 0.0]], 50.0)
    s.sig_x[0] = s.sig_y[0] = s.sig_z[0] = 1.0
    s.sig_x[1] = s.sig_y[1] = s.sig_z[1] = 3.0
    out, _ = s.pair(0, 1, O.pair_params(O.ECP, cutoff=3.0, solver=O.SOLVER_TIGHT))
    assert abs(out[10] - 0.25) < 1e-12


def test_gay_berne_contact_distances():
    # kappa = 3: side by side the well minimum is at sigma0 = 1, end to end at 3
    sig, eps = (1.0, 1.0, 3.0), (1.0, 1.0, 0.2)
    for d, ax in ((1.0, 0), (3.0, 2)):
        r = np.zeros((2, 3))
        r[1, ax] = d
        s = system_from(r, 60.0, sig=sig, eps=eps)
        out, _ = s.pair(0, 1, O.pair_params(O.GB, cutoff=4.0))
        assert abs(out[1 + ax]) < 1e-9                   # force vanishes at the contact (well minimum)
        assert out[0] < 0


def fd_check(kind, sig, eps, q, r, cutoff, h=1e-6, solver=O.SOLVER_TIGHT, **kw):
    s = system_from(r, 80.0, sig=sig, eps=eps, q=q)
    pp = O.pair_params(kind, cutoff=cutoff, solver=solver, **kw)
    out, _ = s.pair(0, 1, pp)
    F = out[1:4]
    num = np.zeros(3)
    for d in range(3):
        for sgn in (1, -1):
            rr = np.array(r, dtype=np.float64)
            rr[0, d] += sgn * h
            s2 = system_from(rr, 80.0, sig=sig, eps=eps, q=q)
            o2, _ = s2.pair(0, 1, pp)
            num[d] -= sgn * o2[0] / (2 * h)
    return F, num, out[0]


@pytest.mark.parametrize("kind", [O.GB, O.GBR])
def test_gay_berne_force_is_minus_gradient(kind):
    # with eps_z = 1: the reference's de2/dr omits the 1/eps_z(I) factor that
    # its energy carries (force.f90:367 vs :393), so F = -grad U only then
    rng = np.random.default_rng(1)
    q = rng.normal(size=(2, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    r = np.array([[0.0, 0.0, 0.0], [1.3, 0.6, 0.4]]) * (0.7 if kind == O.GBR else 1.0)
    F, num, pe = fd_check(kind, (1.0, 1.0, 3.0), (1.0, 1.0, 1.0), q, r, 4.0)
    assert pe != 0.0
    assert np.allclose(F, num, rtol=1e-5, atol=1e-6 * np.abs(F).max())
    if kind == O.GB:
        # and the quirk is reproduced when eps_z != 1
        F2, num2, _ = fd_check(kind, (1.0, 1.0, 3.0), (1.0, 1.0, 0.2), q, r, 4.0)
        assert not np.allclose(F2, num2, rtol=1e-3)


@pytest.mark.parametrize("kind", [O.ECP, O.ECPR])
def test_ecp_force_is_minus_gradient(kind):
    # Two parallel identical ellipsoids: lambda = 1/2 for every separation, so
    # d lambda / d r = 0 and F = -grad U exactly. (For general pairs the
    # reference's forces omit d eps2/d lambda * d lambda/d r, because eps2 is
    # evaluated at the distance optimum lambda_R, force.f90:1308.)
    rng = np.random.default_rng(2)
    q0 = rng.normal(size=4)
    q0 /= np.linalg.norm(q0)
    q = np.stack([q0, q0])
    r = np.array([[0.0, 0.0, 0.0], [2.1, 1.1, 0.5]]) * (0.52 if kind == O.ECPR else 1.0)
    F, num, pe = fd_check(kind, (3.0, 2.0, 1.0), (1.0, 1.0, 1.0), q, r, 3.0)
    assert pe != 0.0
    assert np.allclose(F, num, rtol=2e-5, atol=1e-6 * np.abs(F).max())


def _rotation_rows(q):
    w, x, y, z = q
    return np.array([[w * w + x * x - y * y - z * z, 2 * (x * y + w * z), 2 * (x * z - w * y)],
                     [2 * (x * y - w * z), w * w - x * x + y * y - z * z, 2 * (y * z + w * x)],
                     [2 * (x * z + w * y), 2 * (y * z - w * x), w * w - x * x - y * y + z * z]])


@pytest.mark.parametrize("kind,kw,extra", [(O.ECPR, {}, 0.0), (O.ECP, {}, 2.0), (O.ECPW, {"wf": 0.5}, 2.5)],
                         ids=["ecpr", "ecp", "ecpw"])
def test_ecp_range_test_bounds_hold_at_the_converged_lambda(kind, kw, extra):
    """The two upper bounds on the contact distance that the filtered ECP
    launch tests before any solve: sigma = |r| / sqrt(F(lambda*)) with
    F(l) = l(1-l) r.((1-l)A + lB)^-1 r, A = U^T S^2 U (the AR of fortran/force.f90:1294), is at
    most h_A + h_B (the support functions along r) and at most |r| / sqrt(F(l0))
    at l0 = h_A / (h_A + h_B), because lambda* maximises F. The converged
    lambda here is the oracle's; a pair beyond sigma + extra (reach - sigma:
    cutoff - 1, plus wf welded, 0 repulsive) has no energy, force or torque, so
    turning it away before the solve changes nothing."""
    rng = np.random.default_rng(5)
    sig = np.array([3.0, 2.0, 1.0])
    S2 = np.diag((sig / 2) ** 2)
    grid = np.linspace(1e-4, 1 - 1e-4, 801)
    beyond = 0
    for _ in range(150):
        q = rng.normal(size=(2, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        d = rng.normal(size=3)
        d *= rng.uniform(0.8, 6.0) / np.linalg.norm(d)
        s = system_from([[0, 0, 0], d], 80.0, sig=tuple(sig), q=q)
        out, _ = s.pair(0, 1, O.pair_params(kind, cutoff=3.0, solver=O.SOLVER_TIGHT, **kw))
        A, B = (_rotation_rows(qq).T @ S2 @ _rotation_rows(qq) for qq in q)

        def F(lam):
            return lam * (1 - lam) * d @ np.linalg.solve((1 - lam) * A + lam * B, d)

        lam = out[10]
        assert max(F(g) for g in grid) <= F(lam) * (1 + 1e-12)     # the oracle's lambda is the maximum
        rm = np.linalg.norm(d)
        sigma = rm / np.sqrt(F(lam))
        ha, hb = np.sqrt(d @ A @ d) / rm, np.sqrt(d @ B @ d) / rm
        assert sigma <= (ha + hb) * (1 + 1e-12)
        assert sigma <= rm / np.sqrt(F(ha / (ha + hb))) * (1 + 1e-12)
        if rm > (sigma + extra) * (1 + 1e-9):
            beyond += 1
            assert np.all(out[:10] == 0.0)
    assert beyond > 10


def test_fp16_shape_matrix_widened_by_frobenius_error_bounds_it():
    """The range record's matrix: A rounded to FP16 plus d I with d the
    Frobenius norm of the rounding error (x 1.001, all in FP32) is >= A in
    the positive semi-definite order, so the support functions and 1/F(l)
    taken with it bound those of A from above (the test stays a superset)."""
    rng = np.random.default_rng(9)
    for _ in range(3000):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        U = _rotation_rows(q).astype(np.float32)
        s = rng.uniform(0.05, 20.0, size=3).astype(np.float32)
        A = (U.T @ np.diag((s / 2) ** 2) @ U).astype(np.float32)
        A = (A + A.T) / np.float32(2)
        Ah = A.astype(np.float16).astype(np.float32)
        e = A - Ah
        d = np.float32(np.sqrt(np.float32(np.sum(e * e))) * np.float32(1.001))
        W = Ah + d * np.eye(3, dtype=np.float32)
        assert np.linalg.eigvalsh(W.astype(np.float64) - A.astype(np.float64)).min() >= 0.0


def test_brent_vs_converged_gap_is_the_reference_tolerance():
    # the reference's Brent stops at atol 1e-3 / rtol 1e-2 (force.f90:1065):
    # its lambda differs from the converged one by up to ~1e-2
    rng = np.random.default_rng(3)
    gaps = []
    for k in range(200):
        q = rng.normal(size=(2, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        d = rng.normal(size=3)
        d *= rng.uniform(1.5, 3.3) / np.linalg.norm(d)
        s = system_from([[0, 0, 0], d], 80.0, sig=(3.0, 2.0, 1.0), q=q)
        a, _ = s.pair(0, 1, O.pair_params(O.ECPR, solver=O.SOLVER_BRENT))
        b, _ = s.pair(0, 1, O.pair_params(O.ECPR, solver=O.SOLVER_TIGHT))
        gaps.append(abs(a[10] - b[10]))
    assert 0 < max(gaps) < 2e-2


# ------------------------------------------------------------ neighbour list ---
def test_nlist_against_kdtree():
    from scipy.spatial import cKDTree
    rng = np.random.default_rng(4)
    L = 12.0
    r = rng.uniform(-L / 2, L / 2, size=(400, 3))
    s = system_from(r, L)
    pi, pj = s.pairs(2.5, 0.3)
    got = set(zip(pi.tolist(), pj.tolist()))
    tree = cKDTree((r + L / 2) % L, boxsize=L)
    want = set(map(tuple, np.sort(tree.query_pairs(2.8, output_type="ndarray"), axis=1).tolist()))
    assert got == want
    # reference CSR layout
    nl, off = s.nlist(2.5, 0.3, one_based=True)
    assert off[0] == 1 and off[-1] == len(nl) + 1 and nl.min() >= 2


def test_nlist_cutoff_guard():
    s = system_from(np.zeros((3, 3)), 4.0)
    with pytest.raises(ValueError):
        s.nlist(2.5, 0.3)


def test_third_law_of_pair_loop():
    (rx, ry, rz, *_), L = O.fcc_lattice(3, 0.8442)
    rng = np.random.default_rng(8)
    s = system_from(np.stack([rx, ry, rz], 1) + rng.uniform(-0.1, 0.1, (108, 3)), L)
    pi, pj = s.pairs(2.5, 0.3)
    s.forces(O.pair_params(O.LJ, cutoff=2.5), pi, pj)
    assert np.abs(np.sum(s.fx)) < 1e-10 and np.abs(np.sum(s.fy)) < 1e-10


def test_fp32_prediction_budget():
    # the same formulas in FP32 stay within 1e-5 of FP64, norm-wise, for an ECP cluster
    r, q, box = configs.aligned_lattice((4, 4, 8), (3.0, 2.0, 1.0), 0.1114, seed=3, jitter=0.03, tilt=0.4)
    s = system_from(r.astype(np.float32).astype(np.float64), box, sig=(3.0, 2.0, 1.0),
                    q=q.astype(np.float32).astype(np.float64))
    pi, pj = s.pairs(3.0, 0.3)
    pp = O.pair_params(O.ECP, cutoff=3.0, solver=O.SOLVER_TIGHT)
    s.forces(pp, pi, pj, prec=64)
    F64 = np.stack([s.fx, s.fy, s.fz], 1).copy()
    s.zero_forces()
    s.forces(pp, pi, pj, prec=32)
    F32 = np.stack([s.fx, s.fy, s.fz], 1)
    assert np.linalg.norm(F32 - F64) / np.linalg.norm(F64) < 1e-5


def test_kdtree_reference_pairs_match_the_oracle_build():
    """The k-d tree list used by the full-size tests equals the oracle's
    O(N^2) build_nlist restatement, near-threshold pairs across the
    periodic boundary included."""
    from helpers import kdtree_reference_pairs
    rng = np.random.default_rng(17)
    box = np.array([21.0, 19.5, 23.0])
    base = rng.uniform(-box / 2, box / 2, size=(400, 3))
    d = rng.normal(size=(400, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    partner = base + d * (2.8 + rng.uniform(-3e-6, 3e-6, size=(400, 1)))
    partner -= box * np.round(partner / box)
    r = np.concatenate([base, partner, rng.uniform(-box / 2, box / 2, size=(1200, 3))])
    r = r.astype(np.float32).astype(np.float64)
    s = O.System(len(r), box)
    s.rx[:], s.ry[:], s.rz[:] = r.T
    opi, opj = s.pairs(2.5, 0.3)
    kpi, kpj = kdtree_reference_pairs(r, box, 2.5, 0.3)
    assert len(opi) > 1000
    assert np.array_equal(opi, kpi) and np.array_equal(opj, kpj)
