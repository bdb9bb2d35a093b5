"""The oracle's Morse and charged-particle restatements (morse_, dh_,
coulombic_, dipole_ with the reaction field) pinned against the reference's
C++ Morse, known answers, gradients and a line-by-line numpy transcription of
the Fortran. CPU only."""
import os

import numpy as np
import pytest

import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FOUR_PI = 4.0 * np.pi


def two_body(r_i, r_j, qi=1.0, qj=1.0, quat_i=(1, 0, 0, 0), quat_j=(1, 0, 0, 0), box=50.0, periodic=False):
    s = O.System(2, box, periodic=periodic)
    s.rx[:], s.ry[:], s.rz[:] = np.array([r_i, r_j], dtype=np.float64).T
    s.qw[:], s.qx[:], s.qy[:], s.qz[:] = np.array([quat_i, quat_j], dtype=np.float64).T
    s.charge[:] = (qi, qj)
    return s


def pair(s, params):
    out, _ = s.pair(0, 1, params)
    return out[0], out[1:4], out[4:7], out[7:10]


# ------------------------------------------------------------------ Morse ---
def test_morse_matches_reference_cpp_golden():
    g = np.load(os.path.join(GOLD, "ref_morse.npz"))
    r, L = g["r"], float(g["box"])
    s = O.System(len(r), L)
    s.rx[:], s.ry[:], s.rz[:] = r.T
    pi, pj = np.triu_indices(len(r), 1)
    # the C++ MorsePotential has no cutoff and no shift: morse_ with an infinite cutoff
    s.forces(O.pair_params(O.MORSE, cutoff=np.inf, dissoc=float(g["D"]), rmin=float(g["r0"]),
                           width=float(g["alpha"])), pi, pj)
    F = np.stack([s.fx, s.fy, s.fz], 1)
    Fr = np.stack([g["fx"], g["fy"], g["fz"]], 1)
    assert np.linalg.norm(F - Fr) <= 1e-12 * np.linalg.norm(Fr)
    assert abs(s.s.pot_eng - float(g["pot"])) <= 1e-12 * abs(float(g["pot"]))


def test_morse_known_answer_and_shift():
    D, a, r0, rc = 2.0, 1.5, 1.2, 3.0
    for r in (0.9, 1.2, 2.0, 2.99, 3.0, 3.5):
        s = two_body((0, 0, 0), (r, 0, 0))
        pe, f, _, _ = pair(s, O.pair_params(O.MORSE, cutoff=rc, dissoc=D, width=a, rmin=r0))
        if r < rc:
            e, ec = np.exp(-a * (r - r0)), np.exp(-a * (rc - r0))
            want = D * ((1 - e) ** 2 - 1) - D * ((1 - ec) ** 2 - 1)
            assert pe == pytest.approx(want, rel=1e-14, abs=1e-15)
            # r_ij = r_i - r_j = (-r, 0, 0): the force on I is along -x times -dU/dr
            dudr = 2 * D * a * (1 - e) * e
            assert f[0] == pytest.approx(dudr, rel=1e-13, abs=1e-15)
        else:
            assert pe == 0.0 and not f.any()
    # the well minimum: zero force at r0
    s = two_body((0, 0, 0), (r0, 0, 0))
    assert abs(pair(s, O.pair_params(O.MORSE, cutoff=rc, dissoc=D, width=a, rmin=r0))[1][0]) < 1e-15


# ---------------------------------------------------------- Debye-Hueckel ---
def test_dh_known_answer():
    qi, qj, db, diel, rc = 1.5, -0.75, 1.3, 2.5, 4.0
    for r in (0.6, 1.0, 3.9, 4.0):
        s = two_body((0, 0, 0), (0, r, 0), qi, qj)
        pe, f, _, _ = pair(s, O.pair_params(O.DH, cutoff=rc, db_len=db, dielectric=diel))
        if r < rc:
            want = qi * qj * np.exp(-r / db) / (FOUR_PI * diel * r)
            assert pe == pytest.approx(want, rel=1e-14)
            assert f[1] == pytest.approx(want * (1 + r / db) * (-r) / r ** 2, rel=1e-13)
            assert f[0] == 0.0 and f[2] == 0.0
        else:
            assert pe == 0.0 and not f.any()


def test_dh_force_is_minus_gradient():
    rng = np.random.default_rng(3)
    ri, rj = rng.uniform(0, 2, 3), rng.uniform(0, 2, 3)
    p = O.pair_params(O.DH, cutoff=10.0, db_len=0.9, dielectric=1.7)
    s = two_body(ri, rj, 0.8, 1.1)
    _, f, _, _ = pair(s, p)
    h = 1e-6
    for d in range(3):
        e = []
        for sgn in (1, -1):
            x = ri.copy()
            x[d] += sgn * h
            e.append(pair(two_body(x, rj, 0.8, 1.1), p)[0])
        assert -(e[0] - e[1]) / (2 * h) == pytest.approx(f[d], rel=1e-7, abs=1e-9)


# --------------------------------------------------------------- Coulomb ---
def coulomb_numpy(rij, qi, qj, rc, diel):
    """Line-by-line numpy transcription of coulombic_calculate_forces (force.f90:2627-2665)."""
    rsq = np.sum(rij * rij)
    r = np.sqrt(rsq)
    switch = rc - 2.0
    factor = 1.0 / (rc - switch)
    xx = (r - switch) * factor
    sx = 1.0 - 6.0 * xx ** 5 + 15.0 * xx ** 4 - 10.0 * xx ** 3
    sdx = -30.0 * xx ** 4 + 60.0 * xx ** 3 - 30.0 * xx ** 2
    pe, f = 0.0, np.zeros(3)
    if r < rc:
        pe = qi * qj / (4.0 * np.pi * diel * r)
        f = pe * rij / rsq
        if r >= switch:
            pe = sx * pe
            f = sx * f - sdx * pe * factor
    return pe, f


@pytest.mark.parametrize("r", [0.7, 1.5, 2.0, 2.4, 3.2, 3.99, 4.0, 4.2])
def test_coulomb_against_transcription(r):
    rc, diel = 4.0, 3.0
    d = np.array([0.3, -0.5, 0.81])
    d = r * d / np.linalg.norm(d)
    s = two_body((0, 0, 0), d, -1.0, 0.6)
    pe, f, _, _ = pair(s, O.pair_params(O.COULOMB, cutoff=rc, dielectric=diel))
    pe_t, f_t = coulomb_numpy(-d, -1.0, 0.6, rc, diel)
    assert pe == pytest.approx(pe_t, rel=1e-13, abs=1e-16)
    assert np.allclose(f, f_t, rtol=1e-13, atol=1e-16)


def test_coulomb_switch_term_is_per_component():
    # inside the switch band the reference subtracts the scalar sdx PE factor
    # from each Cartesian component: the force is not central there
    rc = 4.0
    d = np.array([2.7, 0.4, -0.9])
    s = two_body((0, 0, 0), d, 1.0, 1.0)
    _, f, _, _ = pair(s, O.pair_params(O.COULOMB, cutoff=rc, dielectric=1.0))
    rij = -d
    cos = f @ rij / (np.linalg.norm(f) * np.linalg.norm(rij))
    assert abs(abs(cos) - 1.0) > 1e-3
    # below the switch it is the plain central Coulomb force
    d2 = np.array([1.2, 0.4, -0.9])
    _, f2, _, _ = pair(two_body((0, 0, 0), d2, 1.0, 1.0), O.pair_params(O.COULOMB, cutoff=rc, dielectric=1.0))
    assert np.allclose(np.cross(f2, -d2), 0.0, atol=1e-15)


# ---------------------------------------------------------------- dipole ---
def quat_axis_angle(axis, ang):
    axis = np.asarray(axis, dtype=np.float64)
    axis = axis / np.linalg.norm(axis)
    return np.concatenate([[np.cos(ang / 2)], np.sin(ang / 2) * axis])


def qmul(a, b):
    w1, x1, y1, z1 = a
    w2, x2, y2, z2 = b
    return np.array([w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2, w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
                     w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2])


def body_z(q):
    w, x, y, z = q
    return np.array([2 * (x * z + w * y), 2 * (y * z - w * x), w * w - x * x - y * y + z * z])


def test_dipole_energy_known_answer():
    # head-to-tail along z: E = -2 mu1 mu2 / r^3; side by side parallel: +mu1 mu2 / r^3
    mu1, mu2, r = 1.2, 0.7, 1.9
    p = O.pair_params(O.DIPOLE, cutoff=5.0, dielectric=1.0)
    pe, _, _, _ = pair(two_body((0, 0, 0), (0, 0, r), mu1, mu2), p)
    assert pe == pytest.approx(-2 * mu1 * mu2 / r ** 3, rel=1e-14)
    pe, _, _, _ = pair(two_body((0, 0, 0), (r, 0, 0), mu1, mu2), p)
    assert pe == pytest.approx(mu1 * mu2 / r ** 3, rel=1e-14)


def test_dipole_force_and_torque_are_gradients():
    rng = np.random.default_rng(11)
    ri, rj = rng.uniform(0, 1.5, 3), rng.uniform(0, 1.5, 3) + 1.0
    qi = quat_axis_angle(rng.normal(size=3), 1.1)
    qj = quat_axis_angle(rng.normal(size=3), -0.7)
    p = O.pair_params(O.DIPOLE, cutoff=10.0, dielectric=1.0)

    def energy(ri_, qi_, qj_):
        return pair(two_body(ri_, rj, 0.9, 1.3, qi_, qj_), p)[0]

    _, f, ti, tj = pair(two_body(ri, rj, 0.9, 1.3, qi, qj), p)
    h = 1e-6
    for d in range(3):
        e = np.eye(3)[d]
        assert -(energy(ri + h * e, qi, qj) - energy(ri - h * e, qi, qj)) / (2 * h) == pytest.approx(
            f[d], rel=1e-6, abs=1e-9)
        # a space-frame rotation by h about e changes E by -tau.e h
        rp, rm = quat_axis_angle(e, h), quat_axis_angle(e, -h)
        gi = -(energy(ri, qmul(rp, qi), qj) - energy(ri, qmul(rm, qi), qj)) / (2 * h)
        gj = -(energy(ri, qi, qmul(rp, qj)) - energy(ri, qi, qmul(rm, qj))) / (2 * h)
        assert gi == pytest.approx(ti[d], rel=1e-6, abs=1e-9)
        assert gj == pytest.approx(tj[d], rel=1e-6, abs=1e-9)


def test_reaction_field_against_transcription():
    """init_reaction_field, dipole pair loop, eval_reaction_field (force.f90:2677-2766)."""
    rng = np.random.default_rng(21)
    n, L, rc, diel = 40, 6.0, 2.5, 4.0
    r = rng.uniform(0, L, (n, 3))
    q = np.array([quat_axis_angle(rng.normal(size=3), rng.uniform(0, np.pi)) for _ in range(n)])
    ch = rng.choice([0.0, 0.5, 1.0, 1.5], n)
    s = O.System(n, L)
    s.rx[:], s.ry[:], s.rz[:] = r.T
    s.qw[:], s.qx[:], s.qy[:], s.qz[:] = q.T
    s.charge[:] = ch
    s.reaction_field_init()
    pi, pj = [a.astype(np.int32) for a in np.triu_indices(n, 1)]
    p = O.pair_params(O.DIPOLE, cutoff=rc, dielectric=diel)
    s.forces(p, pi, pj)
    s.forces(p, pi, pj)          # RFL keeps accumulating across calls
    pe_pairs = s.s.pot_eng
    t_pairs = np.stack([s.tx, s.ty, s.tz], 1).copy()
    s.reaction_field_eval()

    coeff = (2.0 * (diel - 1.0)) / (2.0 * diel + 1.0) / rc ** 3
    dip = np.zeros((n, 3))
    rfl = np.zeros(3)
    for _ in range(2):
        for i, j in zip(pi, pj):
            d = r[i] - r[j]
            d -= np.round(d / L) * L
            if np.sqrt(d @ d) < rc:
                dip[i] = body_z(q[i]) * ch[i]
                rfl += body_z(q[j]) * ch[j] * coeff
    assert np.allclose(s.rfl, rfl, rtol=1e-13, atol=1e-15)
    assert np.allclose(np.stack([s.dipx, s.dipy, s.dipz], 1), dip, rtol=1e-13, atol=1e-15)
    on = ch != 0.0
    e_rf = 0.5 * np.sum(dip[on] @ rfl)
    assert s.s.pot_eng - pe_pairs == pytest.approx(e_rf, rel=1e-12, abs=1e-15)
    t_rf = np.zeros((n, 3))
    t_rf[on] = -np.cross(dip[on], rfl)
    assert np.allclose(np.stack([s.tx, s.ty, s.tz], 1) - t_pairs, t_rf, rtol=1e-10, atol=1e-14)
