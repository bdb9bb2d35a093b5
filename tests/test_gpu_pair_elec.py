"""Morse and charged pair potentials (morse_, dh_, coulombic_, dipole_ and the
reaction field) on the device against the oracle, same FP32-rounded state.

Tolerances: forces and torques norm-wise relative 1e-5. Energies 1e-5
relative to max(|E|, 0.1 sum|E_pair|): with mixed-sign charges the total is a
sum with cancellation, whose FP32-per-pair rounding is bounded by the sum of
magnitudes rather than by the total."""
import numpy as np
import pytest

import oracle as O
from helpers import Pair, f32, jittered_fcc, per_particle_max, rel
from sucrose_gb300 import capi

pytestmark = pytest.mark.gpu


def mixed_charges(n, seed, positive=False):
    rng = np.random.default_rng(seed)
    vals = [0.5, 1.0, 1.5, 0.0] if positive else [-1.0, -0.5, 0.5, 1.0]
    return f32(rng.choice(vals, n))


def random_quats(n, seed):
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(n, 4))
    return q / np.linalg.norm(q, axis=1, keepdims=True)


def build(seed=4, charges=None, quats=False, cells=6, density=0.8442, amp=0.1):
    r, q, box = jittered_fcc(cells, density, seed=seed, amp=amp)
    if quats:
        q = random_quats(len(r), seed + 1)
    P = Pair(r, q, box)
    if charges is not None:
        P.o.charge[:] = charges
        P.g.set_charges(charges)
    return P


def oracle_pair_sums(P, params, pi, pj):
    """sum |PE_pair| and the pair virial sum r_ij . F_ij from per-pair outputs."""
    out = P.o.pair_batch(params, pi, pj)
    d = P.r[pi] - P.r[pj]
    d -= P.box * np.round(d / P.box)
    return np.abs(out[:, 0]).sum(), float(np.sum(d * out[:, 1:4]))


def run(P, kind_dev, kind_or, cutoff, skin=0.3, **kw):
    P.g.init_nlist(skin, cutoff)
    P.g.zero_forces()
    pe, vir = P.g.pair_forces(P.g.params(kind_dev, cutoff=cutoff, **kw))
    F, T = P.g.forces()
    pi, pj = P.o.pairs(cutoff, skin)
    P.o.zero_forces()
    po = O.pair_params(kind_or, cutoff=cutoff, **kw)
    P.o.forces(po, pi, pj)
    Fo, To = P.oracle_forces()
    sabs, viro = oracle_pair_sums(P, po, pi, pj)
    return dict(pe=pe, vir=vir, F=F, T=T, peo=P.o.s.pot_eng, Fo=Fo, To=To, sabs=sabs, viro=viro)


def check_energy(e, eo, sabs):
    assert abs(e - eo) <= 1e-5 * max(abs(eo), 0.1 * sabs, 1e-12)


CASES = [
    ("morse", capi.MORSE, O.MORSE, 2.5, dict(dissoc=1.3, width=1.7, rmin=1.1), False),
    ("debye_huckel", capi.DH, O.DH, 3.0, dict(db_len=1.0, dielectric=2.0), True),
    ("coulomb_switched", capi.COULOMB, O.COULOMB, 3.5, dict(dielectric=1.5), True),
    ("coulomb_short", capi.COULOMB, O.COULOMB, 2.2, dict(dielectric=0.8), True),
]


@pytest.mark.parametrize("name,kd,ko,rc,kw,charged", CASES, ids=[c[0] for c in CASES])
def test_point_pair_parity(lib, name, kd, ko, rc, kw, charged):
    n = 4 * 6 ** 3
    P = build(charges=mixed_charges(n, 9) if charged else None)
    o = run(P, kd, ko, rc, **kw)
    assert np.linalg.norm(o["Fo"]) > 0
    assert rel(o["F"], o["Fo"]) < 1e-5
    check_energy(o["pe"], o["peo"], o["sabs"])
    assert abs(o["vir"] - o["viro"]) <= 1e-5 * max(abs(o["viro"]), 1e-12) + 1e-5 * o["sabs"]
    assert per_particle_max(o["F"], o["Fo"]) < 5e-4


def test_point_pairs_filtered_launch_agrees(lib):
    # the range-filtered kernel variant gives the same forces
    n = 4 * 6 ** 3
    P = build(charges=mixed_charges(n, 5))
    P.g.set_launch(capi.COULOMB, 128, 1)
    o = run(P, capi.COULOMB, O.COULOMB, 3.5, dielectric=1.0)
    assert rel(o["F"], o["Fo"]) < 1e-5
    check_energy(o["pe"], o["peo"], o["sabs"])


def test_reference_default_charges(lib):
    # initialize_system turns negative charges into 0 (system.f90:595-598)
    n = 4 * 5 ** 3
    q = mixed_charges(n, 2)
    P = build(cells=5)
    P.g.set_charges(q, reference_defaults=True)
    P.o.charge[:] = np.maximum(q, 0.0)
    o = run(P, capi.DH, O.DH, 3.0, db_len=0.7, dielectric=1.0)
    assert rel(o["F"], o["Fo"]) < 1e-5
    check_energy(o["pe"], o["peo"], o["sabs"])


def test_morse_without_cutoff_is_the_cpp_potential(lib):
    # MorsePotential (src/force.cpp:113-140) = morse_ with an infinite cutoff
    P = build(cells=4)
    cutoff_list = 2.8
    P.g.init_nlist(0.2, cutoff_list)
    P.g.zero_forces()
    kw = dict(dissoc=0.9, width=2.1, rmin=1.05)
    pe, _ = P.g.pair_forces(P.g.params(capi.MORSE, cutoff=np.inf, **kw))
    F, _ = P.g.forces()
    pi, pj = P.o.pairs(cutoff_list, 0.2)
    P.o.zero_forces()
    P.o.forces(O.pair_params(O.MORSE, cutoff=np.inf, **kw), pi, pj)
    Fo, _ = P.oracle_forces()
    assert rel(F, Fo) < 1e-5
    assert abs(pe - P.o.s.pot_eng) <= 1e-5 * abs(P.o.s.pot_eng)


def test_dipole_and_reaction_field(lib):
    n = 4 * 6 ** 3
    P = build(charges=mixed_charges(n, 13, positive=True), quats=True, density=0.6)
    rc, diel = 3.0, 5.0
    P.g.reaction_field_init()
    P.o.reaction_field_init()
    o = run(P, capi.DIPOLE, O.DIPOLE, rc, dielectric=diel)
    assert rel(o["F"], o["Fo"]) < 1e-5
    assert rel(o["T"], o["To"]) < 1e-5
    check_energy(o["pe"], o["peo"], o["sabs"])
    rfl, dip = P.g.reaction_field()
    assert np.linalg.norm(rfl - P.o.rfl) <= 1e-5 * np.linalg.norm(P.o.rfl)
    assert rel(dip, np.stack([P.o.dipx, P.o.dipy, P.o.dipz], 1)) < 1e-6
    # a second call keeps accumulating RFL, as the reference's arrays do
    pi, pj = P.o.pairs(rc, 0.3)
    P.g.pair_forces(P.g.params(capi.DIPOLE, cutoff=rc, dielectric=diel))
    P.o.forces(O.pair_params(O.DIPOLE, cutoff=rc, dielectric=diel), pi, pj)
    rfl, _ = P.g.reaction_field()
    assert np.linalg.norm(rfl - P.o.rfl) <= 1e-5 * np.linalg.norm(P.o.rfl)
    # eval_reaction_field: energy and torques
    e_before = P.o.s.pot_eng
    e_rf = P.g.reaction_field_eval()
    P.o.reaction_field_eval()
    assert abs(e_rf - (P.o.s.pot_eng - e_before)) <= 1e-5 * abs(P.o.s.pot_eng - e_before)
    F, T = P.g.forces()
    Fo, To = P.oracle_forces()
    assert rel(T, To) < 1e-5
    assert rel(F, Fo) < 1e-5


def test_dipole_needs_reaction_field_init(lib):
    P = build(cells=3, charges=mixed_charges(108, 1, positive=True))
    P.g.init_nlist(0.3, 2.0)
    with pytest.raises(Exception) as e:
        P.g.pair_forces(P.g.params(capi.DIPOLE, cutoff=2.0, dielectric=2.0))
    assert e.value.code == capi.SG_ENOTREADY


def _oracle_nve_step(P, params, dt, rotations=False, rf=False, skin=0.3):
    o = P.o
    o.vv_initial(dt)
    if rotations:
        o.qq_initial(dt)
    o.zero_forces()
    for p, rc in params:
        pi, pj = o.pairs(rc, skin)
        o.forces(p, pi, pj)
    if rf:
        o.reaction_field_eval()
    o.vv_final(dt)
    if rotations:
        o.qq_final(dt)


def test_step_with_two_pair_sets(lib):
    # one captured step whose pair stage sums WCA and switched Coulomb
    n = 4 * 6 ** 3
    P = build(charges=mixed_charges(n, 17), amp=0.05)
    dt, rc = 0.001, 3.5
    P.g.init_nlist(0.3, rc)
    sets = [P.g.params(capi.WCA, sigma=1.0), P.g.params(capi.COULOMB, cutoff=rc, dielectric=1.0)]
    P.g.configure_step_pairs(sets, integrator=capi.INT_NVE, dt=dt)
    P.g.step(3)
    P.g.step_check()
    po = [(O.pair_params(O.WCA, sigma=1.0, cutoff=1.0), 1.0), (O.pair_params(O.COULOMB, cutoff=rc, dielectric=1.0), rc)]
    for _ in range(3):
        _oracle_nve_step(P, po, dt)
    r, q, v, l = P.g.download()
    vo = np.stack([P.o.vx, P.o.vy, P.o.vz], 1)
    assert rel(v, vo) < 1e-5
    ro = np.stack([P.o.rx, P.o.ry, P.o.rz], 1)
    dr = r - ro
    dr -= P.box * np.round(dr / P.box)
    assert np.max(np.abs(dr)) < 1e-5


def test_step_dipole_with_reaction_field(lib):
    n = 4 * 5 ** 3
    P = build(cells=5, charges=mixed_charges(n, 23, positive=True), quats=True, density=0.5, amp=0.05)
    dt, rc, diel = 0.001, 2.5, 3.0
    P.g.init_nlist(0.3, rc)
    P.g.reaction_field_init()
    P.o.reaction_field_init()
    P.g.configure_step(P.g.params(capi.DIPOLE, cutoff=rc, dielectric=diel), integrator=capi.INT_NVE, dt=dt,
                       rotations=1, flags=capi.STEP_REACTION_FIELD)
    P.g.step(2)
    P.g.step_check()
    for _ in range(2):
        _oracle_nve_step(P, [(O.pair_params(O.DIPOLE, cutoff=rc, dielectric=diel), rc)], dt, rotations=True, rf=True)
    r, q, v, l = P.g.download()
    assert rel(q, np.stack([P.o.qw, P.o.qx, P.o.qy, P.o.qz], 1)) < 1e-5
    assert rel(l, np.stack([P.o.lx, P.o.ly, P.o.lz], 1)) < 1e-5
    assert rel(v, np.stack([P.o.vx, P.o.vy, P.o.vz], 1)) < 1e-5
    rfl, _ = P.g.reaction_field()
    assert np.linalg.norm(rfl - P.o.rfl) <= 1e-5 * np.linalg.norm(P.o.rfl)
