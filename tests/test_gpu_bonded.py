"""Bonded terms (module bonded) on the device against the oracle, and a
polymer step with bonded terms, WCA and RATTLE bonds in one captured graph.
Tolerances: forces norm-wise relative 1e-5, energies 1e-5 relative."""
import numpy as np
import pytest

import oracle as O
from helpers import Pair, rel
from sucrose_gb300 import capi
from sucrose_gb300.molecules import polymer_chains

pytestmark = pytest.mark.gpu
KINDS = [capi.BEND, capi.DIH, capi.COSINE_BEND, capi.COSINE_DIH, capi.ANGLE_BEND, capi.ANGLE_DIH]


def chains(seed=2, jitter=0.12):
    r, box, bonds, bends, dihs = polymer_chains((2, 4, 4), 12, seed, jitter=jitter)
    return Pair(r, None, box), bonds, bends, dihs


@pytest.mark.parametrize("kind", KINDS)
def test_bonded_parity(lib, kind):
    P, bonds, bends, dihs = chains(seed=3 + kind)
    atoms = dihs if kind in (capi.DIH, capi.COSINE_DIH, capi.ANGLE_DIH) else bends
    rng = np.random.default_rng(kind)
    coeff = rng.uniform(0.5, 2.0, len(atoms))
    angle = rng.uniform(100.0, 160.0, len(atoms)) if kind >= capi.COSINE_BEND else None
    P.g.zero_forces()
    P.g.bonded_set(kind, atoms, coeff, angle)
    pe = P.g.bonded_forces(kind)
    F, _ = P.g.forces()
    P.o.zero_forces()
    P.o.bonded_forces(kind, atoms, coeff, angle)
    Fo, _ = P.oracle_forces()
    assert np.linalg.norm(Fo) > 0
    assert rel(F, Fo) < 1e-5
    assert abs(pe - P.o.s.pot_eng) <= 1e-5 * abs(P.o.s.pot_eng) + 1e-7 * len(atoms)
    # internal forces: the total vanishes
    assert np.linalg.norm(F.sum(0)) < 1e-4 * np.linalg.norm(F)


@pytest.mark.parametrize("kind", [capi.DIH, capi.COSINE_DIH])
def test_dihedral_near_straight_bend(lib, kind):
    # one bend of each dihedral straight to within 3e-5 to 3e-4 rad: the FP32
    # dihedral stays finite and matches the FP64 oracle (forces of order
    # 1 / angle there, and FP32 brackets with errors of order 1e-7 / angle,
    # hence the looser bound)
    rng = np.random.default_rng(21)
    quads = []
    for k, eps in enumerate(np.geomspace(3e-5, 3e-4, 12)):
        o = np.array([8.0 * k - 40.0, 0.0, 0.0])
        a = o + np.array([0.0, 0.0, 0.0])
        b = a + np.array([1.0, 0.0, 0.0])
        c = b + np.array([np.cos(eps), np.sin(eps), 0.0])          # bend a-b-c straight to within eps
        ang = rng.uniform(0.5, 2.5)
        d = c + np.array([0.3, np.cos(ang), np.sin(ang)])
        quads.append([a, b, c, d])
    r = np.concatenate(quads)
    P = Pair(r, None, 100.0)
    atoms = np.arange(len(r)).reshape(-1, 4)
    angle = np.full(len(atoms), 150.0) if kind == capi.COSINE_DIH else None
    P.g.zero_forces()
    P.g.bonded_set(kind, atoms, 1.0, angle)
    pe = P.g.bonded_forces(kind)
    F, _ = P.g.forces()
    assert np.isfinite(pe) and np.all(np.isfinite(F))
    P.o.zero_forces()
    P.o.bonded_forces(kind, atoms, np.ones(len(atoms)), angle)
    Fo, _ = P.oracle_forces()
    assert rel(F, Fo) < 2e-2
    assert abs(pe - P.o.s.pot_eng) <= 1e-4 * max(1.0, abs(P.o.s.pot_eng))


def test_angle_bend_near_parallel_bonds(lib):
    # angle_bend_ with the two bond vectors parallel to within 3e-5 to 3e-4
    # rad (a straight chain): finite, and the FP64 oracle's energy and forces
    rng = np.random.default_rng(22)
    tri = []
    for k, eps in enumerate(np.geomspace(3e-5, 3e-4, 12)):
        a = np.array([8.0 * k - 40.0, 0.0, 0.0])
        b = a + np.array([1.0, 0.0, 0.0])
        ax = rng.normal(size=3)
        ax -= ax[0] * np.array([1.0, 0.0, 0.0])
        ax /= np.linalg.norm(ax)
        c = b + np.cos(eps) * np.array([1.0, 0.0, 0.0]) + np.sin(eps) * ax
        tri.append([a, b, c])
    r = np.concatenate(tri)
    P = Pair(r, None, 100.0)
    atoms = np.arange(len(r)).reshape(-1, 3)
    angle = np.full(len(atoms), 60.0)
    P.g.zero_forces()
    P.g.bonded_set(capi.ANGLE_BEND, atoms, 2.0, angle)
    pe = P.g.bonded_forces(capi.ANGLE_BEND)
    F, _ = P.g.forces()
    assert np.isfinite(pe) and np.all(np.isfinite(F))
    P.o.zero_forces()
    P.o.bonded_forces(capi.ANGLE_BEND, atoms, np.full(len(atoms), 2.0), angle)
    Fo, _ = P.oracle_forces()
    assert rel(F, Fo) < 2e-2
    assert abs(pe - P.o.s.pot_eng) <= 1e-4 * max(1.0, abs(P.o.s.pot_eng))


def test_bonded_one_based_indices(lib):
    P, bonds, bends, dihs = chains()
    P.g.zero_forces()
    P.g.bonded_set(capi.BEND, bends + 1, 1.3, one_based=True)
    pe1 = P.g.bonded_forces(capi.BEND)
    P.g.zero_forces()
    P.g.bonded_set(capi.BEND, bends, 1.3)
    pe0 = P.g.bonded_forces(capi.BEND)
    assert pe1 == pytest.approx(pe0, rel=1e-12)


def test_polymer_step_bonded_wca_rattle(lib):
    P, bonds, bends, dihs = chains(seed=9, jitter=0.05)
    sig, dt = 0.9, 0.002
    P.g.set_constraints(bonds[:, 0], bonds[:, 1], 1.0)
    P.o.set_constraints(bonds[:, 0], bonds[:, 1], 1.0)
    P.g.bonded_set(capi.COSINE_BEND, bends, 4.0, 120.0)
    P.g.bonded_set(capi.ANGLE_DIH, dihs, 0.5, 180.0)
    P.g.init_nlist(0.3, sig)
    P.g.zero_forces()
    P.g.pair_forces(P.g.params(capi.WCA, sigma=sig, cutoff=sig))
    P.g.bonded_forces(capi.COSINE_BEND)
    P.g.bonded_forces(capi.ANGLE_DIH)

    def oracle_forces():
        P.o.zero_forces()
        pi, pj = P.o.pairs(sig, 0.3)
        P.o.forces(O.pair_params(O.WCA, sigma=sig, cutoff=sig), pi, pj)
        P.o.bonded_forces(O.COSINE_BEND, bends, 4.0, 120.0)
        P.o.bonded_forces(O.ANGLE_DIH, dihs, 0.5, 180.0)

    oracle_forces()
    F, _ = P.g.forces()
    Fo, _ = P.oracle_forces()
    assert rel(F, Fo) < 1e-5
    P.g.configure_step(P.g.params(capi.WCA, sigma=sig, cutoff=sig), integrator=capi.INT_NVE, dt=dt,
                       flags=capi.STEP_CONSTRAINTS | capi.STEP_BONDED)
    P.g.step(3)
    P.g.step_check()
    for _ in range(3):
        P.o.constraints_save()
        P.o.vv_initial(dt)
        assert P.o.constraints_a(dt) == 0
        oracle_forces()
        P.o.vv_final(dt)
        P.o.constraints_b(dt)
    r, q, v, l = P.g.download()
    vo = np.stack([P.o.vx, P.o.vy, P.o.vz], 1)
    assert rel(v, vo) < 5e-3
    ro = np.stack([P.o.rx, P.o.ry, P.o.rz], 1)
    dr = r - ro
    dr -= P.box * np.round(dr / P.box)
    assert np.max(np.abs(dr)) < 1e-4
