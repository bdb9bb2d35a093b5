"""The oracle's RATTLE restatement (apply_constraints_a / _b,
fortran/system.f90:1055-1210): a line-by-line numpy transcription of the
Fortran, the constraint and momentum properties, and the molecule-by-molecule
evaluation order the device uses giving the same FP64 result as the
reference's single global loop. CPU only."""
import numpy as np
import pytest

import oracle as O
from sucrose_gb300.molecules import molecular_mix


def make(seed=3, cells=3, spacing=3.0, v_scale=1.5):
    r, box, bbi, bbj, ln, mol = molecular_mix(cells, spacing, seed)
    n = len(r)
    rng = np.random.default_rng(seed)
    s = O.System(n, box)
    s.rx[:], s.ry[:], s.rz[:] = r.T
    v = rng.normal(size=(n, 3)) * v_scale
    s.vx[:], s.vy[:], s.vz[:] = v.T
    f = rng.normal(size=(n, 3)) * 5.0
    s.fx[:], s.fy[:], s.fz[:] = f.T
    s.set_constraints(bbi, bbj, ln)
    return s, bbi, bbj, ln, mol


def min_img(d, box):
    return d - np.round(d / box) * box   # ties never occur here


def rattle_a_numpy(r, v, r_old, im, box, bbi, bbj, ln, dt, groups=None):
    """Transcription of apply_constraints_a. groups: run the same loop on each
    molecule's constraints separately (the device's order) instead of once
    over the whole list."""
    r, v = r.copy(), v.copy()
    vir = 0.0
    for idx in (groups if groups is not None else [np.arange(len(bbi))]):
        moved = np.ones(len(r), dtype=bool)
        if groups is not None:   # only this molecule's atoms can be flagged
            moved[:] = False
            moved[bbi[idx]] = True
            moved[bbj[idx]] = True
        rattle = 0
        while moved.any() and rattle < 100:
            for ix in idx:
                i, j, L = bbi[ix], bbj[ix], ln[ix]
                if moved[i] or moved[j]:
                    rij = min_img(r[i] - r[j], box)
                    chi = L ** 2 - np.sum(rij ** 2)
                    if abs(chi) > 2 * 1e-5 * L ** 2:
                        ro = min_img(r_old[i] - r_old[j], box)
                        vdot = rij[0] * ro[0] + rij[1] * ro[1] + rij[2] * ro[2]
                        assert vdot >= 1e-5 * L ** 2
                        lij = chi / (2.0 * vdot * (im[i] + im[j]))
                        vir += (lij * L ** 2) / dt ** 2
                        r[i] += (lij * im[i]) * ro
                        r[j] -= (lij * im[j]) * ro
                        v[i] += (lij * im[i]) * ro / dt
                        v[j] -= (lij * im[j]) * ro / dt
                        moved[i] = moved[j] = True
                    else:
                        moved[i] = moved[j] = False
            rattle += 1
    return r, v, vir


def state(s):
    return (np.stack([s.rx, s.ry, s.rz], 1).copy(), np.stack([s.vx, s.vy, s.vz], 1).copy())


def test_rattle_a_matches_transcription_and_molecule_order():
    s, bbi, bbj, ln, mol = make()
    dt = 0.005
    s.constraints_save()
    r_old = np.stack([s.rx_old, s.ry_old, s.rz_old], 1).copy()
    s.vv_initial(dt)
    r0, v0 = state(s)
    assert s.constraints_a(dt) == 0
    r1, v1 = state(s)
    rt, vt, vir = rattle_a_numpy(r0, v0, r_old, s.inv_mass, s.box, bbi, bbj, ln, dt)
    assert np.array_equal(r1, rt) and np.array_equal(v1, vt)
    assert s.s.virial_bonded == pytest.approx(vir, rel=1e-13)
    # the same sweeps run molecule by molecule (one device thread each) give
    # the same FP64 numbers as the single global loop
    cmol = mol[bbi]
    groups = [np.nonzero(cmol == m)[0] for m in np.unique(cmol)]
    rg, vg, virg = rattle_a_numpy(r0, v0, r_old, s.inv_mass, s.box, bbi, bbj, ln, dt, groups=groups)
    assert np.array_equal(rg, r1) and np.array_equal(vg, v1)
    assert virg == pytest.approx(vir, rel=1e-12)


def test_rattle_a_satisfies_constraints_and_keeps_momentum():
    s, bbi, bbj, ln, _ = make(seed=5)
    dt = 0.005
    p0 = None
    s.constraints_save()
    s.vv_initial(dt)
    p0 = np.stack([s.vx, s.vy, s.vz], 1).sum(0)
    assert s.constraints_a(dt) == 0
    r, v = state(s)
    d = min_img(r[bbi] - r[bbj], s.box)
    assert np.all(np.abs(ln ** 2 - np.sum(d ** 2, 1)) <= 2e-5 * ln ** 2 + 1e-12)
    assert np.allclose(v.sum(0), p0, atol=1e-10)
    # atoms in no constraint keep their initial moved flag, so the reference's
    # any(moved) loop always runs the full 100 sweeps when there are any
    assert s.s.rattle_sweeps == 100


def test_rattle_b_removes_bond_velocity():
    s, bbi, bbj, ln, _ = make(seed=7)
    dt = 0.005
    s.constraints_save()
    s.vv_initial(dt)
    s.constraints_a(dt)
    s.vv_final(dt)
    p0 = np.stack([s.vx, s.vy, s.vz], 1).sum(0)
    s.constraints_b(dt)
    r, v = state(s)
    d = min_img(r[bbi] - r[bbj], s.box)
    vd = np.sum(d * (v[bbi] - v[bbj]), 1)
    # |L| <= r_tol after the last sweep: |r.v| <= r_tol (1/m_i + 1/m_j) len^2
    assert np.all(np.abs(vd) <= 1e-5 * 2.0 * ln ** 2 + 1e-12)
    assert np.allclose(v.sum(0), p0, atol=1e-10)


def test_constraint_failure_is_reported():
    # a dimer whose atoms cross during the drift: the new bond vector opposes
    # the old one and the reference stops (system.f90:1102-1106)
    s = O.System(2, 20.0)
    s.rx[:] = [0.5, -0.5]
    s.vx[:] = [-80.0, 80.0]
    s.set_constraints([0], [1], [1.0])
    s.constraints_save()
    s.vv_initial(0.01)
    assert s.constraints_a(0.01) == 1


def test_virial_bonded_joins_thermo():
    s, bbi, bbj, ln, _ = make(seed=9)
    dt = 0.005
    s.constraints_save()
    s.vv_initial(dt)
    s.constraints_a(dt)
    s.vv_final(dt)
    s.constraints_b(dt)
    s.s.dof = 6 * s.n - len(bbi)
    s.s.density = 0.1
    vb = s.s.virial_bonded
    s.thermo()
    base = np.sum(s.rx * s.fx + s.ry * s.fy + s.rz * s.fz)
    want = base + vb if vb >= 0 else base
    assert s.s.virial == pytest.approx(want, rel=1e-13)
