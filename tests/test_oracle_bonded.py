"""The oracle's bonded terms (module bonded, fortran/force.f90:2238-2581)
pinned by known answers and gradients. bend_, dih_, angle_bend_ and
angle_dih_ return F = -grad PE. cosine_bend_ and cosine_dih_ reuse the bend
and dihedral force expressions with strength = dPE/dcos where those carry
-dPE/dcos, so their forces are +grad PE (they push away from the target
angle): a reference quirk the oracle keeps and these tests pin. CPU only."""
import numpy as np
import pytest

import oracle as O

KINDS = [(O.BEND, 3, -1), (O.DIH, 4, -1), (O.COSINE_BEND, 3, +1), (O.COSINE_DIH, 4, +1), (O.ANGLE_BEND, 3, -1),
         (O.ANGLE_DIH, 4, -1)]


def system(r, periodic=False, box=50.0):
    s = O.System(len(r), box, periodic=periodic)
    s.rx[:], s.ry[:], s.rz[:] = np.asarray(r, dtype=np.float64).T
    return s


def numgrad(r, kind, nat, coeff, angle, h=1e-6):
    G = np.zeros((nat, 3))
    for a in range(nat):
        for d in range(3):
            e = []
            for sg in (1, -1):
                x = r.copy()
                x[a, d] += sg * h
                e.append(system(x).bonded(kind, np.arange(nat), coeff, angle)[0])
            G[a, d] = (e[0] - e[1]) / (2 * h)
    return G


@pytest.mark.parametrize("kind,nat,sign", KINDS)
def test_force_is_signed_gradient(kind, nat, sign):
    rng = np.random.default_rng(10 + kind)
    for _ in range(3):
        r = rng.uniform(0, 2, (nat, 3))
        pe, F = system(r).bonded(kind, np.arange(nat), 1.7, 70.0)
        G = numgrad(r, kind, nat, 1.7, 70.0)
        assert np.allclose(F[:nat], sign * G, rtol=1e-6, atol=1e-8)
        # the terms are internal: the forces sum to zero
        assert np.allclose(F[:nat].sum(0), 0.0, atol=1e-12)


def bent(angle_deg, l1=1.1, l2=0.9):
    a = np.radians(angle_deg)
    return np.array([[l1, 0, 0], [0, 0, 0], [l2 * np.cos(a), l2 * np.sin(a), 0]])


def test_bend_known_answers():
    # straight chain: the bond vectors are parallel, PE = 0; right angle: PE = coeff
    s = system(np.array([[0, 0, 0], [1.0, 0, 0], [2.3, 0, 0]]))
    assert s.bonded(O.BEND, [0, 1, 2], 2.0)[0] == pytest.approx(0.0, abs=1e-15)
    assert system(bent(90.0)).bonded(O.BEND, [0, 1, 2], 2.0)[0] == pytest.approx(2.0, rel=1e-14)


@pytest.mark.parametrize("kind", [O.COSINE_BEND, O.ANGLE_BEND])
def test_bend_minimum_at_target_angle(kind):
    # theta0 = pi - angle: the energy vanishes at bond angle I-J-K = angle
    pe, F = system(bent(109.5)).bonded(kind, [0, 1, 2], 3.0, 109.5)
    assert pe == pytest.approx(0.0, abs=1e-20)
    assert np.allclose(F, 0.0, atol=1e-12)
    pe2, _ = system(bent(100.0)).bonded(kind, [0, 1, 2], 3.0, 109.5)
    if kind == O.ANGLE_BEND:
        assert pe2 == pytest.approx(1.5 * np.radians(9.5) ** 2, rel=1e-12)
    else:
        assert pe2 == pytest.approx(1.5 * (np.cos(np.radians(80.0)) - np.cos(np.radians(70.5))) ** 2, rel=1e-12)


def dihedral(phi_deg):
    """Four atoms with the I-J-K-L dihedral phi (0 = cis, 180 = trans)."""
    p = np.radians(phi_deg)
    return np.array([[1.0, 1.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 0.0], [np.cos(p), 0.0, np.sin(p)]])


def test_dihedral_known_answers():
    for phi in (0.0, 60.0, -60.0, 120.0, 180.0):
        s = system(dihedral(phi))
        # dih_: coeff (1 + prefac fac) = coeff (1 + cos phi)
        assert s.bonded(O.DIH, [0, 1, 2, 3], 1.0)[0] == pytest.approx(1.0 + np.cos(np.radians(phi)), abs=1e-12)
        # angle_dih_: coeff (1 - cos(phi' - phi0)) with phi0 = pi - angle: zero at angle = phi
        assert s.bonded(O.ANGLE_DIH, [0, 1, 2, 3], 1.0, phi)[0] == pytest.approx(0.0, abs=1e-12)
        assert s.bonded(O.ANGLE_DIH, [0, 1, 2, 3], 1.0, phi + 90.0)[0] == pytest.approx(1.0, abs=1e-12)
