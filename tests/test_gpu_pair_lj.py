"""Point-particle pair forces on the device against the oracle."""
import numpy as np
import pytest

import oracle as O
from helpers import Pair, lj_fcc, jittered_fcc, rel, per_particle_max
from sucrose_gb300 import capi

pytestmark = pytest.mark.gpu

KINDS = [(capi.LJ, O.LJ, {}), (capi.LJ12, O.LJ12, {}), (capi.LJW, O.LJW, {"wf": 0.2}), (capi.WCA, O.WCA, {})]


def run(P, kind_dev, kind_or, kw, cutoff=2.5, skin=0.3):
    P.g.init_nlist(skin, cutoff)
    P.g.zero_forces()
    pe, vir = P.g.pair_forces(P.g.params(kind_dev, cutoff=cutoff, **kw))
    F, _ = P.g.forces()
    pi, pj = P.o.pairs(cutoff, skin)
    P.o.zero_forces()
    P.o.forces(O.pair_params(kind_or, cutoff=cutoff, **kw), pi, pj)
    Fo, _ = P.oracle_forces()
    return pe, F, P.o.s.pot_eng, Fo


@pytest.mark.parametrize("kd,ko,kw", KINDS)
def test_lj_family_jittered(lib, kd, ko, kw):
    r, q, box = jittered_fcc(6, 0.8442, seed=4, amp=0.1)
    P = Pair(r, q, box)
    pe, F, peo, Fo = run(P, kd, ko, kw)
    assert rel(F, Fo) < 1e-5
    assert abs(pe - peo) <= 1e-5 * max(abs(peo), 1e-12) + 1e-9
    # per-particle relative error with a floor of 1e-3 rms|F|: diagnostic bound
    assert per_particle_max(F, Fo) < 5e-4


def test_lj_readme_case(lib):
    # README example state (FCC, rho 0.8442, T 0.722, seed 15) after some
    # thermal displacement so that forces are non-zero
    r, q, box, v = lj_fcc()
    P = Pair(r + 0.05 * v, q, box)
    pe, F, peo, Fo = run(P, capi.LJ, O.LJ, {})
    assert rel(F, Fo) < 1e-5
    assert abs(pe - peo) <= 1e-5 * abs(peo)


def test_lj_newton_third_law(lib):
    r, q, box = jittered_fcc(10, 0.8, seed=9, amp=0.1)
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    P.g.zero_forces()
    P.g.pair_forces(P.g.params(capi.LJ, cutoff=2.5))
    F, _ = P.g.forces()
    assert np.linalg.norm(F.sum(0)) < 1e-4 * np.sqrt((F ** 2).sum())


def test_accumulates_like_the_user_loop(lib):
    # two calls add up, exactly as the README loop sums two potentials
    r, q, box = jittered_fcc(6, 0.8442, seed=4, amp=0.1)
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    P.g.zero_forces()
    pe1, _ = P.g.pair_forces(P.g.params(capi.LJ, cutoff=2.5))
    pe2, _ = P.g.pair_forces(P.g.params(capi.WCA, sigma=1.1))
    F, _ = P.g.forces()
    e = P.g.energies()
    assert abs(e[0] - (pe1 + pe2)) < 1e-9 * max(1.0, abs(e[0]))
    pi, pj = P.o.pairs(2.5, 0.3)
    P.o.zero_forces()
    P.o.forces(O.pair_params(O.LJ, cutoff=2.5), pi, pj)
    P.o.forces(O.pair_params(O.WCA, sigma=1.1), pi, pj)
    Fo, _ = P.oracle_forces()
    assert rel(F, Fo) < 1e-5
