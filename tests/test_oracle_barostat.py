"""The oracle's Monte Carlo barostat (mc_barostat, fortran/integrators.f90:
858-945) with Philox draws in place of random_number: the Metropolis
exponent, the scaling on acceptance and the exact restore on rejection. CPU
only."""
import numpy as np
import pytest

import oracle as O
from sucrose_gb300 import configs


def lj_system(cells=4, density=0.7, seed=3):
    r, q, box = configs.fcc_lattice(cells, density)
    rng = np.random.default_rng(seed)
    r = r + rng.normal(scale=0.05, size=r.shape)
    s = O.System(len(r), box)
    s.rx[:], s.ry[:], s.rz[:] = r.T
    return s


@pytest.mark.parametrize("counter", range(8))
def test_exponent_and_decision(counter):
    s = lj_system()
    pi, pj = s.pairs(2.5, 0.3)
    p = O.pair_params(O.LJ, cutoff=2.5)
    r0 = np.stack([s.rx, s.ry, s.rz], 1).copy()
    L0 = s.box.copy()
    T, P, dv = 1.2, 1.0, 0.02
    a, u_old, u_new, v_new = s.mc_barostat([p], pi, pj, P, T, dv, counter=counter)
    w = O.philox4x32(np.array([[counter, 0, 0x4D43, 0]], dtype=np.uint32))[0].astype(np.float64) / 2.0 ** 32
    v_old = np.prod(L0)
    assert v_new == v_old + dv * (2.0 * w[0] - 1.0) * v_old
    expo = -(u_new - u_old) / T - P * (v_new - v_old) / T + s.n * np.log(v_new / v_old)
    assert a == (1 if np.log(w[1]) < expo else 0)
    r1 = np.stack([s.rx, s.ry, s.rz], 1)
    if a == 1:
        sc = (v_new / v_old) ** (1.0 / 3.0)
        assert np.allclose(s.box, L0 * sc, rtol=1e-15)
        assert np.allclose(r1, r0 * sc, rtol=1e-15)
        assert s.s.density == pytest.approx(s.n / v_new, rel=1e-14)
    else:
        assert np.array_equal(s.box, L0) and np.array_equal(r1, r0)


def test_forces_and_energy_left_alone():
    s = lj_system(seed=5)
    s.fx[:] = 1.5
    s.s.pot_eng = -3.0
    pi, pj = s.pairs(2.5, 0.3)
    s.mc_barostat([O.pair_params(O.LJ, cutoff=2.5)], pi, pj, 1.0, 1.0, counter=3)
    assert np.all(s.fx == 1.5) and s.s.pot_eng == -3.0
