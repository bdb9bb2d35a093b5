"""The Monte Carlo barostat on the device against the oracle, and the
Verlet list after box changes. Same FP32-rounded state; the two make the same
decision from the same Philox draws (energies agree to 1e-5 relative)."""
import numpy as np
import pytest

import oracle as O
from helpers import Pair, jittered_fcc, rel
from sucrose_gb300 import capi

pytestmark = pytest.mark.gpu


def lj_pair(seed=3):
    r, q, box = jittered_fcc(8, 0.7, seed=seed, amp=0.05)
    return Pair(r, q, box)


@pytest.mark.parametrize("counter", range(6))
def test_barostat_matches_oracle(lib, counter):
    P = lj_pair()
    P.g.init_nlist(0.3, 2.5)
    P.g.zero_forces()
    P.g.pair_forces(P.g.params(capi.LJ, cutoff=2.5))
    F0, _ = P.g.forces()
    e0 = P.g.energies()
    pi, pj = P.o.pairs(2.5, 0.3)
    T, Pt, dv = 1.2, 1.0, 0.02
    a, vol = P.g.mc_barostat([P.g.params(capi.LJ, cutoff=2.5)], Pt, T, dv, counter=counter)
    ao, u_old, u_new, v_new = P.o.mc_barostat([O.pair_params(O.LJ, cutoff=2.5)], pi, pj, Pt, T, dv, counter=counter)
    expo = -(u_new - u_old) / T - Pt * (v_new - np.prod(P.box)) / T + P.n * np.log(v_new / np.prod(P.box))
    w = O.philox4x32(np.array([[counter, 0, 0x4D43, 0]], dtype=np.uint32))[0].astype(np.float64) / 2.0 ** 32
    if abs(np.log(w[1]) - expo) > 1e-3 * max(1.0, abs(expo)):   # not a borderline draw
        assert a == ao
    r, q, v, l = P.g.download()
    ro = np.stack([P.o.rx, P.o.ry, P.o.rz], 1)
    if a == ao:
        assert vol == pytest.approx(np.prod(P.o.box), rel=1e-14)
        assert np.max(np.abs(r - ro)) < 2e-6 * np.max(P.box)
    # forces and accumulators untouched
    F1, _ = P.g.forces()
    assert np.array_equal(F0, F1)
    assert np.array_equal(e0, P.g.energies())


def test_list_follows_box_changes(lib):
    # shrink the box (and the positions) in steps; each rebuilt list is the
    # oracle's pair set, so the cell grid followed the box
    P = lj_pair(seed=7)
    P.g.init_nlist(0.3, 2.5)
    r0 = P.r.copy()
    box0 = P.box.copy()
    for s in (0.97, 0.92, 0.85):
        r = r0 * s
        box = box0 * s
        P.g.set_box(box)
        P.g.upload(r=r)
        P.g.build_nlist()
        pi, pj = P.g.pairs()
        got = set(zip(pi.tolist(), pj.tolist()))
        o = O.System(P.n, box)
        o.rx[:], o.ry[:], o.rz[:] = np.asarray(r, dtype=np.float32).astype(np.float64).T
        oi, oj = o.pairs(2.5, 0.3)
        assert got == set(zip(oi.tolist(), oj.tolist()))


def test_barostat_inside_a_run(lib):
    # NVT steps with a barostat move every 5 steps: the run stays finite and
    # the captured step follows the box
    P = lj_pair(seed=9)
    P.g.init_nlist(0.3, 2.5)
    p = P.g.params(capi.LJ, cutoff=2.5)
    P.g.configure_step(p, integrator=capi.INT_LANGEVIN, dt=0.003, target_temp=1.0, damping=1.0)
    accepted = 0
    for k in range(6):
        P.g.step(5)
        P.g.step_check()
        a, vol = P.g.mc_barostat([p], 1.0, 1.0, 0.01, counter=k)
        accepted += a == 1
    P.g.step(5)
    P.g.step_check()
    assert np.all(np.isfinite(P.g.download()[0]))
