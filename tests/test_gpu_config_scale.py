"""The ellipsoid workloads at their full size, from their own initial state.

The isotropic placement (configs.isotropic_placement) is checked for
overlaps against the oracle's ECP contact (the repulsive kind is zero for
every pair at or beyond contact), for isotropy (nematic order P2) and for
determinism. Then, at the benchmark sizes and seeds, the device's Verlet
list is compared bit for bit with the reference's acceptance test, and the
forces, torques and energy with the oracle's FP64 evaluation:
  Gay-Berne (3, 5, 2, 1), N = 32 768, rho = 0.30, list radius 6.0 + 0.4;
  ECP (3, 2, 1), ecpr, N = 65 536, phi = 0.35, list radius 3.0 + 0.3,
  plain Newton against the tightly converged FP64 contact parameter.
"""
import numpy as np
import pytest

import oracle as O
from helpers import Pair, kdtree_reference_pairs, rel
from sucrose_gb300 import capi, configs

pytestmark = pytest.mark.gpu

GB = dict(n=32768, sig=(1.0, 1.0, 3.0), eps=(1.0, 1.0, 0.2), density=0.30, seed=1002, cutoff=4.0, list_cutoff=6.0,
          skin=0.4)
ECP = dict(n=65536, sig=(3.0, 2.0, 1.0), eps=(1.0, 1.0, 1.0), density=0.1114, seed=1003, cutoff=3.0,
           list_cutoff=3.0, skin=0.3)


def oracle_sums(n, out, pi, pj):
    F = np.zeros((n, 3))
    T = np.zeros((n, 3))
    np.add.at(F, pi, out[:, 1:4])
    np.add.at(F, pj, -out[:, 1:4])
    np.add.at(T, pi, out[:, 4:7])
    np.add.at(T, pj, out[:, 7:10])
    return F, T, out[:, 0].sum()


@pytest.mark.parametrize("sig,density", [((3.0, 2.0, 1.0), 0.1114), ((1.0, 1.0, 3.0), 0.30)])
def test_isotropic_placement(lib, sig, density):
    n = 4000
    r, q, box, rep = configs.isotropic_placement(n, sig, density, seed=77)
    assert rep.overlaps == 0 and rep.final_scale == 1.0 and rep.min_contact_ratio >= 1.0 - 1e-5
    r2, q2, _, _ = configs.isotropic_placement(n, sig, density, seed=77)
    assert np.array_equal(r, r2) and np.array_equal(q, q2)     # the same bits every run
    assert np.all(np.abs(r) <= box / 2)
    assert np.allclose(np.linalg.norm(q, axis=1), 1.0, atol=1e-12)
    assert configs.nematic_order(q, int(np.argmax(sig))) < 0.06
    # no overlaps: the oracle's repulsive ECP (zero at and beyond contact)
    # over every pair within the largest contact distance
    amax = max(sig)
    pi, pj = kdtree_reference_pairs(r, box, amax, 0.0)
    s = O.System(n, box)
    s.set_defaults(sig=sig)
    s.rx[:], s.ry[:], s.rz[:] = r.T
    s.qw[:], s.qx[:], s.qy[:], s.qz[:] = q.T
    out = s.pair_batch(O.pair_params(O.ECPR, cutoff=amax, solver=O.SOLVER_TIGHT), pi, pj)
    assert len(pi) > n
    assert np.max(out[:, 0]) < 1e-6
    other = configs.isotropic_placement(n, sig, density, seed=78)[0]
    assert not np.array_equal(r, other)


def full_size(w, kind, solver=None, mu=None, nu=None, squeeze=1.0, launch=None):
    """The benchmark's placed state (positions and box scaled by `squeeze`,
    so that repulsive pairs overlap), its list and forces on both sides.
    launch: (block, filter) of the pair kernel (sg_pair_set_launch)."""
    r, q, box, rep = configs.isotropic_placement(w["n"], w["sig"], w["density"], seed=w["seed"])
    assert rep.overlaps == 0
    P = Pair(r * squeeze, q, box * squeeze, sig=w["sig"], eps=w["eps"])
    P.g.init_nlist(w["skin"], w["list_cutoff"])
    gpi, gpj = P.g.pairs()
    opi, opj = kdtree_reference_pairs(P.r, P.box, w["list_cutoff"], w["skin"])
    assert len(gpi) == len(opi)
    assert np.array_equal(gpi, opi) and np.array_equal(gpj, opj)
    kw = {} if mu is None else {"mu": mu, "nu": nu}
    if launch is not None:
        P.g.set_launch(getattr(capi, kind), *launch)
    P.g.zero_forces()
    pe, _ = P.g.pair_forces(P.g.params(getattr(capi, kind), cutoff=w["cutoff"],
                                       **({"solver": solver} if solver is not None else {}), **kw))
    F, T = P.g.forces()
    po = O.pair_params(getattr(O, kind), cutoff=w["cutoff"], **({"solver": O.SOLVER_TIGHT} if solver else {}), **kw)
    out = P.o.pair_batch(po, opi, opj)
    Fo, To, peo = oracle_sums(P.n, out, opi, opj)
    return len(opi), F, T, pe, Fo, To, peo, int(np.count_nonzero(out[:, 0]))


def test_gay_berne_full_size_list_and_forces(lib):
    npairs, F, T, pe, Fo, To, peo, active = full_size(GB, "GB", mu=2, nu=1)
    assert npairs > 4_000_000 and active > 1_000_000
    assert rel(F, Fo) < 1e-5
    assert rel(T, To) < 1e-5
    assert abs(pe - peo) <= 1e-5 * abs(peo)


@pytest.mark.parametrize("solver,filt", [(capi.SOLVER_NEWTON, 0), (capi.SOLVER_NEWTON_SUPPORT, 0),
                                         (capi.SOLVER_NEWTON_SUPPORT, 2)], ids=["half", "support", "support_filtered"])
def test_ecp_full_size_list_and_forces(lib, solver, filt):
    # positions and box 3 % closer: tens of thousands of pairs in contact;
    # filt 2: the support-function range test in front of the solve
    npairs, F, T, pe, Fo, To, peo, active = full_size(ECP, "ECPR", solver=solver, squeeze=0.97, launch=(256, filt))
    assert npairs > 400_000 and active > 10_000
    assert rel(F, Fo) < 1e-5
    assert rel(T, To) < 1e-5
    assert abs(pe - peo) <= 1e-5 * abs(peo)
