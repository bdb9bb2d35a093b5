"""Gay-Berne and ECP pair forces and torques on the device against the oracle.

Tolerance: norm-wise relative error over the whole system,
||F_dev - F_oracle|| / ||F_oracle|| <= 1e-5 (same for torques and the summed
potential energy). The device evaluates each pair in FP32; the oracle in FP64
on the same FP32 state.
"""
import numpy as np
import pytest

import oracle as O
from helpers import Pair, ellipsoids, rel, per_particle_max
from sucrose_gb300 import capi

pytestmark = pytest.mark.gpu
TOL = 1e-5

GB_SIG, GB_EPS = (1.0, 1.0, 3.0), (1.0, 1.0, 0.2)
ECP_SIG = (3.0, 2.0, 1.0)


def gb_state(seed=1):
    r, q, box = ellipsoids((14, 14, 5), GB_SIG, 0.2, seed=seed, tilt=0.3)
    return Pair(r, q, box, sig=GB_SIG, eps=GB_EPS)


def ecp_state(seed=3, tilt=0.4, counts=(6, 8, 12)):
    r, q, box = ellipsoids(counts, ECP_SIG, 0.1114, seed=seed, tilt=tilt)
    return Pair(r, q, box, sig=ECP_SIG)


def compare(P, pdev, por, cutoff_list, skin):
    P.g.init_nlist(skin, cutoff_list)
    P.g.zero_forces()
    pe, vir, st = P.g.pair_forces(pdev, want_stats=True, allow=(capi.SG_OK,))
    F, T = P.g.forces()
    pi, pj = P.o.pairs(cutoff_list, skin)
    P.o.zero_forces()
    P.o.forces(por, pi, pj)
    Fo, To = P.oracle_forces()
    peo = P.o.s.pot_eng
    return F, T, pe, Fo, To, peo, st


GB_KINDS = [(capi.GB, O.GB, {}), (capi.GBR, O.GBR, {}), (capi.GBW, O.GBW, {"wf": 0.3}),
            (capi.GBC, O.GBC, {"chirality": 0.4}), (capi.GBWC, O.GBWC, {"wf": 0.3, "chirality": 0.4})]


@pytest.mark.parametrize("kd,ko,kw", GB_KINDS)
@pytest.mark.parametrize("mu,nu", [(1, 2), (2, 1)])
def test_gay_berne(lib, kd, ko, kw, mu, nu):
    P = gb_state()
    pdev = P.g.params(kd, cutoff=4.0, mu=mu, nu=nu, **kw)
    por = O.pair_params(ko, cutoff=4.0, mu=mu, nu=nu, **kw)
    F, T, pe, Fo, To, peo, _ = compare(P, pdev, por, 3.0 + 4.0 - 1.0 + kw.get("wf", 0.0), 0.4)
    assert np.linalg.norm(Fo) > 0
    assert rel(F, Fo) < TOL and rel(T, To) < TOL
    assert abs(pe - peo) <= TOL * max(abs(peo), 1e-12)


ECP_KINDS = [(capi.ECP, O.ECP, {}), (capi.ECPR, O.ECPR, {}), (capi.ECPW, O.ECPW, {"wf": 0.2}),
             (capi.ECPC, O.ECPC, {"chirality": 0.3}), (capi.ECPWC, O.ECPWC, {"wf": 0.2, "chirality": 0.3})]


@pytest.mark.parametrize("kd,ko,kw", ECP_KINDS)
@pytest.mark.parametrize("split", [1, 0, 2], ids=["split", "fused", "filtered"])
@pytest.mark.parametrize("check", [1, 2], ids=["fp64", "double_float"])
def test_ecp_newton_vs_converged_fp64(lib, kd, ko, kw, split, check):
    # split: Newton solve kernel, then the force kernel from its lambda; fused:
    # one kernel solves and evaluates each pair; filtered: the same behind the
    # support-function range test
    P = ecp_state()
    P.g.set_launch(kd, 256, split)
    pdev = P.g.params(kd, cutoff=3.0, solver=capi.SOLVER_NEWTON, **kw)
    pdev.fp64_check = check
    por = O.pair_params(ko, cutoff=3.0, solver=O.SOLVER_TIGHT, **kw)
    F, T, pe, Fo, To, peo, st = compare(P, pdev, por, 3.0, 0.3)
    assert np.linalg.norm(Fo) > 0
    assert rel(F, Fo) < TOL and rel(T, To) < TOL
    assert abs(pe - peo) <= TOL * max(abs(peo), 1e-12)
    assert st.nonconverged == 0 and st.pairs == len(P.o.pairs(3.0, 0.3)[0])


@pytest.mark.parametrize("kd,ko,kw", ECP_KINDS)
@pytest.mark.parametrize("split", [1, 0, 2], ids=["split", "fused", "filtered"])
def test_ecp_newton_support_start_vs_converged_fp64(lib, kd, ko, kw, split):
    # Newton from the support-function start: same tolerance, same bound
    P = ecp_state(seed=5)
    P.g.set_launch(kd, 256, split)
    pdev = P.g.params(kd, cutoff=3.0, solver=capi.SOLVER_NEWTON_SUPPORT, **kw)
    por = O.pair_params(ko, cutoff=3.0, solver=O.SOLVER_TIGHT, **kw)
    F, T, pe, Fo, To, peo, st = compare(P, pdev, por, 3.0, 0.3)
    assert rel(F, Fo) < TOL and rel(T, To) < TOL
    assert abs(pe - peo) <= TOL * max(abs(peo), 1e-12)
    assert st.nonconverged == 0 and st.pairs == len(P.o.pairs(3.0, 0.3)[0])


def _contact_distance(P, pi, pj, lam):
    """|r_ij| and the contact distance sigma = |r| / sqrt(F(lambda)) along r_ij
    in FP64, F(l) = l(1-l) r.((1-l)A + lB)^-1 r with A = R^T S^2 R (the body axes
    as the rows of each quaternion's rotation matrix, S the semi-axes), at the
    oracle's converged lambda."""
    w, x, y, z = P.q.T.astype(np.float64)
    R = np.stack([np.stack([w * w + x * x - y * y - z * z, 2 * (x * y + w * z), 2 * (x * z - w * y)], -1),
                  np.stack([2 * (x * y - w * z), w * w - x * x + y * y - z * z, 2 * (y * z + w * x)], -1),
                  np.stack([2 * (x * z + w * y), 2 * (y * z - w * x), w * w - x * x - y * y + z * z], -1)], 1)
    S2 = np.diag((0.5 * np.asarray(ECP_SIG)) ** 2)
    A = np.einsum("mki,kl,mlj->mij", R, S2, R)
    d = P.r[pj].astype(np.float64) - P.r[pi].astype(np.float64)
    d -= np.round(d / P.box) * P.box
    rm = np.linalg.norm(d, axis=1)
    G = (1 - lam)[:, None, None] * A[pi] + lam[:, None, None] * A[pj]
    F = lam * (1 - lam) * np.einsum("mi,mi->m", d, np.linalg.solve(G, d[:, :, None])[:, :, 0])
    return rm, rm / np.sqrt(F)


@pytest.mark.parametrize("kd,ko,extra", [(capi.ECPR, O.ECPR, 0.0), (capi.ECP, O.ECP, 2.0)], ids=["ecpr", "ecp"])
def test_ecp_support_filter(lib, kd, ko, extra):
    """The filtered launch: the same forces as the launch that solves every
    pair; the pairs its range test turns away are beyond sigma + (reach -
    sigma) at the oracle's converged lambda, count in iteration bin 0 and read
    NaN as lambda; the others carry the lambda of the full launch."""
    P = ecp_state(seed=8)
    P.g.init_nlist(0.3, 3.0)
    p = P.g.params(kd, cutoff=3.0, solver=capi.SOLVER_NEWTON_SUPPORT)
    out = {}
    for filt in (0, 2):
        P.g.set_launch(kd, 256, filt)
        P.g.zero_forces()
        pe, _, st = P.g.pair_forces(p, want_stats=True)
        out[filt] = (pe, *P.g.forces(), st, P.g.ecp_lambda().astype(np.float64))
    pe0, F0, T0, st0, lam0 = out[0]
    pe2, F2, T2, st2, lam2 = out[2]
    assert np.linalg.norm(F0) > 0
    assert rel(F2, F0) < 3e-6 and rel(T2, T0) < 3e-6
    assert abs(pe2 - pe0) <= 1e-6 * max(abs(pe0), 1e-12)
    k = P.g.npairs()
    away = np.isnan(lam2)
    assert st0.pairs == st2.pairs == k and st0.iter_hist[0] == 0
    # repulsive kind: contact only, most listed pairs are turned away;
    # cutoff 3 (reach = sigma + 2): few are
    assert st2.iter_hist[0] == away.sum() and (0.5 * k if kd == capi.ECPR else 0) <= away.sum() < k
    assert sum(st2.iter_hist) == k and st2.solver_evals < st0.solver_evals
    assert np.max(np.abs(lam2[~away] - lam0[~away])) < 1e-6
    pi, pj = P.g.raw_pairs()
    lam_ref, _ = P.o.forces(O.pair_params(ko, cutoff=3.0, solver=O.SOLVER_TIGHT), pi, pj, want_lambda=True)
    rm, sigma = _contact_distance(P, pi, pj, lam_ref)
    assert np.all(rm[away] >= sigma[away] + extra)


def test_ecp_support_start_saves_evaluations(lib):
    # the support-function start needs fewer Newton evaluations than 1/2 on
    # random orientations, and lands on the same lambda
    P = ecp_state(seed=11, tilt=3.0, counts=(8, 10, 16))
    P.g.init_nlist(0.3, 3.0)
    out = {}
    for solver in (capi.SOLVER_NEWTON, capi.SOLVER_NEWTON_SUPPORT):
        P.g.zero_forces()
        _, _, st = P.g.pair_forces(P.g.params(capi.ECPR, cutoff=3.0, solver=solver), want_stats=True)
        out[solver] = (st.solver_evals / st.pairs, P.g.ecp_lambda().astype(np.float64))
    assert out[capi.SOLVER_NEWTON_SUPPORT][0] < out[capi.SOLVER_NEWTON][0] - 0.2
    assert np.max(np.abs(out[capi.SOLVER_NEWTON_SUPPORT][1] - out[capi.SOLVER_NEWTON][1])) < 4e-6


@pytest.mark.parametrize("kd,ko,kw", ECP_KINDS)
def test_ecp_brent_compat_vs_reference(lib, kd, ko, kw):
    P = ecp_state(seed=4)
    pdev = P.g.params(kd, cutoff=3.0, solver=capi.SOLVER_BRENT_COMPAT, **kw)
    por = O.pair_params(ko, cutoff=3.0, solver=O.SOLVER_BRENT, **kw)
    F, T, pe, Fo, To, peo, st = compare(P, pdev, por, 3.0, 0.3)
    assert rel(F, Fo) < TOL and rel(T, To) < TOL
    assert abs(pe - peo) <= TOL * max(abs(peo), 1e-12)


def test_ecp_brent_lambda_bits(lib):
    # the FP64 Brent on the device lands on the reference's lambda exactly
    P = ecp_state(seed=6)
    P.g.init_nlist(0.3, 3.0)
    P.g.zero_forces()
    P.g.pair_forces(P.g.params(capi.ECPR, solver=capi.SOLVER_BRENT_COMPAT))
    lam_dev = P.g.ecp_lambda()
    pi, pj = P.g.raw_pairs()
    P.o.zero_forces()
    lam_ref, nev = P.o.forces(O.pair_params(O.ECPR, solver=O.SOLVER_BRENT), pi, pj, want_lambda=True)
    assert np.array_equal(lam_dev, lam_ref.astype(np.float32))


@pytest.mark.parametrize("solver", [capi.SOLVER_NEWTON, capi.SOLVER_NEWTON_SUPPORT], ids=["half", "support"])
def test_ecp_newton_lambda_accuracy(lib, solver):
    P = ecp_state(seed=8)
    P.g.init_nlist(0.3, 3.0)
    P.g.zero_forces()
    P.g.pair_forces(P.g.params(capi.ECPR, solver=solver))
    lam_dev = P.g.ecp_lambda().astype(np.float64)
    pi, pj = P.g.raw_pairs()
    lam_ref, _ = P.o.forces(O.pair_params(O.ECPR, solver=O.SOLVER_TIGHT), pi, pj, want_lambda=True)
    assert np.max(np.abs(lam_dev - lam_ref)) < 2e-6


def test_ecp_identical_spheres(lib):
    # equal spheres: lambda = 1/2 exactly, contact distance = sum of radii
    r = np.array([[0.0, 0.0, 0.0], [1.7, 0.3, -0.2], [-1.5, 1.0, 0.4]])
    P = Pair(r, None, 40.0, sig=(2.0, 2.0, 2.0))
    P.g.init_nlist(0.3, 3.0)
    P.g.zero_forces()
    P.g.pair_forces(P.g.params(capi.ECP, cutoff=3.0, solver=capi.SOLVER_NEWTON))
    assert np.allclose(P.g.ecp_lambda(), 0.5, atol=1e-6)


def test_ecp_angular_momentum_balance(lib):
    # ecpr has no taper: sum_i (r_i x F_i + T_i) = 0 for a rotation-invariant pair potential
    P = ecp_state(seed=9, counts=(10, 12, 20))
    P.g.init_nlist(0.3, 3.0)
    P.g.zero_forces()
    P.g.pair_forces(P.g.params(capi.ECPR, solver=capi.SOLVER_NEWTON))
    F, T = P.g.forces()
    pi, pj = P.g.pairs()
    # use pair-relative positions (minimum image) for the balance
    dr = P.r[pi] - P.r[pj]
    dr -= P.box * np.round(dr / P.box)
    scale = np.linalg.norm(np.cross(P.r, F)) + np.linalg.norm(T)
    assert np.linalg.norm(F.sum(0)) < 1e-5 * np.linalg.norm(F) * np.sqrt(len(F))
    assert scale > 0
