"""Batched replicas against their own single-system runs.

Each replica of a batched context must list exactly the pairs of the same
system run alone (same rows, same order), draw exactly the same Philox
numbers in the Langevin update (per-replica key, temperature and 1-based
index within the replica), and get the same forces within 1e-5 relative
(only the order of float atomics differs). The captured step runs every
replica, LJ and GB families together, and is compared with the single
systems stepped one by one."""
import numpy as np
import pytest

from helpers import f32, rel
from sucrose_gb300 import GpuSystem, capi, configs

pytestmark = pytest.mark.gpu

LJ = dict(configs.LJ_REPLICA)
# smaller Gay-Berne range than the benchmark so that small boxes pass the cut-off guard
GB = dict(configs.GB_REPLICA, cutoff=2.0, list_cutoff=4.0, skin=0.3)
FAM = (LJ, GB)
DT = 0.002


def pair_params(f):
    if f == 0:
        return GpuSystem.params(capi.LJ, cutoff=LJ["cutoff"])
    return GpuSystem.params(capi.GB, cutoff=GB["cutoff"], mu=2, nu=1)


def ensemble(nrep=10, seed=11):
    return configs.replica_ensemble(nrep, seed=seed, nmin=100, nmax=700, lj=LJ, gb=GB)


def replica_state(e, k, seed=5):
    """Per-replica arrays: positions, quaternions, velocities, angular momenta,
    per-particle shape, energy axes and inertia."""
    a, b = e["off"][k], e["off"][k + 1]
    n = b - a
    p = FAM[e["family"][k]]
    T = e["temp"][k]
    r = f32(e["r"][a:b])
    q = f32(e["q"][a:b])
    v = f32(configs.velocities_to_temperature(n, T, seed + k))
    I = configs.default_inertia(p["sig"])
    l = f32(configs.angular_momenta(q, I, T, seed + k)) if e["family"][k] == 1 else np.zeros((n, 3))
    sig = np.tile(p["sig"], (n, 1))
    eps = np.tile(p["eps"], (n, 1))
    inert = np.tile(I, (n, 1))
    return r, q, v, l, sig, eps, inert


def batched(e):
    g = GpuSystem.replicas(e["n"], e["box"], e["family"], e["temp"], e["key"])
    parts = [replica_state(e, k) for k in range(len(e["n"]))]
    cat = [np.concatenate([p[c] for p in parts]) for c in range(7)]
    g.set_particles(mass=1.0, sig=cat[4], eps=cat[5], inertia=cat[6])
    g.upload(r=cat[0], q=cat[1], v=cat[2], l=cat[3])
    g.init_rep_nlist([LJ["skin"], GB["skin"], 0.3], [LJ["list_cutoff"], GB["list_cutoff"], 3.0], trigger_mode=1)
    return g


def single(e, k):
    r, q, v, l, sig, eps, inert = replica_state(e, k)
    p = FAM[e["family"][k]]
    s = GpuSystem(len(r), e["box"][k])
    s.set_particles(mass=1.0, sig=sig, eps=eps, inertia=inert)
    s.upload(r=r, q=q, v=v, l=l)
    s.init_nlist(p["skin"], p["list_cutoff"], trigger_mode=1)
    return s


@pytest.fixture(scope="module")
def ens():
    return ensemble()


def test_ensemble_is_grouped_and_legal(ens):
    assert np.all(np.diff(ens["family"]) >= 0)
    for k in range(len(ens["n"])):
        assert ens["box"][k].min() >= 2 * FAM[ens["family"][k]]["list_cutoff"]


def test_lists_match_single_runs(lib, ens):
    g = batched(ens)
    pi, pj = g.raw_pairs()
    assert np.all(np.diff(pi) >= 0)
    for k in range(len(ens["n"])):
        a, b = ens["off"][k], ens["off"][k + 1]
        m = (pi >= a) & (pi < b)
        assert np.all((pj[m] >= a) & (pj[m] < b)), "a pair crosses replicas"
        s = single(ens, k)
        si, sj = s.raw_pairs()
        assert np.array_equal(pi[m] - a, si), k
        assert np.array_equal(pj[m] - a, sj), k
        s.close()
    g.close()


def test_forces_match_single_runs(lib, ens):
    g = batched(ens)
    g.zero_forces()
    pe_lj, _ = g.pair_forces(pair_params(0))
    pe_gb, _ = g.pair_forces(pair_params(1))
    F, T = g.forces()
    pe_single = [0.0, 0.0]
    for k in range(len(ens["n"])):
        a, b = ens["off"][k], ens["off"][k + 1]
        f = ens["family"][k]
        s = single(ens, k)
        s.zero_forces()
        pe, _ = s.pair_forces(pair_params(f))
        pe_single[f] += pe
        Fs, Ts = s.forces()
        assert rel(F[a:b], Fs) < 1e-5, k
        if f == 1:
            assert rel(T[a:b], Ts) < 1e-5, k
        s.close()
    assert abs(pe_lj - pe_single[0]) <= 1e-9 * max(1.0, abs(pe_single[0]))
    assert abs(pe_gb - pe_single[1]) <= 1e-9 * max(1.0, abs(pe_single[1]))
    g.close()


def test_charged_kinds_on_replicas(lib, ens):
    # the charge and Morse kinds belong to the LJ-like family: on a replica
    # context they act on the LJ replicas, charges riding in pos.w
    g = batched(ens)
    rng = np.random.default_rng(4)
    q = f32(rng.choice([-1.0, 1.0], g.n))
    g.set_charges(q)
    kinds = [GpuSystem.params(capi.COULOMB, cutoff=LJ["cutoff"], dielectric=2.0),
             GpuSystem.params(capi.MORSE, cutoff=LJ["cutoff"], dissoc=1.0, width=1.5, rmin=1.1)]
    for p in kinds:
        g.zero_forces()
        pe, _ = g.pair_forces(p)
        F, _ = g.forces()
        pe_single = 0.0
        for k in range(len(ens["n"])):
            if ens["family"][k] != 0:
                continue
            a, b = ens["off"][k], ens["off"][k + 1]
            s = single(ens, k)
            s.set_charges(q[a:b])
            s.zero_forces()
            pk, _ = s.pair_forces(p)
            pe_single += pk
            Fs, _ = s.forces()
            assert rel(F[a:b], Fs) < 1e-5, k
            s.close()
        assert abs(pe - pe_single) <= 1e-6 * max(1.0, abs(pe_single))
    g.close()


def test_langevin_streams_bit_exact(lib, ens):
    """Zero forces, one Langevin half step: every number in the update comes
    from the per-replica Philox stream, so the state must be bit-identical."""
    g = batched(ens)
    g.zero_forces()
    g.lgv_initial(DT, 7, damping=1.0)
    r, q, v, l = g.download()
    for k in range(len(ens["n"])):
        a, b = ens["off"][k], ens["off"][k + 1]
        s = single(ens, k)
        s.zero_forces()
        s.lgv_initial(DT, 7, damping=1.0, target_temp=ens["temp"][k], key=ens["key"][k])
        rs, qs, vs, ls = s.download()
        for x, y in ((r, rs), (q, qs), (v, vs), (l, ls)):
            assert np.array_equal(x[a:b], y), k
        s.close()
    g.close()


def test_captured_step_matches_single_runs(lib, ens):
    nsteps = 4
    g = batched(ens)
    g.configure_step_pairs([pair_params(0), pair_params(1)], integrator=capi.INT_LANGEVIN, dt=DT, damping=1.0,
                           rotations=1)
    g.step(nsteps)
    g.step_check()
    r, q, v, l = g.download()
    ke = g.rep_kinetic()
    assert g.step_kernel_count() > 0
    for k in range(len(ens["n"])):
        a, b = ens["off"][k], ens["off"][k + 1]
        f = ens["family"][k]
        s = single(ens, k)
        s.configure_step(pair_params(f), integrator=capi.INT_LANGEVIN, dt=DT, damping=1.0, rotations=1,
                         target_temp=ens["temp"][k], key=ens["key"][k])
        s.step(nsteps)
        s.step_check()
        rs, qs, vs, ls = s.download()
        box = ens["box"][k]
        dr = r[a:b] - rs
        dr -= box * np.round(dr / box)
        assert np.max(np.abs(dr)) < 1e-5 * box.max(), k
        assert rel(v[a:b], vs) < 1e-4, k
        assert rel(q[a:b], qs) < 1e-5, k
        ke_host = 0.5 * np.sum(v[a:b].astype(np.float64) ** 2)
        assert abs(ke[k, 0] - ke_host) < 1e-6 * ke_host, k
        s.close()
    g.close()


def test_replica_context_rejects_single_system_calls(lib, ens):
    g = batched(ens)
    with pytest.raises(capi.SgError):
        g.set_box((10.0, 10.0, 10.0))
    with pytest.raises(capi.SgError):
        g.init_nlist(0.3, 2.5)
    with pytest.raises(capi.SgError):
        g.nht_initial(DT, 1.0, 0.0)
    with pytest.raises(capi.SgError):
        g.set_velocity_to_temperature(1.0, 5)
    g.close()


def test_only_moved_replicas_rebuild(lib, ens):
    """Displace one replica past its skin: the update rebuilds that replica's
    rows (matching its own single run from the new positions) and keeps every
    other replica's rows."""
    g = batched(ens)
    pi0, pj0 = g.raw_pairs()
    r, q, v, l = g.download()
    k = 1
    a, b = ens["off"][k], ens["off"][k + 1]
    rng = np.random.default_rng(3)
    box = ens["box"][k]
    r2 = r.copy()
    r2[a:b] = f32(r[a:b] + rng.uniform(-0.5, 0.5, size=(b - a, 3)) * box)
    r2[a:b] -= box * np.round(r2[a:b] / box)
    r2 = f32(r2)
    g.upload(r=r2)
    assert g.needs_rebuild()
    builds = g.nlist_builds()
    assert np.array_equal(g.rep_nlist_builds(), np.ones(len(ens["n"]), dtype=np.int64))   # the initial build
    g.update_nlist()
    assert g.nlist_builds() == builds + 1
    counts = g.rep_nlist_builds()
    assert counts[k] == 2 and np.all(np.delete(counts, k) == 1)
    pi1, pj1 = g.raw_pairs()
    for kk in range(len(ens["n"])):
        lo, hi = ens["off"][kk], ens["off"][kk + 1]
        m0 = (pi0 >= lo) & (pi0 < hi)
        m1 = (pi1 >= lo) & (pi1 < hi)
        if kk != k:
            assert np.array_equal(pi0[m0], pi1[m1]) and np.array_equal(pj0[m0], pj1[m1]), kk
        else:
            s = single(ens, kk)
            s.upload(r=r2[lo:hi])
            s.build_nlist()
            si, sj = s.raw_pairs()
            assert np.array_equal(pi1[m1] - lo, si) and np.array_equal(pj1[m1] - lo, sj)
            s.close()
    g.close()
