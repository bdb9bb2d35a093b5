"""Launch variants of the pair kernels and the autotuner.

Every variant (block 64 / 128 / 256, with or without the range filter; for
ECP, the split Newton path, the one-kernel path or the one kernel behind the
support-function range test) must give
the same forces, torques and energies (only the order of float atomics
differs), the same listed / in-range counts, and the autotuner must leave the
caller's forces and accumulators as they were."""
import numpy as np
import pytest

from helpers import ellipsoids, f32, jittered_fcc, rel
from sucrose_gb300 import GpuSystem, capi, configs

pytestmark = pytest.mark.gpu
VARIANTS = [(256, 0), (128, 0), (256, 1), (128, 1), (64, 0), (64, 1)]
ECP_VARIANTS = VARIANTS + [(256, 2), (128, 2), (64, 2)]


def lj_system():
    r, q, box = jittered_fcc(8, 0.8442, seed=4)
    g = GpuSystem(len(r), box)
    g.upload(r=f32(r))
    g.init_nlist(0.3, 2.5)
    return g, GpuSystem.params(capi.LJ, cutoff=2.5)


def gb_system(kind=capi.GB, sig=(1.0, 1.0, 3.0)):
    prolate = sig[2] > sig[0]
    counts = (16, 16, 8) if prolate else (8, 8, 24)
    r, q, box = ellipsoids(counts, sig, 0.3 if prolate else 0.1, seed=6, tilt=0.6 if prolate else 0.05)
    g = GpuSystem(len(r), box)
    g.set_particles(sig=sig, eps=(1.0, 1.0, 0.2))
    g.upload(r=f32(r), q=f32(q))
    g.init_nlist(0.4, 6.0)
    return g, GpuSystem.params(kind, cutoff=4.0, mu=2, nu=1)


def ecp_system():
    # a compressed lattice (density 0.13): pairs in contact for the repulsive kind
    r, q, box = ellipsoids((6, 8, 12), (3.0, 2.0, 1.0), 0.13, seed=3, tilt=0.4)
    g = GpuSystem(len(r), box)
    g.set_particles(sig=(3.0, 2.0, 1.0))
    g.upload(r=f32(r), q=f32(q))
    g.init_nlist(0.3, 3.0)
    return g, GpuSystem.params(capi.ECPR, cutoff=3.0, solver=capi.SOLVER_NEWTON)


def forces_with(g, p, block, filt):
    g.set_launch(p.kind, block, filt)
    g.zero_forces()
    pe, vir, st = g.pair_forces(p, want_stats=True)
    F, T = g.forces()
    return pe, vir, F, T, (st.pairs, st.solver_evals)


@pytest.mark.parametrize("make", [lj_system, gb_system, lambda: gb_system(capi.GBR), lambda: gb_system(capi.GBW),
                                  lambda: gb_system(capi.GB, (3.0, 3.0, 1.0)), ecp_system],
                         ids=["lj", "gb", "gbr", "gbw", "gb_oblate", "ecp_split"])
def test_variants_agree(lib, make):
    g, p = make()
    ref = forces_with(g, p, *VARIANTS[0])
    if p.kind >= capi.ECP:   # solver_evals: Newton evaluations, several per pair
        assert ref[4][0] == g.npairs() and ref[4][1] >= ref[4][0]
    else:                    # solver_evals: pairs in range
        assert ref[4][0] == g.npairs() and 0 < ref[4][1] <= ref[4][0]
    ecp = p.kind >= capi.ECP
    if ecp:
        assert np.linalg.norm(ref[2]) > 0
    for v in (ECP_VARIANTS if ecp else VARIANTS)[1:]:
        pe, vir, F, T, counts = forces_with(g, p, *v)
        if ecp and v[1] == 2:   # the support filter: fewer pairs solved
            assert counts[0] == ref[4][0] and counts[1] < ref[4][1], v
        else:   # the filter's range test and eval's may round differently on the boundary
            assert counts[0] == ref[4][0] and abs(counts[1] - ref[4][1]) <= 2, v
        assert abs(pe - ref[0]) <= 1e-6 * max(1.0, abs(ref[0])), v
        assert abs(vir - ref[1]) <= 1e-6 * max(1.0, abs(ref[1])), v
        # float atomics in another order: ~1e-7 per pair force, amplified where
        # a particle's net force is much smaller than its pair forces
        assert rel(F, ref[2]) < 3e-6, v
        if p.kind != capi.LJ:
            assert rel(T, ref[3]) < 3e-6, v
    g.close()


def test_autotune_restores_state(lib):
    g, p = gb_system()
    g.zero_forces()
    g.pair_forces(p)
    F0, T0 = g.forces()
    e0 = g.energies()
    res = g.autotune(p, reps=3)
    assert res.candidates == 6 and res.block in (64, 128, 256) and res.filter in (0, 1)
    assert all(res.ms[k] > 0 for k in range(6))
    F1, T1 = g.forces()
    assert np.array_equal(F0, F1) and np.array_equal(T0, T1)
    assert np.array_equal(e0, g.energies())
    # the tuned shape is used and agrees with the default one
    g.zero_forces()
    pe = g.pair_forces(p)[0]
    F2, _ = g.forces()
    assert rel(F2, F0) < 1e-6
    g.close()


def test_autotune_ecp_variants(lib):
    """ECP with a Newton solver: eight variants (the support-filtered kernel,
    the one kernel, the split path), the state restored."""
    g, p = ecp_system()
    p.solver = capi.SOLVER_NEWTON_SUPPORT
    g.zero_forces()
    g.pair_forces(p)
    F0, T0 = g.forces()
    res = g.autotune(p, reps=2)
    assert res.candidates == 8 and res.block in (64, 128, 256) and res.filter in (0, 1, 2)
    assert all(res.ms[k] > 0 for k in range(8))
    F1, T1 = g.forces()
    assert np.array_equal(F0, F1) and np.array_equal(T0, T1)
    g.close()


def test_autotuned_captured_step(lib):
    """A tuned launch shape invalidates the captured step, which re-captures."""
    sig = (1.0, 1.0, 3.0)
    r, q, box = ellipsoids((16, 16, 8), sig, 0.3, seed=6, tilt=0.05)
    g = GpuSystem(len(r), box)
    g.set_particles(sig=sig, eps=(1.0, 1.0, 0.2), inertia=configs.default_inertia(sig))
    g.upload(r=f32(r), q=f32(q))
    g.init_nlist(0.4, 6.0)
    p = GpuSystem.params(capi.GB, cutoff=4.0, mu=2, nu=1)
    g.configure_step(p, integrator=capi.INT_LANGEVIN, dt=0.0005, rotations=1)
    g.step(2)
    g.step_check()
    g.autotune(p, reps=2)
    g.step(3)
    g.step_check()
    g.close()
