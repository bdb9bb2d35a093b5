"""One step of each integrator on the device against the oracle, same state."""
import numpy as np
import pytest

import oracle as O
from helpers import Pair, ellipsoids, jittered_fcc, rel, f32
from sucrose_gb300 import configs

pytestmark = pytest.mark.gpu
SIG = (3.0, 2.0, 1.0)


def state(seed=2):
    r, q, box = ellipsoids((6, 8, 12), SIG, 0.1114, seed=seed, tilt=0.4)
    n = len(r)
    v = configs.velocities_to_temperature(n, 1.2, seed)
    I = configs.default_inertia(SIG)
    l = configs.angular_momenta(q, I, 1.2, seed)
    P = Pair(r, q, box, sig=SIG, v=v, l=l)
    rng = np.random.default_rng(seed)
    F = f32(rng.normal(size=(n, 3)) * 5.0)
    T = f32(rng.normal(size=(n, 3)) * 2.0)
    P.g.set_forces(F, T)
    P.set_oracle_forces(F, T)
    return P


def compare_state(P, tol=2e-6):
    r, q, v, l = P.g.download()
    o = P.o
    ro = np.stack([o.rx, o.ry, o.rz], 1)
    dr = r - ro
    dr -= P.box * np.round(dr / P.box)
    assert np.max(np.abs(dr)) < tol * np.max(P.box)
    assert rel(v, np.stack([o.vx, o.vy, o.vz], 1)) < tol
    assert rel(q, np.stack([o.qw, o.qx, o.qy, o.qz], 1)) < tol
    lo = np.stack([o.lx, o.ly, o.lz], 1)
    if np.linalg.norm(lo) > 0:
        assert rel(l, lo) < tol


def test_vv(lib):
    P = state()
    P.g.vv_initial(0.001)
    P.o.vv_initial(0.001)
    compare_state(P)
    ke = P.g.vv_final(0.001)
    P.o.vv_final(0.001)
    compare_state(P)
    assert abs(ke - P.o.s.kin_eng) < 1e-6 * P.o.s.kin_eng


def test_quaternion(lib):
    P = state(3)
    P.g.qq_initial(0.001)
    P.o.qq_initial(0.001)
    compare_state(P)
    kr = P.g.qq_final(0.001)
    P.o.qq_final(0.001)
    compare_state(P)
    assert abs(kr - P.o.s.kin_rot) < 1e-5 * P.o.s.kin_rot


def test_langevin(lib):
    P = state(4)
    P.o.s.target_temp = 1.0
    P.g.lgv_initial(0.002, 17, damping=1.0, target_temp=1.0)
    P.o.lgv_initial(0.002, 17, damping=1.0)
    compare_state(P, tol=5e-6)
    ke, kr = P.g.lgv_final(0.002, 1.0)
    P.o.lgv_final(0.002)
    compare_state(P, tol=5e-6)
    assert abs(ke - P.o.s.kin_eng) < 1e-5 * P.o.s.kin_eng
    assert abs(kr - P.o.s.kin_rot) < 1e-5 * P.o.s.kin_rot


def test_langevin_replica_key(lib):
    P = state(5)
    key = (0x1234ABCD, 0x0BADF00D)
    P.o.s.target_temp = 1.0
    P.g.lgv_initial(0.002, 3, damping=1.0, target_temp=1.0, key=key)
    P.o.lgv_initial(0.002, 3, damping=1.0, key=key)
    compare_state(P, tol=5e-6)


@pytest.mark.parametrize("mode", [0, 1])
def test_nose_hoover(lib, mode):
    P = state(6)
    P.o.s.target_temp = 1.2
    # non-zero chain momenta so the thermostat acts
    chain = np.array([0.0, 0.0, 0.0, 0.3, -0.2, 0.1, 0, 0, 0, 0, 0, 0])
    P.g.nht_state(chain)
    P.o.s.p_eta[0], P.o.s.p_eta[1], P.o.s.p_eta[2] = 0.3, -0.2, 0.1
    P.g.nht_initial(0.001, 1.2, mode=mode)
    P.o.nht_initial(0.001, mode=mode)
    compare_state(P, tol=5e-6)
    st = P.g.nht_state()
    np.testing.assert_allclose(st[:6], list(P.o.s.eta) + list(P.o.s.p_eta), rtol=1e-6, atol=1e-9)
    ke = P.g.nht_final(0.001, 1.2, mode=mode)
    P.o.nht_final(0.001, mode=mode)
    compare_state(P, tol=5e-6)
    assert abs(ke - P.o.s.kin_eng) < 1e-5 * P.o.s.kin_eng
    st = P.g.nht_state()
    np.testing.assert_allclose(st[:6], list(P.o.s.eta) + list(P.o.s.p_eta), rtol=1e-6, atol=1e-9)


def test_nose_hoover_rotational_chain_against_the_oracle(lib):
    """The standard chain on translation and rotation (rot_chain = 1, the
    thermostat of the ECP benchmark) against the oracle's translational chain
    plus its rotational chain (or_nhr_half: the same propagator on
    G1 = sum L_b^2 / I - 3 N T, scaling every angular momentum): particle
    state, all twelve chain variables and the kinetic energy, both halves."""
    P = state(7)
    P.o.s.target_temp = 1.2
    # first chain momenta of order Q1 / dt, so that one half step scales the
    # velocities and angular momenta by about 1e-3 (far above the tolerance)
    chain = np.array([0.01, -0.02, 0.03, 1.0e4, 3.0, -2.0, -0.01, 0.02, 0.0, 2.0e4, 5.0, -3.0])

    def run(sys, rot_chain, oracle):
        sys.g.nht_state(chain)
        for k in range(3):
            sys.o.s.eta[k], sys.o.s.p_eta[k] = chain[k], chain[3 + k]
            sys.o.s.eta_r[k], sys.o.s.p_eta_r[k] = chain[6 + k], chain[9 + k]
        sys.g.nht_initial(0.001, 1.2, mode=1, rot_chain=rot_chain)
        if oracle:
            sys.o.nht_initial(0.001, mode=1)
            sys.o.nhr_half(0.001)
            compare_state(sys, tol=5e-6)
            np.testing.assert_allclose(sys.g.nht_state(), oracle_chain(sys), rtol=1e-6, atol=1e-9)
        ke = sys.g.nht_final(0.001, 1.2, mode=1, rot_chain=rot_chain)
        if oracle:
            sys.o.nht_final(0.001, mode=1)
            sys.o.nhr_half(0.001)
            compare_state(sys, tol=5e-6)
            np.testing.assert_allclose(sys.g.nht_state(), oracle_chain(sys), rtol=1e-6, atol=1e-9)
            assert abs(ke - sys.o.s.kin_eng) < 1e-5 * sys.o.s.kin_eng

    def oracle_chain(sys):
        o = sys.o.s
        return np.array(list(o.eta) + list(o.p_eta) + list(o.eta_r) + list(o.p_eta_r))

    run(P, 1, True)
    # the rotational chain did act: without it the angular momenta differ
    Q = state(7)
    run(Q, 0, False)
    assert rel(Q.g.download()[3], P.g.download()[3]) > 1e-4


def test_thermo(lib):
    r, q, box = jittered_fcc(3, 0.8442, seed=1)
    v = configs.velocities_to_temperature(108, 0.722, 15)
    P = Pair(r, q, box, v=v)
    rng = np.random.default_rng(1)
    F = f32(rng.normal(size=(108, 3)))
    P.g.set_forces(F, np.zeros((108, 3)))
    P.set_oracle_forces(F, np.zeros((108, 3)))
    P.g.vv_final(0.0)
    P.o.vv_final(0.0)
    P.o.s.dof = 6 * 108 - 3
    P.o.s.density = 0.8442
    P.o.thermo()
    t = P.g.thermo(6 * 108 - 3, 0.8442)
    assert abs(t[0] - P.o.s.temp) < 1e-6 * P.o.s.temp
    assert abs(t[1] - P.o.s.virial) < 1e-5 * max(1.0, abs(P.o.s.virial))
    assert abs(t[2] - P.o.s.pressure) < 1e-5 * max(1.0, abs(P.o.s.pressure))


def _nh_system(seed=4):
    sig = (3.0, 2.0, 1.0)
    r, q, box = ellipsoids((8, 8, 12), sig, 0.1114, seed=seed, tilt=0.3)
    n = len(r)
    v = configs.velocities_to_temperature(n, 1.2, seed)
    I = configs.default_inertia(sig)
    l = configs.angular_momenta(q, I, 1.2, seed)
    from sucrose_gb300 import GpuSystem
    g = GpuSystem(n, box)
    g.set_particles(sig=sig, inertia=I)
    g.upload(r=f32(r), q=f32(q), v=f32(v), l=f32(l))
    g.init_nlist(0.3, 3.0)
    return g


def test_fused_nose_hoover_step_matches_separate_calls(lib):
    """The captured step's fused Nose-Hoover kernels against the drop-in entry
    points called one by one (chain on translation and rotation)."""
    from sucrose_gb300 import capi
    dt, T = 0.001, 1.2
    a, b = _nh_system(), _nh_system()
    p = a.params(capi.ECPR, cutoff=3.0, solver=capi.SOLVER_NEWTON)
    for g in (a, b):
        g.zero_forces()
        g.pair_forces(p)
    a.configure_step(p, integrator=capi.INT_NH, dt=dt, target_temp=T, rotations=1, rot_chain=1)
    a.step(1)                       # the first step runs eagerly through the same kernels as the graph
    a.synchronize()
    b.nht_initial(dt, T, 0.0, mode=1, rot_chain=1)
    b.qq_initial(dt)
    b.update_nlist()
    b.zero_forces()
    b.pair_forces(p)
    ke_b = b.nht_final(dt, T, 0.0, mode=1, rot_chain=1)
    kr_b = b.qq_final(dt)
    sa, sb = a.download(), b.download()
    for x, y in zip(sa, sb):
        assert rel(x, y) < 1e-6
    assert rel(a.nht_state(), b.nht_state()) < 1e-9
    e = a.energies()
    assert abs(e[2] - ke_b) < 1e-6 * ke_b and abs(e[3] - kr_b) < 1e-6 * kr_b
    # and the captured graph keeps stepping
    a.step(3)
    a.step_check()


def _nh_configured(p, dt, T):
    from sucrose_gb300 import capi
    g = _nh_system()
    g.zero_forces()
    g.pair_forces(p)
    g.configure_step(p, integrator=capi.INT_NH, dt=dt, target_temp=T, rotations=1, rot_chain=1)
    return g


def test_nose_hoover_steps_take_the_stored_sums_bit_for_bit(lib):
    """Launches after the first of a step call start their chain from the
    kinetic sums the previous final half stored (no grid-wide sum): the same
    bits as steps that recompute them, whether the steps come in one call, in
    calls of one step, or after a state write that forces the sums again."""
    from sucrose_gb300 import capi
    dt, T = 0.001, 1.2
    p = _nh_system().params(capi.ECPR, cutoff=3.0, solver=capi.SOLVER_NEWTON)
    a, b, c = _nh_configured(p, dt, T), _nh_configured(p, dt, T), _nh_configured(p, dt, T)
    a.step(6)                       # one call: five launches take the stored sums
    for _ in range(6):
        b.step(1)                   # calls of one step, nothing written between
    for k in range(6):
        c.configure_step(p, integrator=capi.INT_NH, dt=dt, target_temp=T, rotations=1, rot_chain=1)
        c.step(1)                   # re-captured each time: every step sums the state itself
    for g in (a, b, c):
        g.step_check()
    sa, sb, sc = a.download(), b.download(), c.download()
    for x, y, z in zip(sa, sb, sc):
        assert np.array_equal(x, y) and np.array_equal(x, z)
    assert np.array_equal(a.nht_state(), b.nht_state()) and np.array_equal(a.nht_state(), c.nht_state())
    # a host write between calls: the next step must sum the written state
    r, q, v, l = a.download()
    for g in (a, c):
        g.upload(v=f32(1.05 * v))
    c.configure_step(p, integrator=capi.INT_NH, dt=dt, target_temp=T, rotations=1, rot_chain=1)
    a.step(2)
    c.step(2)
    for x, y in zip(a.download(), c.download()):
        assert np.array_equal(x, y)
    assert np.array_equal(a.nht_state(), c.nht_state())


def _gb_system(seed=6):
    sig, eps = (1.0, 1.0, 3.0), (1.0, 1.0, 0.2)
    r, q, box = ellipsoids((16, 16, 8), sig, 0.3, seed=seed, tilt=0.05)
    n = len(r)
    v = configs.velocities_to_temperature(n, 1.0, seed)
    I = configs.default_inertia(sig)
    l = configs.angular_momenta(q, I, 1.0, seed)
    from sucrose_gb300 import GpuSystem
    g = GpuSystem(n, box)
    g.set_particles(sig=sig, eps=eps, inertia=I)
    g.upload(r=f32(r), q=f32(q), v=f32(v), l=f32(l))
    g.init_nlist(0.4, 6.0, trigger_mode=1)
    return g


@pytest.mark.parametrize("flat", [0, 1], ids=["conditional", "flat"])
def test_fused_langevin_step_matches_separate_calls(lib, flat):
    """The captured Langevin step, whose initial half step also runs the list
    test, zeroes the forces and writes the Gay-Berne prep, against the drop-in
    entry points called one by one; then a step whose list test requests a
    rebuild."""
    from sucrose_gb300 import capi
    dt, T = 0.002, 1.0
    a, b = _gb_system(), _gb_system()
    p = a.params(capi.GB, cutoff=4.0, mu=2, nu=1)
    for g in (a, b):
        g.zero_forces()
        g.pair_forces(p)
    a.configure_step(p, integrator=capi.INT_LANGEVIN, dt=dt, target_temp=T, damping=1.0, rotations=1,
                     first_step=7, flags=flat)
    a.step(1)                       # the first step runs eagerly through the same kernels as the graph
    a.synchronize()
    b.lgv_initial(dt, 7, damping=1.0, target_temp=T)
    b.update_nlist()
    b.zero_forces()
    pe_b, _ = b.pair_forces(p)
    ke_b, kr_b = b.lgv_final(dt, damping=1.0)
    sa, sb = a.download(), b.download()
    for x, y in zip(sa, sb):
        assert np.array_equal(x, y) or rel(x, y) < 1e-6
    fa, ta = a.forces()
    fb, tb = b.forces()
    assert rel(fa, fb) < 1e-6 and rel(ta, tb) < 1e-6
    e = a.energies()
    assert abs(e[0] - pe_b) < 1e-6 * abs(pe_b)
    assert abs(e[2] - ke_b) < 1e-6 * ke_b and abs(e[3] - kr_b) < 1e-6 * kr_b
    # a displacement beyond the skin: the fused test requests the rebuild
    builds = a.nlist_builds()
    r, q, v, l = a.download()
    a.upload(r=r, q=q, v=v + 150.0, l=l)   # a uniform drift of 0.3 per step
    a.step(1)
    a.step_check()
    assert a.nlist_builds() == builds + 1
    a.step(3)
    a.step_check()
