"""Reporters (fortran/reporters.f90) written asynchronously by the library,
checked byte for byte against the test restatement of the record layouts
(oracle/reporters_ref.py) on the same device state; checkpoint round trips."""
import numpy as np
import pytest

from helpers import Pair, f32, jittered_fcc
from oracle import reporters_ref as R
from sucrose_gb300 import GpuSystem, capi
from sucrose_gb300.molecules import molecular_mix

pytestmark = pytest.mark.gpu


def system(seed=3):
    r, box, bbi, bbj, ln, mol = molecular_mix(3, 3.0, seed)
    n = len(r)
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    sig = (1.0, 1.0, 1.0)
    P = Pair(r, q, box, v=rng.normal(size=(n, 3)), l=rng.normal(size=(n, 3)))
    types = rng.integers(0, 3, n)
    P.g.set_types(types)
    charge = f32(rng.choice([0.0, 0.5, 1.0], n))
    P.g.set_charges(charge)
    P.g.set_constraints(bbi, bbj, ln)
    P.g.init_nlist(0.3, 0.9)
    P.g.zero_forces()
    P.g.pair_forces(P.g.params(capi.WCA, sigma=0.9, cutoff=0.9))
    return P, types, charge, (bbi, bbj, ln)


def device_state(g):
    r, q, v, l = g.download()
    F, T = g.forces()
    return r, q, v, l, F


def test_trajectory_config_checkpoint_bytes(lib, tmp_path):
    P, types, charge, bonds = system()
    g = P.g
    paths = {k: tmp_path / f"{k}.txt" for k in ("traj", "conf", "ckpt")}
    with g.reporter(capi.REPORT_TRAJECTORY, paths["traj"]) as rt, g.reporter(capi.REPORT_CONFIG, paths["conf"]) as rc, \
            g.reporter(capi.REPORT_CHECKPOINT, paths["ckpt"]) as rk:
        rt.write(7)
        rc.write(7)
        rk.write(7)
    r, q, v, l, F = device_state(g)
    n = g.n
    shape = np.ones((n, 3))
    assert paths["traj"].read_text() == R.trajectory(7, g.box, types, shape, r, q, F)
    assert paths["conf"].read_text() == R.config(r, v, l, q)
    I = np.full((n, 3), f32(0.1))   # default inertia (s_y^2 + s_z^2) / 20 of unit spheres
    want = R.checkpoint(g.box, types, np.ones(n), charge, shape, np.ones((n, 3)), I, r, v, l, q,
                        list(zip(*bonds)))
    assert paths["ckpt"].read_text() == want


def test_state_data_lines(lib, tmp_path):
    P, types, charge, bonds = system(seed=5)
    g = P.g
    path = tmp_path / "state.txt"
    n = g.n
    dof = 6 * n - len(bonds[0])
    dens = n / np.prod(g.box)
    with g.reporter(capi.REPORT_STATE, path, dof=dof, density=dens) as rs:
        ke = g.vv_final(0.001)
        rs.write(1)
        rs.flush()
        e = g.energies()
        t = g.thermo(dof, dens)
    lines = path.read_text().splitlines(keepends=True)
    assert lines[0] == R.state_header()
    assert lines[1] == R.state_line(1, n, e[0], e[2], e[3], t[0], t[2], dens)


def test_async_writes_follow_the_stream(lib, tmp_path):
    # snapshots taken between steps hold the state of that point of the
    # stream, not of the host's later view
    r, q, box = jittered_fcc(6, 0.8, seed=2, amp=0.05)
    g = GpuSystem(len(r), box)
    g.upload(r=r, q=q)
    g.init_nlist(0.3, 2.5)
    g.configure_step(g.params(capi.LJ, cutoff=2.5), integrator=capi.INT_LANGEVIN, dt=0.002)
    path = tmp_path / "conf.txt"
    snaps = []
    with g.reporter(capi.REPORT_CONFIG, path) as rc:
        for k in range(4):
            g.step(3)
            rc.write(k)
            rr, qq, vv, ll = g.download()
            snaps.append(R.config(rr, vv, ll, qq))
    assert path.read_text() == "".join(snaps)


def test_checkpoint_round_trip(lib, tmp_path):
    P, types, charge, bonds = system(seed=7)
    g = P.g
    path = tmp_path / "ck.txt"
    with g.reporter(capi.REPORT_CHECKPOINT, path) as rk:
        rk.write(0)
    h, cfg = GpuSystem.load_checkpoint(path)
    assert cfg == 0 and h.n == g.n
    r0, q0, v0, l0 = g.download()
    r1, q1, v1, l1 = h.download()
    # the text carries 10 decimals
    for a, b in ((r0, r1), (q0, q1), (v0, v1), (l0, l1)):
        assert np.max(np.abs(a - b)) < 1e-9 + 1e-7 * np.max(np.abs(a))
    # and writing it again gives the same file
    path2 = tmp_path / "ck2.txt"
    with h.reporter(capi.REPORT_CHECKPOINT, path2) as rk:
        rk.write(0)
    assert path2.read_text() == path.read_text()


def test_binary_state_is_exact(lib, tmp_path):
    r, q, box = jittered_fcc(6, 0.8, seed=4, amp=0.05)
    g = GpuSystem(len(r), box)
    g.upload(r=r, q=q)
    g.init_nlist(0.3, 2.5)
    g.configure_step(g.params(capi.LJ, cutoff=2.5), integrator=capi.INT_LANGEVIN, dt=0.002)
    g.step(10)
    g.save_state(tmp_path / "s.bin")
    a = g.download()
    g.step(5)
    g.load_state(tmp_path / "s.bin")
    b = g.download()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
