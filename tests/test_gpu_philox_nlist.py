"""Device Philox words and Verlet-list pair sets against the oracle (bit-exact)."""
import numpy as np
import pytest

import oracle as O
from helpers import Pair, lj_fcc, jittered_fcc, ellipsoids
from sucrose_gb300 import GpuSystem, SgError, capi

pytestmark = pytest.mark.gpu


def test_philox_words_bit_exact(lib):
    g = GpuSystem(4, 10.0)
    rng = np.random.default_rng(7)
    ctr = rng.integers(0, 2 ** 32, size=(1 << 20, 4), dtype=np.uint64).astype(np.uint32)
    ctr[:4] = [[0, 0, 0, 0], [0xFFFFFFFF] * 4, [1, 2, 3, 4], [108, 20000, 722, 1]]
    for key in ((0x6D2B79F5, 0x1B873593), (0xDEADBEEF, 0x12345678)):
        assert np.array_equal(g.philox(ctr, key), O.philox4x32(ctr, key))


def test_philox_normals(lib):
    g = GpuSystem(4, 10.0)
    idx = np.arange(1, 5001)
    ctr = np.stack([idx, np.full_like(idx, 17), np.full_like(idx, 1000), idx % 2], 1)
    dev = g.normal_3seq(ctr)
    ref = np.array([O.philox_normal_3seq(*c) for c in ctr])
    np.testing.assert_allclose(dev, ref, rtol=1e-13, atol=1e-13)


def _velocities_reference(n, temp, seed, nc=0, nrigid=1, remove_com=True):
    """The oracle's set_velocity_to_temperature (fortran/system.f90:361-421),
    FP64, with the module's NC and Nrigid set."""
    o = O.System(n, 60.0)
    o.s.nc, o.s.nrigid = nc, nrigid
    o.set_velocity_to_temperature(temp, seed, remove_com)
    return np.stack([o.vx, o.vy, o.vz], 1).copy()


def test_velocity_init_matches_readme_golden(lib):
    """The device set_velocity_to_temperature against the committed fixture of
    the README system (108 particles, T = 0.722, seed 15; the oracle's
    restatement of system.f90:361-421), to the FP32 rounding of the state."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "readme_velocities.npz"))["v"]
    s = GpuSystem(108, 10.0)
    s.set_velocity_to_temperature(0.722, 15)
    v = s.download()[2]
    np.testing.assert_allclose(v, g, rtol=1e-7, atol=2e-7)
    assert abs(np.sum(v ** 2) - (6 * 108 - 3) * 0.722) < 1e-5 * (6 * 108 - 3) * 0.722


@pytest.mark.parametrize("n,temp,seed,nc,nrigid,com", [(20000, 1.37, -3, 5000, 2, False),
                                                        (70001, 0.8, 2024, 0, 1, True)])
def test_velocity_init_options(lib, n, temp, seed, nc, nrigid, com):
    """Constraints counted in n_dof, no mean removal, Nrigid, a negative seed,
    and a grid of many blocks; the inverse mass in the velocity slot is kept
    (a half kick afterwards moves v by dt/2 F / m)."""
    s = GpuSystem(n, 60.0)
    s.set_particles(mass=np.full(n, 2.5))
    if nc:
        s.set_constraints(2 * np.arange(nc), 2 * np.arange(nc) + 1, 1.0)
    s.set_velocity_to_temperature(temp, seed, remove_com_velocity=com, nrigid=nrigid)
    v = s.download()[2]
    ref = _velocities_reference(n, temp, seed, nc, nrigid, com)
    np.testing.assert_allclose(v, ref, rtol=1e-7, atol=1e-6)
    f = np.tile([1.0, -2.0, 0.5], (n, 1))
    s.set_forces(f, np.zeros((n, 3)))
    s.vv_final(0.1)
    v2 = s.download()[2]
    np.testing.assert_allclose(v2 - v, 0.05 * f / 2.5, rtol=0, atol=1e-6)


def test_velocity_init_refusals(lib):
    s = GpuSystem(1, 10.0)
    with pytest.raises(SgError):
        s.set_velocity_to_temperature(1.0, 5)              # mean removal with one particle
    s.set_velocity_to_temperature(1.0, 5, remove_com_velocity=False)
    assert abs(np.sum(s.download()[2] ** 2) - 6.0) < 1e-5
    s = GpuSystem(10, 10.0)
    for t in (0.0, -1.0, float("nan")):
        with pytest.raises(SgError):
            s.set_velocity_to_temperature(t, 5)
    with pytest.raises(SgError):
        s.set_velocity_to_temperature(1.0, 5, nrigid=0)


def _pairs_equal(P, cutoff, skin):
    opi, opj = P.o.pairs(cutoff, skin)
    gpi, gpj = P.g.pairs()
    assert len(gpi) == len(opi)
    assert np.array_equal(gpi, opi) and np.array_equal(gpj, opj)
    return len(opi)


def test_nlist_readme_fcc(lib):
    r, q, box, v = lj_fcc()
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    assert _pairs_equal(P, 2.5, 0.3) == 3564
    # reference CSR, 1-based, exactly as build_nlist leaves nlist/offset
    onl, ooff = P.o.nlist(2.5, 0.3, one_based=True)
    gnl, goff = P.g.export_nlist(one_based=True)
    assert np.array_equal(onl, gnl) and np.array_equal(ooff, goff)
    assert goff[-1] == len(gnl) + 1


@pytest.mark.parametrize("cells,density", [(6, 0.8), (10, 0.7)])
def test_nlist_cells_jittered(lib, cells, density):
    r, q, box = jittered_fcc(cells, density, seed=cells)
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    assert _pairs_equal(P, 2.5, 0.3) > 0


def test_nlist_dense_cells_long_range(lib):
    # ~150 particles per cell (list radius 6.4 at density 0.3): rows built by
    # one warp per particle
    rng = np.random.default_rng(11)
    box = (4096 / 0.3) ** (1 / 3)
    r = rng.uniform(-box / 2, box / 2, size=(4096, 3))
    P = Pair(r, None, box)
    P.g.init_nlist(0.4, 6.0)
    assert _pairs_equal(P, 6.0, 0.4) > 100000


def test_nlist_dense_cells_follow_box_changes(lib):
    # a dense system (a warp per row over the stencil's x ranges) through a
    # shrinking and a growing box: each rebuilt list is the oracle's pair set,
    # so the cell grid followed the box
    rng = np.random.default_rng(12)
    box0 = (4096 / 0.3) ** (1 / 3)
    r0 = rng.uniform(-box0 / 2, box0 / 2, size=(4096, 3))
    P = Pair(r0, None, box0)
    P.g.init_nlist(0.4, 6.0)
    assert _pairs_equal(P, 6.0, 0.4) > 100000
    for s in (0.97, 1.1, 1.0, 0.9):
        r = np.asarray(r0 * s, dtype=np.float32).astype(np.float64)
        box = box0 * s
        P.g.set_box((box, box, box))
        P.g.upload(r=r)
        P.g.build_nlist()
        pi, pj = P.g.pairs()
        o = O.System(P.n, box)
        o.rx[:], o.ry[:], o.rz[:] = r.T
        oi, oj = o.pairs(6.0, 0.4)
        assert np.array_equal(pi, oi) and np.array_equal(pj, oj), s


def test_nlist_threshold_pairs(lib):
    # pairs placed within a few ulps of (rc+skin) on both sides, across the
    # periodic boundary: the FP64 re-test must decide them like the reference
    rng = np.random.default_rng(3)
    box = 20.0
    rl = 2.8
    base = rng.uniform(-box / 2, box / 2, size=(200, 3))
    d = rng.normal(size=(200, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    eps = rng.uniform(-3e-6, 3e-6, size=(200, 1))
    partner = base + d * (rl + eps)
    partner -= box * np.round(partner / box)
    r = np.concatenate([base, partner])
    P = Pair(r, None, box)
    P.g.init_nlist(0.3, 2.5)
    _pairs_equal(P, 2.5, 0.3)


@pytest.mark.parametrize("box", [60.0, 400.0])
def test_nlist_threshold_pairs_large_box(lib, box):
    # the same near-threshold pairs in boxes of 20 and 140 list radii, across
    # the boundary: the FP32 image shift with an FP32 box is furthest from
    # FP64 there, and the guard band widens with the box
    rng = np.random.default_rng(int(box))
    rl = 2.8
    base = rng.uniform(-box / 2, box / 2, size=(300, 3))
    base[:100, 0] = box / 2 - rng.uniform(0.0, 1.0, 100)   # partners wrap around in x
    d = rng.normal(size=(300, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[:100, 0] = np.abs(d[:100, 0])
    eps = rng.uniform(-3e-5, 3e-5, size=(300, 1))
    partner = base + d * (rl + eps)
    partner -= box * np.round(partner / box)
    r = np.concatenate([base, partner])
    P = Pair(r, None, box)
    P.g.init_nlist(0.3, 2.5)
    _pairs_equal(P, 2.5, 0.3)


def test_nlist_ellipsoid_cells(lib):
    r, q, box = ellipsoids((12, 16, 24), (3.0, 2.0, 1.0), 0.1114, seed=5, tilt=0.4)
    P = Pair(r, q, box, sig=(3.0, 2.0, 1.0))
    P.g.init_nlist(0.3, 3.0)
    _pairs_equal(P, 3.0, 0.3)


def test_nlist_open_boundaries(lib):
    rng = np.random.default_rng(11)
    r = rng.uniform(-6, 6, size=(300, 3))
    P = Pair(r, None, 100.0, periodic=False)
    P.g.init_nlist(0.3, 2.5)
    _pairs_equal(P, 2.5, 0.3)


def test_nlist_small_and_empty(lib):
    for n in (1, 2, 3, 8):
        r = np.arange(3 * n, dtype=np.float64).reshape(n, 3) * 0.7
        P = Pair(r, None, 30.0)
        P.g.init_nlist(0.3, 2.5)
        _pairs_equal(P, 2.5, 0.3)
    P = Pair(np.array([[0.0, 0, 0], [10.0, 0, 0]]), None, 30.0)
    P.g.init_nlist(0.3, 2.5)
    assert P.g.npairs() == 0


def test_nlist_cutoff_guard(lib):
    P = Pair(np.zeros((4, 3)) + np.arange(4)[:, None], None, 4.0)
    with pytest.raises(SgError) as e:
        P.g.init_nlist(0.3, 2.5)
    assert e.value.code == capi.SG_ECUTOFF_GT_HALFBOX


def test_nlist_trigger_matches_reference(lib):
    r, q, box = jittered_fcc(6, 0.8, seed=2)
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5, trigger_mode=0)
    last = P.r.copy()
    for amp in (0.1, 0.5, 1.3, 1.5):
        d = np.zeros_like(P.r)
        d[7, 0] = amp
        rn = P.r + d
        P.g.upload(r=rn)
        P.o.rx[:], P.o.ry[:], P.o.rz[:] = rn.T
        expect = P.o.needs_rebuild(last[:, 0].copy(), last[:, 1].copy(), last[:, 2].copy(), 2.5, 0.3, 0)
        assert P.g.needs_rebuild() == expect
    # skin trigger
    P.g.init_nlist(0.3, 2.5, trigger_mode=1)
    P.g.upload(r=P.r + np.array([0.16, 0, 0]) * (np.arange(P.n)[:, None] == 0))
    assert P.g.needs_rebuild()


def test_nlist_regrows_capacity(lib):
    # a dense blob forces rows far above the density estimate
    rng = np.random.default_rng(5)
    r = np.concatenate([rng.uniform(-1.0, 1.0, size=(400, 3)), rng.uniform(-15, 15, size=(200, 3))])
    P = Pair(r, None, 30.0)
    P.g.init_nlist(0.3, 2.5)
    _pairs_equal(P, 2.5, 0.3)
