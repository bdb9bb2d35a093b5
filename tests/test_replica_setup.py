"""Host-side set-up of the batched replica ensemble (no GPU)."""
import numpy as np

from sucrose_gb300 import configs


def test_ensemble_rules():
    e = configs.replica_ensemble(64, seed=1005)
    assert len(e["n"]) == 64
    assert np.all((e["n"] >= 64) & (e["n"] <= 2048))
    assert np.all(e["family"][:32] == 0) and np.all(e["family"][32:] == 1)
    for k in range(64):
        p = configs.LJ_REPLICA if e["family"][k] == 0 else configs.GB_REPLICA
        # the reference's init_nlist guard: cut-off at most half the box
        assert e["box"][k].min() >= 2.0 * p["list_cutoff"]
        assert p["rho"][0] <= e["density"][k] <= p["rho"][1]
        assert p["T"][0] <= e["temp"][k] <= p["T"][1]
        vol = np.prod(e["box"][k])
        assert abs(e["n"][k] / vol - e["density"][k]) < 1e-9 * e["density"][k]
        a, b = e["off"][k], e["off"][k + 1]
        assert np.all(np.abs(e["r"][a:b]) <= e["box"][k] / 2 + 0.1)
    assert len(np.unique(e["key"], axis=0)) == 64
    assert np.allclose(np.linalg.norm(e["q"], axis=1), 1.0)


def test_ensemble_is_seeded():
    a = configs.replica_ensemble(16, seed=3)
    b = configs.replica_ensemble(16, seed=3)
    c = configs.replica_ensemble(16, seed=4)
    assert np.array_equal(a["n"], b["n"]) and np.array_equal(a["r"], b["r"]) and np.array_equal(a["key"], b["key"])
    assert not np.array_equal(a["n"], c["n"])


def test_lattice_has_no_close_pairs():
    """Placement is overlap-free: nearest centres at least 0.8 of the lattice cell."""
    from scipy.spatial import cKDTree
    e = configs.replica_ensemble(8, seed=9, nmax=600)
    for k in range(8):
        a, b = e["off"][k], e["off"][k + 1]
        box = e["box"][k]
        t = cKDTree(e["r"][a:b] + box / 2, boxsize=box * (1 + 1e-12))
        d, _ = t.query(e["r"][a:b] + box / 2, k=2)
        cell = (1.0 / e["density"][k]) ** (1 / 3) * (0.5 if e["family"][k] == 1 else 1.0)
        assert d[:, 1].min() > 0.8 * cell * 0.85, k
