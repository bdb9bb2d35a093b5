"""Host arrays in and out of the C ABI.

Page-locked (mapped) host arrays are read and written in place by the
conversion kernels; pageable ones are staged through device copies. Both
paths must give the same FP32 state and the same FP64 arrays back, bit for
bit, for the state and for the forces."""
import ctypes as C

import numpy as np
import pytest

from sucrose_gb300 import GpuSystem

pytestmark = pytest.mark.gpu
D = C.POINTER(C.c_double)


def _pinned(torch, n, offset=0):
    # offset 1: the column starts 8 bytes into the allocation (8-byte aligned only)
    return torch.empty(n + offset, dtype=torch.float64, pin_memory=True).numpy()[offset:]


def _state(n, seed):
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    cols = [rng.uniform(-9.0, 9.0, n) for _ in range(3)] + [q[:, k].copy() for k in range(4)]
    cols += [rng.normal(size=n) for _ in range(6)]
    return cols


@pytest.mark.parametrize("offset", [0, 1])
@pytest.mark.parametrize("n", [1, 37, 4096])
def test_pinned_state_round_trip_matches_pageable(lib, n, offset):
    torch = pytest.importorskip("torch")
    cols = _state(n, n)
    g = GpuSystem(n, 20.0)
    # pageable: staged copies
    g.L.sg_upload_state(g.ctx, *[c.ctypes.data_as(D) for c in cols])
    ref = [np.empty(n) for _ in range(13)]
    assert g.L.sg_download_state(g.ctx, *[a.ctypes.data_as(D) for a in ref]) == 0
    # page-locked: in place
    g.L.sg_upload_state(g.ctx, *[np.zeros(n).ctypes.data_as(D) for _ in range(13)])
    pin_in = [_pinned(torch, n, offset if k % 2 else 0) for k in range(13)]
    for p, c in zip(pin_in, cols):
        p[:] = c
    assert g.L.sg_upload_state(g.ctx, *[p.ctypes.data_as(D) for p in pin_in]) == 0
    pin_out = [_pinned(torch, n, offset if k % 3 == 0 else 0) for k in range(13)]
    for p in pin_out:
        p[:] = np.nan
    assert g.L.sg_download_state(g.ctx, *[p.ctypes.data_as(D) for p in pin_out]) == 0
    for k in range(13):
        assert np.array_equal(pin_out[k], ref[k]), k
        assert np.array_equal(ref[k], cols[k].astype(np.float32).astype(np.float64)), k
    g.close()


def test_mixed_pinned_and_pageable_columns(lib):
    # one pageable column among page-locked ones: the whole group is staged
    torch = pytest.importorskip("torch")
    n = 513
    cols = _state(n, 5)
    g = GpuSystem(n, 20.0)
    arrs = []
    for k, c in enumerate(cols):
        if k == 1:
            arrs.append(c.copy())
        else:
            p = _pinned(torch, n)
            p[:] = c
            arrs.append(p)
    assert g.L.sg_upload_state(g.ctx, *[a.ctypes.data_as(D) for a in arrs]) == 0
    r, q, v, l = g.download()
    got = np.concatenate([r.T, q.T, v.T, l.T])
    want = np.array([c.astype(np.float32).astype(np.float64) for c in cols])
    assert np.array_equal(got, want)
    g.close()


def test_pinned_forces_round_trip(lib):
    torch = pytest.importorskip("torch")
    n = 1000
    rng = np.random.default_rng(9)
    cols = [rng.normal(size=n) for _ in range(6)]
    g = GpuSystem(n, 20.0)
    pin = [_pinned(torch, n) for _ in range(6)]
    for p, c in zip(pin, cols):
        p[:] = c
    assert g.L.sg_upload_forces(g.ctx, *[p.ctypes.data_as(D) for p in pin]) == 0
    out = [_pinned(torch, n) for _ in range(6)]
    assert g.L.sg_download_forces(g.ctx, *[p.ctypes.data_as(D) for p in out]) == 0
    F, T = g.forces()
    for k in range(3):
        assert np.array_equal(out[k], F[:, k]) and np.array_equal(out[3 + k], T[:, k])
        assert np.array_equal(F[:, k], cols[k].astype(np.float32).astype(np.float64))
    g.close()
