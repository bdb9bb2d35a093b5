"""sg_lj_forces_noalloc: the pair-force entry point that allocates nothing.

Some callers cannot call cudaMalloc where they need forces: code that runs
while another library is capturing the stream into a CUDA graph, hosts whose
device memory all comes from their own pool, and OpenACC / CUDA Fortran
programs that keep the reference's RX..FZ module arrays resident on the
device. This entry point takes their device arrays as they are and keeps its
scratch in a fixed array inside the library.

Checked against the oracle (the reference's lj_ / wca_ / ljw_ restated in
FP64) and against the existing sg_pair_forces, on two calls in a row, with
the library's own list, with the list shuffled and its pairs turned round,
with 1-based indices, and with bad indices that must be skipped and counted.

Collected last on purpose: it shares the library's fixed scratch and runs
after every other test, and also passes when run alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from helpers import Pair, jittered_fcc, lj_fcc, rel
from sucrose_gb300 import capi

pytestmark = pytest.mark.gpu
TOL = 1e-5   # norm-wise relative error, as in the other force tests

KINDS = [(capi.LJ, O.LJ, {}), (capi.WCA, O.WCA, {"sigma": 1.1}), (capi.LJW, O.LJW, {"wf": 0.2})]


def call(L, n, dev, pi, pj, box, params, out, stream, one_based=0, bad=None):
    err = C.create_string_buffer(256)
    b = np.ascontiguousarray(box, dtype=np.float64)
    rc = L.sg_lj_forces_noalloc(n, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), pi.data_ptr(),
                                pj.data_ptr(), int(pi.numel()), one_based, b.ctypes.data_as(C.POINTER(C.c_double)), 1,
                                C.byref(params), out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(),
                                out[3].data_ptr(), None if bad is None else bad.data_ptr(), stream, err, 256)
    return rc, err.value.decode()


def device_arrays(P, pi_h, pj_h):
    import torch
    dev = [torch.tensor(P.r[:, k], dtype=torch.float64, device="cuda") for k in range(3)]
    pi = torch.tensor(np.asarray(pi_h), dtype=torch.int32, device="cuda")
    pj = torch.tensor(np.asarray(pj_h), dtype=torch.int32, device="cuda")
    out = [torch.zeros(P.n, dtype=torch.float64, device="cuda") for _ in range(3)]
    out.append(torch.zeros(2, dtype=torch.float64, device="cuda"))
    return dev, pi, pj, out


def oracle_forces(P, ko, kw, pi, pj, cutoff=2.5):
    P.o.zero_forces()
    P.o.forces(O.pair_params(ko, cutoff=cutoff, **kw), np.asarray(pi), np.asarray(pj))
    F, _ = P.oracle_forces()
    return F, P.o.s.pot_eng


def readme_state():
    # README example state (FCC, rho 0.8442, T 0.722, seed 15) after some
    # thermal displacement, so that forces are non-zero
    r, q, box, v = lj_fcc()
    return r + 0.05 * v, q, box


@pytest.mark.parametrize("kd,ko,kw", KINDS)
@pytest.mark.parametrize("state", ["readme", "jittered"])
def test_noalloc_matches_oracle_twice(lib, kd, ko, kw, state):
    import torch
    r, q, box = readme_state() if state == "readme" else jittered_fcc(6, 0.8442, seed=12, amp=0.1)
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    P.g.zero_forces()
    params = P.g.params(kd, cutoff=2.5, **kw)
    pe_lib, _ = P.g.pair_forces(params)
    F_lib, _ = P.g.forces()
    pi_h, pj_h = P.g.raw_pairs()
    F_or, pe_or = oracle_forces(P, ko, kw, pi_h, pj_h)

    dev, pi, pj, out = device_arrays(P, pi_h, pj_h)
    bad = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):   # the second call must not see the first call's scratch
        for t in out:
            t.zero_()
        rc, msg = call(lib, P.n, dev, pi, pj, P.box, params, out, stream, bad=bad)
        assert rc == capi.SG_OK, msg
        torch.cuda.synchronize()
        F = torch.stack(out[:3], 1).cpu().numpy()
        pe, vir = out[3].cpu().numpy()
        assert int(bad.item()) == 0
        assert rel(F, F_or) < TOL
        assert abs(pe - pe_or) <= TOL * abs(pe_or)
        # and the library's own entry point on the same list
        assert rel(F, F_lib) < TOL
        assert abs(pe - pe_lib) <= TOL * abs(pe_lib)


@pytest.mark.parametrize("kd,ko,kw", KINDS)
def test_noalloc_shuffled_turned_and_one_based(lib, kd, ko, kw):
    """The same pairs in a random order, a random half of them written j, i,
    and the indices 1-based: a row's pairs are no longer next to each other."""
    import torch
    r, q, box = jittered_fcc(6, 0.8442, seed=21, amp=0.1)
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    pi_h, pj_h = P.g.raw_pairs()
    F_or, pe_or = oracle_forces(P, ko, kw, pi_h, pj_h)
    rng = np.random.default_rng(5)
    perm = rng.permutation(len(pi_h))
    a, b = np.asarray(pi_h)[perm], np.asarray(pj_h)[perm]
    swap = rng.random(len(a)) < 0.5
    a, b = np.where(swap, b, a), np.where(swap, a, b)
    # runs of one i that are not next to each other inside a warp
    assert any(len(set(a[k:k + 32])) < len(a[k:k + 32]) for k in range(0, len(a), 32))
    dev, pi, pj, out = device_arrays(P, a + 1, b + 1)
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    params = P.g.params(kd, cutoff=2.5, **kw)
    rc, msg = call(lib, P.n, dev, pi, pj, P.box, params, out, torch.cuda.current_stream().cuda_stream,
                   one_based=1, bad=bad)
    assert rc == capi.SG_OK, msg
    torch.cuda.synchronize()
    F = torch.stack(out[:3], 1).cpu().numpy()
    assert int(bad.item()) == 0
    assert rel(F, F_or) < TOL
    assert abs(out[3][0].item() - pe_or) <= TOL * abs(pe_or)


def test_noalloc_skips_and_counts_bad_indices(lib):
    import torch
    r, q, box = jittered_fcc(5, 0.8442, seed=8, amp=0.1)
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    pi_h, pj_h = (np.asarray(x) for x in P.g.raw_pairs())
    F_or, pe_or = oracle_forces(P, O.LJ, {}, pi_h, pj_h)
    n = P.n
    junk_i = np.array([n, -1, 3, 131072 + 5, 2 ** 31 - 1, 7], dtype=np.int64)
    junk_j = np.array([0, 4, 3, 1, 2, -2 ** 31], dtype=np.int64)
    a = np.insert(pi_h.astype(np.int64), [5, 40, 41, 300, 301, len(pi_h)], junk_i)
    b = np.insert(pj_h.astype(np.int64), [5, 40, 41, 300, 301, len(pj_h)], junk_j)
    dev, pi, pj, out = device_arrays(P, a, b)
    bad = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc, msg = call(lib, n, dev, pi, pj, P.box, P.g.params(capi.LJ, cutoff=2.5), out,
                   torch.cuda.current_stream().cuda_stream, bad=bad)
    assert rc == capi.SG_OK, msg
    torch.cuda.synchronize()
    assert int(bad.item()) == len(junk_i)
    F = torch.stack(out[:3], 1).cpu().numpy()
    assert rel(F, F_or) < TOL
    assert abs(out[3][0].item() - pe_or) <= TOL * abs(pe_or)


def test_noalloc_adds_into_the_outputs_and_allocates_nothing(lib):
    import torch
    r, q, box = readme_state()
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    pi_h, pj_h = P.g.raw_pairs()
    params = P.g.params(capi.LJ, cutoff=2.5)
    dev, pi, pj, out = device_arrays(P, pi_h, pj_h)
    stream = torch.cuda.current_stream().cuda_stream
    assert call(lib, P.n, dev, pi, pj, P.box, params, out, stream)[0] == capi.SG_OK
    torch.cuda.synchronize()
    once = [t.clone() for t in out]
    free0, _ = torch.cuda.mem_get_info()
    assert call(lib, P.n, dev, pi, pj, P.box, params, out, stream)[0] == capi.SG_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    # FP32 atomics sum in a different order each call: compare norm-wise
    for a, b in zip(out, once):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert rel(a, 2 * b) < TOL


def test_noalloc_rejects_oversize(lib):
    import torch
    params = capi.PairParams(capi.LJ, 0, 0, 0, 1.0, 1.0, 2.5, 0.0, 0.0, 0.0, 0, 0)
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    ij = torch.zeros(1, dtype=torch.int32, device="cuda")
    err = C.create_string_buffer(256)
    b = np.array([10.0, 10.0, 10.0])
    rc = lib.sg_lj_forces_noalloc(131073, x.data_ptr(), x.data_ptr(), x.data_ptr(), ij.data_ptr(), ij.data_ptr(), 0, 0,
                                  b.ctypes.data_as(C.POINTER(C.c_double)), 1, C.byref(params), x.data_ptr(),
                                  x.data_ptr(), x.data_ptr(), x.data_ptr(), None, None, err, 256)
    assert rc == capi.SG_EINVAL
    assert b"131072" in err.value
