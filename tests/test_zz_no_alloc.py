"""sg_lj_forces_noalloc: the pair-force entry point that allocates nothing,
for callers that already hold their particle data on the device and cannot
call cudaMalloc where they call it (inside another library's stream capture,
with a pooled allocator, from OpenACC/CUDA Fortran with device-resident module
arrays). Checked against the existing sg_pair_forces on two calls in a row.

Collected last on purpose: it shares the library's fixed scratch and runs
after every other test, and also passes when run alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import Pair, jittered_fcc, rel
from sucrose_gb300 import capi

pytestmark = pytest.mark.gpu
TOL = 1e-5   # norm-wise relative error, as in the other force tests


def call(L, n, dev, pi, pj, box, params, out, stream):
    err = C.create_string_buffer(256)
    b = np.ascontiguousarray(box, dtype=np.float64)
    rc = L.sg_lj_forces_noalloc(n, dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(), pi.data_ptr(),
                                pj.data_ptr(), int(pi.numel()), b.ctypes.data_as(C.POINTER(C.c_double)), 1,
                                C.byref(params), out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(),
                                out[3].data_ptr(), stream, err, 256)
    return rc, err.value.decode()


@pytest.mark.parametrize("kind,kw", [(capi.LJ, {}), (capi.WCA, {"sigma": 1.1}), (capi.LJW, {"wf": 0.2})])
def test_noalloc_matches_pair_forces_twice(lib, kind, kw):
    import torch
    r, q, box = jittered_fcc(6, 0.8442, seed=12, amp=0.1)
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    P.g.zero_forces()
    params = P.g.params(kind, cutoff=2.5, **kw)
    pe_ref, vir_ref = P.g.pair_forces(params)
    F_ref, _ = P.g.forces()
    pi_h, pj_h = P.g.raw_pairs()

    n = P.n
    dev = [torch.tensor(P.r[:, k], dtype=torch.float64, device="cuda") for k in range(3)]
    pi = torch.tensor(pi_h, dtype=torch.int32, device="cuda")
    pj = torch.tensor(pj_h, dtype=torch.int32, device="cuda")
    out = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    out.append(torch.zeros(2, dtype=torch.float64, device="cuda"))
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):   # the second call must not see the first call's scratch
        for t in out:
            t.zero_()
        rc, msg = call(lib, n, dev, pi, pj, P.box, params, out, stream)
        assert rc == capi.SG_OK, msg
        torch.cuda.synchronize()
        F = torch.stack(out[:3], 1).cpu().numpy()
        pe, vir = out[3].cpu().numpy()
        assert rel(F, F_ref) < TOL
        assert abs(pe - pe_ref) <= TOL * abs(pe_ref)
        assert abs(vir - vir_ref) <= TOL * abs(vir_ref)


def test_noalloc_adds_into_the_outputs(lib):
    import torch
    r, q, box = jittered_fcc(4, 0.8, seed=3, amp=0.1)
    P = Pair(r, q, box)
    P.g.init_nlist(0.3, 2.5)
    pi_h, pj_h = P.g.raw_pairs()
    params = P.g.params(capi.LJ, cutoff=2.5)
    dev = [torch.tensor(P.r[:, k], dtype=torch.float64, device="cuda") for k in range(3)]
    pi = torch.tensor(pi_h, dtype=torch.int32, device="cuda")
    pj = torch.tensor(pj_h, dtype=torch.int32, device="cuda")
    out = [torch.zeros(P.n, dtype=torch.float64, device="cuda") for _ in range(3)]
    out.append(torch.zeros(2, dtype=torch.float64, device="cuda"))
    stream = torch.cuda.current_stream().cuda_stream
    assert call(lib, P.n, dev, pi, pj, P.box, params, out, stream)[0] == capi.SG_OK
    torch.cuda.synchronize()
    once = [t.clone() for t in out]
    assert call(lib, P.n, dev, pi, pj, P.box, params, out, stream)[0] == capi.SG_OK
    torch.cuda.synchronize()
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
    rc = lib.sg_lj_forces_noalloc(131073, x.data_ptr(), x.data_ptr(), x.data_ptr(), ij.data_ptr(), ij.data_ptr(), 0,
                                  b.ctypes.data_as(C.POINTER(C.c_double)), 1, C.byref(params), x.data_ptr(),
                                  x.data_ptr(), x.data_ptr(), x.data_ptr(), None, err, 256)
    assert rc == capi.SG_EINVAL
    assert b"131072" in err.value
