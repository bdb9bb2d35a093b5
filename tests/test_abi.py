"""The C-ABI library: it loads (no GPU needed to dlopen) and exports every
entry point that include/sucrose_gpu.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(sg_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def built_lib():
    import __graft_entry__
    __graft_entry__.build_library()
    from sucrose_gb300 import capi
    return capi.load()


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("sg_create", "sg_pair_forces", "sg_nlist_init", "sg_vv_initial", "sg_lgv_initial", "sg_nht_initial",
                 "sg_philox4x32", "sg_nlist_export"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    missing = [n for n in sorted(declared_symbols()) if not hasattr(built_lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built_lib):
    from sucrose_gb300 import capi
    bound = {s[0] for s in capi.SIGNATURES}
    assert declared_symbols() <= bound, sorted(declared_symbols() - bound)


def test_host_philox_matches_oracle(built_lib):
    # sg_philox4x32 is host code: callable without a GPU
    import numpy as np
    import oracle as O
    rng = np.random.default_rng(0)
    for _ in range(200):
        c = rng.integers(0, 2 ** 32, size=4, dtype=np.uint64).astype(np.uint32)
        k = rng.integers(0, 2 ** 32, size=2, dtype=np.uint64).astype(np.uint32)
        out = (ctypes.c_uint32 * 4)()
        built_lib.sg_philox4x32((ctypes.c_uint32 * 4)(*c), (ctypes.c_uint32 * 2)(*k), out)
        assert list(out) == list(O.philox4x32(c[None], k)[0])


def test_create_without_gpu_fails_cleanly(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ctx = ctypes.c_void_p()
    rc = built_lib.sg_create(ctypes.byref(ctx), 16, 0)
    assert rc != 0
    msg = built_lib.sg_last_error(ctx)
    assert msg
    built_lib.sg_destroy(ctx)


def test_null_context_is_refused_by_every_entry_point(built_lib):
    """Every entry point whose first argument is the context returns
    SG_EINVAL for a NULL context (other arguments zero or NULL) before any
    device work; sg_destroy and sg_reporter_close accept NULL like free."""
    from sucrose_gb300 import capi
    ok_null = {"sg_destroy": 0, "sg_reporter_close": 0}
    checked = 0
    for name, res, args in capi.SIGNATURES:
        if not args or args[0] is not capi._P or name in ("sg_last_error", "sg_stream"):
            continue
        f = getattr(built_lib, name)
        f.restype, f.argtypes = res, args
        vals = []
        for t in args:
            if t in (ctypes.c_int32, ctypes.c_int, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint64):
                vals.append(0)
            elif t in (ctypes.c_double, ctypes.c_float):
                vals.append(0.0)
            else:
                vals.append(None)
        assert f(*vals) == ok_null.get(name, capi.SG_EINVAL), name
        checked += 1
    assert checked > 80
    f = built_lib.sg_last_error
    f.restype, f.argtypes = ctypes.c_char_p, [ctypes.c_void_p]
    assert f(None)
