"""The Fortran ISO_C_BINDING module (include/sucrose_gpu.f90) against the C
header and the library, without a Fortran compiler: every bind(c) name is a
declared and exported entry point, each interface has the C prototype's
argument count and passes each argument by value or by reference as the C
type requires, and the bind(c) derived types have the size and field offsets
of the C structures (computed with the C alignment rules, compared with the
ctypes mirrors)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "include", "sucrose_gpu.f90")
HDR = os.path.join(ROOT, "include", "sucrose_gpu.h")


def fortran_source():
    lines = []
    for ln in open(F90).read().splitlines():
        code = ln.split("!", 1)[0] if '"' not in ln.split("!", 1)[0] else ln
        lines.append(code)
    return re.sub(r"&\s*\n\s*", " ", "\n".join(lines))


def fortran_interfaces():
    """name -> (dummy argument names, {arg: declaration line})."""
    src = fortran_source()
    out = {}
    pat = re.compile(r"(?:function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*bind\(c,\s*name=\"(\w+)\"\)(.*?)end\s+(?:function|subroutine)",
                     re.S | re.I)
    for m in pat.finditer(src):
        args = [a.strip().lower() for a in m.group(2).split(",") if a.strip()]
        decl = {}
        for line in m.group(4).splitlines():
            if "::" not in line:
                continue
            spec, names = line.split("::", 1)
            for nm in re.split(r",\s*", names.strip()):
                nm = re.sub(r"\(.*", "", nm).strip().lower()
                if nm:
                    decl[nm] = spec.strip().lower()
        out[m.group(3)] = (m.group(1), args, decl)
    return out


def c_prototypes():
    txt = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    protos = {}
    for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(sg_\w+)\s*\(([^;]*?)\)\s*;", txt, flags=re.M):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        protos[m.group(1)] = params
    return protos


def test_every_binding_names_an_exported_entry_point():
    from sucrose_gb300 import capi
    import __graft_entry__
    __graft_entry__.build_library()
    lib = capi.load()
    ifs = fortran_interfaces()
    protos = c_prototypes()
    assert len(ifs) >= 30
    for cname in ifs:
        if cname == "strlen":
            continue
        assert cname in protos, f"{cname} is not declared in sucrose_gpu.h"
        assert hasattr(lib, cname), f"{cname} is not exported"


def test_argument_counts_and_passing_match_the_header():
    ifs = fortran_interfaces()
    protos = c_prototypes()
    for cname, (_, args, decl) in ifs.items():
        if cname == "strlen":
            continue
        params = protos[cname]
        assert len(args) == len(params), (cname, args, params)
        for a, p in zip(args, params):
            d = decl[a]
            is_ptr = "*" in p or "[" in p
            by_value = "value" in d
            if is_ptr:
                # a C pointer is a Fortran reference, or a c_ptr passed by value
                assert (not by_value) or "type(c_ptr)" in d, (cname, a, p, d)
            else:
                assert by_value, (cname, a, p, d)
            if "double" in p and not is_ptr:
                assert "real(c_double)" in d, (cname, a, p, d)
            if re.search(r"\bint32_t\b", p) and not is_ptr:
                assert "integer(c_int32_t)" in d, (cname, a, p, d)
            if re.search(r"\b(u?int64_t)\b", p) and not is_ptr:
                assert "integer(c_int64_t)" in d, (cname, a, p, d)


KIND_SIZE = {"integer(c_int32_t)": 4, "integer(c_int64_t)": 8, "real(c_double)": 8, "integer(c_int)": 4}


def fortran_type_layout(name, types):
    """(size, [(field, offset)]) of a bind(c) derived type, C alignment rules."""
    src = fortran_source()
    m = re.search(r"type,\s*bind\(c\)\s*::\s*%s\s*\n(.*?)end type" % name, src, re.S | re.I)
    assert m, name
    off, align_max, fields = 0, 1, []
    for line in m.group(1).splitlines():
        if "::" not in line:
            continue
        spec, names = (s.strip().lower() for s in line.split("::", 1))
        spec = spec.split(",")[0].strip()
        for nm in re.split(r",\s*(?![^()]*\))", names):
            nm = re.sub(r"=.*", "", nm).strip()
            if not nm:
                continue
            count = 1
            dm = re.match(r"(\w+)\((\d+)\)", nm)
            if dm:
                nm, count = dm.group(1), int(dm.group(2))
            if spec.startswith("type("):
                sub = spec[5:-1]
                size, _ = types[sub]
                al = 8
            else:
                size = KIND_SIZE[spec]
                al = size
            off = (off + al - 1) // al * al
            fields.append((nm, off))
            off += size * count
            align_max = max(align_max, al)
    size = (off + align_max - 1) // align_max * align_max
    return size, fields


def test_derived_types_match_the_c_structures():
    from sucrose_gb300 import capi
    types = {}
    for fname, cty in (("sg_pair_params", capi.PairParams), ("sg_ecp_stats", capi.EcpStats),
                       ("sg_step_config", capi.StepConfig)):
        size, fields = fortran_type_layout(fname, types)
        types[fname] = (size, fields)
        assert size == C.sizeof(cty), (fname, size, C.sizeof(cty))
        cfields = [f[0] for f in cty._fields_]
        assert [f for f, _ in fields] == cfields, (fname, fields, cfields)
        for f, o in fields:
            assert getattr(cty, f).offset == o, (fname, f, o, getattr(cty, f).offset)


@pytest.mark.parametrize("const", ["SG_LJ", "SG_WCA", "SG_GB", "SG_ECPR", "SG_SOLVER_NEWTON", "SG_INT_NH"])
def test_constants_match_the_header(const):
    src = fortran_source()
    m = re.search(r"\b%s\s*=\s*(\d+)" % const, src)
    hdr = open(HDR).read()
    h = re.search(r"\b%s\s*=\s*(\d+)" % const, hdr)
    assert m and h and m.group(1) == h.group(1), const
