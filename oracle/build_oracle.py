"""Build recipe for the oracle (test infrastructure only).

Produces, with plain g++ and no build system:
  oracle/_build/liboracle.so       FP64 restatement, strict IEEE (no FMA contraction,
                                   no fast-math): the checker used by the tests.
  oracle/_build/liboracle_fast.so  the same source at -O3 -ffast-math: the timed
                                   single-core CPU baseline (mirrors the reference's
                                   own -Ofast build flags, makefile_f90_linux.py:4).
  oracle/_ref/libsucrose_ref.so    the reference's C++ port compiled in place from
                                   its own sources (src/force.cpp, src/xmath.cpp,
                                   src/system.cpp, src/integrators.cpp) plus
                                   ref_shim.cpp, when the reference tree is present.
The reference's Fortran cannot be built: no Fortran compiler exists in this
image or on the GPU host. The reference tree is read from the directory named
by the SUCROSE_REFERENCE environment variable, else from /root/reference.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("SUCROSE_REFERENCE", "/root/reference")

STRICT = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]
FAST = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffast-math", "-fopenmp"]


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "sucrose_oracle.cpp")
    jobs = []
    for name, flags in (("liboracle.so", STRICT), ("liboracle_fast.so", FAST)):
        out = os.path.join(BUILD, name)
        if force or _stale(out, [src]):
            jobs.append(["g++", *flags, src, "-o", out])
    ref_src = os.path.join(REFERENCE_ROOT, "src")
    if os.path.isdir(ref_src):
        os.makedirs(REF_OUT, exist_ok=True)
        srcs = [os.path.join(ref_src, f) for f in ("force.cpp", "xmath.cpp", "system.cpp", "integrators.cpp")]
        srcs.append(os.path.join(HERE, "ref_shim.cpp"))
        out = os.path.join(REF_OUT, "libsucrose_ref.so")
        if force or _stale(out, srcs):
            jobs.append(["g++", *STRICT, "-I", os.path.join(REFERENCE_ROOT, "include"), *srcs, "-o", out])
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append(subprocess.Popen(cmd))
    for p, cmd in zip(procs, jobs):
        if p.wait() != 0:
            raise RuntimeError("oracle build failed: " + " ".join(cmd))


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
