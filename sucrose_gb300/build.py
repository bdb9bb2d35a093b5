"""Build recipe for libsucrose_gb300.so: nvcc for sm_103a, no build system.

Every CUDA translation unit under csrc/ is compiled in parallel to an object
with one -gencode (compute_103a -> sm_103a) and linked into one shared
library with a plain C ABI (include/sucrose_gpu.h). Objects and the library
stay in-tree (sucrose_gb300/_build/, sucrose_gb300/lib/), git-ignored.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libsucrose_gb300.so")
ROOT = os.path.dirname(HERE)

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction, so host arithmetic rounds as written (the
# reporters' text must match other FP64 evaluations digit for digit)
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-ffp-contract=off",
         "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _deps():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(ROOT, "include", "sucrose_gpu.h")])


def _needs(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force=False, verbose=False, extra_flags=None):
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    deps = _deps()
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or _needs(obj, [src] + deps):
            jobs.append([NVCC, *ARCH, *FLAGS, *(extra_flags or []), "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.stderr

    with ThreadPoolExecutor(max_workers=min(16, max(1, os.cpu_count() or 4))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg.strip():
                print(msg)
    if force or jobs or _needs(LIB, objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        run(cmd)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None)
