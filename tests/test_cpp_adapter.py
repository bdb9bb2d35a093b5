"""The C++ adapters (include/sucrose_gpu.hpp): the README's LJ loop written in
C++ against them compiles and links here; on the GPU it runs and gives the
energies of the same loop driven through the Python bindings."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "readme_lj.cpp")


def build_exe(tmp_path):
    import __graft_entry__
    __graft_entry__.build_library()
    lib = os.path.join(ROOT, "sucrose_gb300", "lib")
    exe = str(tmp_path / "readme_lj")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", lib, "-lsucrose_gb300", "-Wl,-rpath," + lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_adapter_compiles_and_links(tmp_path):
    build_exe(tmp_path)


@pytest.mark.gpu
def test_readme_loop_in_cpp_matches_python(tmp_path):
    from sucrose_gb300 import GpuSystem, capi, configs
    exe = build_exe(tmp_path)
    r, q, box = configs.fcc_lattice(3, 0.8442)
    box = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)).copy()
    v = configs.velocities_to_temperature(len(r), 0.722, 15)
    state = tmp_path / "state.bin"
    with open(state, "wb") as f:
        np.concatenate([[len(r)], box, r[:, 0], r[:, 1], r[:, 2], v[:, 0], v[:, 1], v[:, 2]]).astype(np.float64).tofile(f)
    out = subprocess.run([exe, str(state), "200", "50"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    rows = [ln.split() for ln in out.stdout.splitlines() if not ln.startswith("final")]
    cpp = np.array([[float(x) for x in row[1:]] for row in rows])

    g = GpuSystem(len(r), box)
    g.upload(r=r, v=v)
    g.init_nlist(0.3, 2.5)
    p = g.params(capi.LJ, cutoff=2.5)
    g.zero_forces()
    g.pair_forces(p)
    py = []
    for step in range(1, 201):
        g.vv_initial(0.0005)
        if g.needs_rebuild():
            g.build_nlist()
        g.zero_forces()
        pe, _ = g.pair_forces(p)
        ke = g.vv_final(0.0005)
        if step % 50 == 0:
            py.append((pe, ke))
    py = np.array(py)
    assert cpp.shape == py.shape
    # the same device code on the same inputs; only float atomics may reorder
    assert np.allclose(cpp, py, rtol=1e-5, atol=1e-8)
