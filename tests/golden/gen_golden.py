"""Generates the committed golden fixtures (run in the build container, where
the reference tree is present):

  ref_lj_untruncated.npz  forces and energy of the reference's own C++
                          LennardJones::calculate_forces (src/force.cpp:6-37),
                          compiled from the reference sources into oracle/_ref,
                          over all pairs of a jittered 108-particle FCC box.
  ref_vv_step.npz         one VerletIntegrator initial_step / final_step of the
                          same C++ port (src/integrators.cpp:7-38), unit mass.
  ref_morse.npz           forces and energy of the reference's C++
                          MorsePotential::calculate_forces (src/force.cpp:113-140,
                          no cutoff, no shift), all pairs of the same box,
                          D = 1.3, r0 = 1.1, alpha = 1.7.
  philox_words.npz        Philox4x32-10 words of the reference key for fixed
                          counters, from the oracle restatement (xmath.f90:42-76),
                          as a regression anchor for the device and host copies.
  readme_velocities.npz   set_velocity_to_temperature(0.722, seed=15) of the
                          README example (system.f90:362-421), oracle restatement.

Usage: python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def jittered_fcc():
    (rx, ry, rz, qw, qx, qy, qz), L = O.fcc_lattice(3, 0.8442)
    rng = np.random.default_rng(2024)
    r = np.stack([rx, ry, rz], 1) + rng.uniform(-0.15, 0.15, size=(108, 3))
    return r, L


def main():
    R = O.ref_lib()
    if R is None:
        raise SystemExit("the reference C++ port is not built (oracle/_ref missing)")
    r, L = jittered_fcc()
    n = len(r)
    pi, pj = np.triu_indices(n, 1)
    pi = pi.astype(np.int32)
    pj = pj.astype(np.int32)
    rx, ry, rz = (np.ascontiguousarray(r[:, k]) for k in range(3))
    fx, fy, fz, pot = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(1)
    R.ref_lj_forces(n, L, 1, O.dptr(rx), O.dptr(ry), O.dptr(rz), 1.0, 1.0, len(pi), O.iptr(pi), O.iptr(pj),
                    O.dptr(fx), O.dptr(fy), O.dptr(fz), O.dptr(pot))
    np.savez(os.path.join(HERE, "ref_lj_untruncated.npz"), r=r, box=L, fx=fx, fy=fy, fz=fz, pot=pot[0])

    rng = np.random.default_rng(7)
    v = rng.normal(size=(n, 3))
    f = rng.normal(size=(n, 3)) * 10.0
    out = {}
    for which in (0, 1):
        a = [np.ascontiguousarray(x) for x in (r[:, 0], r[:, 1], r[:, 2], v[:, 0], v[:, 1], v[:, 2])]
        fa = [np.ascontiguousarray(f[:, k]) for k in range(3)]
        R.ref_vv_step(n, L, 1, 0.005, *[O.dptr(x) for x in a], *[O.dptr(x) for x in fa], which)
        out[f"r{which}"] = np.stack(a[:3], 1)
        out[f"v{which}"] = np.stack(a[3:], 1)
    np.savez(os.path.join(HERE, "ref_vv_step.npz"), r=r, v=v, f=f, box=L, dt=0.005, **out)

    ctr = rng.integers(0, 2 ** 32, size=(256, 4), dtype=np.uint64).astype(np.uint32)
    ctr[0] = 0
    np.savez(os.path.join(HERE, "philox_words.npz"), ctr=ctr, words=O.philox4x32(ctr))

    s = O.System(108, L)
    s.set_velocity_to_temperature(0.722, 15)
    np.savez(os.path.join(HERE, "readme_velocities.npz"), v=np.stack([s.vx, s.vy, s.vz], 1))

    fx, fy, fz, pot = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(1)
    R.ref_morse_forces(n, L, 1, O.dptr(rx), O.dptr(ry), O.dptr(rz), 1.3, 1.1, 1.7, len(pi), O.iptr(pi), O.iptr(pj),
                       O.dptr(fx), O.dptr(fy), O.dptr(fz), O.dptr(pot))
    np.savez(os.path.join(HERE, "ref_morse.npz"), r=r, box=L, D=1.3, r0=1.1, alpha=1.7, fx=fx, fy=fy, fz=fz,
             pot=pot[0])


if __name__ == "__main__":
    main()
