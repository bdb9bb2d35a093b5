"""Small, self-contained launches of each kernel family, for profiling.

    python -m sucrose_gb300.profile_case <case> [--reps K]

Each case builds one seeded system at the size of its benchmark workload (or
smaller where noted), runs one untimed launch sequence, then K launches of
the kernels of interest and exits. A profiler selects the kernel with its own
filter (for example ncu -k regex:k_pair -c 2). Cases:

  ecp       ECP (3,2,1) ellipsoids, N = 65 536, repulsive kind, Newton solve
  ecp_mlp   the same with the learned guess (weights from a short training)
  gb        Gay-Berne (3,5,2,1), N = 32 768, filtered launch
  lj        Lennard-Jones fcc, N = 32 000
  list      neighbour-list rebuild of the ECP system (forced, every launch)
  gb_list   neighbour-list rebuild of the Gay-Berne system (list radius 6.4)
  langevin  Langevin step (initial + final) with rotations, N = 32 768
  nhc       Nose-Hoover chain step with rotations, N = 65 536
  mlp_train one MLP training step on 65 536 samples
  ecp_step  captured Nose-Hoover steps of the ECP system (list build as
            flag-gated kernels, so that a profiler sees every kernel)
  replicas  captured steps of --nrep replicas (default 1 024, LJ + GB), same flag
"""
import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from sucrose_gb300 import GpuSystem, capi, configs  # noqa: E402


def ecp_system():
    sig = (3.0, 2.0, 1.0)
    r, q, box = configs.aligned_lattice((32, 32, 64), sig, 0.1114, seed=1003, jitter=0.02, tilt=0.2)
    g = GpuSystem(len(r), box)
    g.set_particles(sig=sig, inertia=configs.default_inertia(sig))
    g.upload(r=r, q=q, v=configs.velocities_to_temperature(len(r), 1.2, 3))
    g.init_nlist(0.3, 3.0, trigger_mode=1)
    return g, g.params(capi.ECPR, cutoff=3.0, solver=capi.SOLVER_NEWTON)


def gb_system():
    sig = (1.0, 1.0, 3.0)
    r, q, box = configs.aligned_lattice((64, 32, 16), sig, 0.30, seed=1002, jitter=0.02, tilt=0.15)
    g = GpuSystem(len(r), box)
    g.set_particles(sig=sig, eps=(1.0, 1.0, 0.2), inertia=configs.default_inertia(sig))
    g.upload(r=r, q=q, v=configs.velocities_to_temperature(len(r), 1.0, 2))
    g.init_nlist(0.4, 6.0, trigger_mode=1)
    return g, g.params(capi.GB, cutoff=4.0, mu=2, nu=1)


def lj_system():
    r, q, box = configs.fcc_lattice(20, 0.8442)
    g = GpuSystem(len(r), box)
    g.upload(r=r, v=configs.velocities_to_temperature(len(r), 0.722, 15))
    g.init_nlist(0.3, 2.5, trigger_mode=1)
    return g, g.params(capi.LJ, cutoff=2.5)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--nrep", type=int, default=1024, help="replicas (case replicas)")
    ap.add_argument("--equil", type=int, default=0, help="untimed steps before the profiled ones (case replicas)")
    a = ap.parse_args()
    if a.case in ("ecp", "ecp_mlp", "list", "nhc", "ecp_step"):
        g, p = ecp_system()
    elif a.case in ("gb", "langevin", "gb_list"):
        g, p = gb_system()
    elif a.case == "lj":
        g, p = lj_system()
    elif a.case == "mlp_train":
        g, p = ecp_system()
    elif a.case == "replicas":
        g = None
    else:
        raise SystemExit("unknown case " + a.case)

    if a.case in ("ecp", "gb", "lj"):
        for _ in range(1 + a.reps):
            g.zero_forces()
            g.pair_forces(p)
    elif a.case == "ecp_mlp":
        from sucrose_gb300 import mlp
        newton = p

        def langevin(T):
            g.configure_step(newton, integrator=capi.INT_LANGEVIN, dt=0.001, target_temp=T, rotations=1)

        X, y = mlp.generate(g, newton, langevin, samples=200_000, every=10, equil=20)
        mlp.train(g, X, y, epochs=1, batch=65536, lr=2e-3, seed=1)
        g.build_nlist()
        pm = g.params(capi.ECPR, cutoff=3.0, solver=capi.SOLVER_MLP_NEWTON)
        for _ in range(1 + a.reps):
            g.zero_forces()
            g.pair_forces(pm)
    elif a.case in ("list", "gb_list"):
        for _ in range(1 + a.reps):
            g.build_nlist()
    elif a.case == "langevin":
        g.zero_forces()
        g.pair_forces(p)
        for k in range(1 + a.reps):
            g.lgv_initial(0.002, k + 1, damping=1.0, target_temp=1.0)
            g.lgv_final(0.002, damping=1.0)
    elif a.case == "nhc":
        g.zero_forces()
        g.pair_forces(p)
        for _ in range(1 + a.reps):
            g.nht_initial(0.001, 1.2, 0.0, mode=1, rot_chain=1)
            g.qq_initial(0.001)
            g.nht_final(0.001, 1.2, 0.0, mode=1, rot_chain=1)
            g.qq_final(0.001)
    elif a.case == "ecp_step":
        g.configure_step(p, integrator=capi.INT_NH, dt=0.001, target_temp=1.2, rotations=1, rot_chain=1,
                         flags=capi.STEP_FLAT)
        g.step(1 + a.reps)
    elif a.case == "mlp_train":
        from sucrose_gb300 import mlp

        def langevin(T):
            g.configure_step(p, integrator=capi.INT_LANGEVIN, dt=0.001, target_temp=T, rotations=1)

        X, y = mlp.generate(g, p, langevin, samples=65536, every=2, equil=2)
        mlp.train(g, X, y, epochs=1 + a.reps, batch=65536, lr=2e-3, seed=1)
    elif a.case == "replicas":
        e = configs.replica_ensemble(a.nrep, seed=1005)
        import bench  # the benchmark's replica set-up, reused
        sig, eps, inert, v0, l0 = bench.replica_arrays(e)
        g = GpuSystem.replicas(e["n"], e["box"], e["family"], e["temp"], e["key"])
        g.set_particles(mass=1.0, sig=sig, eps=eps, inertia=inert)
        g.upload(r=e["r"], q=e["q"], v=v0, l=l0)
        LJ, GB = configs.LJ_REPLICA, configs.GB_REPLICA
        g.init_rep_nlist([LJ["skin"], GB["skin"], 0.3], [LJ["list_cutoff"], GB["list_cutoff"], 3.0], trigger_mode=1)
        pairs = bench.replica_pair_params()
        g.configure_step_pairs(pairs, integrator=capi.INT_LANGEVIN, dt=bench.REPLICAS["dt"], damping=1.0, rotations=1,
                               flags=capi.STEP_FLAT)
        if a.equil:   # untimed steps first, until replicas start to rebuild their lists
            g.step(a.equil)
        g.step(1 + a.reps)
    g.synchronize()
    print("profile case", a.case, "done")


if __name__ == "__main__":
    main()
