"""Benchmark: ECP pair-evaluations per second and ns/day on one GB300.

Workload (default "ecp"): N = 65536 biaxial ellipsoids, semi-axes (1.5, 1, 0.5)
(full axes sig = (3, 2, 1)), packing fraction 0.35 (number density 0.1114),
repulsive ECP (ecpr) with the Newton contact solve from the support-function
start (the autotuner's launch: pairs beyond two upper bounds on the contact
distance skip the solve, forces unchanged), Nose-Hoover chains
of length 3 on translation and rotation, T* = 1.2, dt = 0.001, Verlet list
rc 3.0 + skin 0.3. Synthetic, seeded: uniform random orientations and
non-overlapping positions from the isotropic placement
(configs.isotropic_placement: growth from a fifth of full size with overlap
relaxation), thermal velocities and angular momenta; the reference publishes
no placement routine and no benchmark data set. Both arms start from the same
bits of that state.

A step is one full timestep (integrators, list check and rebuild when due,
forces) launched as one captured CUDA graph. value = listed pairs x
steps / device time of those steps; e2e repeats the measurement through the
C ABI with FP64 host arrays copied in and out every step. The default line
also carries the Gay-Berne fluid ("gb") and the 4096-replica ensemble
("replicas") as sub-objects, each with its own roofline and CPU baseline.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

TAU_PS = 2.156  # argon LJ time unit sigma*sqrt(m/eps) in ps (sigma 3.405 A, eps/kB 119.8 K, m 39.948 u)

WORKLOADS = {
    "ecp": dict(workload="ecp_biaxial_ecpr_nhc_N65536_phi0.35", n=65536, sig=(3.0, 2.0, 1.0),
                eps=(1.0, 1.0, 1.0), density=0.1114, kind="ECPR", cutoff=3.0, list_cutoff=3.0, skin=0.3,
                integrator="NH", T=1.2, dt=0.001, seed=1003),
    "gb": dict(workload="gay_berne_3_5_2_1_langevin_N32768_rho0.30", n=32768, sig=(1.0, 1.0, 3.0),
               eps=(1.0, 1.0, 0.2), density=0.30, kind="GB", cutoff=4.0, list_cutoff=6.0, skin=0.4,
               integrator="LANGEVIN", T=1.0, dt=0.002, mu=2, nu=1, seed=1002),
}

# one metric string per workload, printed identically by both arms
METRICS = {
    "ecp": "ECP pair-evals/s (ecpr, N=65536, phi=0.35)",
    "gb": "GB pair-evals/s (GB(3,5,2,1), N=32768, rho=0.30)",
    "replicas": "replica-ensemble pair-evals/s (4096 LJ + GB replicas)",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="ecp", choices=sorted(WORKLOADS) + ["replicas", "charged", "constrained", "polymer"])
    ap.add_argument("--nrep", type=int, default=4096, help="replicas (config replicas)")
    ap.add_argument("--rep-equil", type=int, default=300, help="untimed equilibration steps (config replicas)")
    ap.add_argument("--flat-graph", action="store_true",
                    help="replica contexts: list build as flag-gated kernels instead of a conditional graph node (for ncu launch lists)")
    ap.add_argument("--solver", default="support", choices=["support", "newton", "brent", "mlp"],
                    help="ECP contact solve: Newton from the support-function start (default), from 1/2, "
                         "the reference's Brent, or from the learned guess")
    ap.add_argument("--equil", type=int, default=1500, help="untimed Langevin equilibration steps")
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="bounded CPU-baseline sample")
    ap.add_argument("--no-extras", action="store_true", help="skip the secondary measurements")
    ap.add_argument("--no-mlp", action="store_true", help="skip the learned-guess leg")
    ap.add_argument("--no-sub", action="store_true", help="skip the gb and replicas sub-objects of the ecp line")
    ap.add_argument("--profile-case", default=None, help="run one small profiling case and exit (see PROFILE_CASES)")
    ap.add_argument("--reps", type=int, default=3, help="launches of the profiled kernels (--profile-case)")
    ap.add_argument("--ecp-path", default=None, choices=["split", "fused", "filtered"],
                    help="ECP profile cases: the split Newton path, the one-kernel path or the one kernel behind the support-function range test (default: untuned)")
    ap.add_argument("--launch", default=None,
                    help="block,filter of the headline pair kernel instead of autotuning (e.g. 128,2)")
    ap.add_argument("--state-equil", type=int, default=0,
                    help="untimed Langevin steps from the placed state before timing (ecp, gb)")
    ap.add_argument("--mlp-samples", type=int, default=10_000_000)
    ap.add_argument("--mlp-epochs", type=int, default=3)
    return ap.parse_args()


# ------------------------------------------------------------------ clocks ---
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for name, val in zip(names, p[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- workload ---
def initial_state(w, seed=None):
    """The workload's seeded initial state, the same bits in both arms:
    isotropic non-overlapping placement (uniform orientations), velocities by
    the reference's set_velocity_to_temperature convention, thermal
    body-frame angular momenta. Returns r, q, box, v, l, placement report."""
    from sucrose_gb300 import configs
    seed = w["seed"] if seed is None else seed
    r, q, box, rep = configs.isotropic_placement(w["n"], w["sig"], w["density"], seed=seed)
    n = len(r)
    v = configs.velocities_to_temperature(n, w["T"], seed)
    l = configs.angular_momenta(q, configs.default_inertia(w["sig"]), w["T"], seed)
    return r, q, box, v, l, rep


def long_axis(w):
    return int(np.argmax(w["sig"]))


def make_system(w, seed=None):
    from sucrose_gb300 import GpuSystem
    t0 = time.perf_counter()
    r, q, box, v, l, rep = initial_state(w, seed)
    t_place = time.perf_counter() - t0
    g = GpuSystem(len(r), box)
    g.set_particles(sig=w["sig"], eps=w["eps"])
    g.upload(r=r, q=q, v=v, l=l)
    g.init_nlist(w["skin"], w["list_cutoff"], trigger_mode=1)
    info = {"placement_s": t_place, "placement_sweeps": int(rep.sweeps),
            "placement_min_contact_ratio": float(rep.min_contact_ratio)}
    return g, box, info


def pair_params(g, w, solver):
    from sucrose_gb300 import capi
    kind = getattr(capi, w["kind"])
    s = {"newton": capi.SOLVER_NEWTON, "support": capi.SOLVER_NEWTON_SUPPORT, "brent": capi.SOLVER_BRENT_COMPAT,
         "mlp": capi.SOLVER_MLP_NEWTON}[solver]
    return g.params(kind, cutoff=w["cutoff"], mu=w.get("mu", 0), nu=w.get("nu", 0), solver=s)


FLAGS = 0   # step-graph flags (capi.STEP_FLAT under --flat-graph)

# DRAM bytes (read + write) of one launch of the dominant kernel, from the
# committed ncu captures of these workloads (traffic is not measurable from
# inside a timed run)
NCU_TRAFFIC = {
    "EC": {"bytes": 12.60e6, "pairs": 0.46e6,
           "source": "profiles/k_pair_ecp_newton_N65536.md: ncu, 0.46 M listed pairs"},
    "GB": {"bytes": 45.26e6, "pairs": 5.32e6,
           "source": "profiles/k_pair_gb_filtered_N32768.md: ncu, 5.32 M listed pairs"},
    "COULOMB": {"bytes": 65.06e6, "pairs": 7.57e6,
                "source": "profiles/k_pair_coulomb_charged_N131072.md: ncu, 7.57 M listed pairs"},
}


def configure(g, w, pp, langevin=False, first_step=1):
    from sucrose_gb300 import capi
    if langevin or w["integrator"] == "LANGEVIN":
        g.configure_step(pp, integrator=capi.INT_LANGEVIN, dt=w["dt"], target_temp=w["T"], damping=1.0,
                         rotations=1, first_step=first_step, flags=FLAGS)
    else:
        g.configure_step(pp, integrator=capi.INT_NH, dt=w["dt"], target_temp=w["T"], rotations=1, rot_chain=1,
                         flags=FLAGS)


def pair_flops(kind, listed, in_range, mean_evals=0.0, support=False, solved=None):
    """Algorithmic FP32 flops of one pair-force launch, counted from the kernel
    sources (FMA = 2 flops, sqrt / rsqrt / division = 1). Every listed pair
    pays the distance and, for Gay-Berne, the orientation terms up to the range
    test; pairs in range pay the force and torque terms. ECP: `solved` pairs
    (all listed ones unless the support-filtered launch turned some away) pay
    the contact solve and the force terms, mean_evals Newton evaluations each;
    with the filter every listed pair pays its test (70: the distance, two
    quadratic forms, two square roots)."""
    if kind.startswith("ECP"):
        if solved is None or solved >= listed:
            return ecp_flops_per_pair(mean_evals, support) * listed
        return 70.0 * listed + ecp_flops_per_pair(mean_evals, support) * solved
    if kind.startswith("GB"):
        return 80.0 * listed + 240.0 * in_range
    return 20.0 * listed + 20.0 * in_range


def ecp_flops_per_pair(mean_evals, support=False):
    """Algorithmic FP32 flops of one ECP pair (Newton), counted from the kernel
    source: setup 60, per Newton evaluation 110, final factorisation 30, force
    and torque terms 420 (FMA = 2 flops, rsqrt/div = 1); the support-function
    start adds 44 (two quadratic forms, two square roots, one division)."""
    return 60.0 + (44.0 if support else 0.0) + 110.0 * mean_evals + 30.0 + 420.0


def timed_steps(g, torch, stream, steps, flush):
    import ctypes
    start = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    end = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for k in range(steps):
            start[k].record(stream)
            g.step(1)
            end[k].record(stream)
            flush.add_(1.0)   # write 256 MB (> L2) between timed steps
    torch.cuda.synchronize()
    return sum(s.elapsed_time(e) for s, e in zip(start, end)) / 1e3


def timed_forces(g, torch, stream, pp, reps, flush):
    """Device time of one force call (prep and pair kernels), L2 flushed before
    each: the flush is enqueued first, so that the host has enqueued the
    call's launches while the device still runs it and the interval between
    the events holds the call's kernels back to back (an idle device between
    the events would time the host's launch rate instead)."""
    start = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    end = [torch.cuda.Event(enable_timing=True) for _ in range(reps)]
    with torch.cuda.stream(stream):
        for k in range(reps):
            flush.add_(1.0)
            g.zero_forces()
            start[k].record(stream)
            g.pair_forces_async(pp)
            end[k].record(stream)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) / 1e3 for s, e in zip(start, end)]


def cpu_baseline(g, w, seconds, nthreads=1):
    """The oracle's faithful restatement of the reference pair routine (the
    reference's Brent, per-pair setup, FP64) over a bounded sample of the
    device's current pair list, on host cores."""
    import oracle as O
    r, q, v, l = g.download()
    pi, pj = g.pairs()
    s = O.System(g.n, g.box, fast=True)
    s.set_defaults(sig=w["sig"], eps=w["eps"])
    s.rx[:], s.ry[:], s.rz[:] = r.T
    s.qw[:], s.qx[:], s.qy[:], s.qz[:] = q.T
    kind = getattr(O, w["kind"])
    pp = O.pair_params(kind, cutoff=w["cutoff"], solver=O.SOLVER_BRENT, mu=w.get("mu"), nu=w.get("nu"))
    # calibrate on a small slice, then run a sample of about `seconds`
    m0 = min(len(pi), 4000 * nthreads)
    t = time.perf_counter()
    s.pair_batch(pp, pi[:m0], pj[:m0], nthreads)
    per = (time.perf_counter() - t) / max(m0, 1)
    m = int(min(len(pi), max(m0, seconds / max(per, 1e-9))))
    t = time.perf_counter()
    s.pair_batch(pp, pi[:m], pj[:m], nthreads)
    dt = time.perf_counter() - t
    return m / dt, m


def force_error_vs_fp64(g, w, pp, nthreads=None):
    """Norm-wise relative error of the device forces and torques against the
    oracle's FP64 evaluation with the tightly converged contact parameter, on
    the same FP32 state and list."""
    import oracle as O
    r, q, v, l = g.download()
    pi, pj = g.pairs()
    g.zero_forces()
    pe, _ = g.pair_forces(pp)
    F, T = g.forces()
    s = O.System(g.n, g.box, fast=True)
    s.set_defaults(sig=w["sig"], eps=w["eps"])
    s.rx[:], s.ry[:], s.rz[:] = r.T
    s.qw[:], s.qx[:], s.qy[:], s.qz[:] = q.T
    kind = getattr(O, w["kind"])
    out = s.pair_batch(O.pair_params(kind, cutoff=w["cutoff"], solver=O.SOLVER_TIGHT, mu=w.get("mu"), nu=w.get("nu")),
                       pi, pj, nthreads or os.cpu_count() or 1)
    Fo = np.zeros((g.n, 3))
    To = np.zeros((g.n, 3))
    np.add.at(Fo, pi, out[:, 1:4])
    np.add.at(Fo, pj, -out[:, 1:4])
    np.add.at(To, pi, out[:, 4:7])
    np.add.at(To, pj, out[:, 7:10])
    peo = out[:, 0].sum()
    nf = lambda a, b: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    return {"force": nf(F, Fo), "torque": nf(T, To), "pot_eng": abs(pe - peo) / max(abs(peo), 1e-300)}


def mlp_leg(a, g, w, torch, stream, flush, npairs, tune):
    """Train the learned guess on plain-Newton samples at T* 0.8, 1.2, 1.6 and
    time the MLP-guess path against the plain path on the same state, both
    with the one-kernel launch that solves every pair (the samples need every
    pair's lambda); the tuned launch is restored at the end."""
    import ctypes
    from sucrose_gb300 import capi, mlp
    r, q, v, l = g.download()          # restore the timed state afterwards
    newton = pair_params(g, w, "newton")
    g.set_launch(newton.kind, 256, 0)

    def langevin(T):
        g.configure_step(newton, integrator=capi.INT_LANGEVIN, dt=w["dt"], target_temp=T, damping=1.0, rotations=1)

    t0 = time.perf_counter()
    X, y = mlp.generate(g, newton, langevin, samples=a.mlp_samples, every=25, equil=200)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    hist = mlp.train(g, X, y, epochs=a.mlp_epochs, batch=65536, lr=2e-3, seed=1)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del X, y
    g.upload(r=r, q=q, v=v, l=l)
    g.build_nlist()
    pm = pair_params(g, w, "mlp")
    _, _, sm = g.pair_forces(pm, want_stats=True)
    _, _, sp = g.pair_forces(newton, want_stats=True)
    tm = statistics.median(timed_forces(g, torch, stream, pm, 10, flush))
    tp = statistics.median(timed_forces(g, torch, stream, newton, 10, flush))
    # the tensor-core guess pass alone (part of tm)
    guess_buf = torch.empty(max(npairs_int := g.npairs(), 1), dtype=torch.float32, device="cuda")
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tg = []
    with torch.cuda.stream(stream):
        for _ in range(10):
            ev0.record(stream)
            capi.check(g.ctx, g.L.sg_mlp_guess_tc(g.ctx, ctypes.c_void_p(guess_buf.data_ptr()), guess_buf.numel()))
            ev1.record(stream)
            torch.cuda.synchronize()
            tg.append(ev0.elapsed_time(ev1) / 1e3)
    t_guess = statistics.median(tg)
    # the same network in the ECP kernel itself (warp mma.sync, one kernel)
    capi.check(g.ctx, g.L.sg_mlp_set_inline(g.ctx, 1))
    ti = statistics.median(timed_forces(g, torch, stream, pm, 10, flush))
    capi.check(g.ctx, g.L.sg_mlp_set_inline(g.ctx, 0))
    configure(g, w, pm)
    g.step(5)
    g.step_check()
    t_step = timed_steps(g, torch, stream, 50, flush)
    g.set_launch(newton.kind, tune.block, tune.filter)
    return {"samples": a.mlp_samples, "epochs": a.mlp_epochs, "train_mse": hist, "gen_s": t_gen, "train_s": t_train,
            "force_kernel_ms": 1e3 * tm, "pair_evals_per_s_force_kernel": npairs / tm,
            "guess_pass_ms_tcgen05": 1e3 * t_guess,
            "guess_tensor_tflops": 18560.0 * npairs_int / t_guess / 1e12,
            "inline_mma_sync_force_kernel_ms": 1e3 * ti,
            "plain_force_kernel_ms_same_state": 1e3 * tp, "speedup_vs_plain_force_kernel": tp / tm,
            "full_step_pair_evals_per_s": npairs * 50 / t_step,
            "mean_evals_per_pair": sm.solver_evals / max(sm.pairs, 1),
            "plain_mean_evals_per_pair": sp.solver_evals / max(sp.pairs, 1),
            "fallback_rate": sm.fallbacks / max(sm.pairs, 1), "nonconverged": int(sm.nonconverged),
            "iter_hist": [int(x) for x in sm.iter_hist], "force_error_vs_fp64": force_error_vs_fp64(g, w, pm)}


# -------------------------------------------------------------------- ours ---
def ellipsoid_line(a, name, rank=0, world=1, local=0, dist=None, steps=None, extras_on=True):
    """One ellipsoid workload (ecp or gb) from the shared seeded state: the
    captured step timed on the device, the force kernel alone, e2e through
    the C ABI with host arrays, the CPU baseline. Returns the JSON line."""
    import torch
    from sucrose_gb300 import capi, configs, ranks
    w = WORKLOADS[name]
    steps = steps or a.steps
    # replicas only: every rank runs its own independent system
    g, box, info = make_system(w, seed=ranks.replica_seed(w["seed"], rank))
    p2_initial = configs.nematic_order(g.download()[1], long_axis(w))
    stream = torch.cuda.ExternalStream(g.stream_ptr())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    solver = a.solver if name == "ecp" else "newton"
    pp = pair_params(g, w, solver)
    if a.state_equil:
        # optional untimed Langevin steps from the placed state
        configure(g, w, pair_params(g, w, "newton"), langevin=True, first_step=1)
        g.step(a.state_equil)
        g.step_check()
    if a.launch:
        # a fixed launch shape instead of the autotuner's pick (profiling
        # under ncu, whose per-kernel overhead would skew the tuner's timings)
        from sucrose_gb300 import capi as _c
        tune = _c.TuneResult()
        tune.block, tune.filter = [int(x) for x in a.launch.split(",")]
        g.set_launch(pp.kind, tune.block, tune.filter)
    else:
        tune = g.autotune(pp, reps=5)      # launch shape of the pair kernel on the live list
    configure(g, w, pp, first_step=a.state_equil + 1)
    g.step(max(a.warmup, 3))
    g.step_check()
    kernels_per_step = g.step_kernel_count()
    p_before = g.npairs()
    builds0 = g.nlist_builds()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_dev = timed_steps(g, torch, stream, steps, flush)
    g.step_check()
    p_after = g.npairs()
    builds = g.nlist_builds() - builds0
    npairs = 0.5 * (p_before + p_after)
    if dist is not None:
        t_dev = ranks.max_over_ranks(t_dev, device="cuda")
    ms_per_step = 1e3 * t_dev / steps
    value = npairs * steps * world / t_dev
    steps_per_s = steps / t_dev
    ns_day = steps_per_s * w["dt"] * TAU_PS * 1e-3 * 86400.0
    p2_timed = configs.nematic_order(g.download()[1], long_axis(w))

    # dominant kernel: the pair-force kernel timed alone (same stream, L2 flushed)
    _, _, st = g.pair_forces(pp, want_stats=True)
    # ECP: pairs solved (iteration bin 0 holds the pairs the support-filtered
    # launch turned away) and Newton evaluations per solved pair
    solved = st.pairs - int(st.iter_hist[0]) if w["kind"].startswith("ECP") else st.pairs
    mean_evals = st.solver_evals / max(solved, 1)
    tf = timed_forces(g, torch, stream, pp, 20, flush)
    t_force = statistics.median(tf)
    peak32 = g.peak_fma(False)
    flops = pair_flops(w["kind"], st.pairs, st.solver_evals, mean_evals, support=solver == "support",
                       solved=solved)
    achieved = flops / t_force / 1e12

    # e2e: FP64 host arrays in and out through the C ABI every step
    n = g.n
    pin = lambda: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    host = [pin() for _ in range(13)]
    r, q, v, l = g.download()
    for k in range(3):
        host[k][:] = r[:, k]
        host[7 + k][:] = v[:, k]
        host[10 + k][:] = l[:, k]
    for k in range(4):
        host[3 + k][:] = q[:, k]
    import ctypes as C
    D = C.POINTER(C.c_double)
    ptrs = [h.ctypes.data_as(D) for h in host]
    L = g.L
    energies = np.zeros(4)
    e_steps = max(10, steps // 4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e_steps):
        capi.check(g.ctx, L.sg_upload_state(g.ctx, *ptrs))
        g.step(1)
        capi.check(g.ctx, L.sg_download_state(g.ctx, *ptrs))
        capi.check(g.ctx, L.sg_read_energies(g.ctx, energies.ctypes.data_as(D)))
    t_e2e = time.perf_counter() - t0
    e2e_value = npairs * e_steps / t_e2e
    h2d = 13 * 8 * n
    d2h = 13 * 8 * n + 32

    extras = {}
    if extras_on and rank == 0:
        extras["force_kernel_pair_evals_per_s"] = npairs / t_force
        extras["force_kernel_ms"] = 1e3 * t_force
        if w["kind"].startswith("ECP"):
            extras["newton_mean_evals_per_solved_pair"] = mean_evals
            extras["pairs_solved_frac"] = solved / max(st.pairs, 1)
            extras["newton_iter_hist"] = [int(x) for x in st.iter_hist]
            extras["newton_fp64_refined_frac"] = st.fp64_refined / max(st.pairs, 1)
            extras["nonconverged"] = int(st.nonconverged)
        else:
            extras["pairs_in_range_frac"] = st.solver_evals / max(st.pairs, 1)
            extras["pairs_near_contact_frac"] = st.fallbacks / max(st.pairs, 1)
        extras["fp64_peak_tflops_measured"] = g.peak_fma(True)
        extras["list_rebuilds_in_timed_region"] = int(builds)
        extras["stage_ms_in_graph"] = g.step_stage_times(20)
        ecp = w["kind"].startswith("ECP")
        pick = {"block": tune.block, "filter": tune.filter}
        if ecp:
            pick["path"] = {0: "fused", 1: "split", 2: "support_filtered"}[tune.filter]
        extras["autotune"] = {"pick": pick, "variant_ms": tune_variants(tune, ecp)}
        extras["force_error_vs_fp64"] = force_error_vs_fp64(g, w, pp)
        if name == "ecp" and a.solver in ("newton", "support"):
            # Newton from lambda = 1/2 on the same list (the support start is the headline)
            if a.solver == "support":
                ph = pair_params(g, w, "newton")
                _, _, sth = g.pair_forces(ph, want_stats=True)
                th = statistics.median(timed_forces(g, torch, stream, ph, 10, flush))
                extras["newton_half_start"] = {
                    "force_kernel_ms": 1e3 * th, "pair_evals_per_s": npairs / th,
                    "mean_evals_per_solved_pair": sth.solver_evals / max(sth.pairs - int(sth.iter_hist[0]), 1),
                    "iter_hist": [int(x) for x in sth.iter_hist]}
            # residual check variants of the same kernel
            for mode, mname in ((2, "double_float"), (0, "none")):
                pv = pair_params(g, w, a.solver)
                pv.fp64_check = mode
                tv = statistics.median(timed_forces(g, torch, stream, pv, 10, flush))
                extras[f"newton_check_{mname}_force_kernel_ms"] = 1e3 * tv
                extras[f"newton_check_{mname}_pair_evals_per_s"] = npairs / tv
            pb = pair_params(g, w, "brent")
            _, _, stb = g.pair_forces(pb, want_stats=True)
            tb = statistics.median(timed_forces(g, torch, stream, pb, 5, flush))
            extras["brent_compat_force_kernel_ms"] = 1e3 * tb
            extras["brent_compat_pair_evals_per_s"] = npairs / tb
            extras["brent_mean_evals_per_pair"] = stb.solver_evals / max(stb.pairs, 1)
            extras["nh_modes"] = nh_modes(g, w, pp, torch, stream, flush)
            if not a.no_mlp:
                extras["mlp"] = mlp_leg(a, g, w, torch, stream, flush, npairs, tune)

    cpu = None
    if rank == 0:
        cpu_rate, m = cpu_baseline(g, w, a.cpu_seconds, nthreads=1)
        routine = ("the reference's ecpr_ with its Brent solve and per-pair setup" if w["kind"].startswith("ECP")
                   else "the reference's gb_ (mu 2, nu 1)")
        cpu = {"value": cpu_rate, "unit": "pair-evals/s", "cores": 1, "kind": "port",
               "sample": f"{m} listed pairs of this workload's list, {routine}, FP64, "
                         f"oracle restatement built -O3 -ffast-math, 1 thread"}
    g.close()
    kname = "k_pair<PotECP>" if w["kind"].startswith("ECP") else "k_pair<PotGB>"
    line = {
        "metric": METRICS[name],
        "value": value, "unit": "pair-evals/s", "n_gpus": world, "steps": steps, "warmup": a.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 (fp64 totals and residual check)",
        "data": "synthetic (seeded isotropic placement, the same state as the reference arm)",
        "config": {"workload": w["workload"], "n": n, "listed_pairs": npairs, "solver": solver,
                   "dt": w["dt"], "T": w["T"], "seed": w["seed"],
                   "integrator": "Nose-Hoover chains (3) on translation and rotation" if w["integrator"] == "NH"
                   else "Langevin on translation and rotation",
                   "timed": "the full MD step (integrators, list check and rebuild when due, forces), "
                            "one captured CUDA graph per step",
                   "pair_launch": {"block": int(tune.block), "filter": int(tune.filter)},
                   "nematic_P2_initial": p2_initial, "nematic_P2_timed_state": p2_timed, **info,
                   "untimed_equilibration_steps": a.state_equil,
                   "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": "replicas only" if world > 1 else "single GPU"},
        "ns_per_day": ns_day, "tau_per_day": steps_per_s * w["dt"] * 86400.0,
        "e2e": {"value": e2e_value, "unit": "pair-evals/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(kernels_per_step * steps),
        "roofline": {"bound": "fp32", "kernel": kname, "achieved": achieved, "peak": peak32,
                     "unit": "TFLOP/s", "frac": achieved / peak32,
                     "peak_source": "measured FMA throughput (sg_peak_fma) on this GPU",
                     "traffic": NCU_TRAFFIC[w["kind"][:2]]["bytes"] * st.pairs / NCU_TRAFFIC[w["kind"][:2]]["pairs"],
                     "traffic_source": NCU_TRAFFIC[w["kind"][:2]]["source"]
                     + " (scaled to this launch's listed pairs)"},
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
    }
    line.update(extras)
    return line


def tune_variants(tune, ecp=False):
    """The autotuner's timed launch variants, by block size and range filter
    (ECP: the one-kernel path, the split Newton path, or the one kernel behind
    the support-function range test)."""
    shapes = ((256, 0), (128, 0), (256, 1), (128, 1), (64, 0), (64, 1))
    if tune.candidates == 3:
        shapes = ((256, 0), (128, 0), (64, 0))
    if tune.candidates == 8:
        shapes = ((256, 2), (128, 2), (256, 0), (128, 0), (256, 1), (128, 1), (64, 2), (64, 0))
    names = {0: "fused", 1: "split", 2: "support_filtered"}
    tag = (lambda f: names[f]) if ecp else (lambda f: f"f{f}")
    return {f"b{b}_{tag(f)}": float(tune.ms[k]) for k, (b, f) in enumerate(shapes[:tune.candidates])}


def nh_modes(g, w, pp, torch, stream, flush, steps=20):
    """The Nose-Hoover step in both modes on the same state: the reference's
    per-particle chain recurrence (mode 0) and the standard chain (mode 1)."""
    from sucrose_gb300 import capi
    r, q, v, l = g.download()
    out = {}
    for mode, label in ((capi.INT_NH_REF, "reference_per_particle_chain"), (capi.INT_NH, "standard_chain")):
        g.upload(r=r, q=q, v=v, l=l)
        g.build_nlist()
        g.configure_step(pp, integrator=mode, dt=w["dt"], target_temp=w["T"], rotations=1,
                         rot_chain=0 if mode == capi.INT_NH_REF else 1, flags=FLAGS)
        g.step(3)
        g.step_check()
        t = timed_steps(g, torch, stream, steps, flush)
        g.step_check()
        out[label] = {"ms_per_step": 1e3 * t / steps}
    g.upload(r=r, q=q, v=v, l=l)
    g.build_nlist()
    configure(g, w, pp)
    return out


def run_ours(a):
    import torch
    import __graft_entry__
    __graft_entry__.build_library()
    from sucrose_gb300 import ranks
    rank, world, local = ranks.rank_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist.barrier()
    line = ellipsoid_line(a, a.config, rank, world, local, dist, extras_on=not a.no_extras)
    if a.config == "ecp" and not a.no_extras and not a.no_sub:
        # the other two headline workloads, each timed over fewer steps
        sub = min(a.steps, 50)
        line["gb"] = ellipsoid_line(a, "gb", rank, world, local, dist, steps=sub, extras_on=rank == 0)
        line["replicas"] = replicas_line(a, rank, world, local, dist, steps=min(a.steps, 20))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ----------------------------------------------------------------- charged ---
CHARGED = dict(workload="charged_wca_coulomb_langevin_N131072_rho0.5", cells=32, density=0.5, cutoff=3.5, skin=0.3,
               dielectric=1.0, T=1.0, dt=0.002, damping=1.0, seed=1007)

# FP32 flops per pair, counted from pair_elec.cu (FMA = 2, sqrt / div / exp = 1):
# every listed pair pays the minimum image and the range test; pairs in range
# pay the potential's terms
ELEC_FLOPS = {"COULOMB": (20.0, 40.0), "DH": (20.0, 45.0), "MORSE": (20.0, 45.0), "DIPOLE": (20.0, 130.0)}


def charged_state(seed):
    from sucrose_gb300 import configs
    w = CHARGED
    r, q, box = configs.fcc_lattice(w["cells"], w["density"])
    n = len(r)
    rng = np.random.default_rng(seed)
    charge = rng.permutation(np.repeat([1.0, -1.0], n // 2))
    v = configs.velocities_to_temperature(n, w["T"], seed)
    return r, q, box, v, charge


def charged_params(g):
    from sucrose_gb300 import capi
    w = CHARGED
    return [g.params(capi.WCA, sigma=1.0), g.params(capi.COULOMB, cutoff=w["cutoff"], dielectric=w["dielectric"])]


def run_charged(a):
    """Charged spheres: WCA plus the switched Coulomb of coulombic_ summed in
    one captured Langevin step; the other charge and Morse kinds timed alone
    on the same list."""
    import ctypes as C
    import torch
    import __graft_entry__
    __graft_entry__.build_library()
    from sucrose_gb300 import GpuSystem, capi, ranks
    rank, world, local = ranks.rank_info()
    torch.cuda.set_device(local)
    w = CHARGED
    r, q, box, v, charge = charged_state(ranks.replica_seed(w["seed"], rank))
    n = len(r)
    g = GpuSystem(n, box)
    g.upload(r=r, q=q, v=v)
    g.set_charges(charge)
    g.init_nlist(w["skin"], w["cutoff"], trigger_mode=1)
    stream = torch.cuda.ExternalStream(g.stream_ptr())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    sets = charged_params(g)
    g.configure_step_pairs(sets, integrator=capi.INT_LANGEVIN, dt=w["dt"], target_temp=w["T"],
                           damping=w["damping"], rotations=0, flags=FLAGS)
    g.step(a.equil)
    g.step_check()
    tunes = [g.autotune(p, reps=5) for p in sets]
    g.configure_step_pairs(sets, integrator=capi.INT_LANGEVIN, dt=w["dt"], target_temp=w["T"],
                           damping=w["damping"], rotations=0, first_step=a.equil + 1, flags=FLAGS)
    g.step(max(a.warmup, 3))
    g.step_check()
    kernels_per_step = g.step_kernel_count()
    p_before = g.npairs()
    builds0 = g.nlist_builds()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_dev = timed_steps(g, torch, stream, a.steps, flush)
    g.step_check()
    builds = g.nlist_builds() - builds0
    npairs = 0.5 * (p_before + g.npairs())
    if dist is not None:
        t_dev = ranks.max_over_ranks(t_dev, device="cuda")
    # pair-evals of one step: each listed pair is evaluated by both sets
    evals_per_step = 2.0 * npairs
    value = evals_per_step * a.steps * world / t_dev
    steps_per_s = a.steps / t_dev

    # the Coulomb kernel alone (dominant), then the other kinds on the same list
    peak32 = g.peak_fma(False)
    hbm = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs") \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    kinds = {}
    extra_params = {
        "COULOMB": sets[1],
        "DH": g.params(capi.DH, cutoff=w["cutoff"], db_len=1.0, dielectric=w["dielectric"]),
        "MORSE": g.params(capi.MORSE, cutoff=w["cutoff"], dissoc=1.0, width=2.0, rmin=1.1),
        "DIPOLE": g.params(capi.DIPOLE, cutoff=w["cutoff"], dielectric=4.0),
    }
    g.reaction_field_init()
    for name, p in extra_params.items():
        if name != "COULOMB":
            g.autotune(p, reps=3)
        _, _, st = g.pair_forces(p, want_stats=True)
        t = statistics.median(timed_forces(g, torch, stream, p, 20, flush))
        fl = ELEC_FLOPS[name][0] * st.pairs + ELEC_FLOPS[name][1] * st.solver_evals
        # minimum DRAM bytes of one launch: the list (i, j int32 per pair), the
        # positions read once and the forces read and written once
        by = 8.0 * st.pairs + 48.0 * n + (48.0 * n if name == "DIPOLE" else 0.0)
        kinds[name] = {"kernel_ms": 1e3 * t, "pair_evals_per_s": st.pairs / t,
                       "in_range_frac": st.solver_evals / max(st.pairs, 1),
                       "fp32_tflops": fl / t / 1e12, "fp32_frac": fl / t / 1e12 / peak32,
                       "min_dram_gbs": by / t / 1e9, "min_dram_frac": (by / t / 1e9 / hbm) if hbm else None}
    c = kinds["COULOMB"]

    # Monte Carlo barostat (mc_barostat) with the step's two pair sets: one
    # trial move = two energy evaluations + scaling + restore, host-driven
    accepted = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nb = 10
    for k in range(nb):
        acc_k, _ = g.mc_barostat(sets, target_pressure=0.5, temperature=w["T"], max_dv=0.002, counter=k)
        accepted += acc_k == 1
    baro_ms = 1e3 * (time.perf_counter() - t0) / nb

    # asynchronous trajectory reporter: wall time of 100 steps writing a
    # LAMMPS-style frame every 10 steps, against the same steps without
    import tempfile
    def run_steps(rep):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for k in range(10):
            g.step(10)
            if rep is not None:
                rep.write(k)
        torch.cuda.synchronize()
        if rep is not None:
            t_issue = time.perf_counter() - t
            rep.flush()
            return t_issue, time.perf_counter() - t
        return time.perf_counter() - t
    t_plain = run_steps(None)
    with tempfile.TemporaryDirectory() as td:
        with g.reporter(capi.REPORT_TRAJECTORY, os.path.join(td, "traj.lammpstrj")) as rep:
            t_rep_steps, t_rep_all = run_steps(rep)
        traj_bytes = os.path.getsize(os.path.join(td, "traj.lammpstrj"))

    e2e_value, h2d, d2h = e2e_rate(g, torch, max(10, a.steps // 4), evals_per_step)

    cpu = None
    if rank == 0:
        rate, m = charged_cpu_sample(g, charge, a.cpu_seconds, 1)
        cpu = {"value": rate, "unit": "pair-evals/s", "cores": 1, "kind": "port",
               "sample": f"{m} listed pairs of this workload's list through the reference's coulombic_ "
                         "(FP64, oracle restatement built -O3 -ffast-math), 1 thread"}
        line = {
            "metric": "charged pair-evals/s (WCA + switched Coulomb, full MD step)",
            "value": value, "unit": "pair-evals/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * t_dev / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 (fp64 totals)", "data": "synthetic (seeded FCC lattice, +-1 charges, device-equilibrated)",
            "config": {"workload": w["workload"], "n": n, "listed_pairs": npairs, "pair_sets": ["WCA", "COULOMB"],
                       "dt": w["dt"], "T": w["T"], "cutoff": w["cutoff"], "skin": w["skin"],
                       "l2": "flushed between timed steps (256 MB write)",
                       "parallelism": "replicas only" if world > 1 else "single GPU"},
            "ns_per_day": steps_per_s * w["dt"] * TAU_PS * 1e-3 * 86400.0,
            "tau_per_day": steps_per_s * w["dt"] * 86400.0,
            "e2e": {"value": e2e_value, "unit": "pair-evals/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": int(kernels_per_step * a.steps),
            "roofline": {"bound": "hbm", "kernel": "k_pair<PotElec> (COULOMB)", "achieved": c["min_dram_gbs"],
                         "peak": hbm, "unit": "GB/s", "frac": c["min_dram_frac"],
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)",
                         "bytes_per_launch": "8 per listed pair + 48 per particle",
                         "traffic": NCU_TRAFFIC["COULOMB"]["bytes"], "traffic_source": NCU_TRAFFIC["COULOMB"]["source"],
                         "fp32_tflops": c["fp32_tflops"], "fp32_frac_of_measured": c["fp32_frac"]},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "kinds_alone": kinds,
            "mc_barostat": {"ms_per_trial_move": baro_ms, "accepted": int(accepted), "moves": nb,
                            "note": "host wall time per call: two energy passes over both pair sets"},
            "trajectory_reporter": {"steps_ms_without": 1e3 * t_plain, "steps_ms_with_10_frames": 1e3 * t_rep_steps,
                                    "ms_until_written": 1e3 * t_rep_all, "bytes": traj_bytes,
                                    "note": "100 steps, a frame every 10; frames formatted on a host thread"},
            "list_rebuilds_in_timed_region": int(builds),
            "autotune": [{"block": t.block, "filter": t.filter} for t in tunes],
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ------------------------------------------------------------- constrained ---
MOLECULAR = {
    # rigid dimers: RATTLE bonds and WCA between all atoms
    "constrained": dict(workload="constrained_dimers_wca_langevin_N128000", cells=40, spacing=1.6, sigma=0.9,
                        bond=1.0, skin=0.3, T=1.0, dt=0.002, damping=1.0, seed=1009,
                        metric="constraint-solves/s (rigid WCA dimers, RATTLE a + b, full MD step)"),
    # bead chains of 10: RATTLE bonds, harmonic bends (angle_bend_, 4, 120 deg), dihedrals (dih_, 0.5), WCA
    "polymer": dict(workload="polymer_chains10_wca_bend_dih_rattle_langevin_N96000", counts=(6, 40, 40), length=10,
                    sigma=0.9, bond=1.0, skin=0.3, T=1.0, dt=0.002, damping=1.0, seed=1011,
                    metric="constraint-solves/s (WCA bead chains, bends, dihedrals, RATTLE, full MD step)"),
}
CONSTRAINED = MOLECULAR["constrained"]


def molecular_state(name, seed):
    """Positions, box, bond constraints (bbi, bbj, length) and the bonded
    term lists [(kind, atoms, coeff, angle)] of a molecular workload."""
    from sucrose_gb300 import capi
    from sucrose_gb300.molecules import molecular_mix, polymer_chains
    w = MOLECULAR[name]
    if name == "constrained":
        r, box, bbi, bbj, ln, mol = molecular_mix(w["cells"], w["spacing"], seed, bond=w["bond"], kinds=("dimer",))
        return r, box, bbi, bbj, ln, []
    r, box, bonds, bends, dihs = polymer_chains(w["counts"], w["length"], seed, bond=w["bond"])
    terms = [(capi.ANGLE_BEND, bends, 4.0, 120.0), (capi.DIH, dihs, 0.5, None)]
    return r, box, bonds[:, 0].copy(), bonds[:, 1].copy(), np.full(len(bonds), w["bond"]), terms


def run_constrained(a):
    """Molecular workloads (config constrained: rigid dimers; polymer: bead
    chains with bonded terms) with RATTLE bonds and WCA between all atoms:
    one captured Langevin step with the constraint (and bonded) stages."""
    import torch
    import __graft_entry__
    __graft_entry__.build_library()
    from sucrose_gb300 import GpuSystem, capi, configs, ranks
    rank, world, local = ranks.rank_info()
    torch.cuda.set_device(local)
    w = MOLECULAR[a.config]
    seed = ranks.replica_seed(w["seed"], rank)
    r, box, bbi, bbj, ln, terms = molecular_state(a.config, seed)
    n = len(r)
    v = configs.velocities_to_temperature(n, w["T"], seed)
    g = GpuSystem(n, box)
    g.upload(r=r, v=v)
    g.set_constraints(bbi, bbj, ln)
    for kind, atoms, coeff, angle in terms:
        g.bonded_set(kind, atoms, coeff, angle)
    g.init_nlist(w["skin"], w["sigma"], trigger_mode=1)
    stream = torch.cuda.ExternalStream(g.stream_ptr())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    pp = g.params(capi.WCA, sigma=w["sigma"], cutoff=w["sigma"])
    cfg = dict(integrator=capi.INT_LANGEVIN, dt=w["dt"], target_temp=w["T"], damping=w["damping"], rotations=0,
               flags=FLAGS | capi.STEP_CONSTRAINTS | (capi.STEP_BONDED if terms else 0))
    g.configure_step(pp, first_step=1, **cfg)
    g.step(a.equil)
    g.step_check()
    tune = g.autotune(pp, reps=5)
    g.configure_step(pp, first_step=a.equil + 1, **cfg)
    g.step(max(a.warmup, 3))
    g.step_check()
    kernels_per_step = g.step_kernel_count()
    p_before = g.npairs()
    builds0 = g.nlist_builds()
    g.constraint_stats(reset=True)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_dev = timed_steps(g, torch, stream, a.steps, flush)
    g.step_check()
    cst = g.constraint_stats(reset=True)
    builds = g.nlist_builds() - builds0
    npairs = 0.5 * (p_before + g.npairs())
    if dist is not None:
        t_dev = ranks.max_over_ranks(t_dev, device="cuda")
    nc = len(bbi)
    value = nc * a.steps * world / t_dev
    steps_per_s = a.steps / t_dev
    stages = g.step_stage_times(20)
    # RATTLE pass a: per correction it reads and writes two positions and two
    # velocities and reads two start-of-step positions (16 B each), plus the
    # constraint record (12 B); HBM-bound at best, latency-bound per molecule
    hbm = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs") \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    ta = stages["constraints_a"] * 1e-3
    bytes_a = nc * (2 * 16 * 2 + 2 * 16 * 2 + 2 * 16 + 12)
    e2e_value, h2d, d2h = e2e_rate(g, torch, max(10, a.steps // 4), nc)
    if rank == 0:
        line = {
            "metric": w["metric"],
            "value": value, "unit": "constraint-solves/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * t_dev / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 (fp64 totals)", "data": "synthetic (seeded molecule lattice, device-equilibrated)",
            "config": {"workload": w["workload"], "n": n, "constraints": nc,
                       "bonded_terms": {int(k): int(len(at)) for k, at, _, _ in terms},
                       "listed_pairs": npairs, "dt": w["dt"], "T": w["T"],
                       "l2": "flushed between timed steps (256 MB write)",
                       "parallelism": "replicas only" if world > 1 else "single GPU"},
            "ns_per_day": steps_per_s * w["dt"] * TAU_PS * 1e-3 * 86400.0,
            "tau_per_day": steps_per_s * w["dt"] * 86400.0,
            "pair_evals_per_s": npairs * a.steps * world / t_dev,
            "e2e": {"value": e2e_value, "unit": "constraint-solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(kernels_per_step * a.steps),
            "roofline": {"bound": "hbm", "kernel": "k_rattle_a", "achieved": bytes_a / ta / 1e9 if ta > 0 else None,
                         "peak": hbm, "unit": "GB/s", "frac": (bytes_a / ta / 1e9 / hbm) if (hbm and ta > 0) else None,
                         "bytes_per_launch": "124 per constraint (one correction)", "traffic": None,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)"},
            "cpu_baseline": None,
            "clocks": clk.summary(),
            "stage_ms_in_graph": stages,
            "constraint_stats_timed": cst,
            "list_rebuilds_in_timed_region": int(builds),
            "autotune": {"block": tune.block, "filter": tune.filter},
        }
        if terms:
            line["bonded_kernel_ms"] = bonded_kernel_ms(g, torch, stream, terms, flush)
        line["cpu_baseline"] = constrained_cpu_sample(g, bbi, bbj, ln, w, a.cpu_seconds)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def bonded_kernel_ms(g, torch, stream, terms, flush, reps=20):
    """Median CUDA-event time of each registered bonded list's kernel."""
    out = {}
    for kind, atoms, _, _ in terms:
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        with torch.cuda.stream(stream):
            for s, e in ev:
                s.record(stream)
                g.L.sg_bonded_forces_async(g.ctx, int(kind))
                e.record(stream)
                flush.add_(1.0)
        torch.cuda.synchronize()
        out[str(int(kind))] = statistics.median(s.elapsed_time(e) for s, e in ev)
    return out


def constrained_cpu_sample(g, bbi, bbj, ln, w, seconds):
    """The oracle's apply_constraints_a (the reference's global Gauss-Seidel
    loop, FP64, one core) on the device's current state after one drift."""
    import oracle as O
    r, q, v, l = g.download()
    s = O.System(g.n, g.box, fast=True)
    s.rx[:], s.ry[:], s.rz[:] = r.T
    s.vx[:], s.vy[:], s.vz[:] = v.T
    s.set_constraints(bbi, bbj, ln)
    calls, t = 0, 0.0
    while t < seconds and calls < 50:
        s.constraints_save()
        s.vv_initial(w["dt"])
        t0 = time.perf_counter()
        s.constraints_a(w["dt"])
        t += time.perf_counter() - t0
        calls += 1
    rate = len(bbi) * calls / t
    return {"value": rate, "unit": "constraint-solves/s", "cores": 1, "kind": "port",
            "sample": f"{calls} apply_constraints_a calls on this workload's state (oracle restatement, FP64, "
                      "-O3 -ffast-math, 1 thread), the RATTLE pass alone"}


def e2e_rate(g, torch, steps, units_per_step):
    """The metric through the C ABI with FP64 host arrays (pinned) copied in
    and out every step, and the energies read back. Returns (rate, h2d bytes
    per step, d2h bytes per step)."""
    import ctypes as C
    from sucrose_gb300 import capi
    n = g.n
    pin = lambda: torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    host = [pin() for _ in range(13)]
    rr, qq, vv, ll = g.download()
    for k in range(3):
        host[k][:] = rr[:, k]
        host[7 + k][:] = vv[:, k]
        host[10 + k][:] = ll[:, k]
    for k in range(4):
        host[3 + k][:] = qq[:, k]
    D = C.POINTER(C.c_double)
    ptrs = [h.ctypes.data_as(D) for h in host]
    energies = np.zeros(4)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        capi.check(g.ctx, g.L.sg_upload_state(g.ctx, *ptrs))
        g.step(1)
        capi.check(g.ctx, g.L.sg_download_state(g.ctx, *ptrs))
        capi.check(g.ctx, g.L.sg_read_energies(g.ctx, energies.ctypes.data_as(D)))
    t = time.perf_counter() - t0
    return units_per_step * steps / t, 13 * 8 * n, 13 * 8 * n + 32


def charged_cpu_sample(g, charge, seconds, nthreads):
    """The oracle's coulombic_ over a bounded sample of the device's list."""
    import oracle as O
    r, q, v, l = g.download()
    pi, pj = g.pairs()
    s = O.System(g.n, g.box, fast=True)
    s.rx[:], s.ry[:], s.rz[:] = r.T
    s.charge[:] = charge
    pp = O.pair_params(O.COULOMB, cutoff=CHARGED["cutoff"], dielectric=CHARGED["dielectric"])
    m0 = min(len(pi), 20000 * nthreads)
    t = time.perf_counter()
    s.pair_batch(pp, pi[:m0], pj[:m0], nthreads)
    per = (time.perf_counter() - t) / max(m0, 1)
    m = int(min(len(pi), max(m0, seconds / max(per, 1e-9))))
    t = time.perf_counter()
    s.pair_batch(pp, pi[:m], pj[:m], nthreads)
    return m / (time.perf_counter() - t), m


def run_reference_charged(a):
    """Reference arm for the charged workload: the restated coulombic_ on all
    host cores over the lattice's list, a fixed slice per step."""
    import oracle as O
    from scipy.spatial import cKDTree
    w = CHARGED
    r, q, box, v, charge = charged_state(w["seed"])
    n = len(r)
    b = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
    tree = cKDTree((r + b / 2.0) % b, boxsize=b)
    pairs = tree.query_pairs(w["cutoff"] + w["skin"], output_type="ndarray")
    pairs.sort(axis=1)
    pairs = pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]
    pi, pj = pairs[:, 0].astype(np.int32), pairs[:, 1].astype(np.int32)
    s = O.System(n, box, fast=True)
    s.rx[:], s.ry[:], s.rz[:] = r.T
    s.charge[:] = charge
    pp = O.pair_params(O.COULOMB, cutoff=w["cutoff"], dielectric=w["dielectric"])
    nth = os.cpu_count() or 1
    per_step = min(len(pi), 2000000)
    for _ in range(a.warmup):
        s.pair_batch(pp, pi[:per_step // 10], pj[:per_step // 10], nth)
    t0 = time.perf_counter()
    for k in range(a.steps):
        off = (k * per_step) % max(1, len(pi) - per_step + 1)
        s.pair_batch(pp, pi[off:off + per_step], pj[off:off + per_step], nth)
    dt = time.perf_counter() - t0
    value = per_step * a.steps / dt
    line = {"impl": "reference", "metric": "charged pair-evals/s (WCA + switched Coulomb, full MD step)",
            "value": value, "unit": "pair-evals/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * dt / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp64", "data": "synthetic (seeded FCC lattice, +-1 charges)",
            "config": {"workload": w["workload"], "n": n, "listed_pairs": int(len(pi)), "per_step_pairs": per_step},
            "cpu_baseline": {"value": value, "unit": "pair-evals/s", "cores": nth, "kind": "port",
                             "sample": f"{per_step} pairs per step of the {len(pi)}-pair list; the reference "
                                       "coulombic_ (FP64) restated in C++, OpenMP"},
            "e2e": {"value": value, "unit": "pair-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_constrained(a):
    """Reference arm for the molecular workloads: the restated
    apply_constraints_a (one global Gauss-Seidel loop, FP64) on the lattice
    state after one drift, each step one call."""
    import oracle as O
    from sucrose_gb300 import configs
    w = MOLECULAR[a.config]
    r, box, bbi, bbj, ln, terms = molecular_state(a.config, w["seed"])
    n = len(r)
    v = configs.velocities_to_temperature(n, w["T"], w["seed"])
    s = O.System(n, box, fast=True)
    s.set_constraints(bbi, bbj, ln)

    def one():
        s.rx[:], s.ry[:], s.rz[:] = r.T
        s.vx[:], s.vy[:], s.vz[:] = v.T
        s.constraints_save()
        s.vv_initial(w["dt"])
        t0 = time.perf_counter()
        s.constraints_a(w["dt"])
        return time.perf_counter() - t0

    for _ in range(a.warmup):
        one()
    dt = sum(one() for _ in range(a.steps))
    value = len(bbi) * a.steps / dt
    line = {"impl": "reference", "metric": w["metric"],
            "value": value, "unit": "constraint-solves/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * dt / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp64", "data": "synthetic (seeded molecule lattice)",
            "config": {"workload": w["workload"], "n": n, "constraints": int(len(bbi))},
            "cpu_baseline": {"value": value, "unit": "constraint-solves/s", "cores": 1, "kind": "port",
                             "sample": "apply_constraints_a alone per step (the reference's loop is serial), "
                                       "FP64 restatement; favours the CPU (no forces, no pass b)"},
            "e2e": {"value": value, "unit": "constraint-solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- replicas ---
REPLICAS = dict(workload="replicas_4096_lj_gb_langevin_n64to2048", nrep=4096, seed=1005, dt=0.002, damping=1.0)


def replica_arrays(e):
    """Per-particle constants and initial velocities / angular momenta of an
    ensemble from configs.replica_ensemble (seeded per replica)."""
    from sucrose_gb300 import configs
    fams = (configs.LJ_REPLICA, configs.GB_REPLICA)
    sig, eps, inert, v, l = [], [], [], [], []
    for k in range(len(e["n"])):
        n = int(e["n"][k])
        p = fams[e["family"][k]]
        I = configs.default_inertia(p["sig"])
        sig.append(np.tile(p["sig"], (n, 1)))
        eps.append(np.tile(p["eps"], (n, 1)))
        inert.append(np.tile(I, (n, 1)))
        v.append(configs.velocities_to_temperature(n, e["temp"][k], 1 + k))
        a, b = e["off"][k], e["off"][k + 1]
        l.append(configs.angular_momenta(e["q"][a:b], I, e["temp"][k], 1 + k) if e["family"][k] == 1
                 else np.zeros((n, 3)))
    return [np.concatenate(x) for x in (sig, eps, inert, v, l)]


def replica_pair_params():
    from sucrose_gb300 import GpuSystem, capi, configs
    return [GpuSystem.params(capi.LJ, cutoff=configs.LJ_REPLICA["cutoff"]),
            GpuSystem.params(capi.GB, cutoff=configs.GB_REPLICA["cutoff"], mu=2, nu=1)]


def run_replicas(a):
    import torch
    import __graft_entry__
    __graft_entry__.build_library()
    from sucrose_gb300 import ranks
    rank, world, local = ranks.rank_info()
    torch.cuda.set_device(local)
    line = replicas_line(a, rank, world, local)
    if rank == 0:
        print(json.dumps(line), flush=True)


def replicas_line(a, rank=0, world=1, local=0, dist=None, steps=None):
    """Batched replicas: one captured step advances all 4096 replicas; the
    same replicas as 4096 single-system contexts, each stepped by its own
    captured graph one after another, give the sequential-launch comparison.
    Returns the JSON line."""
    import torch
    from sucrose_gb300 import GpuSystem, capi, configs, ranks
    steps = steps or steps
    W = REPLICAS
    t0 = time.perf_counter()
    e = configs.replica_ensemble(a.nrep, seed=ranks.replica_seed(W["seed"], rank))
    sig, eps, inert, v0, l0 = replica_arrays(e)
    t_setup_host = time.perf_counter() - t0
    LJ, GB = configs.LJ_REPLICA, configs.GB_REPLICA
    skins = [LJ["skin"], GB["skin"], 0.3]
    cuts = [LJ["list_cutoff"], GB["list_cutoff"], 3.0]
    g = GpuSystem.replicas(e["n"], e["box"], e["family"], e["temp"], e["key"])
    g.set_particles(mass=1.0, sig=sig, eps=eps, inertia=inert)
    g.upload(r=e["r"], q=e["q"], v=v0, l=l0)
    g.init_rep_nlist(skins, cuts, trigger_mode=1)
    pairs = replica_pair_params()
    stream = torch.cuda.ExternalStream(g.stream_ptr())
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    dt = W["dt"]

    def configure(step_dt, first):
        g.configure_step_pairs(pairs, integrator=capi.INT_LANGEVIN, dt=step_dt, damping=W["damping"], rotations=1,
                               first_step=first, flags=FLAGS)

    # untimed equilibration from the lattice: short steps first
    configure(dt / 4, 1)
    g.step(a.rep_equil // 2)
    g.step_check()
    configure(dt, 1 + a.rep_equil // 2)
    g.step(a.rep_equil - a.rep_equil // 2)
    g.step_check()
    tunes = {}
    for pp, name in zip(pairs, ("LJ", "GB")):
        t = g.autotune(pp, reps=3)
        tunes[name] = {"block": t.block, "filter": t.filter, "variant_ms": [float(t.ms[k]) for k in range(t.candidates)]}
    g.step(max(a.warmup, 3))
    g.step_check()
    kernels_per_step = g.step_kernel_count()
    p_before = g.npairs()
    builds0 = g.nlist_builds()
    rep_builds0 = g.rep_nlist_builds()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_dev = timed_steps(g, torch, stream, steps, flush)
    g.step_check()
    npairs = 0.5 * (p_before + g.npairs())
    builds = g.nlist_builds() - builds0
    rep_builds = g.rep_nlist_builds() - rep_builds0
    fam_of = np.asarray(e["family"])
    rebuilt_per_step = {name: float(rep_builds[fam_of == f].sum()) / steps for f, name in ((0, "LJ"), (1, "GB"))}
    if world > 1:
        t_dev = ranks.max_over_ranks(t_dev, device="cuda")
    ms_per_step = 1e3 * t_dev / steps
    value = npairs * steps * world / t_dev

    # where a step's time goes: the same step enqueued stage by stage (no graph)
    stages = ("lgv_initial", "list_check_and_rebuild", "zero_forces", "pair_LJ", "pair_GB", "lgv_final")
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(stages) + 1)] for _ in range(10)]
    builds_b = g.nlist_builds()
    with torch.cuda.stream(stream):
        for k in range(10):
            evk = ev[k]
            evk[0].record(stream)
            g.lgv_initial(dt, 10_000 + k, damping=W["damping"])
            evk[1].record(stream)
            g.update_nlist()
            evk[2].record(stream)
            g.zero_forces()
            evk[3].record(stream)
            g.pair_forces_async(pairs[0])
            evk[4].record(stream)
            g.pair_forces_async(pairs[1])
            evk[5].record(stream)
            g.L.sg_lgv_final(g.ctx, dt, W["damping"], None, None)
            evk[6].record(stream)
    torch.cuda.synchronize()
    g.step_check()
    breakdown = {name: statistics.mean(ev[k][s].elapsed_time(ev[k][s + 1]) for k in range(10))
                 for s, name in enumerate(stages)}
    breakdown["rebuilds_in_10_steps"] = int(g.nlist_builds() - builds_b)

    # dominant kernels: each family's pair launch timed alone
    fam = {}
    peak32 = g.peak_fma(False)
    for pp, name in zip(pairs, ("LJ", "GB")):
        _, _, st = g.pair_forces(pp, want_stats=True)
        tk = statistics.median(timed_forces(g, torch, stream, pp, 10, flush))
        fl = pair_flops(name, st.pairs, st.solver_evals)
        fam[name] = {"listed_pairs": int(st.pairs), "in_range": int(st.solver_evals), "force_kernel_ms": 1e3 * tk,
                     "tflops": fl / tk / 1e12}
    top = max(fam, key=lambda k: fam[k]["force_kernel_ms"])

    # e2e through the C ABI: FP64 host state in and out every step
    n = g.n
    host = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(13)]
    import ctypes as C
    D = C.POINTER(C.c_double)
    r, q, v, l = g.download()
    for k in range(3):
        host[k][:], host[7 + k][:], host[10 + k][:] = r[:, k], v[:, k], l[:, k]
    for k in range(4):
        host[3 + k][:] = q[:, k]
    ptrs = [h.ctypes.data_as(D) for h in host]
    energies = np.zeros(4)
    e_steps = 10
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(e_steps):
        capi.check(g.ctx, g.L.sg_upload_state(g.ctx, *ptrs))
        g.step(1)
        capi.check(g.ctx, g.L.sg_download_state(g.ctx, *ptrs))
        capi.check(g.ctx, g.L.sg_read_energies(g.ctx, energies.ctypes.data_as(D)))
    t_e2e = time.perf_counter() - t0

    # the same replicas one context each, stepped one after another
    seq = None
    if rank == 0 and not a.no_extras:
        r, q, v, l = g.download()
        t0 = time.perf_counter()
        singles = []
        fams = (LJ, GB)
        for k in range(len(e["n"])):
            lo, hi = e["off"][k], e["off"][k + 1]
            f = int(e["family"][k])
            s = GpuSystem(int(e["n"][k]), e["box"][k])
            s.set_particles(mass=1.0, sig=sig[lo:hi], eps=eps[lo:hi], inertia=inert[lo:hi])
            s.upload(r=r[lo:hi], q=q[lo:hi], v=v[lo:hi], l=l[lo:hi])
            s.init_nlist(fams[f]["skin"], fams[f]["list_cutoff"], trigger_mode=1)
            s.configure_step(pairs[f], integrator=capi.INT_LANGEVIN, dt=dt, damping=W["damping"], rotations=1,
                             target_temp=e["temp"][k], key=e["key"][k], first_step=1000)
            s.step(1)          # eager step + capture of the single-system graph
            singles.append(s)
        torch.cuda.synchronize()
        t_seq_setup = time.perf_counter() - t0
        seq_steps = 3
        t0 = time.perf_counter()
        for _ in range(seq_steps):
            for s in singles:
                s.step(1)
        torch.cuda.synchronize()
        t_seq = (time.perf_counter() - t0) / seq_steps
        for s in singles:
            s.step_check()
            s.close()
        seq = {"ms_per_step": 1e3 * t_seq, "contexts": len(singles), "setup_s": t_seq_setup,
               "batched_speedup": t_seq / (t_dev / steps),
               "how": "one context and one captured step graph per replica, launched one after another from the "
                      "host each step (each context on its own stream); host wall clock over 3 steps with device "
                      "synchronisation at both ends"}

    cpu = None
    if rank == 0:
        cpu = replica_cpu_sample(e, a.cpu_seconds, nthreads=1)
    if rank == 0:
        nrep_total = len(e["n"]) * world
        line = {
            "metric": METRICS["replicas"],
            "value": value, "unit": "pair-evals/s", "n_gpus": world, "steps": steps, "warmup": a.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 (fp64 totals)", "data": "synthetic (seeded replica ensemble, device-equilibrated)",
            "config": {"workload": W["workload"], "replicas": len(e["n"]), "particles": int(n),
                       "listed_pairs": npairs, "lj_replicas": int(np.sum(e["family"] == 0)),
                       "gb_replicas": int(np.sum(e["family"] == 1)), "count_redraws": int(e["redraws"]),
                       "dt": dt, "integrator": "Langevin (translation + rotation), per-replica T and Philox key",
                       "l2": "inputs larger than L2 (and a 256 MB write between timed steps)",
                       "parallelism": "replicas only" if world > 1 else "single GPU"},
            "replica_steps_per_s": nrep_total * steps / t_dev,
            "e2e": {"value": npairs * e_steps / t_e2e, "unit": "pair-evals/s", "h2d_bytes_per_step": 13 * 8 * n,
                    "d2h_bytes_per_step": 13 * 8 * n + 32},
            "gpu_launches": int(kernels_per_step * steps),
            "roofline": {"bound": "fp32", "kernel": f"k_pair<Pot{top}> (replica family range)",
                         "achieved": fam[top]["tflops"], "peak": peak32, "unit": "TFLOP/s",
                         "frac": fam[top]["tflops"] / peak32,
                         "peak_source": "measured FMA throughput (sg_peak_fma) on this GPU", "traffic": None},
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "families": fam,
            "autotune": tunes,
            "stage_ms_in_graph": breakdown,
            "list_rebuilds_in_timed_region": int(builds),
            "replicas_rebuilt_per_step": rebuilt_per_step,
            "sequential_single_system": seq,
            "host_setup_s": t_setup_host,
        }
    g.close()
    return line if rank == 0 else None


def replica_cpu_systems(e, stride=97):
    """Oracle systems and k-d-tree lists (the reference's list contents) for
    every stride-th LJ and GB replica, interleaved."""
    import oracle as O
    from scipy.spatial import cKDTree
    from sucrose_gb300 import configs
    fams = (configs.LJ_REPLICA, configs.GB_REPLICA)
    R = len(e["n"])
    lj, gb = list(range(0, R // 2, stride)), list(range(R // 2, R, stride))
    idx = [k for pair in zip(lj, gb) for k in pair] + lj[len(gb):] + gb[len(lj):]
    out = []
    for k in idx:
        f = int(e["family"][k])
        p = fams[f]
        lo, hi = e["off"][k], e["off"][k + 1]
        box = e["box"][k]
        r = e["r"][lo:hi]
        t = cKDTree((r + box / 2) % box, boxsize=box)
        pr = t.query_pairs(p["list_cutoff"] + p["skin"], output_type="ndarray")
        if len(pr) == 0:
            continue
        pr.sort(axis=1)
        s = O.System(hi - lo, box, fast=True)
        s.set_defaults(sig=p["sig"], eps=p["eps"])
        s.rx[:], s.ry[:], s.rz[:] = r.T
        s.qw[:], s.qx[:], s.qy[:], s.qz[:] = e["q"][lo:hi].T
        pp = O.pair_params(O.LJ if f == 0 else O.GB, cutoff=p["cutoff"], mu=2 if f else None, nu=1 if f else None)
        out.append((s, pp, pr[:, 0].astype(np.int32).copy(), pr[:, 1].astype(np.int32).copy()))
    return out


def replica_cpu_sample(e, seconds, nthreads=1):
    """The oracle's restatement of the reference pair routines (lj_, gb_) on
    whole replicas, one after another, until about `seconds` have passed."""
    done, spent, reps = 0, 0.0, 0
    for s, pp, pi, pj in replica_cpu_systems(e):
        t0 = time.perf_counter()
        s.pair_batch(pp, pi, pj, nthreads)
        spent += time.perf_counter() - t0
        done += len(pi)
        reps += 1
        if spent > seconds:
            break
    return {"value": done / max(spent, 1e-9), "unit": "pair-evals/s", "cores": nthreads, "kind": "port",
            "sample": f"{reps} whole replicas (every 97th LJ and GB replica, interleaved), {done} listed pairs, the "
                      "reference's lj_ / gb_ restated in C++ (FP64), oracle built -O3 -ffast-math"}


def reference_replicas_line(a, steps=None):
    """Reference arm for the replica ensemble: the restated lj_ / gb_ on the
    host cores (OpenMP), each step one pass over a fixed sample of whole
    replicas."""
    from sucrose_gb300 import configs
    steps = steps or a.steps
    e = configs.replica_ensemble(a.nrep, seed=REPLICAS["seed"])
    systems = replica_cpu_systems(e)
    nth = os.cpu_count() or 1
    per_step = 0
    chosen = []
    for sy in systems:          # about 2M pairs per step
        chosen.append(sy)
        per_step += len(sy[2])
        if per_step > 2000000:
            break
    for _ in range(a.warmup):
        for s, pp, pi, pj in chosen[:2]:
            s.pair_batch(pp, pi, pj, nth)
    t0 = time.perf_counter()
    for _ in range(steps):
        for s, pp, pi, pj in chosen:
            s.pair_batch(pp, pi, pj, nth)
    dt = time.perf_counter() - t0
    value = per_step * steps / dt
    line = {"impl": "reference", "metric": METRICS["replicas"],
            "value": value, "unit": "pair-evals/s", "n_gpus": a.gpus, "steps": steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * dt / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp64", "data": "synthetic (seeded replica ensemble, lattice state)",
            "config": {"workload": REPLICAS["workload"], "replicas_sampled": len(chosen), "per_step_pairs": per_step},
            "cpu_baseline": {"value": value, "unit": "pair-evals/s", "cores": nth, "kind": "port",
                             "sample": f"{len(chosen)} whole replicas per step ({per_step} pairs); the reference "
                                       "lj_ / gb_ restated in C++, OpenMP"},
            "e2e": {"value": value, "unit": "pair-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


# --------------------------------------------------------------- reference ---
def reference_ellipsoid_line(a, name, steps=None):
    """The reference's pair routine (ecpr_ with its Brent solve and per-pair
    setup, or gb_) restated on the CPU (its Fortran has no compiler here), on
    all host threads, over the whole listed pair set of the same seeded state
    the GPU arm starts from (the list built by a k-d tree with the
    reference's acceptance test), once per step."""
    import oracle as O
    from scipy.spatial import cKDTree
    w = WORKLOADS[name]
    steps = steps or a.steps
    r, q, box, v, l, rep = initial_state(w)
    n = len(r)
    rw = (r + box / 2.0) % box
    tree = cKDTree(rw, boxsize=box)
    pairs = tree.query_pairs(w["list_cutoff"] + w["skin"], output_type="ndarray")
    pairs.sort(axis=1)
    pairs = pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]
    pi, pj = pairs[:, 0].astype(np.int32), pairs[:, 1].astype(np.int32)
    s = O.System(n, box, fast=True)
    s.set_defaults(sig=w["sig"], eps=w["eps"])
    s.rx[:], s.ry[:], s.rz[:] = r.T
    s.qw[:], s.qx[:], s.qy[:], s.qz[:] = q.T
    kind = getattr(O, w["kind"])
    pp = O.pair_params(kind, cutoff=w["cutoff"], solver=O.SOLVER_BRENT, mu=w.get("mu"), nu=w.get("nu"))
    nth = os.cpu_count() or 1
    for _ in range(a.warmup):
        s.pair_batch(pp, pi[:len(pi) // 10], pj[:len(pj) // 10], nth)
    t0 = time.perf_counter()
    for k in range(steps):
        s.pair_batch(pp, pi, pj, nth)
    dt = time.perf_counter() - t0
    value = len(pi) * steps / dt
    routine = "ecpr_: Brent, per-pair setup" if name == "ecp" else "gb_ (mu 2, nu 1)"
    return {"impl": "reference", "metric": METRICS[name],
            "value": value, "unit": "pair-evals/s", "n_gpus": a.gpus, "steps": steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * dt / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp64", "data": "synthetic (seeded isotropic placement, the same state as the GPU arm)",
            "config": {"workload": w["workload"], "n": n, "listed_pairs": int(len(pi)), "seed": w["seed"],
                       "timed": "the reference pair routine over every listed pair, once per step",
                       "placement_sweeps": int(rep.sweeps)},
            "cpu_baseline": {"value": value, "unit": "pair-evals/s", "cores": nth, "kind": "port",
                             "sample": f"all {len(pi)} listed pairs per step; the reference pair routine ("
                                       + routine + ", FP64) restated in C++, OpenMP"},
            "e2e": {"value": value, "unit": "pair-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if a.config == "replicas":
        print(json.dumps(reference_replicas_line(a)), flush=True)
        return
    if a.config == "charged":
        return run_reference_charged(a)
    if a.config in ("constrained", "polymer"):
        return run_reference_constrained(a)
    import __graft_entry__
    __graft_entry__.build_library()     # the seeded placement runs on the device (input set-up only)
    line = reference_ellipsoid_line(a, a.config)
    if a.config == "ecp" and not a.no_extras and not a.no_sub:
        line["gb"] = reference_ellipsoid_line(a, "gb", steps=min(a.steps, 50))
        line["replicas"] = reference_replicas_line(a, steps=min(a.steps, 20))
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------- profile cases ---
PROFILE_CASES = """Small, self-contained launches of each kernel family, for profiling:
python bench.py --profile-case <case> [--reps K]. Each case builds one seeded
system at the size of its benchmark workload (the same isotropic ECP and GB
states as the benchmark), runs one untimed launch sequence, then K launches
of the kernels of interest and exits. A profiler selects the kernel with its
own filter (for example ncu -k regex:k_pair -c 2). Cases:
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
  replicas  captured steps of --nrep replicas (LJ + GB), same flag"""


def profile_case(a):
    import __graft_entry__
    __graft_entry__.build_library()
    from sucrose_gb300 import GpuSystem, capi, configs
    case = a.profile_case
    g = p = None
    if case in ("ecp", "ecp_mlp", "list", "nhc", "ecp_step", "mlp_train"):
        w = WORKLOADS["ecp"]
        g, _, _ = make_system(w)
        p = pair_params(g, w, a.solver if a.solver in ("newton", "support") else "newton")
        if a.ecp_path:
            g.set_launch(p.kind, 256, {"fused": 0, "split": 1, "filtered": 2}[a.ecp_path])
    elif case in ("gb", "langevin", "gb_list"):
        w = WORKLOADS["gb"]
        g, _, _ = make_system(w)
        p = pair_params(g, w, "newton")
    elif case == "lj":
        r, q, box = configs.fcc_lattice(20, 0.8442)
        g = GpuSystem(len(r), box)
        g.upload(r=r, v=configs.velocities_to_temperature(len(r), 0.722, 15))
        g.init_nlist(0.3, 2.5, trigger_mode=1)
        p = g.params(capi.LJ, cutoff=2.5)
    elif case != "replicas":
        raise SystemExit("unknown case " + case + "\n" + PROFILE_CASES)
    reps = a.reps
    if case in ("ecp", "gb", "lj"):
        for _ in range(1 + reps):
            g.zero_forces()
            g.pair_forces(p)
    elif case == "ecp_mlp":
        from sucrose_gb300 import mlp

        def langevin(T):
            g.configure_step(p, integrator=capi.INT_LANGEVIN, dt=0.001, target_temp=T, rotations=1)

        X, y = mlp.generate(g, p, langevin, samples=200_000, every=10, equil=20)
        mlp.train(g, X, y, epochs=1, batch=65536, lr=2e-3, seed=1)
        g.build_nlist()
        pm = pair_params(g, WORKLOADS["ecp"], "mlp")
        for _ in range(1 + reps):
            g.zero_forces()
            g.pair_forces(pm)
    elif case in ("list", "gb_list"):
        for _ in range(1 + reps):
            g.build_nlist()
    elif case == "langevin":
        g.zero_forces()
        g.pair_forces(p)
        for k in range(1 + reps):
            g.lgv_initial(0.002, k + 1, damping=1.0, target_temp=1.0)
            g.lgv_final(0.002, damping=1.0)
    elif case == "nhc":
        g.zero_forces()
        g.pair_forces(p)
        for _ in range(1 + reps):
            g.nht_initial(0.001, 1.2, 0.0, mode=1, rot_chain=1)
            g.qq_initial(0.001)
            g.nht_final(0.001, 1.2, 0.0, mode=1, rot_chain=1)
            g.qq_final(0.001)
    elif case == "ecp_step":
        g.configure_step(p, integrator=capi.INT_NH, dt=0.001, target_temp=1.2, rotations=1, rot_chain=1,
                         flags=capi.STEP_FLAT)
        g.step(1 + reps)
    elif case == "mlp_train":
        from sucrose_gb300 import mlp

        def langevin(T):
            g.configure_step(p, integrator=capi.INT_LANGEVIN, dt=0.001, target_temp=T, rotations=1)

        X, y = mlp.generate(g, p, langevin, samples=65536, every=2, equil=2)
        mlp.train(g, X, y, epochs=1 + reps, batch=65536, lr=2e-3, seed=1)
    elif case == "replicas":
        e = configs.replica_ensemble(a.nrep, seed=REPLICAS["seed"])
        sig, eps, inert, v0, l0 = replica_arrays(e)
        g = GpuSystem.replicas(e["n"], e["box"], e["family"], e["temp"], e["key"])
        g.set_particles(mass=1.0, sig=sig, eps=eps, inertia=inert)
        g.upload(r=e["r"], q=e["q"], v=v0, l=l0)
        LJ, GB = configs.LJ_REPLICA, configs.GB_REPLICA
        g.init_rep_nlist([LJ["skin"], GB["skin"], 0.3], [LJ["list_cutoff"], GB["list_cutoff"], 3.0], trigger_mode=1)
        pairs = replica_pair_params()
        g.configure_step_pairs(pairs, integrator=capi.INT_LANGEVIN, dt=REPLICAS["dt"], damping=1.0, rotations=1,
                               flags=capi.STEP_FLAT)
        if a.rep_equil:   # untimed steps first, until replicas start to rebuild their lists
            g.step(a.rep_equil)
        g.step(1 + reps)
    g.synchronize()
    print("profile case", case, "done")


if __name__ == "__main__":
    args = parse()
    if args.flat_graph:
        FLAGS = 1
    if args.profile_case:
        profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.config == "replicas":
        run_replicas(args)
    elif args.config == "charged":
        run_charged(args)
    elif args.config in ("constrained", "polymer"):
        run_constrained(args)
    else:
        run_ours(args)
