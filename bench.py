"""Benchmark of the GB300 force-evaluation path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME]

Prints ONE JSON line (rank 0).  A step is one integrator step of the
workload (drift + force evaluation + kick) over the whole particle set.

Workloads (seeded synthetic inputs -- grav_sim publishes no dataset):
  galaxy1048576_learned -- the default and the headline line: the two-galaxy
                    collision (exponential disk, Hernquist bulge and halo;
                    equal masses) at N = 1,048,576, run as the theta = 1.0
                    group walk plus the learned residual, judged every step
                    by a 4,096-particle direct sum with the theta = 0.5 walk
                    as fallback (method 104; collection and GPU training
                    happen before the timed region; when the network did not
                    earn its place on the held-out snapshot, every step is
                    the fallback walk alone, with nothing to judge).  The same line times
                    the plain Barnes-Hut comparators on the same GPU: the
                    group walk at theta = 0.5 (method 106) and the
                    reference-style monopole walk (method 103) at theta =
                    0.5 and at theta = 0.3, where it meets the 1e-3 median
                    error bound; and the learned pipeline at work: method
                    104 at theta_cheap = 0.75 with the network forced on
                    (features, forward pass, correction and judge every
                    step) beside the plain group walk at theta = 0.75.
  galaxy1048576_learned_t075 -- that learned arm alone (method 104 at
                    theta_cheap = 0.75, the network forced on), for its
                    launch list.
  plummer1024_fp64 -- the reference's CPU-sized case: Plummer N = 1,024, the
                    FP64 direct sum in the reference's order (bit-exact),
                    leapfrog dt = 1e-3; every step is one CUDA-graph replay.
  plummer262144  -- equal-mass Plummer sphere, N = 262,144, G = M = a = 1,
                    compensated-FP32 direct sum, eps = 0.01, leapfrog,
                    dt = 1e-3 (the mixed-precision direct-sum workload).
  galaxy2097152 / galaxy1048576 -- the galaxy pair, Barnes-Hut with monopole
                    + quadrupole cells, theta = 0.5, eps = 0.01, leapfrog
                    dt = 1e-3.
  galaxy1048576_plain -- the same at N = 1,048,576 with the monopole walk.
  galaxy2097152_group / galaxy1048576_group -- the group walk with
                    interaction lists (quadrupole cells), theta = 0.5; the
                    2,097,152-particle one is the Barnes-Hut galaxy-collision
                    workload (200 steps in the original brief).
  galaxy16777216_group -- the group walk at N = 16,777,216 (about 4 GB of
                    state and tree in HBM).
  galaxy2097152_group_leaf1 / _t065, galaxy1048576_group_leaf1 -- with one
                    particle per leaf (the reference's default tree), or at
                    theta = 0.65 (median error 6.4e-4, inside the 1e-3 bound).
                    The group workloads use up to 16 particles per leaf, the
                    library's default for methods 104, 106 and 107.
  galaxy1048576_group_mono[_t035] -- the group walk with monopole cells
                    only, theta = 0.5 (0.35).
  ensemble8192 / ensemble8192_leapfrog -- 8,192 planetary systems (Sun, 8
                    planets, 0-4,096 massless test particles each), WHFast or
                    leapfrog with the massless accelerations, dt = 1 day.
  cosmo_pm256    -- cosmological particle-mesh run: 256^3 particles on a
                    perturbed lattice in a periodic box, 256^3 mesh, h = 0.7,
                    Omega_m = 0.3, Omega_Lambda = 0.7, a = 1/8 in steps of
                    1/256 (exact in binary, so K steps are ceil(K da / da) = K;
                    launch_cosmological_simulation).

value      particle-steps/s over all ranks, state resident in HBM, device
           time of K steps from CUDA events on the simulation's stream
           (L2 flushed by a 256 MiB write before every timed step, outside
           the step's events).
e2e        the same metric through launch_simulation_python with host numpy
           buffers: allocation, host->device copy of x, v, m, K steps and the
           device->host copy of x, v inside the timed region.
roofline   dominant kernel: the direct sum (20 FLOP per pair interaction x
           N(N-1) per launch) or the Barnes-Hut walk (20 FLOP per accepted
           cell or leaf pair term, counted on the device) / mean launch time
           (CUDA events around the kernel on its stream), against the FP32
           FMA peak measured on this GPU by the library's probe.
accuracy   median / p99 relative acceleration error of the last step's
           forces against an FP64 direct sum of 4,096 sampled particles
           (512 for the direct-sum workloads), computed on the GPU in FP64.
cpu_baseline  the reference's algorithm restated by the oracle, timed on
           this machine's host cores: the symmetric pairwise loop (one
           thread: the reference's pairwise sum has no OpenMP) for the
           direct-sum workloads; Barnes-Hut at theta = 0.5 as the reference
           computes it (serial octree build, OpenMP walk over all cores) for
           the galaxy workloads; the per-system WHFast or leapfrog loop (one
           system per thread) for the ensembles.  Each on a bounded sample,
           extrapolated to a full step.
Multi-GPU: replicas only (each rank runs the whole workload); value sums
ranks; time is the max over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import importlib.util
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "gravity-simulator_gb300"
METRIC = "particle-steps/s at ≤1e-3 median accel err vs FP64 sum; learned vs plain BH"


def _module(name):
    key = f"gsgpu_{name}"
    if key in sys.modules:
        return sys.modules[key]
    spec = importlib.util.spec_from_file_location(key, PKG / f"{name}.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[key] = mod
    spec.loader.exec_module(mod)
    return mod


WORKLOADS = {
    "plummer262144": dict(ic="plummer", n=262144, seed=2, G=1.0, eps=0.01, dt=1e-3, integrator=4,
                          method=101, flop_per_interaction=20),
    # the reference's own CPU-sized case (N = 1,024, leapfrog, 1,000 steps in the
    # parity test), FP64 reference-order forces: launch- and graph-bound
    "plummer1024_fp64": dict(ic="plummer", n=1024, seed=1, G=1.0, eps=0.01, dt=1e-3,
                             integrator=4, method=111, flop_per_interaction=20),
    # small case of the same kernel, for profiler captures
    "plummer65536": dict(ic="plummer", n=65536, seed=2, G=1.0, eps=0.01, dt=1e-3, integrator=4,
                         method=101, flop_per_interaction=20),
    "galaxy2097152": dict(ic="galaxy", n=2097152, seed=4, G=1.0, eps=0.01, dt=1e-3, integrator=4,
                          method=105, theta=0.5, leaf=1, flop_per_interaction=20),
    "galaxy1048576": dict(ic="galaxy", n=1048576, seed=5, G=1.0, eps=0.01, dt=1e-3, integrator=4,
                          method=105, theta=0.5, leaf=1, flop_per_interaction=20),
    "galaxy1048576_plain": dict(ic="galaxy", n=1048576, seed=5, G=1.0, eps=0.01, dt=1e-3,
                                integrator=4, method=103, theta=0.5, leaf=1,
                                flop_per_interaction=20),
    # the headline: theta = 1.0 walk + learned residual against plain
    # Barnes-Hut on the same GPU (the group walk, and the reference-style
    # monopole walk at theta = 0.5 and at the theta where it meets 1e-3)
    "galaxy1048576_learned": dict(ic="galaxy", n=1048576, seed=5, G=1.0, eps=0.01, dt=1e-3,
                                  integrator=4, method=104, theta=1.0, leaf=16,
                                  flop_per_interaction=20, plain_key="plain_group_theta0.5",
                                  compare=[("plain_group_theta0.5",
                                            dict(method=106, theta=0.5, leaf=16)),
                                           ("plain_monopole_theta0.5",
                                            dict(method=103, theta=0.5, leaf=1)),
                                           ("plain_monopole_theta0.3",
                                            dict(method=103, theta=0.3, leaf=1)),
                                           # the learned pipeline at work: a cheap angle
                                           # where the corrected error meets the bound,
                                           # the network forced on, beside the plain walk
                                           # at the same angle
                                           ("learned_forced_theta0.75",
                                            dict(method=104, theta=0.75, leaf=16, policy=1)),
                                           ("plain_group_theta0.75",
                                            dict(method=106, theta=0.75, leaf=16))]),
    # the learned pipeline alone (the headline's learned_forced_theta0.75 arm)
    "galaxy1048576_learned_t075": dict(ic="galaxy", n=1048576, seed=5, G=1.0, eps=0.01,
                                       dt=1e-3, integrator=4, method=104, theta=0.75, leaf=16,
                                       policy=1, flop_per_interaction=20),
    "galaxy2097152_group": dict(ic="galaxy", n=2097152, seed=4, G=1.0, eps=0.01, dt=1e-3,
                                integrator=4, method=106, theta=0.5, leaf=16,
                                flop_per_interaction=20),
    "galaxy16777216_group": dict(ic="galaxy", n=16777216, seed=8, G=1.0, eps=0.01, dt=1e-3,
                                 integrator=4, method=106, theta=0.5, leaf=16,
                                 flop_per_interaction=20),
    "galaxy2097152_group_leaf1": dict(ic="galaxy", n=2097152, seed=4, G=1.0, eps=0.01, dt=1e-3,
                                      integrator=4, method=106, theta=0.5, leaf=1,
                                      flop_per_interaction=20),
    "galaxy2097152_group_t065": dict(ic="galaxy", n=2097152, seed=4, G=1.0, eps=0.01, dt=1e-3,
                                     integrator=4, method=106, theta=0.65, leaf=16,
                                     flop_per_interaction=20),
    "galaxy1048576_group": dict(ic="galaxy", n=1048576, seed=5, G=1.0, eps=0.01, dt=1e-3,
                                integrator=4, method=106, theta=0.5, leaf=16,
                                flop_per_interaction=20),
    "galaxy1048576_group_leaf1": dict(ic="galaxy", n=1048576, seed=5, G=1.0, eps=0.01, dt=1e-3,
                                      integrator=4, method=106, theta=0.5, leaf=1,
                                      flop_per_interaction=20),
    "galaxy1048576_group_mono": dict(ic="galaxy", n=1048576, seed=5, G=1.0, eps=0.01, dt=1e-3,
                                     integrator=4, method=107, theta=0.5, leaf=16,
                                     flop_per_interaction=20),
    "galaxy1048576_group_mono_t035": dict(ic="galaxy", n=1048576, seed=5, G=1.0, eps=0.01,
                                          dt=1e-3, integrator=4, method=107, theta=0.35,
                                          leaf=16, flop_per_interaction=20),
    # small cases of the walks, for profiler captures
    "galaxy262144": dict(ic="galaxy", n=262144, seed=6, G=1.0, eps=0.01, dt=1e-3, integrator=4,
                         method=105, theta=0.5, leaf=1, flop_per_interaction=20),
    "galaxy262144_group": dict(ic="galaxy", n=262144, seed=6, G=1.0, eps=0.01, dt=1e-3,
                               integrator=4, method=106, theta=0.5, leaf=16,
                               flop_per_interaction=20),
    "ensemble8192": dict(ic="ensemble", systems=8192, seed=3, max_test=4096, dt=1.0,
                         integrator=10, method=102),
    "cosmo_pm256": dict(ic="cosmo", n=256 ** 3, grid=256, seed=7, box_width=50.0, h=0.7,
                        omega_m=0.3, omega_lambda=0.7, a_begin=0.125, da=1.0 / 256),
    "ensemble8192_leapfrog": dict(ic="ensemble", systems=8192, seed=3, max_test=4096, dt=1.0,
                                  integrator=4, method=102),
}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(values, world):
    """Each value's maximum over the ranks (replicas: the slowest rank sets
    the job's time).  Uses whichever torch.distributed backend is up: NCCL on
    CUDA tensors, gloo on CPU tensors."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu().tolist()]


def cpu_baseline_pairwise(wk, x, m, target_s=12.0):
    """Time the reference's pairwise loop (oracle restatement, 1 thread) on a
    bounded slice of outer rows and extrapolate to one full leapfrog step."""
    sys.path.insert(0, str(ROOT))
    from oracle import restatement as orc
    orc.load()
    n = wk["n"]
    rows = 64
    _, pairs = orc.pairwise_slice(x, m, wk["G"], wk["eps"], 0, rows)
    t0 = time.perf_counter()
    _, pairs = orc.pairwise_slice(x, m, wk["G"], wk["eps"], 0, rows)
    dt0 = time.perf_counter() - t0
    rows = max(64, min(n, int(rows * target_s / max(dt0, 1e-3))))
    t0 = time.perf_counter()
    _, pairs = orc.pairwise_slice(x, m, wk["G"], wk["eps"], 0, rows)
    el = time.perf_counter() - t0
    pair_rate = pairs / el
    t_eval = (n * (n - 1) / 2) / pair_rate
    return {"value": n / t_eval, "unit": "particle-steps/s", "cores": 1, "kind": "port",
            "sample": f"grav_sim symmetric pairwise loop over outer rows 0..{rows} of N={n} "
                      f"({pairs} pair evaluations, {el:.1f} s), extrapolated to N(N-1)/2 pairs "
                      f"per step; kick/drift (O(N)) neglected",
            "pair_evals_per_s": pair_rate}


# The reference's Barnes-Hut as the CPU baseline of the galaxy workloads:
# opening angle 0.5, one particle per leaf (its default tree), its own cell
# membership test and leaf multipoles (compat mode), serial octree build and
# an OpenMP walk (src/acceleration_barnes_hut.c:33-248).
CPU_BH_THETA = 0.5
CPU_BH_LEAF = 1


def cpu_baseline_bh(wk, x, m, target_s=10.0):
    """Time grav_sim's Barnes-Hut (oracle restatement: serial build, OpenMP
    walk over the host's cores) on a strided sample of the sorted particles;
    a step is the build plus N walks (kick/drift, O(N), neglected)."""
    sys.path.insert(0, str(ROOT))
    from oracle import restatement as orc
    n = wk["n"]
    r = orc.bh_cpu_timing(x, m, wk["G"], wk["eps"], CPU_BH_THETA, CPU_BH_LEAF, True,
                          target_s=target_s)
    step_s = r["build_s"] + n * r["walk_s_per_particle"]
    return {"value": n / step_s, "unit": "particle-steps/s", "cores": r["threads"],
            "kind": "port",
            "sample": f"grav_sim Barnes-Hut (theta={CPU_BH_THETA}, {CPU_BH_LEAF} particle per leaf, "
                      f"the reference's membership test and leaf multipoles) at N={n}: octree "
                      f"build {r['build_s']:.2f} s (serial, as the reference), walk of "
                      f"{r['sample']} strided sorted particles in {r['walk_s']:.1f} s on "
                      f"{r['threads']} OpenMP threads, extrapolated to N walks per step",
            "step_s": step_s}


def fp64_rows(x, m, rows, G, eps):
    """FP64 direct-sum accelerations of the given rows (numpy in, numpy
    out), computed with torch in FP64 on the current GPU."""
    import torch
    X = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    M = torch.from_numpy(np.ascontiguousarray(m)).cuda()
    out = torch.empty((len(rows), 3), dtype=torch.float64, device="cuda")
    idx = torch.from_numpy(np.asarray(rows, dtype=np.int64)).cuda()
    chunk = max(1, int(2 ** 27 // max(x.shape[0], 1)))
    for b in range(0, len(rows), chunk):
        r = idx[b:b + chunk]
        d = X[None, :, :] - X[r][:, None, :]              # x_j - x_i
        r2 = (d * d).sum(-1) + eps * eps
        w = M[None, :] / (r2 * torch.sqrt(r2))
        w[torch.arange(len(r), device="cuda"), r] = 0.0    # no self term
        out[b:b + chunk] = G * (w[:, :, None] * d).sum(1)
        del d, r2, w
    res = out.cpu().numpy()
    del X, M, out, idx
    torch.cuda.empty_cache()
    return res


def accuracy_sample(a_gpu, x, m, G, eps, rows=4096, seed=0):
    """Median / p99 relative error of GPU accelerations on sampled particles
    against an FP64 direct sum."""
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(x.shape[0], min(rows, x.shape[0]), replace=False))
    ref = fp64_rows(x, m, idx, G, eps)
    errs = np.linalg.norm(a_gpu[idx] - ref, axis=1) / np.linalg.norm(ref, axis=1)
    return float(np.median(errs)), float(np.quantile(errs, 0.99))


def profile_traffic(kernel, workload, summary=None, field="traffic_bytes_per_launch"):
    """DRAM bytes (read + write) per launch of `kernel` on `workload`, from
    the ncu capture summarised in profiles/<kernel>_<workload>.md (or the
    named summary), or None.  field="l2_bytes_per_launch" gives the L2
    traffic (lts__t_bytes.sum) where the summary records it."""
    prof = ROOT / "profiles" / f"{summary or kernel + '_' + workload}.md"
    if prof.exists():
        for ln in prof.read_text().splitlines():
            if ln.startswith(field + ":"):
                return float(ln.split(":", 1)[1])
    return None


BH_METHODS = (103, 104, 105, 106, 107, 113)
FLOP_QUAD_CELL = 56


def _bind_sim(lib, g):
    dp = ctypes.POINTER(ctypes.c_double)
    lib.gsgpu_sim_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                     ctypes.c_double, ctypes.POINTER(g.AccelerationParam),
                                     ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    lib.gsgpu_sim_upload.argtypes = [ctypes.c_void_p, dp, dp, dp]
    lib.gsgpu_sim_run.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    lib.gsgpu_sim_download.argtypes = [ctypes.c_void_p, dp, dp]
    lib.gsgpu_sim_set_force_timing.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.gsgpu_sim_force_timing.argtypes = [ctypes.c_void_p, dp, ctypes.POINTER(ctypes.c_int64)]
    lib.gsgpu_sim_kernels_per_step.argtypes = [ctypes.c_void_p]
    lib.gsgpu_sim_destroy.argtypes = [ctypes.c_void_p]
    lib.gsgpu_sim_download_acceleration.argtypes = [ctypes.c_void_p, dp]
    lib.gsgpu_measure_fma_peak.argtypes = [ctypes.c_int, dp, dp]
    lib.gsgpu_sim_interaction_counts.argtypes = [ctypes.c_void_p,
                                                 ctypes.POINTER(ctypes.c_longlong)]
    lib.gsgpu_sim_warmup_until_ready.argtypes = [ctypes.c_void_p, ctypes.c_int64,
                                                 ctypes.POINTER(ctypes.c_int64)]
    lib.gsgpu_sim_report.argtypes = [ctypes.c_void_p, dp, ctypes.c_int]
    return dp


def sim_arm(args, lib, g, wk, x, v, m, stream, flush, world, local, sample_clocks=False,
            acc_rows=4096):
    """One method on the device-resident loop: (training), W warm-up steps,
    K timed steps (CUDA events on the simulation's stream, L2 flushed before
    each), K more steps with events around the dominant kernel, then the
    accuracy of the last step's forces."""
    import torch
    dp = _bind_sim(lib, g)
    n = x.shape[0]
    sim = ctypes.c_void_p()
    p = g.AccelerationParam(wk["method"], wk.get("theta", 1.0), wk["eps"], wk.get("leaf", -1))
    rc = lib.gsgpu_sim_create(ctypes.byref(sim), n, wk["G"], ctypes.byref(p), wk["integrator"],
                              wk["dt"], ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, rc
    out = {}
    try:
        assert lib.gsgpu_sim_upload(sim, x.ctypes.data_as(dp), v.ctypes.data_as(dp),
                                    m.ctypes.data_as(dp)) == 0
        if wk["method"] == 104:
            # collection snapshots and GPU training happen before the timed region
            t0 = time.perf_counter()
            spent = ctypes.c_int64()
            assert lib.gsgpu_sim_warmup_until_ready(sim, 1000, ctypes.byref(spent)) == 0
            out["training_s"] = time.perf_counter() - t0
            out["training_steps"] = spent.value
            if wk.get("policy") is not None:   # 1: the network at every step, judged
                lib.gsgpu_sim_set_learned_policy.argtypes = [ctypes.c_void_p, ctypes.c_int]
                assert lib.gsgpu_sim_set_learned_policy(sim, int(wk["policy"])) == 0
        # warm-up (includes the leapfrog half kick and graph capture)
        assert lib.gsgpu_sim_run(sim, args.warmup) == 0
        torch.cuda.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        clocks = ClockSampler(local) if sample_clocks else None
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
            time.sleep(0.3)
        # the primary arm's timed steps are the profiler range (a launch list
        # taken with ncu --profile-from-start off covers exactly them)
        if sample_clocks:
            torch.cuda.profiler.start()
        wall0 = time.perf_counter()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.fill_(k & 0xFF)                 # evict L2 between steps (not timed)
                starts[k].record(stream)
                assert lib.gsgpu_sim_run(sim, 1) == 0
                ends[k].record(stream)
        torch.cuda.synchronize()
        out["wall_s"] = time.perf_counter() - wall0
        if sample_clocks:
            torch.cuda.profiler.stop()
        if clocks:
            out["clocks"] = clocks.stop()
        if world > 1:
            torch.distributed.barrier()
        total_ms = float(sum(s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)))
        total_ms, = max_over_ranks([total_ms], world)
        out["total_ms"] = total_ms
        out["ms_per_step"] = total_ms / args.steps
        out["kernels_per_step"] = lib.gsgpu_sim_kernels_per_step(sim)
        # The dominant kernel's duration, for the roofline: K more steps with
        # CUDA events around each force kernel (launched directly, not from
        # the graph; outside the timed region).
        lib.gsgpu_sim_set_force_timing(sim, 1)
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.fill_(k & 0xFF)
                assert lib.gsgpu_sim_run(sim, 1) == 0
        torch.cuda.synchronize()
        force_ms = ctypes.c_double()
        force_n = ctypes.c_int64()
        lib.gsgpu_sim_force_timing(sim, ctypes.byref(force_ms), ctypes.byref(force_n))
        if wk["method"] in BH_METHODS:
            mo_ms, so_ms, builds = ctypes.c_double(), ctypes.c_double(), ctypes.c_int64()
            lib.gsgpu_sim_build_timing.argtypes = [ctypes.c_void_p, dp, dp,
                                                   ctypes.POINTER(ctypes.c_int64)]
            lib.gsgpu_sim_build_timing(sim, ctypes.byref(mo_ms), ctypes.byref(so_ms),
                                       ctypes.byref(builds))
            out["morton_ms"] = mo_ms.value / max(builds.value, 1)
            out["sort_ms"] = so_ms.value / max(builds.value, 1)
        lib.gsgpu_sim_set_force_timing(sim, 0)
        out["mean_force_ms"] = force_ms.value / max(force_n.value, 1)
        interactions = float(n) * (n - 1)
        out["interaction_cells"], out["interaction_pairs"] = 0.0, interactions
        if wk["method"] in BH_METHODS:
            cnt = (ctypes.c_longlong * 2)()
            lib.gsgpu_sim_interaction_counts(sim, cnt)
            interactions = float(cnt[0] + cnt[1])
            out["interaction_cells"], out["interaction_pairs"] = float(cnt[0]), float(cnt[1])
        out["interactions"] = interactions
        if wk["method"] == 104:
            rep = np.zeros(13)
            k = lib.gsgpu_sim_report(sim, rep.ctypes.data_as(dp), 13)
            rep = rep[:max(k, 0)].tolist()
            names = ["trained", "snapshots", "loss_first_epoch", "loss_last_epoch",
                     "heldout_median_residual_before", "heldout_median_residual_after",
                     "last_judged_median_err", "steps_judged", "steps_fallen_back",
                     "theta_cheap", "training_seconds", "adam_steps", "network_in_use"]
            out["learned_report"] = dict(zip(names, rep))
        a_host = np.empty((n, 3))
        torch.cuda.synchronize()
        assert lib.gsgpu_sim_download_acceleration(sim, a_host.ctypes.data_as(dp)) == 0
        xs = np.empty((n, 3))
        vs = np.empty((n, 3))
        lib.gsgpu_sim_download(sim, xs.ctypes.data_as(dp), vs.ctypes.data_as(dp))
    finally:
        lib.gsgpu_sim_destroy(sim)
    med, p99 = accuracy_sample(a_host, xs, m, wk["G"], wk["eps"], rows=acc_rows)
    out["median_rel_err"] = med
    out["p99_rel_err"] = p99
    out["xs"], out["vs"] = xs, vs
    # steps from the uploaded state to xs, vs: training, warm-up, timed, force-timing
    out["steps_run"] = out.get("training_steps", 0) + args.warmup + 2 * args.steps
    return out


def _arm_summary(wk, r, n):
    d = {"method": wk["method"], "theta": wk.get("theta"), "leaf": wk.get("leaf"),
         "ms_per_step": r["ms_per_step"], "particle_steps_per_s": n / (r["ms_per_step"] / 1e3),
         "median_rel_err": r["median_rel_err"], "p99_rel_err": r["p99_rel_err"],
         "walk_ms": r["mean_force_ms"], "interactions": r["interactions"]}
    if wk["method"] == 104:
        lr = r.get("learned_report", {})
        d.update({"policy": wk.get("policy", 0), "network_in_use": lr.get("network_in_use"),
                  "steps_judged": lr.get("steps_judged"),
                  "steps_fallen_back": lr.get("steps_fallen_back"),
                  "heldout_median_residual_before": lr.get("heldout_median_residual_before"),
                  "heldout_median_residual_after": lr.get("heldout_median_residual_after")})
    return d


def run_ours(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    g = _module("gsgpu")
    wl = _module("workloads")
    lib = g.load_c_lib()
    wk = WORKLOADS[args.workload]
    if wk["ic"] == "ensemble":
        return run_ensemble(args, world, rank, local, wk, g, wl, lib)
    if wk["ic"] == "cosmo":
        return run_cosmo(args, world, rank, local, wk, g, lib)
    n = wk["n"]
    x, v, m = (wl.plummer if wk["ic"] == "plummer" else wl.galaxy_pair)(n, wk["seed"])
    bh = wk["method"] in BH_METHODS
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    acc_rows = 4096 if bh else 512
    r = sim_arm(args, lib, g, wk, x, v, m, stream, flush, world, local, sample_clocks=True,
                acc_rows=acc_rows)
    value = world * n * args.steps / (r["total_ms"] / 1e3)
    interactions = r["interactions"]
    mean_force_ms = r["mean_force_ms"]
    # Algorithmic FLOP of one launch of the dominant kernel: 20 per pair
    # interaction (direct sum, leaf pair terms, monopole cells); a cell term
    # with its traceless quadrupole adds 36 (the contraction Q d, 15; d.Q.d,
    # 5; r^-5, r^-7 and the scale, 4; the two vector terms, 12): 56.
    quad_cells = wk["method"] in (104, 105, 106)
    flop_cell = FLOP_QUAD_CELL if quad_cells else wk["flop_per_interaction"]
    flop_launch = (wk["flop_per_interaction"] * r["interaction_pairs"]
                   + flop_cell * r["interaction_cells"])
    achieved_tflops = flop_launch / (mean_force_ms / 1e3) / 1e12
    achieved_20 = wk["flop_per_interaction"] * interactions / (mean_force_ms / 1e3) / 1e12
    fp64 = wk["method"] == 111   # the FP64 reference-order direct sum
    dp = ctypes.POINTER(ctypes.c_double)
    peak = ctypes.c_double()
    lib.gsgpu_measure_fma_peak(1 if fp64 else 0, ctypes.byref(peak), None)

    # the comparators of this workload, on the same GPU
    comparison = None
    if wk.get("compare"):
        comparison = {"this_line": _arm_summary(wk, r, n)}
        if wk["method"] == 104:
            comparison["this_line"]["training_s"] = r.get("training_s")
            comparison["this_line"]["network_in_use"] = bool(
                r.get("learned_report", {}).get("network_in_use", 0))
        for name, over in wk["compare"]:
            wc = dict(wk, **over)
            rc_ = sim_arm(args, lib, g, wc, x, v, m, stream, flush, world, local,
                          acc_rows=acc_rows)
            comparison[name] = _arm_summary(wc, rc_, n)
        plain = comparison.get(wk.get("plain_key"))
        if plain:
            comparison["this_over_plain_speed"] = (comparison["this_line"]["particle_steps_per_s"]
                                                  / plain["particle_steps_per_s"])

    energy = None
    if wk["ic"] == "plummer":
        # FP64 energies (unsoftened potential, src/utils.c:27-59) of the initial
        # state and of the state after the warm-up and timed steps, on the GPU
        state = np.zeros((2, n, 7))
        state[:, :, 0] = m
        state[0, :, 1:4], state[0, :, 4:7] = x, v
        state[1, :, 1:4], state[1, :, 4:7] = r["xs"], r["vs"]
        e = np.zeros(2)
        lib.compute_energy_python.argtypes = [dp, ctypes.c_double, dp, ctypes.c_int32,
                                              ctypes.c_int32]
        lib.compute_energy_python(e.ctypes.data_as(dp), ctypes.c_double(wk["G"]),
                                  np.ascontiguousarray(state).ctypes.data_as(dp), 2, n)
        energy = {"e0": float(e[0]), "e1": float(e[1]),
                  "rel_drift": float(abs(e[1] - e[0]) / abs(e[0])),
                  "steps": args.warmup + 2 * args.steps,
                  "note": "unsoftened potential while the force is softened (eps=0.01), "
                          "as the reference's compute_energy"}
    elif bh and "xs" in r:
        # softened energies (the force's own potential) of the initial state and
        # of the state after the warm-up and timed steps: the FP64 O(N^2) sum is
        # too slow at these sizes, so the pair terms are compensated FP32 on
        # double-float coordinates (gsgpu_softened_energy, ~1e-7 relative)
        lib.gsgpu_softened_energy.restype = ctypes.c_int
        lib.gsgpu_softened_energy.argtypes = [dp, dp, dp, ctypes.c_int, ctypes.c_double,
                                              ctypes.c_double, dp]
        e = np.zeros(2)
        for k, (xx, vv) in enumerate(((x, v), (r["xs"], r["vs"]))):
            xx, vv = np.ascontiguousarray(xx), np.ascontiguousarray(vv)
            ek = ctypes.c_double()
            if lib.gsgpu_softened_energy(xx.ctypes.data_as(dp), vv.ctypes.data_as(dp),
                                         m.ctypes.data_as(dp), n, wk["G"], wk["eps"],
                                         ctypes.byref(ek)) == 0:
                e[k] = ek.value
        if e[0] != 0.0:
            energy = {"e0": float(e[0]), "e1": float(e[1]),
                      "rel_drift": float(abs(e[1] - e[0]) / abs(e[0])),
                      "steps": r["steps_run"],
                      "note": "softened potential (the force's eps); pair terms in "
                              "compensated FP32 on double-float coordinates"}

    # end to end through the reference-facing entry point
    xe, ve, me = x.copy(), v.copy(), m.copy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g.launch_simulation(lib, xe, ve, me, wk["G"], integrator=wk["integrator"], dt=wk["dt"],
                        tf=wk["dt"] * args.steps * (1 - 1e-9), method=wk["method"],
                        opening_angle=wk.get("theta", 1.0), softening_length=wk["eps"],
                        max_num_particles_per_leaf=wk.get("leaf", -1))
    e2e_s, = max_over_ranks([time.perf_counter() - t0], world)
    e2e_val = world * n * args.steps / e2e_s

    kernel = ("k_bh_group" if wk["method"] in (104, 106, 107) else "k_bh_walk") if bh else \
        ("k_direct_fp64_reference_order" if fp64 else "k_direct_sum")
    traffic = profile_traffic(kernel, args.workload)
    l2_bytes = profile_traffic(kernel, args.workload, field="l2_bytes_per_launch")
    if bh:
        desc = (f"{args.workload}: galaxy pair N={n}, Barnes-Hut method {wk['method']} "
                f"theta={wk['theta']} leaf={wk['leaf']}, eps={wk['eps']}, leapfrog dt={wk['dt']}")
        if wk["method"] == 104:
            desc += (" (theta=1.0 group walk + learned residual, judged by a 4096-particle "
                     "direct sum per step, theta=0.5 group walk as fallback; a network that "
                     "did not earn its place leaves the fallback walk alone)")
        data = "synthetic (seeded two-galaxy model: exponential disk, Hernquist bulge and halo)"
        dtype = "f32 walk terms (Kahan), f64 tree multipoles and state"
    elif fp64:
        desc = (f"{args.workload}: Plummer N={n}, FP64 direct sum in the reference's order "
                f"(bit-exact), eps={wk['eps']}, leapfrog dt={wk['dt']}")
        data = "synthetic (seeded Plummer sphere)"
        dtype = "f64"
    else:
        desc = (f"{args.workload}: Plummer N={n}, compensated-FP32 direct sum, "
                f"eps={wk['eps']}, leapfrog dt={wk['dt']}")
        data = "synthetic (seeded Plummer sphere)"
        dtype = "f32 pair terms (Kahan), f64 state"

    out = {
        "metric": METRIC,
        "value": value,
        "unit": "particle-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": r["total_ms"] / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": dtype,
        "data": data,
        "config": {"workload": desc,
                   "parallelism": f"replicas x{world}", "l2": "flushed between steps (256 MiB write)",
                   "interactions_per_s": value / n * interactions,
                   "accuracy": {"median_rel_err": r["median_rel_err"],
                                "p99_rel_err": r["p99_rel_err"],
                                "sample": f"{acc_rows} particles vs FP64 direct sum"},
                   "energy": energy},
        "roofline": {"bound": "fp64" if fp64 else "fp32", "achieved": achieved_tflops,
                     "peak": peak.value,
                     "unit": "TFLOP/s", "frac": achieved_tflops / peak.value if peak.value else None,
                     "traffic": traffic,
                     "kernel": kernel, "mean_launch_ms": mean_force_ms,
                     "peak_source": ("FP64" if fp64 else "FP32") + " FMA probe on this GPU "
                                    "(gsgpu_measure_fma_peak), not in MEASURED_PEAKS.json",
                     "flop_per_interaction": {"pair": wk["flop_per_interaction"],
                                              "cell": flop_cell},
                     "interactions_per_launch": {"cells": r["interaction_cells"],
                                                 "pairs": r["interaction_pairs"]},
                     "achieved_at_20_flop_per_interaction": achieved_20,
                     "l2": ({"bytes_per_launch": l2_bytes,
                             "achieved_gbs": l2_bytes / (mean_force_ms * 1e6),
                             "source": "lts__t_bytes.sum of one launch (profiles/)"}
                            if l2_bytes and mean_force_ms else None)},
        "e2e": {"value": e2e_val, "unit": "particle-steps/s",
                "h2d_bytes_per_step": (7 * n * 8) / args.steps,
                "d2h_bytes_per_step": (6 * n * 8) / args.steps,
                "note": "one launch_simulation_python call of K steps; its copies and setup "
                        "amortised over the K steps"},
        "gpu_launches": args.steps * r["kernels_per_step"],
        "clocks": r.get("clocks"),
        "wall_s": r["wall_s"],
    }
    if bh:
        out["config"]["interactions"] = "accepted cells + leaf pair terms of the last step "\
                                        "(device counters); FLOP per term in roofline"
        # Tree build against HBM: algorithmic bytes per particle of the Morton
        # keys (24 B of positions read, 8 B of key written) and of the key
        # sort (grav_sim's 7 radix passes of 9 bits, each reading and writing
        # an 8 B key and a 4 B index: 168 B), over the kernels' event times.
        hbm = measured_peaks().get("hbm_gbs")
        mo_gbs = 32.0 * n / (r["morton_ms"] / 1e3) / 1e9 if r.get("morton_ms") else None
        so_gbs = 168.0 * n / (r["sort_ms"] / 1e3) / 1e9 if r.get("sort_ms") else None
        out["roofline"]["tree_build"] = {
            "bound": "hbm", "unit": "GB/s", "peak": hbm,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs",
            "morton": {"ms": r.get("morton_ms"), "achieved": mo_gbs,
                       "frac": mo_gbs / hbm if mo_gbs and hbm else None,
                       "bytes_per_particle": 32},
            "sort": {"ms": r.get("sort_ms"), "achieved": so_gbs,
                     "frac": so_gbs / hbm if so_gbs and hbm else None,
                     "bytes_per_particle": 168}}
    if wk["method"] == 104:
        out["config"]["training_s"] = r.get("training_s")
        out["config"]["learned_report"] = r.get("learned_report")
        out["e2e"]["note"] += ("; with method 104 a leapfrog call of at most 252 steps ends "
                               "before its network could be trained (after the 64th "
                               "65,536-row snapshot, the 253rd force evaluation) and applied, "
                               "so it skips the collection: every step is the fallback walk")
    if comparison:
        out["config"]["comparison"] = comparison
    if rank == 0:
        if wk["ic"] == "plummer":
            out["cpu_baseline"] = cpu_baseline_pairwise(wk, x, m)
        else:
            out["cpu_baseline"] = cpu_baseline_bh(wk, x, m)
        print(json.dumps(out), flush=True)


def cpu_baseline_ensemble(wk, systems, target_s=10.0, sample_systems=128):
    """The reference's per-system loop (oracle restatement of WHFast or
    leapfrog with the massless acceleration) on a stratified sample of the
    systems -- every (S / sample)-th system in order of size -- one system
    per OpenMP thread (the fair-share baseline of one system per core),
    for a number of steps sized to about target_s seconds."""
    sys.path.insert(0, str(ROOT))
    from oracle import restatement as orc
    G = _module("workloads").G_AU_MSUN_DAY
    order = np.argsort([s_[2].size for s_ in systems], kind="stable")
    pick = order[np.linspace(0, len(systems) - 1, min(sample_systems, len(systems))).astype(int)]
    sample = [systems[i] for i in pick]
    P = int(sum(s_[2].size for s_ in sample))
    steps = 4
    el, threads = orc.ensemble_cpu_timing(sample, G, wk["dt"], steps, wk["integrator"])
    steps = max(4, min(10000, int(steps * target_s / max(el, 1e-3))))
    el, threads = orc.ensemble_cpu_timing(sample, G, wk["dt"], steps, wk["integrator"])
    name = "WHFast" if wk["integrator"] == 10 else "leapfrog"
    return {"value": P * steps / el, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"grav_sim {name} + massless acceleration, each system alone as "
                      f"launch_simulation_python runs it: {len(sample)} of {len(systems)} systems "
                      f"stratified by size ({P} particles), {steps} steps each, {el:.1f} s on "
                      f"{threads} threads (one system per thread); particle-steps/s of the "
                      f"sample, whose size distribution is the ensemble's"}


def reference_ensemble(args, wk, wl):
    systems = wl.planetary_ensemble(wk["systems"], wk["seed"], max_test=wk["max_test"])
    for _ in range(args.warmup):
        cpu_baseline_ensemble(wk, systems, target_s=0.5)
    vals = [cpu_baseline_ensemble(wk, systems, target_s=3.0) for _ in range(args.steps)]
    value = statistics.median(r["value"] for r in vals)
    P = int(sum(s_[2].size for s_ in systems))
    name = "WHFast" if wk["integrator"] == 10 else "leapfrog"
    return {"value": value, "ms_per_step": 1e3 * P / value,
            "data": "synthetic (seeded planetary systems)",
            "config": {"workload": f"{args.workload}: {wk['systems']} systems, {P} particles, "
                                   f"grav_sim {name} + massless accelerations, dt={wk['dt']} day"},
            "cpu_baseline": {"value": value, "unit": "particle-steps/s",
                             "cores": vals[-1]["cores"], "kind": "port",
                             "sample": vals[-1]["sample"]},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def run_ensemble(args, world, rank, local, wk, g, wl, lib):
    """Batched planetary ensembles: every phase of a step is one launch over
    all systems; a step is captured in a CUDA graph and replayed."""
    import torch
    systems = wl.planetary_ensemble(wk["systems"], wk["seed"], max_test=wk["max_test"])
    counts = np.array([s_[2].size for s_ in systems], dtype=np.int32)
    ids = np.concatenate([np.arange(c, dtype=np.int32) for c in counts])
    x = np.concatenate([s_[0] for s_ in systems])
    v = np.concatenate([s_[1] for s_ in systems])
    m = np.concatenate([s_[2] for s_ in systems])
    P = int(counts.sum())
    G = wl.G_AU_MSUN_DAY
    ens = g.Ensemble(lib, counts, G, integrator=wk["integrator"], method=wk["method"], dt=wk["dt"])
    ens.upload(ids, x, v, m)
    ens.run(args.warmup)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    torch.cuda.profiler.start()   # the timed steps are the profiler range
    t0 = time.perf_counter()
    ens.run(args.steps)
    torch.cuda.synchronize()
    total_s = time.perf_counter() - t0
    torch.cuda.profiler.stop()
    clk = clocks.stop()
    total_s, = max_over_ranks([total_s], world)
    kps = ens.kernels_per_step()
    accel_tpb, drift_tpb = ens.tuning()
    tuning = {"accel_threads_per_block": accel_tpb, "drift_threads_per_block": drift_tpb,
              "sort_threads_per_system": [{"class_capacity": c, "threads": t}
                                          for c, t in ens.sort_tuning()]}
    # the acceleration kernels' own time, for the roofline: K more steps
    # launched directly with CUDA events around them (outside the timed region)
    ens.set_kernel_timing(True)
    ens.run(args.steps)
    torch.cuda.synchronize()
    drift_ms, accel_ms, timed = ens.kernel_timing()
    ens.set_kernel_timing(False)
    ens.close()
    # Algorithmic work of one acceleration step, at 20 FLOP per pair term:
    # WHFast (src/integrator_whfast.c:959-1264) gives every particle but the
    # primary its M - 1 interior / exterior massive terms and its 2 primary
    # terms, and each system its M (M - 1) / 2 massive pair terms (summed once
    # per system here); leapfrog's massless acceleration
    # (src/acceleration.c:236-367) has L M + M (M - 1) / 2 terms per system
    # (M massive bodies, L massless particles).
    terms = 0
    for s_ in systems:
        n_s = s_[2].size
        M = int(np.count_nonzero(s_[2]))
        if wk["integrator"] == 10:
            terms += (n_s - 1) * (M + 1) + M * (M - 1) // 2
        else:
            terms += (n_s - M) * M + M * (M - 1) // 2
    lib.gsgpu_measure_fma_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double)]
    peak64 = ctypes.c_double()
    lib.gsgpu_measure_fma_peak(1, ctypes.byref(peak64), None)
    accel_launch_ms = accel_ms / max(timed, 1)
    achieved = 20.0 * terms / (accel_launch_ms / 1e3) / 1e12
    value = world * P * args.steps / total_s
    # end to end: launch, upload, K steps, download through the ensemble API
    t0 = time.perf_counter()
    e2 = g.Ensemble(lib, counts, G, integrator=wk["integrator"], method=wk["method"], dt=wk["dt"])
    e2.upload(ids, x, v, m)
    e2.run(args.steps)
    e2.download()
    e2e_s, = max_over_ranks([time.perf_counter() - t0], world)
    e2.close()
    name = "WHFast" if wk["integrator"] == 10 else "leapfrog"
    out = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded planetary systems)",
        "config": {"workload": f"{args.workload}: {wk['systems']} systems, {P} particles, "
                               f"{name} + massless accelerations, dt={wk['dt']} day",
                   "parallelism": f"replicas x{world}",
                   "l2": f"working set {P * 250 / 2**20:.0f} MiB > L2",
                   "accuracy": "bit-exact to the reference per system (tests/test_gpu_ensemble.py)",
                   "timing": "host clock around K graph replays with device synchronisation",
                   "autotune": tuning},
        "e2e": {"value": world * P * args.steps / e2e_s, "unit": "particle-steps/s",
                "h2d_bytes_per_step": (P * 60) / args.steps,
                "d2h_bytes_per_step": (P * 60) / args.steps,
                "note": "create + upload + K steps + download through gsgpu_ensemble_*"},
        "gpu_launches": args.steps * kps,
        "clocks": clk,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64.value,
                     "unit": "TFLOP/s", "frac": achieved / peak64.value if peak64.value else None,
                     "traffic": profile_traffic("k_wh_accel", args.workload,
                                                "ensemble_whfast_" + args.workload)
                                if wk["integrator"] == 10 else None,
                     "kernel": "k_wh_pairs + k_wh_accel" if wk["integrator"] == 10
                               else "k_ens_massless_accel",
                     "mean_launch_ms": accel_launch_ms, "pair_terms_per_step": terms,
                     "flop_per_pair_term": 20,
                     "drift_ms_per_step": drift_ms / max(timed, 1) if wk["integrator"] == 10
                                          else None,
                     "peak_source": "FP64 FMA probe on this GPU (gsgpu_measure_fma_peak), "
                                    "not in MEASURED_PEAKS.json",
                     "note": "every pair term holds three correctly rounded FP64 divisions and a "
                             "square root (bit-exact to the reference), which the 20-FLOP "
                             "convention counts as single operations"},
    }
    if rank == 0:
        out["cpu_baseline"] = cpu_baseline_ensemble(wk, systems)
        print(json.dumps(out), flush=True)


def run_cosmo(args, world, rank, local, wk, g, lib):
    """Cosmological particle-mesh run through launch_cosmological_simulation:
    value from the device time of the step loop (CUDA events on the
    library's stream), e2e from the wall time of the whole call (host->device
    copies, allocation, K steps, device->host copy of x)."""
    import torch
    n, grid, bw = wk["n"], wk["grid"], wk["box_width"]
    rng = np.random.default_rng(wk["seed"])
    side = round(n ** (1.0 / 3.0))
    spacing = 2.0 * bw / side
    centre = np.zeros(3)
    lattice = np.indices((side, side, side)).reshape(3, -1).T.astype(np.float64)
    x = np.ascontiguousarray(centre - bw + (lattice + 0.5 + rng.uniform(-0.3, 0.3, (n, 3)))
                             * spacing)
    v = np.ascontiguousarray(rng.normal(0.0, 5.0, (n, 3)))
    m = np.ones(n)
    del lattice
    kw = dict(h=wk["h"], omega_m=wk["omega_m"], omega_lambda=wk["omega_lambda"],
              box_center=centre, box_width=bw, dt=wk["da"], a_begin=wk["a_begin"],
              pm_grid_size=grid)
    lib.gsgpu_cosmology_last_timing.argtypes = [ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_int64),
                                                ctypes.POINTER(ctypes.c_int)]
    xw = x.copy()
    g.launch_cosmological_simulation(lib, xw, v.copy(), m,
                                     a_final=wk["a_begin"] + args.warmup * wk["da"], **kw)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    clocks.start()
    time.sleep(0.3)
    xt = x.copy()
    t0 = time.perf_counter()
    st = g.launch_cosmological_simulation(lib, xt, v.copy(), m,
                                          a_final=wk["a_begin"] + args.steps * wk["da"], **kw)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    loop_ms, steps, kps = ctypes.c_double(), ctypes.c_int64(), ctypes.c_int()
    assert lib.gsgpu_cosmology_last_timing(ctypes.byref(loop_ms), ctypes.byref(steps),
                                           ctypes.byref(kps)) == 0
    assert steps.value == args.steps == st.num_steps, (steps.value, st.num_steps)
    dev_s = loop_ms.value / 1e3
    dev_s, wall = max_over_ranks([dev_s, wall], world)
    # The step is bound by the FP64 pipe (1/64 of the FP32 rate on this GPU).
    # Algorithmic FP64 work per step (an FMA counts 2): per particle the two
    # cloud-in-cell weight sets (2 x 15), the deposit products (14), the
    # interpolation (8 products + 24 FMA = 56), two kicks and the drift
    # (3 x 6) = 118; per mesh cell the contrast (2), the gradient (15) and the
    # Green's function (~3) = 20; the r2c and c2r transforms 2.5 N log2 N each.
    cells = grid ** 3
    flop_step = 118.0 * n + 20.0 * cells + 2 * 2.5 * cells * math.log2(cells)
    lib.gsgpu_measure_fma_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double)]
    peak64 = ctypes.c_double()
    lib.gsgpu_measure_fma_peak(1, ctypes.byref(peak64), None)
    achieved = flop_step / (dev_s / args.steps) / 1e12
    out = {
        "metric": METRIC, "value": world * n * args.steps / dev_s, "unit": "particle-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded perturbed lattice)",
        "config": {"workload": f"{args.workload}: {n} particles, {grid}^3 mesh, periodic box "
                               f"width {2 * bw}, a from {wk['a_begin']} in steps of {wk['da']}",
                   "parallelism": f"replicas x{world}",
                   "l2": f"inputs larger than L2 ({n * 24 / 2**20:.0f} MiB of positions, "
                         f"{grid ** 3 * 56 / 2**20:.0f} MiB of meshes)",
                   "accuracy": "within 1e-10 of the largest acceleration of the reference's "
                               "particle-mesh code (tests/test_gpu_pm.py)"},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64.value,
                     "unit": "TFLOP/s", "frac": achieved / peak64.value, "traffic": None,
                     "kernel": "whole step (8 kernels + 2 cuFFT transforms)",
                     "algorithmic_flop_per_step": flop_step,
                     "peak_source": "FP64 FMA probe on this GPU (gsgpu_measure_fma_peak), "
                                    "not in MEASURED_PEAKS.json"},
        "e2e": {"value": world * n * args.steps / wall, "unit": "particle-steps/s",
                "h2d_bytes_per_step": n * 56 / args.steps, "d2h_bytes_per_step": n * 24 / args.steps,
                "note": "one launch_cosmological_simulation call of K steps"},
        "gpu_launches": args.steps * kps.value,
        "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_reference(args, world, rank, local):
    """The reference's CPU implementation of the workload's path (the
    oracle's restatement of grav_sim, built on this machine), on the host
    cores, each step a bounded sample of the workload extrapolated to a
    full step.  Rank 0 alone runs it."""
    if rank != 0:
        return
    wl = _module("workloads")
    wk = WORKLOADS[args.workload]
    base = {"metric": METRIC, "unit": "particle-steps/s", "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64"}
    if wk["ic"] == "ensemble":
        out = dict(base, **reference_ensemble(args, wk, wl))
        print(json.dumps(out), flush=True)
        return
    if wk["ic"] == "cosmo":
        print(json.dumps({"impl": "reference", "unavailable":
                          "the reference's particle-mesh path needs FFTW 3, absent on this "
                          "machine; its restatement runs a direct DFT, far too slow for a "
                          "256^3 mesh"}), flush=True)
        return
    if wk["ic"] == "plummer":
        x, v, m = wl.plummer(wk["n"], wk["seed"])
        for _ in range(args.warmup):
            cpu_baseline_pairwise(wk, x, m, target_s=1.0)
        vals = [cpu_baseline_pairwise(wk, x, m, target_s=4.0) for _ in range(args.steps)]
        desc = (f"{args.workload}: Plummer N={wk['n']}, grav_sim pairwise "
                f"(acceleration.c:177-234) + leapfrog dt={wk['dt']}")
        data = "synthetic (seeded Plummer sphere)"
        cores = 1
    else:
        x, v, m = wl.galaxy_pair(wk["n"], wk["seed"])
        for _ in range(args.warmup):
            cpu_baseline_bh(wk, x, m, target_s=0.5)
        vals = [cpu_baseline_bh(wk, x, m, target_s=3.0) for _ in range(args.steps)]
        desc = (f"{args.workload}: galaxy pair N={wk['n']}, grav_sim Barnes-Hut "
                f"(acceleration_barnes_hut.c:33-248, linear_octree.c) theta={CPU_BH_THETA} "
                f"leaf={CPU_BH_LEAF}, eps={wk['eps']}, leapfrog dt={wk['dt']}")
        data = "synthetic (seeded two-galaxy model: exponential disk, Hernquist bulge and halo)"
        cores = vals[-1]["cores"]
    value = statistics.median(r["value"] for r in vals)
    out = dict(base, **{
        "value": value, "ms_per_step": 1e3 * wk["n"] / value, "data": data,
        "config": {"workload": desc},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores,
                         "kind": "port", "sample": vals[-1]["sample"]},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    })
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="galaxy1048576_learned", choices=sorted(WORKLOADS))
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, local)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    try:
        run_ours(args, world, rank, local)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
