#!/usr/bin/env python3
"""PBF step benchmark on GB300: 1M-particle dam-break steps per second.

One step = AkuaEngine's PBFSolver::step over the attached 108-byte particle records: predict, hash,
sort, neighbour lists, 4 Jacobi iterations (density, lambda, delta with artificial pressure,
correct + clamp), update, boundary damping, vorticity confinement, XSPH, written back into the
records in hash order.  Workload: 100x100x100 lattice block at spacing 0.5h with seeded jitter of
+-0.01h in a box 3 x 1.5 x 1.5 block widths, dt 0.0083, seeded synthetic data.

  python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference]

Under torchrun each rank steps its own replica of the scene (no data exchange: replicas only) and
rank 0 prints one JSON line.  `--impl reference` times the reference algorithm's CPU restatement
(the oracle; the reference's own code is GPU-only and cannot run on host cores) with all host
threads, on rank 0 only.
"""
from __future__ import annotations

import argparse
import csv
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "1M-particle PBF steps/s"
# per workload: metric name, lattice block(s), box in block widths
WORKLOADS = {
    "dam_break_27k": ("27k-particle PBF steps/s", [30, 30, 30], [4.0, 4.0, 4.0]),
    "dam_break_1m": (METRIC, [100, 100, 100], [3.0, 1.5, 1.5]),
    "double_dam_break_8m": ("8M-particle PBF steps/s", [[200, 100, 200], [200, 100, 200]],
                            [6.0, 2.0, 2.0]),
}
UNIT = "steps/s"
WORKLOAD = "dam_break_1m"

# Algorithmic bytes per particle moved by each kernel: the compulsory traffic of the SoA design,
# every array a kernel reads or writes counted once per particle; neighbour positions gathered
# through the lists are assumed cache-served and not counted, the lists themselves are.  `L` is
# the mean bytes of one particle's list tiles (16 * ceil(count / 4)), `B` the mean number of bucket
# table entries per particle (one 8-byte entry per occupied bucket), both taken from the run.
KERNEL_BYTES = {
    # R record 108; W x|m, v, colour, size, rank, hash key and Morton key with their payloads
    "k_import": lambda L, B: 108 + 16 + 16 + 16 + 4 + 4 + 16,
    # R x|m, v, rank; W hash key, index, Morton key
    "k_keys": lambda L, B: 16 + 16 + 4 + 16,
    "radix_upsweep": lambda L, B: 4,                  # R key (per pass)
    "radix_downsweep": lambda L, B: 16,               # R key, value; W key, value (per pass)
    # R two permutations, x|m, v, colour, size, old rank; W x|m, colour, size, x*|m, rank->slot,
    # slot->rank, reference-ordered x*|m, order
    "k_gather": lambda L, B: 8 + 16 + 16 + 16 + 4 + 4 + 16 + 16 + 4 + 16 + 4 + 4 + 16 + 4,
    "k_table_build": lambda L, B: 4 + 4 + 8 * B,      # R keys, slots; W entry
    # R x*|m, 27 bucket entries per cell run; W lists, count, rho, lambda, x*|lambda
    "k_search": lambda L, B: 16 + 27 * 8 * B + L + 4 + 8 + 16,
    # R x*|m, count, lists; W rho, lambda, x*|lambda
    "k_density_lambda": lambda L, B: 16 + 4 + L + 8 + 16,
    # R x*|m, lambda, count, lists; W x*|m, delta
    "k_delta_correct": lambda L, B: 16 + 4 + 4 + L + 16 + 16,
    # R x*|m, lambda, count, lists, x|m, colour, size, rank; W x, v, v*, delta, colour, size, rank,
    # record (x|m, v)
    "k_delta_final": lambda L, B: 16 + 4 + 4 + L + 16 + 16 + 4 + 4 + 16 * 4 + 16 + 4 + 4 + 32,
    "k_vorticity": lambda L, B: 16 + 16 + 4 + L + 16 + 16,   # R x, v, count, lists; W omega, x|omega
    # R x, v, omega, rho, count, lists; W record (x|m/rho, v)
    "k_confine": lambda L, B: 16 + 16 + 16 + 4 + 4 + L + 32,
    # R record, count, lists, keys; W v, emptied bucket entries
    "k_xsph": lambda L, B: 32 + 4 + L + 16 + 4 + 8 * B,
    # R slot, key, x, v, v*, delta, omega, colour, rho, lambda, size; W record 108
    "k_export": lambda L, B: 4 + 4 + 16 * 6 + 4 + 4 + 4 + 108,
}


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--profile-steps", type=int, default=10)
    ap.add_argument("--preroll", type=int, default=240,
                    help="untimed steps before warm-up: the timed window then lies in the middle "
                         "of the workload's 500-step run (developed flow), not at rest")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip timing the reference's own kernels (baseline leg)")
    ap.add_argument("--pair-blocks", default=None,
                    help="six comma-separated block sizes of the pair kernels instead of the "
                         "autotuner's choice (profiling runs)")
    ap.add_argument("--search-shape", default=None,
                    help="the walk's block size and staged entries, e.g. 128,32 (with "
                         "--pair-blocks: profiling runs; default: the autotuner's choice)")
    ap.add_argument("--table-size", type=int, default=None,
                    help="hash table buckets (default: the reference's maxNeighbours * N)")
    ap.add_argument("--resident", action="store_true",
                    help="records read only on the first step (the key kernel replaces the import "
                         "on later steps)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--exact", action="store_true", help="IEEE math in pair terms")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned warm-start comparison")
    ap.add_argument("--learned-iterations", type=int, default=2)
    return ap.parse_args(argv)


def dist_env():
    from akuaengine_gb300 import replicas

    e = replicas.dist_env()
    return e.world, e.rank, e.local_rank


SM_COUNT = 152
FP32_PEAK_TFLOPS = round(SM_COUNT * 128 * 2 * 2.07e9 / 1e12, 1)  # nominal: no FP32 peak is measured


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = None

    def start(self):
        try:
            self.out = open(self._path(), "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def _path(self):
        # the raw samples: AKUA_BENCH_CLOCKS_DIR when set, else the temporary directory
        d = os.environ.get("AKUA_BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        return os.path.join(d, "bench_clocks_%d_%d.csv" % (self.device, os.getpid()))

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.out.close()
        rows = []
        with open(self._path()) as f:
            for r in csv.reader(f):
                if len(r) >= 9:
                    rows.append([x.strip() for x in r])
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "", 1).isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------------- oracle arm
def time_oracle(sc, cfg, corr, steps, budget_s, threads=0, table_size=None):
    """Times the CPU restatement on `steps` steps, on a sub-block when the full scene would take
    longer than `budget_s`.  Returns (steps/s at full size, cores, sample description)."""
    import numpy as np

    import oracle

    P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=sc.n, num_threads=threads,
                           table_size=table_size)
    cores = threads if threads > 0 else oracle.max_threads()
    p = sc.particles.copy()
    t0 = time.perf_counter()
    oracle.step(p, P)
    t1 = time.perf_counter() - t0
    n_sample = sc.n
    parts = p
    if t1 * steps > budget_s:
        frac = max(budget_s / (t1 * steps), 0.02)
        n_sample = max(int(sc.n * frac), 4096)
        parts = p[:n_sample].copy()  # a contiguous slab of the hash-sorted particle set
        P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=n_sample,
                               num_threads=threads,
                               table_size=None if table_size is None else
                               max(1, int(table_size * n_sample / sc.n)))
        oracle.step(parts, P)
    t0 = time.perf_counter()
    for _ in range(steps):
        oracle.step(parts, P)
    el = time.perf_counter() - t0
    psps = n_sample * steps / el
    sample = "%d steps of %d particles%s (%.1f s)" % (
        steps, n_sample, "" if n_sample == sc.n else " (first particles of the sorted scene)", el)
    return psps / sc.n, psps, cores, sample


def step_error_vs_fp64(solver, sc, cfg, corr, table_size=None):
    """One fast-math GPU step of the scene's state against the same step of the restatement in
    FP64 and in FP32 (the checker; outside every timed region): per-particle position error
    quantiles, so the GPU's error is read against the FP32 arithmetic's own."""
    import numpy as np

    import oracle

    gpu = sc.particles.copy()
    solver.step_host(gpu, sc.dt, sc.box_min, sc.box_max)
    out = {}
    for name, flags in (("fp32_oracle", oracle.FMA), ("fp64_oracle", oracle.FMA | oracle.FP64)):
        p = sc.particles.copy()
        oracle.step(p, oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=sc.n,
                                          flags=flags, table_size=table_size))
        out[name] = p
    def q(a, b):
        d = np.abs(a["position"].astype(np.float64) - b["position"]).max(axis=1)
        return {"p50": float(np.quantile(d, 0.5)), "p99": float(np.quantile(d, 0.99)),
                "max": float(d.max())}
    return {"gpu_fast_vs_fp64": q(gpu, out["fp64_oracle"]),
            "fp32_oracle_vs_fp64": q(out["fp32_oracle"], out["fp64_oracle"]),
            "gpu_fast_vs_fp32_oracle": q(gpu, out["fp32_oracle"]),
            "what": "position error after one step of the timed window's state, per particle "
                    "max over x, y, z"}


def time_reference_gpu(sc, cfg, corr, value, e2e, table_size=None):
    """The reference's unchanged CUDA kernels (compiled from its sources into cubins, driven by a
    re-sequenced PBFSolver::step) on this GPU and the same state: the faithful form (host-resident
    neighbour lists, per-step table allocation, as the reference's wrappers do) and the form with
    device-resident lists.  A baseline leg; returns None-valued entries with the reason when the
    cubins are absent."""
    try:
        from oracle import ref_gpu
        sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
        from make_ref_gpu_golden import params
    except Exception as exc:  # noqa: BLE001
        return {"unavailable": "reference harness not importable: %s" % exc}
    if not ref_gpu.have_cubins():
        return {"unavailable": "the reference's kernels were not compiled (oracle/_ref)"}
    out = {"unit": UNIT}
    sampler = ClockSampler(0)
    sampler.start()
    try:
        for mode, steps in (("faithful", 10), ("resident", 20)):
            p = sc.particles.copy()
            pr = params(cfg, corr, sc, sc.n)
            if table_size:
                pr["table"] = int(table_size)
            pr["warmup"] = 1
            info = ref_gpu.run(p, pr, steps, mode=mode)
            v = 1000.0 / info["ms_per_step"]
            out[mode] = {"steps_per_s": round(v, 3), "ms_per_step": round(info["ms_per_step"], 3),
                         "steps": steps, "ours_over_reference": round(value / v, 2)}
            if e2e:
                out[mode]["ours_e2e_over_reference"] = round(e2e["value"] / v, 2)
    except Exception as exc:  # noqa: BLE001
        out["unavailable"] = "reference harness failed: %s" % str(exc)[:200]
    out["clocks"] = sampler.stop()
    out["note"] = ("faithful = the reference's wrappers' traffic (host neighbour arrays copied "
                   "per wrapper, table allocated and filled per step); resident = the same kernels "
                   "with lists kept on the device")
    return out


def run_reference(args, sc, cfg, corr):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    budget = 150.0
    per_step_budget = budget / max(args.steps, 1)
    # warm-up: W steps of a small sample (the oracle has no caches to warm beyond the first call)
    sps, psps, cores, sample = time_oracle(sc, cfg, corr, args.steps, budget,
                                           table_size=args.table_size)
    line = {
        "impl": "reference", "metric": WORKLOADS[args.workload][0], "value": sps, "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / sps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded lattice + jitter)",
        "config": {"workload": args.workload, "particles": sc.n, "solver_iterations": 4,
                   "dt": sc.dt, "hardware": "host CPU cores", "per_step_budget_s": per_step_budget},
        "cpu_baseline": {"value": sps, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample, "particle_steps_per_s": psps,
                         "precision": "fp32: the reference's arithmetic and contractions, "
                                      "restated for the host (OpenMP over particles)",
                         "state": "the workload's initial state (the GPU arm's pre-roll into the "
                                  "developed flow would take minutes on the host cores)"},
        "e2e": {"value": sps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's step is CUDA-only; its algorithm restated on the CPU is timed",
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------------- learned
def _family(cfg, seed, count):
    """The `count` largest dam breaks of a batched-family draw (config 3's scene distribution),
    each with its own gravity."""
    import numpy as np

    from akuaengine_gb300 import PBFConfig, scene

    batch = scene.batched_dam_breaks(count=256, seed=seed)
    order = np.argsort([-d["numParticles"] for d in batch.scenes])[:count]
    return [(batch.scene(int(k)),
             PBFConfig(**{**cfg.__dict__, "gravity": tuple(batch.scenes[int(k)]["gravity"])}))
            for k in order]


def run_learned(args, sc, cfg, corr, stream, plain_value, plain_ms, sc_timed=None):
    """Learned warm start against the plain 4-iteration step at equal max density error.  Training
    pairs come from a differently seeded copy of the workload and from dam breaks of the batched
    family (other block shapes, boxes and gravities).  For k = 1, 2, 3 warm-started iterations
    (fewest first) a network is trained on a teacher of 4 - k + 1 plain iterations (the learned
    first iteration stands in for the iterations it saves) and its blend is calibrated on the
    training scenes with zero tolerance against the plain solver's max error on each; the first k
    that reaches it is the equal-error result.  Reported beside it: the k = 3 network timed and
    evaluated whether or not it qualified.  Steps are device-timed like the main line, from the
    same state; errors come from scenes not trained on (the benchmark scene, and a batched-family
    scene of another draw)."""
    import numpy as np
    import torch

    from akuaengine_gb300 import PBFSolver, scene
    from akuaengine_gb300.warm_start import fewest_iterations_at_equal_error, rollout_errors

    t0 = time.perf_counter()
    train_scenes = [(scene.workload(args.workload, seed=1), cfg)] + _family(cfg, 3, 4)
    plain_it = cfg.solverIterations
    steps = 60
    k, net, report = fewest_iterations_at_equal_error(
        train_scenes, corr, plain_iterations=plain_it, candidates=(1, 2, 3), steps=steps,
        stream=stream, collect={"steps": 123, "capture_every": 40, "first_capture": 2},
        keep_last=True)
    last = report.pop("last", None)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    timed = sc_timed if sc_timed is not None else sc

    def time_solver(iterations, network):
        solver = PBFSolver(sc.n, cfg, corr, stream=stream)
        solver.set_solver_iterations(iterations)
        if network is not None:
            solver.set_warm_start(network)
        buf = torch.from_numpy(timed.particles.view(np.uint8).copy()).cuda()
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                solver.step(buf, sc.dt, sc.box_min, sc.box_max)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            solver.step(buf, sc.dt, sc.box_min, sc.box_max)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        launches = solver.kernels_per_step()
        solver.profile_begin(3)
        for _ in range(3):
            solver.step(buf, sc.dt, sc.box_min, sc.box_max)
        prof = solver.profile_end()
        solver.close()
        return args.steps / (ms / 1000.0), ms / args.steps, launches, prof

    evals = {"benchmark_scene_seed0": (sc, cfg), "batched_family_scene": _family(cfg, 7, 1)[0]}

    def accuracy(iterations, network):
        out = {}
        for name, (esc, ecfg) in evals.items():
            e_plain = rollout_errors(esc, ecfg, corr, plain_it, None, steps, stream)
            e_warm = rollout_errors(esc, ecfg, corr, iterations, network, steps, stream)
            e_same = rollout_errors(esc, ecfg, corr, iterations, None, steps, stream)
            out[name] = {
                "particles": int(esc.n),
                "warm": {"max": round(float(e_warm[:, 0].mean()), 5),
                         "mean_abs": round(float(e_warm[:, 1].mean()), 5)},
                "plain": {"max": round(float(e_plain[:, 0].mean()), 5),
                          "mean_abs": round(float(e_plain[:, 1].mean()), 5)},
                "plain_same_iterations": {"max": round(float(e_same[:, 0].mean()), 5),
                                          "mean_abs": round(float(e_same[:, 1].mean()), 5)},
                "warm_max_within_plain": bool(e_warm[:, 0].mean() <= e_plain[:, 0].mean())}
        return out

    value, ms, launches, prof = time_solver(k, net)
    result = {
        "method": "iteration 1 uses lambda0 + blend * (network estimate - lambda0), then plain "
                  "Jacobi iterations; the fewest iterations (of 1, 2, 3) whose calibrated blend "
                  "keeps the max density error at or below the plain solver's on the calibration "
                  "scene (zero tolerance)",
        "warm_iterations": k, "plain_iterations": plain_it, "network": net is not None,
        "steps_per_s": round(value, 2), "ms_per_step": round(ms, 4),
        "speedup_vs_plain": round(value / plain_value, 4),
        "gpu_launches_per_step": launches,
        "training": {"scenes": ["%s (%d particles)" % (t.name, t.n) for t, _ in train_scenes],
                     "calibration": "zero tolerance against the plain solver's max error on every "
                                    "training scene",
                     "rollout_steps": steps, **report},
        "density_error": {
            "rollout_steps": steps, "scenes": accuracy(k, net),
            "definition": "per step: max_i max(rho_i/rho0 - 1, 0) and mean_i |rho_i/rho0 - 1| at "
                          "the step's final positions over its lists; averaged over the rollout"},
        "train_and_calibrate_s": round(t1 - t0, 2),
    }
    if net is not None:
        net.close()
    if last is not None:  # the k = 3 network, which did not reach the plain max error
        lk, lnet = last
        lv, lms, _, lprof = time_solver(lk, lnet)
        result["best_network_not_qualified"] = {
            "warm_iterations": lk, "blend": lnet.blend, "steps_per_s": round(lv, 2),
            "speedup_vs_plain": round(lv / plain_value, 4),
            "density_error": accuracy(lk, lnet),
            "kernels_us": {k_: round(1000.0 * v[1] / max(v[0], 1), 2) for k_, v in lprof.items()
                           if k_ in ("k_mlp_forward", "k_search", "k_delta_correct",
                                     "k_density_lambda", "k_delta_final")}}
        prof = lprof
        lnet.close()
    result["kernels_us"] = {k_: round(1000.0 * v[1] / max(v[0], 1), 2) for k_, v in prof.items()
                            if k_ in ("k_mlp_forward", "k_search", "k_delta_correct",
                                      "k_density_lambda", "k_delta_final")}
    return result


# ---------------------------------------------------------------------------------- batched scenes
def run_batched(args, cfg, corr):
    """256 independent dam breaks (log-uniform 2k-64k particles, about 5M in all) stepped by one
    batch solver: aggregate particle-steps/s, and the distribution of the batch step time (every
    scene advances once per batch step, so that is each scene's step latency)."""
    import numpy as np
    import torch

    from akuaengine_gb300 import BatchSolver, scene

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    b = scene.batched_dam_breaks(count=256, seed=replicas_seed(rank))
    stream = torch.cuda.Stream()
    solver = BatchSolver(b.scenes, cfg, corr, stream=stream)
    buf = torch.from_numpy(b.particles.view(np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    from akuaengine_gb300.solver import as_particle_buffer

    solver.attach(as_particle_buffer(buf))
    pair_blocks = solver.autotune(b.dt, steps=3)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            solver.step(buf, b.dt)
    torch.cuda.synchronize()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    evs[0].record(stream)
    for k in range(args.steps):
        solver.step(buf, b.dt)
        evs[k + 1].record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    per = np.array([evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)])
    ms = float(per.sum())
    launches = solver.kernels_per_step()
    search_shape = solver.search_shape()
    # what launching costs: the same steps with every kernel launched one by one and bracketed
    # by events (the sum includes each launch's gap) against the graph-launched batch step
    prof_steps = 5
    solver.profile_begin(prof_steps)
    for _ in range(prof_steps):
        solver.step(buf, b.dt)
    prof = solver.profile_end()
    solver.close()
    kernel_sum_ms = sum(v[1] for v in prof.values()) / prof_steps
    node_us = graph_node_us(launches)
    launch_cost = {
        "launches_per_batch_step": launches,
        "graph_step_ms": round(ms / args.steps, 4),
        "kernels_launched_one_by_one_ms": round(kernel_sum_ms, 4),
        "kernels": {k: round(1000.0 * v[1] / max(v[0], 1), 2) for k, v in prof.items()},
        "graph_node_us": round(node_us, 3),
        "launch_bound_ms": round(launches * node_us / 1000.0, 4),
        "what": "the one-by-one figure times each kernel between events with its own launch "
                "(sorts not overlapped); graph_node_us is the replay cost per node of a CUDA graph "
                "of as many tiny kernels, so launches x graph_node_us bounds what a persistent "
                "kernel could save"}
    if rank == 0:
        line = {
            "metric": "batched scenes particle-steps/s", "value": round(b.n * args.steps / (ms / 1e3), 1),
            "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded lattice blocks + uniform jitter 0.01h)",
            "config": {"workload": "batched_256", "scenes": len(b.scenes), "particles": b.n,
                       "scene_particles": [int(min(d["numParticles"] for d in b.scenes)),
                                           int(max(d["numParticles"] for d in b.scenes))],
                       "dt": b.dt, "solver_iterations": cfg.solverIterations,
                       "table_size": int(cfg.maxNeighbours * b.n),
                       "pair_blocks_autotuned": pair_blocks,
                       "walk_shape_autotuned": {"block": search_shape[0],
                                                "staged_entries": search_shape[1]}},
            "launch_cost": launch_cost,
            "batch_step_ms": {"p50": round(float(np.percentile(per, 50)), 4),
                              "p99": round(float(np.percentile(per, 99)), 4),
                              "max": round(float(per.max()), 4)},
            "scene_steps_per_s": round(len(b.scenes) * args.steps / (ms / 1e3), 1),
            "gpu_launches": launches * args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)


def graph_node_us(nodes: int) -> float:
    """Replay cost per node of a CUDA graph of `nodes` tiny kernels (one-element adds), launch and
    the kernels' own run included: what each launch of a graph costs at the least."""
    import torch

    x = torch.zeros(32, device="cuda")
    st = torch.cuda.Stream()
    times = {}
    for k in (1, nodes):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(st):
            for _ in range(k):
                x.add_(1.0)
            torch.cuda.synchronize()
            with torch.cuda.graph(g, stream=st):
                for _ in range(k):
                    x.add_(1.0)
        torch.cuda.synchronize()
        for _ in range(20):
            g.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(200):
            g.replay()
        e1.record()
        torch.cuda.synchronize()
        times[k] = e0.elapsed_time(e1) / 200 * 1000.0
    return (times[nodes] - times[1]) / max(nodes - 1, 1)


def replicas_seed(rank):
    from akuaengine_gb300 import replicas

    return replicas.replica_seed(0, rank)


# ---------------------------------------------------------------------------------- GPU arm
def run_ours(args, sc, cfg, corr):
    import numpy as np
    import torch

    import akuaengine_gb300 as ak
    from akuaengine_gb300 import PBFSolver, replicas
    from akuaengine_gb300.solver import as_particle_buffer

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ak.load_library()

    stream = torch.cuda.Stream()
    opts = (ak.OPT_EXACT_MATH if args.exact else 0) | (ak.OPT_RESIDENT if args.resident else 0)
    solver = PBFSolver(sc.n, cfg, corr, options=opts, stream=stream, table_size=args.table_size)
    table_size = solver.stats()["tableSize"]
    host = sc.particles
    buf = torch.from_numpy(host.view(np.uint8).copy()).cuda()
    torch.cuda.synchronize()
    # launch shapes of the pair kernels, chosen by the solver's autotuner on a copy of the records
    solver.attach(as_particle_buffer(buf))
    if args.pair_blocks:
        solver.set_pair_blocks([int(b) for b in args.pair_blocks.split(",")])
        pair_blocks = solver.pair_blocks()
        solver.set_search_shape(*[int(v) for v in (args.search_shape or "128,32").split(",")])
    else:
        pair_blocks = solver.autotune(sc.dt, sc.box_min, sc.box_max, steps=3)
    search_shape = solver.search_shape()

    def barrier():
        if dist is not None:
            dist.barrier()

    # pre-roll into the developed flow (untimed), then warm-up
    with torch.cuda.stream(stream):
        for _ in range(args.preroll):
            solver.step(buf, sc.dt, sc.box_min, sc.box_max)
    torch.cuda.synchronize()
    sc_initial = sc  # the learned warm start keeps its own protocol from rest
    if args.preroll:
        # every later leg (end to end, baselines) starts from the same developed state
        host = buf.cpu().numpy().view(ak.PARTICLE_DTYPE).copy()
        sc = dataclasses.replace(sc, particles=host)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            solver.step(buf, sc.dt, sc.box_min, sc.box_max)
    torch.cuda.synchronize()
    cnt = solver.read_debug(ak.DEBUG_NEIGHBOUR_COUNTS).astype(np.int64)
    mean_c = float(cnt.mean())
    list_bytes = float((16 * ((cnt + 3) // 4)).mean())
    hashes = solver.read_debug(ak.DEBUG_HASHES)
    buckets_per_particle = float(np.unique(hashes).size) / sc.n

    # timed region: K steps on the solver's stream, events on that stream
    sampler = ClockSampler(local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    ev0.record(stream)
    for _ in range(args.steps):
        solver.step(buf, sc.dt, sc.box_min, sc.box_max)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    barrier()
    ms = ev0.elapsed_time(ev1)
    ms = replicas.max_over_ranks(ms, device="cuda")
    value = replicas.aggregate_rate(args.steps, ms / 1000.0, world)
    launches_per_step = solver.kernels_per_step()

    # per-kernel durations (CUDA events between consecutive kernels on the same stream)
    solver.profile_begin(args.profile_steps)
    for _ in range(args.profile_steps):
        solver.step(buf, sc.dt, sc.box_min, sc.box_max)
    prof = solver.profile_end()
    total = sum(v[1] for v in prof.values())
    kernels = {k: {"launches": v[0], "ms_total": round(v[1], 4),
                   "us_per_launch": round(1000.0 * v[1] / max(v[0], 1), 2),
                   "share": round(v[1] / total, 4)} for k, v in prof.items()}
    dom = max((k for k in prof if k in KERNEL_BYTES), key=lambda k: prof[k][1])
    per_launch_s = prof[dom][1] / prof[dom][0] / 1000.0
    alg = {k: KERNEL_BYTES[k](list_bytes, buckets_per_particle) * sc.n for k in KERNEL_BYTES}
    alg_bytes = alg[dom]
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / per_launch_s / 1e9
    for k, v in kernels.items():
        if k in alg:
            v["algorithmic_bytes"] = int(alg[k])
            v["gbs"] = round(alg[k] / (1e-3 * v["ms_total"] / v["launches"]) / 1e9, 1)
    step_bytes = sum(alg[k] * prof[k][0] for k in prof if k in alg) / args.profile_steps
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic_%s.json" % args.workload)) as f:
            tr = json.load(f)
        traffic = tr["bytes_per_launch"].get(dom)
    except Exception:
        pass
    # the walk is bound by instruction issue: its warp instructions per launch (ncu) over the
    # event-timed duration, against one instruction per scheduler per clock (4 per SM)
    issue = None
    try:
        inst = float(tr["warp_instructions_per_launch"][dom])
        mhz = float(clocks.get("sm_mhz") or 2070.0)
        peak_ips = SM_COUNT * 4 * mhz * 1e6
        issue = {"warp_instructions": int(inst), "achieved_per_s": round(inst / per_launch_s, 1),
                 "peak_per_s": round(peak_ips, 1), "frac": round(inst / per_launch_s / peak_ips, 4),
                 "source": "profiles/traffic_%s.json (ncu smsp__inst_executed.sum); peak at the "
                           "sampled SM clock" % args.workload}
    except Exception:
        pass
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "traffic": traffic, "algorithmic_bytes": int(alg_bytes),
                "peak_source": "measured hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
                else "fallback 6.8 TB/s",
                "issue": issue,
                "step_algorithmic_bytes": int(step_bytes),
                "step_achieved": round(step_bytes / (ms / args.steps / 1000.0) / 1e9, 1)}

    # secondary figure: the step's FP32 arithmetic (counted by ncu per kernel, per particle) against
    # the nominal FP32 rate
    fp32 = None
    try:
        with open(os.path.join(ROOT, "profiles", "fp32_ops_%s.json" % args.workload)) as f:
            fo = json.load(f)
        flops_step = float(fo["flops_per_particle_step"]) * sc.n
        tf = flops_step / (ms / args.steps / 1000.0) / 1e12
        fp32 = {"flops_per_step": int(flops_step), "achieved_tflops": round(tf, 2),
                "peak_tflops": FP32_PEAK_TFLOPS, "frac": round(tf / FP32_PEAK_TFLOPS, 4),
                "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 flops x 2.07 GHz",
                "counts": "profiles/fp32_ops_%s.json" % args.workload}
    except Exception:
        pass

    # end to end through the public API: pinned host records -> device, step, -> host
    e2e = None
    if not args.no_e2e:
        pinned = torch.empty(host.nbytes, dtype=torch.uint8, pin_memory=True)
        pinned.numpy()[:] = host.view(np.uint8)
        hp = pinned.numpy().view(ak.PARTICLE_DTYPE)
        for _ in range(2):
            solver.step_host(hp, sc.dt, sc.box_min, sc.box_max)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            solver.step_host(hp, sc.dt, sc.box_min, sc.box_max)
        el = time.perf_counter() - t0
        el = replicas.max_over_ranks(el, device="cuda")
        e2e = {"value": replicas.aggregate_rate(args.steps, el, world), "unit": UNIT,
               "h2d_bytes_per_step": int(host.nbytes), "d2h_bytes_per_step": int(host.nbytes),
               "api": "akua_pbf_step_host (pinned host records)"}

    learned = None
    if not args.no_learned and cfg.solverIterations > args.learned_iterations:
        learned = run_learned(args, sc_initial, cfg, corr, stream, value / world, ms / args.steps,
                              sc_timed=sc)
        # what fewer iterations can buy at most: the plain step minus the saved Jacobi iterations
        # (one density pass and one delta pass each) plus the network and its features
        t4 = 1000.0 * ms / args.steps
        it_us = (kernels.get("k_density_lambda", {}).get("us_per_launch", 0.0)
                 + kernels.get("k_delta_correct", {}).get("us_per_launch", 0.0))
        net_us = learned["kernels_us"].get("k_mlp_forward", 0.0)
        learned["budget"] = {
            "plain_step_us": round(t4, 1), "iteration_us": round(it_us, 1),
            "network_us": round(net_us, 1),
            "max_speedup": {str(k): round(t4 / (t4 - (cfg.solverIterations - k) * it_us + net_us), 3)
                            for k in (1, 2, 3)},
            "what": "plain step / (plain step - saved iterations x iteration + network): the "
                    "speedup at k warm iterations if the network's accuracy cost nothing"}

    # baseline legs (rank 0 at N=1, after every timed region): the CPU restatement, the error of
    # one fast step against the FP64 restatement, and the reference's own kernels on this GPU
    cpu = fp64_error = reference_gpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # ~10 s of CPU work at 1M on 16 cores (18 steps); larger scenes fall back to a sub-block
        sps, psps, cores, sample = time_oracle(sc, cfg, corr, 18, 30.0, table_size=args.table_size)
        cpu = {"value": sps, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
               "particle_steps_per_s": psps,
               "precision": "fp32: the reference's arithmetic and contractions, restated for the "
                            "host (OpenMP over particles)",
               "state": "the timed window's developed flow (after %d pre-roll steps)"
                        % args.preroll}
        fp64_error = step_error_vs_fp64(solver, sc, cfg, corr, args.table_size)
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        reference_gpu = time_reference_gpu(sc, cfg, corr, value, e2e, args.table_size)

    solver.close()
    if rank == 0:
        line = {
            "metric": WORKLOADS[args.workload][0], "value": round(value, 2), "unit": UNIT,
            "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded lattice block + uniform jitter 0.01h)",
            "config": {"workload": args.workload, "particles": sc.n,
                       "block": WORKLOADS[args.workload][1],
                       "box_block_widths": WORKLOADS[args.workload][2], "dt": sc.dt,
                       "solver_iterations": 4,
                       "max_neighbours": cfg.maxNeighbours, "table_size": table_size,
                       "corr": {"k": corr.k, "n": corr.n, "delta_q": corr.delta_q},
                       "math": "exact" if args.exact else "fast",
                       "parallelism": "replicas x%d" % world,
                       "l2": "per-step working set > L2 (no flush)",
                       "flow_phase": {"preroll_steps": args.preroll,
                                      "timed_steps": [args.preroll + args.warmup + 1,
                                                      args.preroll + args.warmup + args.steps],
                                      "sim_time_s": round((args.preroll + args.warmup) * sc.dt, 3)},
                       "mean_neighbours": round(mean_c, 3),
                       "list_bytes_per_particle": round(list_bytes, 2),
                       "pair_blocks_autotuned": pair_blocks,
                       "walk_shape_autotuned": {"block": search_shape[0],
                                                "staged_entries": search_shape[1]},
                       "buckets_per_particle": round(buckets_per_particle, 4)},
            "roofline": roofline,
            "fp32": fp32,
            "cpu_baseline": cpu,
            "fp64_error": fp64_error,
            "reference_gpu": reference_gpu,
            "e2e": e2e,
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks,
            "kernels": kernels,
            "learned_warm_start": learned,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main(argv=None):
    args = parse_args(argv)
    from akuaengine_gb300 import scene

    if args.workload == "batched_256":
        cfg, corr = scene.benchmark_params()
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batched workload is timed "
                              "on the GPU path only; the CPU arm covers dam_break_1m"}))
            return
        run_batched(args, cfg, corr)
        return

    from akuaengine_gb300 import replicas

    # every rank steps its own replica (rank 0: seed 0); replicas exchange no data
    sc = scene.workload(args.workload, seed=replicas.replica_seed(0, replicas.dist_env().rank))
    cfg, corr = scene.benchmark_params()
    if args.impl == "reference":
        run_reference(args, sc, cfg, corr)
    else:
        run_ours(args, sc, cfg, corr)


if __name__ == "__main__":
    main()
