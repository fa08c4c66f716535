"""Generates the rollout fixtures of the reference's own CUDA kernels (compiled unchanged from the
reference sources into cubins by oracle/ref_gpu.py, driven by oracle/ref_harness.cu):

* tests/golden/ref_gpu_spread.json: the reference's run-to-run spread.  Its XSPH pass reads
  neighbours' velocities while other threads overwrite them (IntegrationCUDA.cu:167-195), so two
  runs of the same input differ; the spread between two runs, as per-particle quantiles of
  |x_A - x_B| and |v_A - v_B| after 1..50 steps, is the floor of the rollout tolerances.
* tests/golden/ref_gpu_rollout_27k.npz: run A's positions and velocities after 20 and 50 steps
  of the 27k dam break, in input order (colour.r carries each particle's input index).
* tests/golden/ref_gpu_aggregates_27k.json: whole-scene quantities of the 27k dam break every 10
  steps over 200 steps, for two runs of the reference kernels (kinetic energy, centre of mass,
  spread, density error): by then the flow is chaotic particle by particle, and these are what two
  runs of the reference still agree on, and how closely.

Run on a GPU machine where oracle/_ref/ holds the cubins:

    python tests/golden/make_ref_gpu_rollout.py [out_dir]
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from akuaengine_gb300 import scene  # noqa: E402
from make_ref_gpu_golden import params, tagged  # noqa: E402
from oracle import ref_gpu  # noqa: E402

QUANTILES = (0.5, 0.9, 0.99, 0.999, 1.0)

# name: (workload, strong artificial pressure, snapshot steps)
ROLLOUTS = {
    "dam_break_27k": ("dam_break_27k", False, (1, 5, 10, 20, 50)),
    "dam_break_27k_strong": ("dam_break_27k", True, (1, 5, 10, 20)),
    "dam_break_1m": ("dam_break_1m", False, (1, 5, 10, 20)),
}


def in_input_order(p):
    """Records sorted back into input order by their colour.r tag."""
    return p[np.argsort(p["color"][:, 0].astype(np.int64), kind="stable")]


def run_chain(sc, cfg, corr, snaps):
    """One run of the reference kernels over max(snaps) steps; the state at each snapshot."""
    p = tagged(sc)
    pr = params(cfg, corr, sc, sc.n)
    out, done = {}, 0
    for s in snaps:
        ref_gpu.run(p, pr, s - done)
        done = s
        out[s] = in_input_order(p.copy())
    return out


def spread_quantiles(a, b):
    dx = np.abs(a["position"].astype(np.float64) - b["position"]).max(axis=1)
    dv = np.abs(a["velocity"].astype(np.float64) - b["velocity"]).max(axis=1)
    return {"position": [float(np.quantile(dx, q)) for q in QUANTILES],
            "velocity": [float(np.quantile(dv, q)) for q in QUANTILES]}


AGG_STEPS = tuple(range(10, 201, 10))


def aggregates(p, rho0=7600.0):
    """Whole-scene quantities of one state (float64 sums)."""
    x = p["position"].astype(np.float64)
    v = p["velocity"].astype(np.float64)
    m = p["mass"].astype(np.float64)
    c = p["density"].astype(np.float64) / rho0 - 1.0
    com = (m[:, None] * x).sum(0) / m.sum()
    return {"kinetic_energy": float(0.5 * (m * (v * v).sum(1)).sum()),
            "com_x": float(com[0]), "com_y": float(com[1]), "com_z": float(com[2]),
            "spread_x": float(np.sqrt((m * (x[:, 0] - com[0]) ** 2).sum() / m.sum())),
            "mean_abs_c": float(np.abs(c).mean()), "max_c": float(c.max())}


def aggregate_runs(out_dir):
    sc = scene.workload("dam_break_27k", seed=0)
    cfg, corr = scene.benchmark_params()
    runs = []
    for _ in range(2):
        states = run_chain(sc, cfg, corr, AGG_STEPS)
        runs.append({str(k): aggregates(states[k], cfg.restDensity) for k in AGG_STEPS})
    with open(os.path.join(out_dir, "ref_gpu_aggregates_27k.json"), "w") as f:
        json.dump({"workload": "dam_break_27k", "seed": 0, "steps": list(AGG_STEPS),
                   "runs": runs}, f, indent=1)


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    spread = {"quantiles": list(QUANTILES),
              "what": "per-particle max-abs-component difference between two runs of the "
                      "reference kernels on the same input",
              "cases": {}}
    for name, (work, strong, snaps) in ROLLOUTS.items():
        sc = scene.workload(work, seed=0)
        cfg, corr = scene.benchmark_params(strong_pressure=strong)
        run_a = run_chain(sc, cfg, corr, snaps)
        run_b = run_chain(sc, cfg, corr, snaps)
        spread["cases"][name] = {
            "workload": work, "strong_pressure": strong, "seed": 0, "n": sc.n,
            "steps": {str(s): spread_quantiles(run_a[s], run_b[s]) for s in snaps}}
        print(name, json.dumps(spread["cases"][name]["steps"]))
        if name == "dam_break_27k":
            np.savez_compressed(
                os.path.join(out_dir, "ref_gpu_rollout_27k.npz"),
                **{"position_%d" % s: run_a[s]["position"] for s in (20, 50)},
                **{"velocity_%d" % s: run_a[s]["velocity"] for s in (20, 50)})
    with open(os.path.join(out_dir, "ref_gpu_spread.json"), "w") as f:
        json.dump(spread, f, indent=1)
    aggregate_runs(out_dir)


if __name__ == "__main__":
    # python make_ref_gpu_rollout.py [out_dir [aggregates]]: with "aggregates", only that fixture
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden")
    if len(sys.argv) > 2 and sys.argv[2] == "aggregates":
        os.makedirs(out, exist_ok=True)
        aggregate_runs(out)
    else:
        main(out)
