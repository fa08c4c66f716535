"""Generates tests/golden/ref_gpu_*.npz: outputs of the reference's own CUDA kernels (compiled
unchanged from the reference sources into cubins by oracle/ref_gpu.py, driven by
oracle/ref_harness.cu) on seeded scenes.  Run on a GPU machine where oracle/_ref/ holds the cubins:

    python tests/golden/make_ref_gpu_golden.py [out_dir]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from akuaengine_gb300 import LambdaCorrParams, PBFConfig, scene  # noqa: E402
from oracle import ref_gpu  # noqa: E402


def params(cfg, corr, sc, n):
    return {"h": cfg.smoothRadius, "cell": cfg.spatialHashCellSize, "rho0": cfg.restDensity,
            "relax": cfg.relaxation, "veps": cfg.vorticityEpsilon, "visc": cfg.viscosity,
            "cap": cfg.maxNeighbours, "iters": cfg.solverIterations, "table": cfg.maxNeighbours * n,
            "k": corr.k, "nexp": corr.n, "dq": corr.delta_q, "dt": sc.dt, "g": cfg.gravity,
            "bmin": sc.box_min, "bmax": sc.box_max}


CASES = {
    # name: (scene factory, config, corr, steps, keep lists)
    "small_it1": (lambda: scene.dam_break((12, 12, 12), (3.0, 3.0, 3.0), seed=0),
                  PBFConfig(solverIterations=1), LambdaCorrParams(), 1, True),
    "small_it4": (lambda: scene.dam_break((12, 12, 12), (3.0, 3.0, 3.0), seed=0),
                  PBFConfig(), LambdaCorrParams(), 1, True),
    "small_it4_3steps": (lambda: scene.dam_break((12, 12, 12), (3.0, 3.0, 3.0), seed=0),
                         PBFConfig(), LambdaCorrParams(), 3, True),
    "refscene_1step": (scene.reference_dam_break, PBFConfig(), LambdaCorrParams(), 1, False),
    "bench27k_1step": (lambda: scene.workload("dam_break_27k", seed=0), PBFConfig(),
                       LambdaCorrParams(), 1, False),
}


def tagged(sc):
    """Particles with colour.r = their input index: colour is carried unchanged through the step,
    so the output colours spell out the sorted order."""
    p = sc.particles.copy()
    p["color"][:, 0] = np.arange(sc.n, dtype=np.float32)
    return p


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    for name, (make, cfg, corr, steps, lists) in CASES.items():
        sc = make()
        p = tagged(sc)
        info = ref_gpu.run(p, params(cfg, corr, sc, sc.n), steps, dump_lists=lists)
        out = {"hash": p["hash"], "position": p["position"], "velocity": p["velocity"],
               "new_velocity": p["new_velocity"], "position_delta": p["position_delta"],
               "vorticity": p["vorticity"], "density": p["density"], "lambda": p["lambda"],
               "color": p["color"]}
        if lists:
            cnt = info["cnt"]
            out["cnt"] = cnt
            out["nbr_flat"] = np.concatenate([info["nbr"][i, : cnt[i]] for i in range(sc.n)])
        np.savez_compressed(os.path.join(out_dir, "ref_gpu_%s.npz" % name), **out)
        print(name, sc.n, "particles", steps, "steps")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"))
