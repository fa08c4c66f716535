"""Generates tests/golden/ref_gpu_*.npz: outputs of the reference's own CUDA kernels (compiled
unchanged from the reference sources into cubins by oracle/ref_gpu.py, driven by
oracle/ref_harness.cu) on seeded scenes.  Run on a GPU machine where oracle/_ref/ holds the cubins:

    python tests/golden/make_ref_gpu_golden.py [out_dir [case ...]]
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
    # the strong artificial pressure k = 0.1, n = 4, delta_q = 0.2h: the block flies apart within
    # a few steps and every FP32 evaluation order (the reference's own runs included) diverges
    # from step 2 on, so these fixtures hold one step
    "small_strong_1step": (lambda: scene.dam_break((12, 12, 12), (3.0, 3.0, 3.0), seed=0),
                           *scene.benchmark_params(strong_pressure=True), 1, True),
    "strong27k_1step": (lambda: scene.workload("dam_break_27k", seed=0),
                        *scene.benchmark_params(strong_pressure=True), 1, False),
    "dam_break_100k_1step": (lambda: scene.workload("dam_break_100k", seed=0), PBFConfig(),
                             LambdaCorrParams(), 1, False),
}

# Fixtures that keep the float fields of every stride-th particle only (by input index, colour.r)
# to stay small; their hashes and sorted order (as `tag`, the output's colour.r) cover every
# particle.
FLOAT_STRIDE = {"strong27k_1step": 2, "dam_break_100k_1step": 8}
FLOAT_KEYS = ("position", "velocity", "new_velocity", "position_delta", "vorticity", "density",
              "lambda")


def kept(p, name):
    """Mask of the particles (in output order) whose float fields the fixture `name` keeps."""
    stride = FLOAT_STRIDE.get(name, 1)
    return p["color"][:, 0].astype(np.int64) % stride == 0


def tagged(sc):
    """Particles with colour.r = their input index: colour is carried unchanged through the step,
    so the output colours spell out the sorted order."""
    p = sc.particles.copy()
    p["color"][:, 0] = np.arange(sc.n, dtype=np.float32)
    return p


def main(out_dir, only=None):
    os.makedirs(out_dir, exist_ok=True)
    for name, (make, cfg, corr, steps, lists) in CASES.items():
        if only and name not in only:
            continue
        sc = make()
        p = tagged(sc)
        info = ref_gpu.run(p, params(cfg, corr, sc, sc.n), steps, dump_lists=lists)
        if name in FLOAT_STRIDE:
            keep = kept(p, name)
            out = {"hash": p["hash"], "tag": p["color"][:, 0]}
            out.update({k: p[k][keep] for k in FLOAT_KEYS})
        else:
            out = {"hash": p["hash"], "color": p["color"]}
            out.update({k: p[k] for k in FLOAT_KEYS})
        if lists:
            cnt = info["cnt"]
            out["cnt"] = cnt
            out["nbr_flat"] = np.concatenate([info["nbr"][i, : cnt[i]] for i in range(sc.n)])
        np.savez_compressed(os.path.join(out_dir, "ref_gpu_%s.npz" % name), **out)
        print(name, sc.n, "particles", steps, "steps")


if __name__ == "__main__":
    # python make_ref_gpu_golden.py [out_dir [case ...]]
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"),
         sys.argv[2:] or None)
