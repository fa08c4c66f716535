"""TEST INFRASTRUCTURE ONLY.  Times the reference's own CUDA step (oracle/ref_harness.cu over the
reference's kernels) on a benchmark workload, in its faithful form (host-resident neighbour
lists, per-step table allocation, as the reference's wrappers do) and with device-resident lists.

    python oracle/ref_gpu_bench.py [workload] [steps]
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from akuaengine_gb300 import scene  # noqa: E402
from oracle import ref_gpu  # noqa: E402
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from make_ref_gpu_golden import params  # noqa: E402


def main(workload="dam_break_1m", steps=3):
    sc = scene.workload(workload, seed=0)
    cfg, corr = scene.benchmark_params()
    out = {"workload": workload, "particles": sc.n, "steps": steps}
    for mode in ("faithful", "resident"):
        p = sc.particles.copy()
        pr = params(cfg, corr, sc, sc.n)
        pr["warmup"] = 1
        info = ref_gpu.run(p, pr, steps, mode=mode)
        out[mode] = {"ms_per_step": info["ms_per_step"], "steps_per_s": 1000.0 / info["ms_per_step"]}
    print(json.dumps(out))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "dam_break_1m",
         int(sys.argv[2]) if len(sys.argv) > 2 else 3)
