"""Rollout parity of the benchmarked (default, fast-math) step: 20-50 steps, not one.

The reference is not deterministic: its XSPH pass reads neighbours' velocities while other threads
overwrite them (IntegrationCUDA.cu:167-195), so two runs of the reference's own kernels on the same
input drift apart, and a dam break amplifies every difference (the flow is chaotic).  Two measured
spreads set the tolerances, per quantile of the per-particle difference (max over the three
components) and per snapshot:

* S_ref: the reference against itself, two runs of its kernels on a GB300
  (tests/golden/ref_gpu_spread.json, written by tests/golden/make_ref_gpu_rollout.py);
* S_fp32: the FP32 restatement of the reference's arithmetic against the same equations in FP64
  (the oracle's two modes, run here): how far FP32 rounding alone moves the rollout.

Bars (every quantile 50%..100%, positions and velocities):
  * fast step vs the FP32 oracle, and vs the reference's own run (27k, stored after 20 and 50
    steps): at most 3 x max(S_ref, S_fp32), floored at two ulps of the coordinates;
  * fast step vs the FP64 oracle: at most 1.5 x S_fp32 (plus the floor), i.e. the benchmarked mode
    is as accurate as the reference's own FP32 arithmetic.
Hashes, order and lists stay bit-exact per step; exact-math mode stays bit-exact over rollouts
(tests/test_gpu_parity.py; 200 steps of the 27k dam break below, where the fast mode is judged on
whole-scene quantities against two runs of the reference's kernels).
"""
import json
import os
import sys

import numpy as np
import pytest

import oracle
import akuaengine_gb300 as ak
from akuaengine_gb300 import PBFSolver, scene

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
from make_ref_gpu_golden import tagged  # noqa: E402
from make_ref_gpu_rollout import QUANTILES, in_input_order  # noqa: E402

with open(os.path.join(GOLDEN, "ref_gpu_spread.json")) as _f:
    SPREAD = json.load(_f)
assert tuple(SPREAD["quantiles"]) == tuple(QUANTILES)


def quantiles(a, b, field):
    d = np.abs(a[field].astype(np.float64) - b[field].astype(np.float64)).max(axis=1)
    return np.array([np.quantile(d, q) for q in QUANTILES])


def run_fast(sc, cfg, corr, snaps):
    p, out = tagged(sc), {}
    with PBFSolver(sc.n, cfg, corr) as s:
        for k in range(1, max(snaps) + 1):
            s.step_host(p, sc.dt, sc.box_min, sc.box_max)
            if k in snaps:
                out[k] = in_input_order(p.copy())
    return out


def run_oracle(sc, cfg, corr, snaps, flags):
    p, out = tagged(sc), {}
    P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=sc.n, flags=flags)
    for k in range(1, max(snaps) + 1):
        oracle.step(p, P)
        if k in snaps:
            out[k] = in_input_order(p.copy())
    return out


def floors(sc):
    """Two ulps of the largest coordinate, and that over dt for velocities."""
    big = float(np.abs(np.asarray(sc.box_max, np.float32)).max())
    pos = 2.0 * float(np.spacing(np.float32(big)))
    return {"position": pos, "velocity": pos / sc.dt}


@pytest.fixture(scope="module", autouse=True)
def _lib(cuda_lib):
    return cuda_lib


@pytest.mark.parametrize("case,snaps", [("dam_break_27k", (5, 20, 50)),
                                        ("dam_break_1m", (5, 20))])
def test_fast_rollout_within_reference_spread(case, snaps):
    spec = SPREAD["cases"][case]
    sc = scene.workload(spec["workload"], seed=spec["seed"])
    cfg, corr = scene.benchmark_params(strong_pressure=spec["strong_pressure"])
    fast = run_fast(sc, cfg, corr, snaps)
    o32 = run_oracle(sc, cfg, corr, snaps, oracle.FMA)
    o64 = run_oracle(sc, cfg, corr, snaps, oracle.FMA | oracle.FP64)
    ref = None
    if case == "dam_break_27k":
        ref = dict(np.load(os.path.join(GOLDEN, "ref_gpu_rollout_27k.npz")))
    fl = floors(sc)
    for s in snaps:
        for field in ("position", "velocity"):
            s_ref = np.array(spec["steps"][str(s)][field])
            s_fp32 = quantiles(o32[s], o64[s], field)
            bound = np.maximum(3.0 * np.maximum(s_ref, s_fp32), fl[field])
            got = quantiles(fast[s], o32[s], field)
            acc = quantiles(fast[s], o64[s], field)
            print("%s step %d %s: fast-oracle %s | bound %s | fast-fp64 %s | fp32-fp64 %s"
                  % (case, s, field, np.array2string(got, precision=2),
                     np.array2string(bound, precision=2), np.array2string(acc, precision=2),
                     np.array2string(s_fp32, precision=2)))
            assert np.all(got <= bound), (case, s, field, got, bound)
            assert np.all(acc <= np.maximum(1.5 * s_fp32, fl[field])), (case, s, field, acc, s_fp32)
            if ref is not None and ("%s_%d" % (field, s)) in ref:
                vs_ref = quantiles(fast[s], {field: ref["%s_%d" % (field, s)]}, field)
                assert np.all(vs_ref <= bound), (case, s, field, "vs reference", vs_ref, bound)


def test_200_steps_of_the_27k_dam_break(cuda_lib):
    """The 27k dam break over 200 steps against the host oracle.  With exact math every record of
    every one of the 200 steps equals the FP32 restatement's (checked every 10 steps).  In the
    benchmarked fast mode the flow has long become chaotic particle by particle, so whole-scene
    quantities are compared: kinetic energy, centre of mass, spread along x, mean and max density
    constraint.  Correct runs scatter around each other: two runs of the reference's kernels
    (tests/golden/ref_gpu_aggregates_27k.json) and the FP32 and FP64 restatements form the
    ensemble; the fast step must lie within 3 x the ensemble's width plus 0.5% of its mean."""
    import akuaengine_gb300 as ak
    from make_ref_gpu_rollout import AGG_STEPS, aggregates

    with open(os.path.join(GOLDEN, "ref_gpu_aggregates_27k.json")) as f:
        ref = json.load(f)
    sc = scene.workload(ref["workload"], seed=ref["seed"])
    cfg, corr = scene.benchmark_params()
    runs = {"refA": ref["runs"][0], "refB": ref["runs"][1]}
    exact_mismatch = []
    for name, flags in (("o32", oracle.FMA), ("o64", oracle.FMA | oracle.FP64)):
        q = sc.particles.copy()
        P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=sc.n, flags=flags)
        g = sc.particles.copy()
        solver = PBFSolver(sc.n, cfg, corr, options=ak.OPT_EXACT_MATH) if name == "o32" else None
        agg = {}
        try:
            for k in range(1, 201):
                oracle.step(q, P)
                if solver is not None:
                    solver.step_host(g, sc.dt, sc.box_min, sc.box_max)
                if k in AGG_STEPS:
                    agg[str(k)] = aggregates(q, cfg.restDensity)
                    if solver is not None and g.tobytes() != q.tobytes():
                        exact_mismatch.append(k)
        finally:
            if solver is not None:
                solver.close()
        runs[name] = agg
    assert not exact_mismatch, "exact-math records differ from the oracle at steps %s" % exact_mismatch
    fast, p = {}, sc.particles.copy()
    with PBFSolver(sc.n, cfg, corr) as s:
        for k in range(1, 201):
            s.step_host(p, sc.dt, sc.box_min, sc.box_max)
            if k in AGG_STEPS:
                fast[str(k)] = aggregates(p, cfg.restDensity)
    worst = 0.0
    for k in map(str, AGG_STEPS):
        for q, v in fast[k].items():
            e = [runs[n][k][q] for n in ("refA", "refB", "o32", "o64")]
            mid, width = sum(e) / len(e), max(e) - min(e)
            bound = 3.0 * width + 5e-3 * abs(mid)
            worst = max(worst, abs(v - mid) / bound)
            assert abs(v - mid) <= bound, (k, q, v, e)
    print("200-step aggregates: worst |fast - ensemble| / bound = %.2f" % worst)
