"""GPU parity: the CUDA step (through the C ABI) against the CPU oracle on the same seeded inputs.

Bars:
  * cell hashes, sorted order, neighbour lists and counts: bit-exact, in both math modes;
  * AKUA_PBF_OPT_EXACT_MATH: every field of every record bit-exact, over many steps;
  * default (fast) math: floats within the tolerances written in each test.
"""
import numpy as np
import pytest

import oracle
import akuaengine_gb300 as ak
from akuaengine_gb300 import LambdaCorrParams, PBFConfig, PBFSolver, scene

pytestmark = pytest.mark.gpu

FLOAT_FIELDS = ["position", "velocity", "new_position", "new_velocity", "position_delta",
                "vorticity", "mass", "density", "lambda", "color", "size"]


def bench_params():
    """Benchmark workloads' parameters: reference scene values, dt 0.0083, reference
    artificial pressure (k=1e-4, n=4, dq=0.03)."""
    return PBFConfig(), LambdaCorrParams()


def strong_corr():
    """The artificial pressure k=0.1, n=4, dq=0.2h; with the reference's rho0 and mass it makes
    the fluid break apart, which exercises sparse neighbourhoods."""
    return LambdaCorrParams(k=0.1, n=4.0, delta_q=0.02)


def run_gpu(sc, cfg, corr, steps=1, options=0, table_size=None, particles=None):
    p = (sc.particles if particles is None else particles).copy()
    with PBFSolver(sc.n, cfg, corr, options=options, table_size=table_size) as s:
        for _ in range(steps):
            s.step_host(p, sc.dt, sc.box_min, sc.box_max)
        extra = {
            "order": s.read_debug(ak.DEBUG_ORDER),
            "hashes": s.read_debug(ak.DEBUG_HASHES),
            "cnt": s.read_debug(ak.DEBUG_NEIGHBOUR_COUNTS),
            "nbr": s.read_debug(ak.DEBUG_NEIGHBOURS),
            "stats": s.stats(),
        }
    return p, extra


def run_oracle(sc, cfg, corr, steps=1, flags=oracle.FMA, table_size=None, particles=None):
    p = (sc.particles if particles is None else particles).copy()
    P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=sc.n, flags=flags,
                           table_size=table_size)
    out = None
    for k in range(steps):
        out = oracle.step(p, P, want_lists=(k == steps - 1))
    perm, nbr, cnt = out
    return p, {"order": perm, "nbr": nbr, "cnt": cnt}


def assert_grid_equal(g, o, cap):
    assert np.array_equal(g["order"], o["order"]), "sorted order differs"
    assert np.array_equal(g["cnt"], o["cnt"]), "neighbour counts differ"
    n = len(g["cnt"])
    mask = np.arange(cap)[None, :] < g["cnt"][:, None]
    assert np.array_equal(np.where(mask, g["nbr"], 0), np.where(mask, o["nbr"], 0)), \
        "neighbour lists differ"


def assert_records_bitexact(a, b):
    for f in FLOAT_FIELDS + ["hash"]:
        x, y = a[f], b[f]
        if not np.array_equal(x.view(np.uint32), y.view(np.uint32)):
            bad = np.argwhere(x.view(np.uint32) != y.view(np.uint32))
            raise AssertionError("%s differs at %d places, first %s: %r vs %r"
                                 % (f, len(bad), bad[0], x[tuple(bad[0])], y[tuple(bad[0])]))


@pytest.fixture(scope="module", autouse=True)
def _lib(cuda_lib):
    return cuda_lib


# --- exact math: bit-exact records -----------------------------------------------------------

def test_exact_one_step_27k_bitexact():
    sc = scene.workload("dam_break_27k", seed=0)
    cfg, corr = bench_params()
    g, ge = run_gpu(sc, cfg, corr, 1, ak.OPT_EXACT_MATH)
    o, oe = run_oracle(sc, cfg, corr, 1)
    assert np.array_equal(ge["hashes"], o["hash"])
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


@pytest.mark.parametrize("strong", [False, True])
def test_exact_many_steps_bitexact(strong):
    sc = scene.dam_break((14, 12, 10), (3.0, 3.0, 3.0), seed=7)
    cfg = PBFConfig()
    corr = strong_corr() if strong else LambdaCorrParams()
    g, ge = run_gpu(sc, cfg, corr, 25, ak.OPT_EXACT_MATH)
    o, oe = run_oracle(sc, cfg, corr, 25)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


def test_exact_reference_scene_bitexact():
    """The reference's own scene (Application.cpp:162-192, no jitter, dt 0.016, default corr)."""
    sc = scene.reference_dam_break()
    cfg, corr = PBFConfig(), LambdaCorrParams()
    g, ge = run_gpu(sc, cfg, corr, 5, ak.OPT_EXACT_MATH)
    o, oe = run_oracle(sc, cfg, corr, 5)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


def test_capacity_truncation_bitexact():
    sc = scene.dam_break((12, 12, 12), (3.0, 3.0, 3.0), seed=2)
    cfg = PBFConfig(maxNeighbours=12)
    corr = LambdaCorrParams()
    g, ge = run_gpu(sc, cfg, corr, 3, ak.OPT_EXACT_MATH)
    o, oe = run_oracle(sc, cfg, corr, 3)
    assert ge["cnt"].max() == 12
    assert ge["stats"]["deviceFlags"] & ak.FLAG_CAP_REACHED
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


def test_dense_pile_up_bitexact():
    """5,000 particles packed into one cell beside a resting block: their run's candidate sequence
    is far longer than any resting cell's, so the walk stops once every list of the run is full;
    lists, records and the overflow flag must still equal the oracle's, which walks everything."""
    sc = scene.dam_break((12, 12, 12), (3.0, 3.0, 3.0), seed=4)
    rng = np.random.default_rng(4)
    pile = np.zeros(5000, dtype=sc.particles.dtype)
    pile["position"] = (np.array([0.95, 0.55, 0.95]) + rng.uniform(0.0, 0.09, (5000, 3))).astype(
        np.float32)
    pile["mass"] = 1.0
    pile["color"] = (1.0, 0.0, 0.0, 1.0)
    pile["size"] = 50.0
    sc.particles = np.concatenate([sc.particles, pile])
    cfg, corr = PBFConfig(), LambdaCorrParams()
    g, ge = run_gpu(sc, cfg, corr, 2, ak.OPT_EXACT_MATH)
    o, oe = run_oracle(sc, cfg, corr, 2)
    assert ge["cnt"].max() == cfg.maxNeighbours
    assert ge["stats"]["deviceFlags"] & ak.FLAG_CAP_REACHED
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


@pytest.mark.parametrize("cap", [128, 100, 200])
@pytest.mark.parametrize("table_size", [None, 4096])
def test_long_lists_bitexact(cap, table_size):
    """A lattice at 0.3h gives ~150 neighbours: lists run past the walk's 64-entry stage (the
    overflow pass) and, for cap 100/128, past the capacity; with a small table the long lists also
    hold duplicated and foreign-cell candidates."""
    p = scene.lattice_block((16, 16, 16), 0.03, (1.0, 1.0, 1.0), jitter=0.001, seed=7)
    sc = scene.Scene(p, (0.0, 0.0, 0.0), (3.0, 3.0, 3.0), 0.0083, "dense")
    cfg = PBFConfig(maxNeighbours=cap)
    corr = LambdaCorrParams()
    g, ge = run_gpu(sc, cfg, corr, 1, ak.OPT_EXACT_MATH, table_size=table_size)
    o, oe = run_oracle(sc, cfg, corr, 1, table_size=table_size)
    assert ge["cnt"].max() > 64
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


@pytest.mark.parametrize("masses", ["uniform_0.7", "varied"])
def test_masses_bitexact(masses):
    """The Jacobi delta gathers (x*, lambda) in one load when every mass has the same bit
    pattern, and positions, masses and lambdas separately otherwise: both bit-exact."""
    sc = scene.workload("dam_break_27k", seed=8)
    p = sc.particles.copy()
    if masses == "varied":
        p["mass"] = np.random.default_rng(1).uniform(0.8, 1.2, sc.n).astype(np.float32)
    else:
        p["mass"] = np.float32(0.7)
    cfg, corr = bench_params()
    cfg.restDensity = float(np.float32(7600.0 * float(p["mass"].mean())))
    g, ge = run_gpu(sc, cfg, corr, 3, ak.OPT_EXACT_MATH, particles=p)
    o, oe = run_oracle(sc, cfg, corr, 3, particles=p)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


SDF_SHAPES = [
    {"type": "sphere", "a": (0.8, 0.0, 0.8), "radius": 0.4},
    {"type": "box", "a": (1.5, 0.1, 0.5), "b": (0.2, 0.3, 0.2), "radius": 0.02},
    {"type": "capsule", "a": (0.2, 0.25, 1.4), "b": (1.2, 0.25, 1.4), "radius": 0.1},
    {"type": "plane", "a": (0.0995037190, 0.995037190, 0.0), "b": (0.06, 0.0, 0.0)},
]


def test_sdf_obstacles_bitexact():
    """A sphere, a rounded box, a capsule and a tilted floor in the tank: 20 steps bit-exact
    against the oracle with the same obstacles, and different from the run without them."""
    import oracle as orc

    sc = scene.workload("dam_break_27k", seed=9)
    cfg, corr = bench_params()
    steps = 20
    g = sc.particles.copy()
    with PBFSolver(sc.n, cfg, corr, options=ak.OPT_EXACT_MATH) as s:
        s.set_sdf_shapes(SDF_SHAPES)
        for _ in range(steps):
            s.step_host(g, sc.dt, sc.box_min, sc.box_max)
    o = sc.particles.copy()
    P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=sc.n)
    orc.set_shapes(P, [{**d, "type": ak.solver.SDF_TYPES[d["type"]]} for d in SDF_SHAPES])
    for _ in range(steps):
        oracle.step(o, P)
    assert_records_bitexact(g, o)
    plain, _ = run_gpu(sc, cfg, corr, steps, ak.OPT_EXACT_MATH)
    moved = np.abs(plain["position"] - g["position"]).max(1)
    assert (moved > 1e-3).sum() > 100  # the obstacles changed the flow


def test_small_table_collisions_bitexact():
    """A 4096-entry table makes many cells share a bucket (duplicated and foreign candidates)."""
    sc = scene.dam_break((12, 12, 12), (3.0, 3.0, 3.0), seed=4)
    cfg, corr = PBFConfig(), LambdaCorrParams()
    g, ge = run_gpu(sc, cfg, corr, 3, ak.OPT_EXACT_MATH, table_size=4096)
    o, oe = run_oracle(sc, cfg, corr, 3, table_size=4096)
    dup = sum(len(set(oe["nbr"][i, : oe["cnt"][i]])) != oe["cnt"][i] for i in range(sc.n))
    assert dup > 0
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


def test_zero_iterations_bitexact():
    sc = scene.dam_break((8, 8, 8), (3.0, 3.0, 3.0), seed=9)
    p = sc.particles.copy()
    p["density"] = np.linspace(7000, 8000, sc.n, dtype=np.float32)
    p["lambda"] = np.linspace(-1e-4, 1e-4, sc.n, dtype=np.float32)
    p["position_delta"] = 1e-3
    cfg, corr = PBFConfig(solverIterations=0), LambdaCorrParams()
    g, ge = run_gpu(sc, cfg, corr, 2, ak.OPT_EXACT_MATH, particles=p)
    o, oe = run_oracle(sc, cfg, corr, 2, particles=p)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


@pytest.mark.parametrize("opts", [0, ak.OPT_EXACT_MATH], ids=["fast", "exact"])
def test_interior_lattice_density_known_answer(opts):
    """The centre of a resting lattice at spacing h/2 has 26 neighbours and density
    W(0) + 6 W(h/2) + 12 W(h/sqrt 2) + 8 W(h sqrt 3/2) = 8082.3 (computed in float64)."""
    from test_oracle import lattice_density_known_answer, lattice_kat_scene

    p, cfg, centre = lattice_kat_scene()
    sc = scene.Scene(p, (0.0, 0.0, 0.0), (3.0, 3.0, 3.0), 0.0083, "lattice_kat")
    g, ge = run_gpu(sc, cfg, LambdaCorrParams(), 1, opts)
    k = int(np.nonzero(ge["order"] == centre)[0][0])
    assert ge["cnt"][k] == 26
    assert float(g["density"][k]) == pytest.approx(lattice_density_known_answer(), rel=2e-5)
    if opts:
        o, _ = run_oracle(sc, cfg, LambdaCorrParams(), 1)
        assert_records_bitexact(g, o)


@pytest.mark.parametrize("n", [1, 2, 7])
def test_tiny_particle_counts(n):
    sc = scene.dam_break((30, 30, 30), seed=1)
    sc.particles = sc.particles[:n].copy()
    cfg, corr = PBFConfig(), LambdaCorrParams()
    g, ge = run_gpu(sc, cfg, corr, 3, ak.OPT_EXACT_MATH)
    o, oe = run_oracle(sc, cfg, corr, 3)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


def test_particles_outside_box_clamped_and_damped_bitexact():
    sc = scene.dam_break((10, 10, 10), (2.0, 2.0, 2.0), seed=5)
    p = sc.particles.copy()
    rng = np.random.default_rng(0)
    p["velocity"] = rng.normal(0, 3, size=(sc.n, 3)).astype(np.float32)
    p["position"][:50] -= 0.2           # some start outside the lower walls
    cfg, corr = PBFConfig(), strong_corr()
    g, ge = run_gpu(sc, cfg, corr, 4, ak.OPT_EXACT_MATH, particles=p)
    o, oe = run_oracle(sc, cfg, corr, 4, particles=p)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


# --- fast math: exact grid, floats within tolerance ------------------------------------------

# Tolerances of the default math against the oracle after one step from the same state.  The
# fast path replaces IEEE sqrt/divide in pair terms by rsqrt-based forms (a few ulp each); the
# four Jacobi iterations carry those differences into positions.
POS_ATOL = 2e-5        # position units (boxes are 6-15 units wide)
VEL_ATOL = 4e-3        # = POS_ATOL / dt plus XSPH/vorticity terms
RHO_RTOL = 2e-5
LAM_ATOL = 2e-8        # lambda magnitudes are ~1e-4
VORT_RTOL = 1e-3      # of the largest |omega|: omega sums nearly cancelling terms of ~|dv| |grad W|


def assert_close_fast(g, o):
    assert np.array_equal(g["hash"], o["hash"])
    assert np.array_equal(g["mass"], o["mass"]) and np.array_equal(g["color"], o["color"])
    err = {
        "position": np.abs(g["position"] - o["position"]).max(),
        "velocity": np.abs(g["velocity"] - o["velocity"]).max(),
        "new_velocity": np.abs(g["new_velocity"] - o["new_velocity"]).max(),
        "density": (np.abs(g["density"] - o["density"]) / np.abs(o["density"])).max(),
        "lambda": np.abs(g["lambda"] - o["lambda"]).max(),
        "vorticity": np.abs(g["vorticity"] - o["vorticity"]).max()
        / max(np.abs(o["vorticity"]).max(), 1e-30),
    }
    print("fast-vs-oracle max errors:", {k: float(v) for k, v in err.items()})
    assert err["position"] <= POS_ATOL
    assert err["velocity"] <= VEL_ATOL and err["new_velocity"] <= VEL_ATOL
    assert err["density"] <= RHO_RTOL
    assert err["lambda"] <= LAM_ATOL
    assert err["vorticity"] <= VORT_RTOL


def test_fast_one_step_27k():
    sc = scene.workload("dam_break_27k", seed=1)
    cfg, corr = bench_params()
    g, ge = run_gpu(sc, cfg, corr, 1, 0)
    o, oe = run_oracle(sc, cfg, corr, 1)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_close_fast(g, o)


def test_fast_one_step_from_evolved_state():
    """Parity from a state 40 steps into the dam break (splashes, compressed regions)."""
    sc = scene.workload("dam_break_27k", seed=2)
    cfg, corr = bench_params()
    start, _ = run_oracle(sc, cfg, corr, 40)
    g, ge = run_gpu(sc, cfg, corr, 1, 0, particles=start)
    o, oe = run_oracle(sc, cfg, corr, 1, particles=start)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_close_fast(g, o)


def test_fast_one_step_1m_full_size():
    """The 1M-particle benchmark workload: grid bit-exact, floats within tolerance."""
    sc = scene.workload("dam_break_1m", seed=0)
    cfg, corr = bench_params()
    g, ge = run_gpu(sc, cfg, corr, 1, 0)
    o, oe = run_oracle(sc, cfg, corr, 1)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_close_fast(g, o)


@pytest.mark.parametrize("shape", [(64, 32), (256, 32), (64, 16), (128, 16), (256, 16), (64, 48),
                                   (128, 48)])
def test_walk_tile_shapes_identical(shape):
    """Every tile shape of the walk the autotuner can pick gives the default shape's records,
    lists and order bit for bit (three steps, both math modes)."""
    sc = scene.workload("dam_break_27k", seed=9)
    cfg, corr = bench_params()
    for opts in (0, ak.OPT_EXACT_MATH):
        outs = []
        for sh in ((128, 32), shape):
            p = sc.particles.copy()
            with PBFSolver(sc.n, cfg, corr, options=opts) as s:
                s.set_search_shape(*sh)
                assert s.search_shape() == sh
                for _ in range(3):
                    s.step_host(p, sc.dt, sc.box_min, sc.box_max)
                outs.append((p, s.read_debug(ak.DEBUG_NEIGHBOURS), s.read_debug(ak.DEBUG_ORDER)))
        assert outs[0][0].tobytes() == outs[1][0].tobytes()
        assert np.array_equal(outs[0][1], outs[1][1]) and np.array_equal(outs[0][2], outs[1][2])


@pytest.mark.parametrize("table_size", [None, 1 << 24], ids=["table_128N", "table_2e24"])
def test_exact_one_step_8m_double_dam_break(table_size):
    """8M particles in two blocks, with the reference's table of 128 N = 1.024e9 buckets and with
    the 2^24-bucket table of the 8M workload (about 61 particles per bucket on average, so most
    buckets hold several cells): one step, grid and every record bit-exact against the oracle at
    the same table size."""
    sc = scene.workload("double_dam_break_8m", seed=0)
    cfg, corr = bench_params()
    g, ge = run_gpu(sc, cfg, corr, 1, ak.OPT_EXACT_MATH, table_size=table_size)
    o, oe = run_oracle(sc, cfg, corr, 1, table_size=table_size)
    assert_grid_equal(ge, oe, cfg.maxNeighbours)
    assert_records_bitexact(g, o)


def test_fast_error_against_fp64_oracle():
    """FP32 error of one GPU step measured against the same equations in double precision."""
    sc = scene.workload("dam_break_27k", seed=3)
    cfg, corr = bench_params()
    g, _ = run_gpu(sc, cfg, corr, 1, 0)
    d, _ = run_oracle(sc, cfg, corr, 1, flags=oracle.FMA | oracle.FP64)
    f, _ = run_oracle(sc, cfg, corr, 1)
    e_gpu = np.abs(g["position"].astype(np.float64) - d["position"]).max()
    e_f32 = np.abs(f["position"].astype(np.float64) - d["position"]).max()
    print("position error vs fp64: gpu fast %.3g, fp32 oracle %.3g" % (e_gpu, e_f32))
    assert e_gpu <= 4 * e_f32 + 1e-6


# --- host logic of the step: graph, resident state, device buffers ---------------------------

def test_step_host_pinned_and_pageable_identical():
    """Pinned host records are stepped in place over the host link; pageable ones through a
    device copy: same bytes, over several steps."""
    import torch

    sc = scene.workload("dam_break_27k", seed=12)
    cfg, corr = bench_params()
    pinned = torch.empty(sc.particles.nbytes, dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = sc.particles.view(np.uint8)
    pv = pinned.numpy().view(ak.PARTICLE_DTYPE)
    pageable = sc.particles.copy()
    with PBFSolver(sc.n, cfg, corr) as a, PBFSolver(sc.n, cfg, corr) as b:
        for _ in range(4):
            a.step_host(pv, sc.dt, sc.box_min, sc.box_max)
            b.step_host(pageable, sc.dt, sc.box_min, sc.box_max)
    assert pv.tobytes() == pageable.tobytes()


def test_autotune_keeps_results_and_user_state():
    """The autotuner picks block sizes from 64/128/256 on a copy of the records: the attached
    records and the step count are untouched, and the tuned step gives the same bytes."""
    import torch

    sc = scene.workload("dam_break_27k", seed=13)
    cfg, corr = bench_params()
    ref = sc.particles.copy()
    with PBFSolver(sc.n, cfg, corr) as s:
        for _ in range(2):
            s.step_host(ref, sc.dt, sc.box_min, sc.box_max)
    buf = torch.from_numpy(sc.particles.view(np.uint8).copy()).cuda()
    with PBFSolver(sc.n, cfg, corr) as s:
        s.step(buf, sc.dt, sc.box_min, sc.box_max)
        before = buf.cpu().numpy().tobytes()
        steps = s.stats()["steps"]
        choice = s.autotune(sc.dt, sc.box_min, sc.box_max, steps=2)
        assert set(choice.values()) <= {64, 128, 256} and s.pair_blocks() == choice
        assert buf.cpu().numpy().tobytes() == before and s.stats()["steps"] == steps
        s.step(buf, sc.dt, sc.box_min, sc.box_max)
        s.set_pair_blocks([64, 256, 64, 256, 64, 256])
        assert buf.cpu().numpy().view(ak.PARTICLE_DTYPE).tobytes() == ref.tobytes()
    with pytest.raises(ak.AkuaError):
        with PBFSolver(sc.n, cfg, corr) as s:
            s.set_pair_blocks([96] * 6)


def test_graph_and_direct_launch_identical():
    sc = scene.dam_break((16, 16, 16), (3.0, 3.0, 3.0), seed=11)
    cfg, corr = bench_params()
    a, _ = run_gpu(sc, cfg, corr, 5, 0)
    b, _ = run_gpu(sc, cfg, corr, 5, ak.OPT_NO_GRAPH)
    assert a.tobytes() == b.tobytes()


def test_resident_mode_matches_reimport():
    torch = pytest.importorskip("torch")
    sc = scene.dam_break((16, 16, 16), (3.0, 3.0, 3.0), seed=12)
    cfg, corr = bench_params()
    outs = []
    for opts in (0, ak.OPT_RESIDENT):
        buf = torch.from_numpy(sc.particles.view(np.uint8).copy()).cuda()
        with PBFSolver(sc.n, cfg, corr, options=opts) as s:
            for _ in range(6):
                s.step(buf, sc.dt, sc.box_min, sc.box_max)
            s.synchronize()
        outs.append(buf.cpu().numpy().tobytes())
    assert outs[0] == outs[1]


def test_device_attach_matches_host_step_and_reports_launches():
    torch = pytest.importorskip("torch")
    sc = scene.dam_break((16, 16, 16), (3.0, 3.0, 3.0), seed=13)
    cfg, corr = bench_params()
    host, _ = run_gpu(sc, cfg, corr, 3, 0)
    buf = torch.from_numpy(sc.particles.view(np.uint8).copy()).cuda()
    with PBFSolver(sc.n, cfg, corr) as s:
        s.set_stream(torch.cuda.current_stream())
        for _ in range(3):
            s.step(buf, sc.dt, sc.box_min, sc.box_max)
        s.synchronize()
        assert s.kernels_per_step() >= 20
        st = s.stats()
        assert st["steps"] == 3 and st["graphCaptures"] == 1
    dev = buf.cpu().numpy().view(ak.PARTICLE_DTYPE)
    assert dev.tobytes() == host.tobytes()


def test_set_gravity_changes_step_without_recapture():
    sc = scene.dam_break((10, 10, 10), (3.0, 3.0, 3.0), seed=14)
    cfg, corr = bench_params()
    p = sc.particles.copy()
    with PBFSolver(sc.n, cfg, corr, options=ak.OPT_EXACT_MATH) as s:
        s.step_host(p, sc.dt, sc.box_min, sc.box_max)
        s.setGravity((0.0, 0.0, -9.8))
        s.step_host(p, sc.dt, sc.box_min, sc.box_max)
        assert s.stats()["graphCaptures"] == 1
    q = sc.particles.copy()
    cfg1 = PBFConfig()
    P = oracle.make_params(cfg1, corr, sc.dt, sc.box_min, sc.box_max, n=sc.n)
    oracle.step(q, P)
    cfg2 = PBFConfig(gravity=(0.0, 0.0, -9.8))
    P = oracle.make_params(cfg2, corr, sc.dt, sc.box_min, sc.box_max, n=sc.n)
    oracle.step(q, P)
    assert_records_bitexact(p, q)


def test_errors_are_reported():
    sc = scene.dam_break((4, 4, 4), seed=0)
    with PBFSolver(sc.n) as s:
        with pytest.raises(ak.AkuaError) as ei:
            s._lib and ak._abi.check(
                s._lib.akua_pbf_step(s._h, 0.01, ak._abi.vec3((0, 0, 0)), ak._abi.vec3((1, 1, 1))),
                "step")
        assert ei.value.status == ak.AKUA_ERR_NOT_ATTACHED
        with pytest.raises(ak.AkuaError):
            s.step_host(sc.particles.copy(), -1.0, sc.box_min, sc.box_max)
        with pytest.raises(ak.AkuaError):
            s.set_options(0x80)


# --- against the reference's own kernels (fixtures from tests/golden/make_ref_gpu_golden.py) ----

def _ref_cases():
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    from make_ref_gpu_golden import CASES
    return CASES


@pytest.mark.parametrize("opts", [0, ak.OPT_EXACT_MATH], ids=["fast", "exact"])
@pytest.mark.parametrize("name", list(_ref_cases()))
def test_cuda_matches_reference_kernels(name, opts):
    from make_ref_gpu_golden import tagged
    from test_reference_golden import (assert_order_equal, compare_floats, fp32_sensitivity,
                                       golden_floats, have_fixture, load)

    make, cfg, corr, steps, lists = _ref_cases()[name]
    if not have_fixture(name):
        pytest.skip("fixture not generated")
    ref = load(name)
    sc = make()
    g, ge = run_gpu(sc, cfg, corr, steps, opts, particles=tagged(sc))
    assert np.array_equal(g["hash"], ref["hash"])
    assert_order_equal(g, ref)
    if lists:
        assert np.array_equal(ge["cnt"], ref["cnt"])
        flat = np.concatenate([ge["nbr"][i, : ge["cnt"][i]] for i in range(sc.n)])
        assert np.array_equal(flat, ref["nbr_flat"])
    # the fast path adds its own rsqrt-level error on top of the oracle's
    compare_floats(golden_floats(g, name), ref, scale=1.0 if opts else 3.0,
                   extra=fp32_sensitivity(name))
