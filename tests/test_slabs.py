"""Slab decomposition with a halo exchange between neighbouring slabs (akuaengine_gb300/slabs.py).

With the host restatement as each rank's local step (CPU), and with the CUDA solver (GPU): every
particle's record after each decomposed step must equal the single-domain step's, byte for byte,
over many steps, with 2 and 3 slabs, in one process and as two gloo ranks exchanging through
point-to-point messages; and the records each rank sends per step are bounded by its halo, not by
the scene.
"""
import os
import socket

import numpy as np
import pytest

import oracle
from akuaengine_gb300 import scene, slabs

STEPS = 12


def _scene():
    sc = scene.dam_break((120, 6, 6), (1.2, 1.0, 1.0), seed=11)
    # distinct colour[3] per particle: the decomposition borrows that field and must restore it
    sc.particles["color"][:, 3] = np.linspace(0.0, 1.0, sc.n, dtype=np.float32)
    return sc


def _plan(sc, cfg, world):
    return slabs.plan_slabs(sc.box_min, sc.box_max, world, cfg, sc.dt, max_speed=5.0)


def _oracle_step(cfg, corr, sc):
    table = cfg.maxNeighbours * sc.n  # the whole scene's table: hashes as in one domain

    def local_step(rec):
        P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=rec.shape[0],
                               table_size=table)
        oracle.step(rec, P)
    return local_step


def _global_by_gid(sc, cfg, corr, steps):
    """The single-domain oracle step; records indexed by particle id after each step."""
    rec = sc.particles.copy()
    slabs.set_gid(rec, np.arange(sc.n, dtype=np.uint32))
    step = _oracle_step(cfg, corr, sc)
    out = []
    for _ in range(steps):
        step(rec)
        by = np.empty_like(rec)
        by[slabs.gid_of(rec).astype(np.int64)] = rec
        by["color"][:, 3] = sc.particles["color"][:, 3]
        out.append(by)
    return out


def test_plan_ownership_and_held_regions():
    cfg, _ = scene.benchmark_params()
    p = slabs.plan_slabs((0.0, 0, 0), (8.0, 1, 1), 4, cfg, 0.01, max_speed=0.0)
    assert p.halo == pytest.approx(1.1 + 0.5 + 3 * 9.8 * 1e-4)
    x = np.array([0.0, 1.99, 2.0, 7.99, -1.0, 9.0])
    assert list(p.owner(x)) == [0, 0, 1, 3, 0, 3]
    lo, hi = p.held_range(1)
    assert lo == pytest.approx(2.0 - p.halo) and hi == pytest.approx(4.0 + p.halo)
    assert p.held_range(0)[0] == -np.inf and p.held_range(3)[1] == np.inf
    with pytest.raises(ValueError):
        slabs.plan_slabs((0.0, 0, 0), (8.0, 1, 1), 8, cfg, 0.01, max_speed=0.0)


def test_cluster_positions():
    h = np.array([1, 1, 1, 2, 3, 3, 3, 3], np.uint32)
    c = np.array([[0, 0, 0], [0, 0, 1], [0, 0, 0], [5, 5, 5],
                  [0, 0, 0], [10, 0, 0], [1, 0, 0], [10, 1, 0]])
    # hash 3 holds two clusters far apart (cells 0-1 and 10): each numbered on its own
    assert list(slabs.cluster_positions(h, c)) == [0, 1, 2, 0, 0, 0, 1, 1]


@pytest.mark.parametrize("world", [2, 3])
def test_decomposed_steps_equal_global(oracle_mod, world):
    sc = _scene()
    cfg, corr = scene.benchmark_params()
    glob = _global_by_gid(sc, cfg, corr, STEPS)
    plan = _plan(sc, cfg, world)
    ranks = [slabs.SlabRank(sc.particles, plan, r) for r in range(world)]
    step = _oracle_step(cfg, corr, sc)
    for k in range(STEPS):
        slabs.step_all(ranks, step)
        got = slabs.gather_by_gid(ranks, sc.n)
        assert got.tobytes() == glob[k].tobytes(), "step %d differs" % (k + 1)
    # each rank held only its slab and halo, and sent per step at most its halo's records
    held = [r.rec.shape[0] for r in ranks]
    assert max(held) < sc.n
    per_step = [r.sent_records / STEPS for r in ranks]
    x = glob[-1]["position"][:, 0]
    for r, sent in zip(ranks, per_step):
        band = 0
        for nb in (r.rank - 1, r.rank + 1):
            if 0 <= nb < world:
                band += int((plan.held(x, nb) & (plan.owner(x) == r.rank)).sum())
        # O(halo): the trusted records inside the neighbours' halos (the band), not the scene
        assert sent <= 1.5 * band + 50


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        oracle.load()
        sc = _scene()
        cfg, corr = scene.benchmark_params()
        plan = _plan(sc, cfg, world)
        me = slabs.SlabRank(sc.particles, plan, rank)
        step = _oracle_step(cfg, corr, sc)
        for _ in range(4):
            me.step(step, lambda sends: slabs.neighbour_exchange(sends, rank, world))
        rec, gid = me.owned_records()
        q.put((rank, rec.tobytes(), gid.tobytes(), me.sent_records))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_equal_global(oracle_mod):
    import torch.multiprocessing as mp

    from akuaengine_gb300 import PARTICLE_DTYPE

    sc = _scene()
    cfg, corr = scene.benchmark_params()
    glob = _global_by_gid(sc, cfg, corr, 4)[-1]
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    parts = [(np.frombuffer(r, dtype=PARTICLE_DTYPE).copy(), np.frombuffer(g, dtype=np.uint32))
             for _, r, g, _ in res]
    got = slabs.gather_by_gid(parts, sc.n)
    assert got.tobytes() == glob.tobytes()
    assert all(0 < sent / 4 < sc.n / 2 for *_, sent in res)  # records sent per step


# ------------------------------------------------------------------------ device-resident form
def _tensor_oracle_step(cfg, corr, sc):
    from akuaengine_gb300 import PARTICLE_DTYPE

    table = cfg.maxNeighbours * sc.n

    def local_step(buf):  # a CPU tensor's memory, stepped in place by the host restatement
        rec = buf.numpy().view(PARTICLE_DTYPE)
        P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=rec.shape[0],
                               table_size=table)
        oracle.step(rec, P)
    return local_step


def _tensor(sc):
    import torch

    return torch.from_numpy(sc.particles.view(np.uint8).copy())


@pytest.mark.parametrize("world", [2, 3])
def test_tensor_form_equals_global(oracle_mod, world):
    """The torch form (here on CPU tensors, the host restatement stepping each slab) equals the
    single-domain step byte for byte per particle."""
    from akuaengine_gb300 import PARTICLE_DTYPE

    sc = _scene()
    cfg, corr = scene.benchmark_params()
    glob = _global_by_gid(sc, cfg, corr, 6)
    plan = _plan(sc, cfg, world)
    ranks = [slabs.SlabRankDevice(_tensor(sc), plan, r) for r in range(world)]
    step = _tensor_oracle_step(cfg, corr, sc)
    for k in range(6):
        slabs.step_all(ranks, step)
        got = slabs.gather_by_gid_device(ranks, sc.n).numpy().view(PARTICLE_DTYPE).reshape(-1)
        assert got.tobytes() == glob[k].tobytes(), "step %d differs" % (k + 1)


def _tensor_rank_main(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        oracle.load()
        sc = _scene()
        cfg, corr = scene.benchmark_params()
        me = slabs.SlabRankDevice(_tensor(sc), _plan(sc, cfg, world), rank)
        step = _tensor_oracle_step(cfg, corr, sc)
        for _ in range(3):
            me.step(step, lambda s: slabs.neighbour_exchange_device(s, rank, world))
        rec, gid = me.owned_records()
        q.put((rank, rec.numpy().tobytes(), gid.numpy().astype(np.uint32).tobytes()))
    finally:
        dist.destroy_process_group()


def test_tensor_form_two_gloo_ranks(oracle_mod):
    import torch.multiprocessing as mp

    from akuaengine_gb300 import PARTICLE_DTYPE

    sc = _scene()
    cfg, corr = scene.benchmark_params()
    glob = _global_by_gid(sc, cfg, corr, 3)[-1]
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_tensor_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in range(world)]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    parts = [(np.frombuffer(r, dtype=PARTICLE_DTYPE).copy(), np.frombuffer(g, dtype=np.uint32))
             for _, r, g in res]
    assert slabs.gather_by_gid(parts, sc.n).tobytes() == glob.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("world", [2, 3])
def test_cuda_solver_slabs_equal_global(cuda_lib, world):
    """Records resident on the GPU, each slab stepped by the CUDA solver (exact math, the whole
    scene's table size), the ranks one after another on one GPU exchanging halos: every particle
    equals the single-domain CUDA step's, byte for byte, over six steps."""
    import torch

    import akuaengine_gb300 as ak
    from akuaengine_gb300 import PARTICLE_DTYPE, PBFSolver

    sc = _scene()
    cfg, corr = scene.benchmark_params()
    table = cfg.maxNeighbours * sc.n

    def local_step(buf):
        with PBFSolver(buf.numel() // 108, cfg, corr, options=ak.OPT_EXACT_MATH,
                       table_size=table) as s:
            s.step(buf, sc.dt, sc.box_min, sc.box_max)
            s.synchronize()

    glob = sc.particles.copy()
    slabs.set_gid(glob, np.arange(sc.n, dtype=np.uint32))
    gbuf = torch.from_numpy(glob.view(np.uint8).copy()).cuda()
    ranks = [slabs.SlabRankDevice(_tensor(sc).cuda(), _plan(sc, cfg, world), r)
             for r in range(world)]
    with PBFSolver(sc.n, cfg, corr, options=ak.OPT_EXACT_MATH) as s:
        for k in range(6):
            s.step(gbuf, sc.dt, sc.box_min, sc.box_max)
            s.synchronize()
            slabs.step_all(ranks, local_step)
            g = gbuf.cpu().numpy().view(PARTICLE_DTYPE).copy()
            want = np.empty_like(g)
            want[slabs.gid_of(g).astype(np.int64)] = g
            want["color"][:, 3] = sc.particles["color"][:, 3]
            got = slabs.gather_by_gid_device(ranks, sc.n).cpu().numpy().view(PARTICLE_DTYPE)
            assert got.reshape(-1).tobytes() == want.tobytes(), "step %d differs" % (k + 1)
