"""Slab decomposition with a wide halo (akuaengine_gb300/slabs.py), with the host restatement as
each rank's local step: every particle's record after a decomposed step must equal the
single-domain step's, byte for byte, over several steps; run in one process and as two gloo
ranks exchanging their owned records."""
import os
import socket

import numpy as np
import pytest

import oracle
from akuaengine_gb300 import scene, slabs


def _scene():
    return scene.dam_break((120, 6, 6), (1.2, 1.0, 1.0), seed=11)


def _stepper(cfg, corr, sc, n_global):
    def local_step(rec):
        P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=n_global)
        oracle.step(rec, P)
    return local_step


def test_halo_width_and_ownership():
    s = slabs.Slabs(4, 0.0, 8.0, 1.1)
    x = np.array([0.0, 1.99, 2.0, 7.99, -1.0, 9.0])
    assert list(s.owner(x)) == [0, 0, 1, 3, 0, 3]
    m = s.local_mask(np.array([0.5, 2.5, 3.05, 3.2, 5.0]), 1)  # slab [2, 4) plus 1.1 either side
    assert list(m) == [False, True, True, True, True]
    m = s.local_mask(np.array([0.85, 0.95, 5.05, 5.15]), 1)
    assert list(m) == [False, True, True, False]
    assert slabs.halo_width(0.1, 4, 0.0, 0.01, 0.0) == pytest.approx(1.1)


@pytest.mark.parametrize("world", [2, 3])
def test_decomposed_steps_equal_global(oracle_mod, world):
    sc = _scene()
    cfg, corr = scene.benchmark_params()
    step = _stepper(cfg, corr, sc, sc.n)
    glob = sc.particles.copy()
    dec = sc.particles.copy()
    for _ in range(3):
        step(glob)
        dec = slabs.decomposed_step(dec, world, cfg, sc.dt, step)
        assert dec.tobytes() == glob.tobytes()
    # the slabs were real: each rank stepped fewer than all particles
    sl = slabs.make_slabs(slabs.tag(dec), world, cfg, sc.dt)
    x = dec["position"][:, 0]
    assert all(sl.local_mask(x, r).sum() < sc.n for r in range(world))


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
        step = _stepper(cfg, corr, sc, sc.n)

        def exchange(mine):
            out = [None] * world
            dist.all_gather_object(out, mine)
            return out

        rec = sc.particles.copy()
        for _ in range(2):
            rec = slabs.decomposed_step(rec, world, cfg, sc.dt, step, exchange=exchange, rank=rank)
        q.put((rank, rec.tobytes()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_equal_global(oracle_mod):
    import torch.multiprocessing as mp

    sc = _scene()
    cfg, corr = scene.benchmark_params()
    glob = sc.particles.copy()
    step = _stepper(cfg, corr, sc, sc.n)
    for _ in range(2):
        step(glob)
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
    for _, b in res:
        assert b == glob.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("world", [2, 3])
def test_decomposed_steps_on_the_cuda_solver_equal_global(cuda_lib, world):
    """Each slab stepped by the CUDA solver (exact math, the whole scene's table size), one slab
    after another on one GPU: the reassembled records equal the single-domain CUDA step's, byte
    for byte, over three steps."""
    import akuaengine_gb300 as ak
    from akuaengine_gb300 import PBFSolver

    sc = _scene()
    cfg, corr = scene.benchmark_params()
    table = cfg.maxNeighbours * sc.n

    def local_step(rec):
        with PBFSolver(rec.shape[0], cfg, corr, options=ak.OPT_EXACT_MATH, table_size=table) as s:
            s.step_host(rec, sc.dt, sc.box_min, sc.box_max)

    glob = sc.particles.copy()
    dec = sc.particles.copy()
    with PBFSolver(sc.n, cfg, corr, options=ak.OPT_EXACT_MATH) as s:
        for _ in range(3):
            s.step_host(glob, sc.dt, sc.box_min, sc.box_max)
            dec = slabs.decomposed_step(dec, world, cfg, sc.dt, local_step)
            assert dec.tobytes() == glob.tobytes()


# ------------------------------------------------------------------------ device-resident form
def _torch_records(sc):
    import torch

    return torch.from_numpy(sc.particles.view(np.uint8).copy()).view(-1)


def _oracle_tensor_step(cfg, corr, sc, n_global):
    def local_step(buf):  # a CPU tensor's memory, stepped in place by the host restatement
        rec = buf.numpy().view(ak_dtype())
        P = oracle.make_params(cfg, corr, sc.dt, sc.box_min, sc.box_max, n=n_global)
        oracle.step(rec, P)
    return local_step


def ak_dtype():
    from akuaengine_gb300 import PARTICLE_DTYPE

    return PARTICLE_DTYPE


@pytest.mark.parametrize("world", [2, 3])
def test_tensor_decomposition_equals_global(oracle_mod, world):
    """The torch form of the decomposition (here on CPU tensors, the host restatement stepping
    each slab) reproduces the single-domain step byte for byte."""
    sc = _scene()
    cfg, corr = scene.benchmark_params()
    step = _stepper(cfg, corr, sc, sc.n)
    glob = sc.particles.copy()
    dec = _torch_records(sc)
    local = _oracle_tensor_step(cfg, corr, sc, sc.n)
    for _ in range(3):
        step(glob)
        dec = slabs.decomposed_step_device(dec, world, cfg, sc.dt, local)
        assert dec.numpy().tobytes() == glob.tobytes()


def _tensor_rank_main(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        oracle.load()
        sc = _scene()
        cfg, corr = scene.benchmark_params()
        local = _oracle_tensor_step(cfg, corr, sc, sc.n)
        rec = _torch_records(sc)
        for _ in range(2):
            rec = slabs.decomposed_step_device(rec, world, cfg, sc.dt, local,
                                               exchange=slabs.all_gather_records, rank=rank)
        q.put((rank, rec.numpy().tobytes()))
    finally:
        dist.destroy_process_group()


def test_tensor_decomposition_two_gloo_ranks(oracle_mod):
    """Two ranks, each stepping its slab and exchanging owned records with all_gather_records
    (variable sizes, padded), end with the single-domain records."""
    import torch.multiprocessing as mp

    sc = _scene()
    cfg, corr = scene.benchmark_params()
    glob = sc.particles.copy()
    step = _stepper(cfg, corr, sc, sc.n)
    for _ in range(2):
        step(glob)
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
    for _, b in res:
        assert b == glob.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("world", [2, 3])
def test_device_decomposition_on_the_cuda_solver_equals_global(cuda_lib, world):
    """Records resident on the GPU, slabs selected and reassembled there, each stepped by the CUDA
    solver (exact math, the whole scene's table size): equal to the single-domain CUDA step."""
    import akuaengine_gb300 as ak
    from akuaengine_gb300 import PBFSolver

    sc = _scene()
    cfg, corr = scene.benchmark_params()
    table = cfg.maxNeighbours * sc.n

    def local_step(buf):
        with PBFSolver(buf.numel() // 108, cfg, corr, options=ak.OPT_EXACT_MATH,
                       table_size=table) as s:
            s.step(buf, sc.dt, sc.box_min, sc.box_max)
            s.synchronize()

    glob = _torch_records(sc).cuda()
    dec = glob.clone()
    with PBFSolver(sc.n, cfg, corr, options=ak.OPT_EXACT_MATH) as s:
        for _ in range(3):
            s.step(glob, sc.dt, sc.box_min, sc.box_max)
            s.synchronize()
            dec = slabs.decomposed_step_device(dec, world, cfg, sc.dt, local_step)
            assert dec.cpu().numpy().tobytes() == glob.cpu().numpy().tobytes()
