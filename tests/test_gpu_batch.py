"""Batches of independent scenes (akua_pbf_create_batch): every scene of a batch step must come out
byte-identical to the same scene stepped alone by its own solver."""
import dataclasses

import numpy as np
import pytest

import akuaengine_gb300 as ak
from akuaengine_gb300 import BatchSolver, PBFSolver, scene


def test_batched_dam_breaks_generator():
    b = scene.batched_dam_breaks(count=16, seed=5)
    ns = np.array([d["numParticles"] for d in b.scenes])
    assert len(b.scenes) == 16 and b.n == ns.sum()
    assert ns.min() >= 1000 and ns.max() <= 80000
    g = np.array([-d["gravity"][1] for d in b.scenes])
    assert (g >= 5).all() and (g <= 15).all()
    for k, d in enumerate(b.scenes):
        sc = b.scene(k)
        lo, hi = sc.particles["position"].min(0), sc.particles["position"].max(0)
        assert (lo > 0).all() and (hi < np.array(d["box_max"])).all()
    assert b.first[3] == ns[:3].sum()


def _alone(b, k, cfg, corr, steps, opts):
    sc = b.scene(k)
    c = dataclasses.replace(cfg, gravity=sc.meta["gravity"])
    s = PBFSolver(sc.n, c, corr, options=opts)
    p = sc.particles.copy()
    for _ in range(steps):
        s.step_host(p, sc.dt, sc.box_min, sc.box_max)
    s.close()
    return p


@pytest.mark.gpu
@pytest.mark.parametrize("opts", [ak.OPT_EXACT_MATH, 0])
def test_batch_matches_scenes_stepped_alone(cuda_lib, opts):
    import torch

    b = scene.batched_dam_breaks(count=7, n_min=300, n_max=9000, seed=3)
    cfg, corr = scene.benchmark_params()
    steps = 4
    bs = BatchSolver(b.scenes, cfg, corr, options=opts)
    buf = torch.from_numpy(b.particles.view(np.uint8).copy()).cuda()
    for _ in range(steps):
        bs.step(buf, b.dt)
    got = buf.cpu().numpy().view(ak.PARTICLE_DTYPE)
    launches = bs.kernels_per_step()
    bs.close()
    for k, d in enumerate(b.scenes):
        f, n = b.first[k], d["numParticles"]
        want = _alone(b, k, cfg, corr, steps, opts)
        assert got[f:f + n].tobytes() == want.tobytes(), "scene %d" % k
    assert launches > 30


@pytest.mark.gpu
def test_batch_set_scene_changes_only_that_scene(cuda_lib):
    import torch

    b = scene.batched_dam_breaks(count=3, n_min=500, n_max=2000, seed=9)
    cfg, corr = scene.benchmark_params()
    bs = BatchSolver(b.scenes, cfg, corr)
    d = dict(b.scenes[1])
    d["gravity"] = (0.0, -20.0, 0.0)
    bs.set_scene(1, d)
    buf = torch.from_numpy(b.particles.view(np.uint8).copy()).cuda()
    bs.step(buf, b.dt)
    got = buf.cpu().numpy().view(ak.PARTICLE_DTYPE)
    bs.close()
    b2 = scene.SceneBatch(b.particles, [b.scenes[0], d, b.scenes[2]], b.dt, b.name)
    for k in range(3):
        f, n = b2.first[k], b2.scenes[k]["numParticles"]
        assert got[f:f + n].tobytes() == _alone(b2, k, cfg, corr, 1, 0).tobytes()


@pytest.mark.gpu
def test_batch_rejects_single_scene_calls(cuda_lib):
    b = scene.batched_dam_breaks(count=2, n_min=500, n_max=1000, seed=1)
    cfg, corr = scene.benchmark_params()
    bs = BatchSolver(b.scenes, cfg, corr)
    with pytest.raises(ak.AkuaError):
        bs.step_host(b.particles.copy(), b.dt, (0, 0, 0), (1, 1, 1))
    with pytest.raises(ak.AkuaError):
        bs.setGravity((0, -1, 0))
    with pytest.raises(ak.AkuaError):
        bs.set_table_size(1000)
    bs.close()


def _alone_with(b, k, cfg, corr, steps, opts, setup):
    sc = b.scene(k)
    c = dataclasses.replace(cfg, gravity=sc.meta["gravity"])
    s = PBFSolver(sc.n, c, corr, options=opts)
    setup(s)
    p = sc.particles.copy()
    for _ in range(steps):
        s.step_host(p, sc.dt, sc.box_min, sc.box_max)
    s.close()
    return p


def _batch_with(b, cfg, corr, steps, opts, setup):
    import torch

    bs = BatchSolver(b.scenes, cfg, corr, options=opts)
    setup(bs)
    buf = torch.from_numpy(b.particles.view(np.uint8).copy()).cuda()
    for _ in range(steps):
        bs.step(buf, b.dt)
    got = buf.cpu().numpy().view(ak.PARTICLE_DTYPE)
    bs.close()
    return got


@pytest.mark.gpu
def test_batch_with_obstacles_equals_scenes_alone(cuda_lib):
    """Obstacles set on a batch apply to every scene: each comes out as if stepped alone with them."""
    b = scene.batched_dam_breaks(count=4, n_min=800, n_max=6000, seed=11)
    cfg, corr = scene.benchmark_params()
    shapes = [{"type": "sphere", "a": (0.25, 0.05, 0.25), "b": (0.0, 0.0, 0.0), "radius": 0.08},
              {"type": "plane", "a": (0.0, 0.02, 0.0), "b": (0.0, 1.0, 0.0), "radius": 0.0}]
    setup = lambda s: s.set_sdf_shapes(shapes)
    steps = 5
    got = _batch_with(b, cfg, corr, steps, ak.OPT_EXACT_MATH, setup)
    for k, d in enumerate(b.scenes):
        f, n = b.first[k], d["numParticles"]
        want = _alone_with(b, k, cfg, corr, steps, ak.OPT_EXACT_MATH, setup)
        assert got[f:f + n].tobytes() == want.tobytes(), "scene %d" % k


@pytest.mark.gpu
def test_batch_with_warm_start_equals_scenes_alone(cuda_lib):
    """The learned warm start on a batch: every quantity the network sees is per particle, so each
    scene comes out as if stepped alone with the same network."""
    from akuaengine_gb300.warm_start import LambdaNet

    net = LambdaNet(seed=3)
    net.set_normalization(np.zeros(8, np.float32), np.ones(8, np.float32), 1e-6, blend=0.5)
    b = scene.batched_dam_breaks(count=3, n_min=800, n_max=5000, seed=12)
    cfg, corr = scene.benchmark_params()
    cfg = dataclasses.replace(cfg, solverIterations=2)

    def setup(s):
        s.set_lambda_tracking(True)
        s.set_warm_start(net)

    steps = 4
    got = _batch_with(b, cfg, corr, steps, 0, setup)
    for k, d in enumerate(b.scenes):
        f, n = b.first[k], d["numParticles"]
        want = _alone_with(b, k, cfg, corr, steps, 0, setup)
        assert got[f:f + n].tobytes() == want.tobytes(), "scene %d" % k
    net.close()
